"""The GoldenC drop-in as a program uses it: a GoldenC-style C driver
(tests/goldnc_driver.c: globals f, v, gDelta; g = A(phantom); MumfordShah)
compiled against libat_engine.so and run, compared with the FP64 oracle of
GoldenC's solver and projector (rel-L2 <= 1e-4)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_goldnc_program_through_the_library(engine, oracle, tmp_path):
    lib_dir = os.path.join(ROOT, "medimage_gb300")
    exe = tmp_path / "driver"
    subprocess.run(["gcc", "-O2", "-std=c99", f"-I{ROOT}/include", os.path.join(ROOT, "tests", "goldnc_driver.c"),
                    f"-L{lib_dir}", "-lat_engine", f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(exe)], check=True)
    ph = engine.phantom.ellipse_phantom(512, seed=61).astype(np.float64)
    (tmp_path / "ph.bin").write_bytes(ph.tobytes())
    subprocess.run([str(exe), str(tmp_path / "ph.bin"), str(tmp_path / "f.bin"), str(tmp_path / "v.bin"), "2"],
                   check=True, timeout=300)
    f = np.fromfile(tmp_path / "f.bin", dtype=np.float64).reshape(512, 512)
    v = np.fromfile(tmp_path / "v.bin", dtype=np.float64).reshape(512, 512)
    g = oracle.gc_A(ph)
    fo, vo, _ = oracle.solve(None, g, 1000.0, 0.002, 1e-4, 2, 10, 10)
    assert np.linalg.norm(f - fo) <= 1e-4 * np.linalg.norm(fo)
    assert np.linalg.norm(v - vo) <= 1e-4 * np.linalg.norm(vo)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_goldnc_text_files_through_the_library(engine, oracle, tmp_path):
    """GoldenC's own input and output files (origin/GoldenC/src/main.c:51-79):
    phantom.dat as whitespace-separated text read with "%lf", I_result.txt and
    E_result.txt written "%f " per value with a newline per row, by the C
    driver linked against the engine.  Values agree with the FP64 oracle to
    rel-L2 1e-4 (beyond the six-decimal quantisation of the format), and the
    files parse as the reference's layout: 512 lines of 512 fields."""
    from medimage_gb300 import io

    lib_dir = os.path.join(ROOT, "medimage_gb300")
    exe = tmp_path / "driver"
    subprocess.run(["gcc", "-O2", "-std=c99", f"-I{ROOT}/include", os.path.join(ROOT, "tests", "goldnc_driver.c"),
                    f"-L{lib_dir}", "-lat_engine", f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(exe)], check=True)
    ph = engine.phantom.ellipse_phantom(512, seed=62).astype(np.float64)
    io.write_goldnc_image(str(tmp_path / "phantom.dat"), ph)
    ph_text = io.read_goldnc_image(str(tmp_path / "phantom.dat"))  # what the program reads
    subprocess.run([str(exe), "--text", str(tmp_path), "2"], check=True, timeout=300)
    for name in ("I_result.txt", "E_result.txt"):
        lines = (tmp_path / name).read_text().split("\n")
        assert len(lines) == 513 and lines[-1] == ""
        assert all(len(ln.split()) == 512 and ln.endswith(" ") for ln in lines[:-1])
    f = io.read_goldnc_image(str(tmp_path / "I_result.txt"))
    v = io.read_goldnc_image(str(tmp_path / "E_result.txt"))
    fo, vo, _ = oracle.solve(None, oracle.gc_A(ph_text), 1000.0, 0.002, 1e-4, 2, 10, 10)
    assert np.linalg.norm(f - fo) <= 1e-4 * np.linalg.norm(fo)
    assert np.linalg.norm(v - vo) <= 1e-4 * np.linalg.norm(vo)

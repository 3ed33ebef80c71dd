"""C-ABI checks that need no GPU: the engine library loads, exports every
function include/*.h declares, rejects bad arguments before touching the
device, and links as a drop-in for GoldenC's proj.c."""
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
REF_ROOT = os.environ.get("MEDIMAGE_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
REF_GOLDNC = os.path.join(REF_ROOT, "origin", "GoldenC", "src")


def declared_functions():
    names = set()
    for fn in sorted(os.listdir(INCLUDE)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof", "defined"):
                names.add(name)
    return names


def test_headers_declare_expected_entry_points():
    names = declared_functions()
    for n in ("A", "AStar", "minimize_in_IMAGE_variable", "minimize_in_EDGE_variable", "medfilt2", "MumfordShah",
              "at_plan_create_fan", "at_forward", "at_back", "at_solver_run", "at_reconstruct_host"):
        assert n in names


def test_library_exports_every_declared_symbol(engine):
    L = engine.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(engine.engine.SIGNATURES) | {"at_solver_set_fv_host"}


def test_bad_geometry_rejected_without_device(engine):
    g = engine.FanGeometry.covering(64, 1.0, 90, 128)
    g.ndets = 127  # must be even
    with pytest.raises(engine.AtError) as ei:
        engine.Plan.fan(g)
    assert ei.value.code == -1
    assert "ndets" in engine.lib().at_last_error().decode()
    g = engine.FanGeometry.covering(64, 1.0, 90, 128)
    g.sod_mm = 10.0
    with pytest.raises(engine.AtError):
        engine.Plan.fan(g)


def test_quality_rejects_mismatched_images_without_device(engine):
    with pytest.raises(ValueError):
        engine.quality(np.zeros((16, 16), np.float32), np.zeros((16, 17), np.float32))
    with pytest.raises(ValueError):
        engine.quality(np.zeros(16, np.float32), np.zeros(16, np.float32))


def test_bad_ray_table_rejected_without_device(engine):
    g = engine.RayGeometry.msbeam_parallel(64, 8, 96)
    bad = g.endpoints.copy()
    bad[5, 2] = np.nan
    with pytest.raises(engine.AtError) as ei:
        engine.Plan.rays(engine.RayGeometry(64, 1.0, 8, 96, bad))
    assert ei.value.code == -1 and "finite" in str(ei.value)
    bad = g.endpoints.copy()
    bad[7, 2:] = bad[7, :2]
    with pytest.raises(engine.AtError) as ei:
        engine.Plan.rays(engine.RayGeometry(64, 1.0, 8, 96, bad))
    assert "coincide" in str(ei.value)
    with pytest.raises(engine.AtError):
        engine.Plan.rays(engine.RayGeometry(4, 1.0, 8, 96, g.endpoints))


def test_null_arguments_rejected(engine):
    L = engine.lib()
    assert L.at_plan_get_stats(None, None) == -1
    assert L.at_solver_run(None, None) == -1
    assert L.at_solver_launches_per_outer(None, None) == -1


def test_goldnc_globals_are_weak_references():
    out = subprocess.run(["nm", "-D", os.path.join(ROOT, "medimage_gb300", "libat_engine.so")],
                         capture_output=True, text=True, check=True).stdout
    for g in ("f", "v", "gDelta"):
        assert re.search(rf"^\s+w {g}$", out, flags=re.M), g


@pytest.mark.skipif(not os.path.isdir(REF_GOLDNC) or shutil.which("gcc") is None,
                    reason="reference GoldenC sources not present on this host")
def test_reference_main_links_against_engine(tmp_path):
    """GoldenC's own main.c, unchanged, links with libat_engine.so in place of
    proj.c (A and AStar resolve to the engine)."""
    lib_dir = os.path.join(ROOT, "medimage_gb300")
    exe = tmp_path / "goldnc_gpu"
    subprocess.run(["gcc", "-O2", "-std=c99", "-w", f"-I{REF_GOLDNC}", os.path.join(REF_GOLDNC, "main.c"),
                    f"-L{lib_dir}", "-lat_engine", f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(exe)], check=True)
    syms = subprocess.run(["nm", str(exe)], capture_output=True, text=True, check=True).stdout
    assert re.search(r"^\s+U A$", syms, flags=re.M) and re.search(r"^\s+U AStar$", syms, flags=re.M)


def test_driver_program_links(tmp_path):
    """The GoldenC-style driver used by the GPU drop-in test compiles and links."""
    lib_dir = os.path.join(ROOT, "medimage_gb300")
    exe = tmp_path / "driver"
    subprocess.run(["gcc", "-O2", "-std=c99", f"-I{INCLUDE}", os.path.join(ROOT, "tests", "goldnc_driver.c"),
                    f"-L{lib_dir}", "-lat_engine", f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(exe)], check=True)
    assert exe.exists()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_struct_layouts_match_the_header(tmp_path):
    """Every struct the Python bindings mirror with ctypes has the size and
    field offsets the C header gives it (a C program compiled with gcc prints
    them), so no field can drift between include/at_engine.h and engine.py."""
    from medimage_gb300 import engine as E

    structs = {
        "at_fan_geometry": E._FanGeom,
        "at_cone_geometry": E._ConeGeom,
        "at_rowaction_params": E._RowActionParams,
        "at_params": E._Params,
        "at_plan_stats": E._PlanStats,
        "at_server_config": E._ServerConfig,
        "at_server_stats": E._ServerStats,
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "at_engine.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {(a, b): int(c) for a, b, c in (line.split() for line in out if line.strip())}
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)

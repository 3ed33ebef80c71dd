"""Reference file layouts (medimage_gb300/io.py) and host-side helpers."""
import numpy as np
import pytest

from medimage_gb300 import io, phantom
from medimage_gb300.engine import FanGeometry


def test_goldnc_text_round_trip(tmp_path):
    img = np.random.default_rng(0).random((512, 512)) * 0.02
    p = tmp_path / "I_result.txt"
    io.write_goldnc_image(str(p), img)
    first = p.read_text().split("\n")[0].split(" ")
    assert first[0] == "%f" % img[0, 0] and len(first) == 513  # "%f " per value, then newline
    back = io.read_goldnc_image(str(p))
    np.testing.assert_allclose(back, img, atol=5e-7)  # six decimals, as GoldenC writes


def test_goldnc_phantom_reader_accepts_any_whitespace(tmp_path):
    vals = np.arange(512 * 512, dtype=np.float64) / 7.0
    p = tmp_path / "phantom.dat"
    p.write_text("\n".join(" \t".join(repr(float(v)) for v in vals[i:i + 1000]) for i in range(0, vals.size, 1000)))
    np.testing.assert_array_equal(io.read_goldnc_image(str(p)), vals.reshape(512, 512))


def test_view_table_and_uniform_angles(tmp_path):
    p = tmp_path / "table"
    ang = 12.5 + 0.5 * np.arange(720)
    io.write_view_table(str(p), np.full(720, 1000.0), ang)
    pos, a = io.read_view_table(str(p))
    np.testing.assert_array_equal(a, ang)
    assert np.all(pos == 1.0)
    v0, step = io.uniform_view_angles(a)
    assert v0 == 12.5 and abs(step - 0.5) < 1e-12
    with pytest.raises(ValueError):
        io.uniform_view_angles(np.array([0.0, 1.0, 3.0]))


def test_text_sinogram_and_dr_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    s = rng.random((36, 64))
    p = tmp_path / "sino.txt"
    io.write_text_sinogram(str(p), s)
    np.testing.assert_array_equal(io.read_text_sinogram(str(p), 36, 64), s)
    counts = rng.integers(0, 65535, size=(4, 6, 5), dtype=np.uint16)
    d = tmp_path / "x.dr"
    io.write_dr(str(d), counts)
    raw = d.read_bytes()
    assert len(raw) == 1024 + counts.size * 2 and raw[:1024] == bytes(1024)
    np.testing.assert_array_equal(io.read_dr(str(d), 4, 6, 5), counts)
    li = io.counts_to_line_integrals(np.array([0, 1, 5000, 10000]), 1e4)
    np.testing.assert_allclose(li, [np.log(1e4), np.log(1e4), np.log(2.0), 0.0], rtol=1e-6)


def test_phantom_and_noise_are_seeded():
    a = phantom.ellipse_phantom(128, seed=3, n_random=5)
    b = phantom.ellipse_phantom(128, seed=3, n_random=5)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0 and 0.015 < a.max() <= 0.0225
    clean = np.full((10, 10), 2.0)
    s1 = phantom.poisson_sinogram(clean, 1e4, 9)
    np.testing.assert_array_equal(s1, phantom.poisson_sinogram(clean, 1e4, 9))
    assert abs(float(s1.mean()) - 2.0) < 0.05


def test_fan_geometry_covers_image():
    g = FanGeometry.covering(512, 0.75, 720, 888)
    half_fan = np.radians(g.det_pitch_deg * g.ndets / 2)
    r = 512 * 0.75 * np.sqrt(2) / 2
    assert abs(np.sin(half_fan) * g.sod_mm - r) < 1e-9
    assert g.view_step_deg == 0.5 and g.off_center == 0.5

"""The msbeam/CPU_OpenMP restatement (the timed OpenMP CPU comparator) and the
ray-table geometry that carries msbeam's parallel beam to the GPU engine.

The restatement is pinned to golden vectors made from the reference's own
sources (tests/golden/make_golden.py: the program's phantom, wray traversals,
A, and f and v after its 10 sweeps with one thread, where it is
deterministic) and, where the reference tree is built, to those sources
directly.
"""
import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from medimage_gb300.engine import RayGeometry

HERE = os.path.dirname(os.path.abspath(__file__))


def digest(x):
    return hashlib.sha1(np.ascontiguousarray(x, np.float32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def gms():
    return np.load(os.path.join(HERE, "golden", "msbeam.npz"))


def wray(oracle, k, r):
    line = np.zeros(2048, np.int32)
    w = np.zeros(2048, np.float32)
    n = oracle.lib().or_ms_wray(k, r, line, w)
    return line[:n].copy(), w[:n].copy()


def test_phantom_golden(oracle, gms):
    assert digest(oracle.ms_phantom()) == str(gms["phantom_digest"])


def test_wray_golden(oracle, gms):
    off = gms["wray_off"]
    for i, (k, r) in enumerate(gms["wray_rays"]):
        line, w = wray(oracle, int(k), int(r))
        np.testing.assert_array_equal(line, gms["wray_ind"][off[i]:off[i + 1]])
        np.testing.assert_array_equal(w.view(np.uint32), gms["wray_w"][off[i]:off[i + 1]].view(np.uint32))


def test_forward_golden(oracle, gms):
    g = oracle.ms_A(oracle.ms_phantom())
    np.testing.assert_array_equal(g[::15], gms["A_rows"])
    assert digest(g) == str(gms["A_digest"])


def test_solve_single_thread_golden(oracle, gms):
    """10 sweeps with one thread: bit-identical to the reference program."""
    g = oracle.ms_A(oracle.ms_phantom())
    f, v = oracle.ms_solve(g, 10, 1)
    np.testing.assert_array_equal(f[216:296, 216:296], gms["f_crop"])
    np.testing.assert_array_equal(v[216:296, 216:296], gms["v_crop"])
    assert digest(f) == str(gms["f_digest"]) and digest(v) == str(gms["v_digest"])


ref_only = pytest.mark.skipif(
    not __import__("oracle.pyoracle", fromlist=["Ref"]).Ref.available(),
    reason="the reference's sources are not built on this host (oracle/_ref)")


@ref_only
def test_wray_equals_reference_everywhere(oracle):
    ref = oracle.Ref()
    ref.ms.wray.argtypes = [C.c_int, C.c_int, oracle._ip, oracle._fp32, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    for k in range(0, 180, 1):
        for r in range(k % 5, 768, 5):
            line, w = wray(oracle, k, r)
            l2 = np.zeros(2048, np.int32)
            w2 = np.zeros(2048, np.float32)
            nb, sn = C.c_int(), C.c_float()
            ref.ms.wray(k, r, l2, w2, C.byref(nb), C.byref(sn))
            assert nb.value == line.size
            np.testing.assert_array_equal(line, l2[: nb.value])
            np.testing.assert_array_equal(w.view(np.uint32), w2[: nb.value].view(np.uint32))


def test_multithreaded_solve_runs_racy_sweeps(oracle):
    """With several threads each thread sweeps its own block of views and the
    updates race on f and v as the reference's do (main.c:377), so the order
    and the result differ from one thread; both stay in the bounds the
    updates clamp to and both approach the phantom."""
    ph = oracle.ms_phantom()
    g = oracle.ms_A(ph)
    for nt in (1, 4):
        f, v = oracle.ms_solve(g, 2, nt)
        assert np.all(np.isfinite(f)) and f.min() >= 0.0
        assert v.min() >= 0.0 and v.max() <= 1.0
        assert 10 * np.log10(ph.max() ** 2 / np.mean((f - ph) ** 2)) > 25.0


def test_ray_table_is_msbeam_geometry(oracle):
    """msbeam's parallel beam as a ray table: the exact-Siddon traversal of
    each ray visits msbeam's pixels (rays that miss the grid miss it in both;
    msbeam drops the ray's last boundary
    pixel, gives the entry pixel a full step and accumulates its crossing
    parameter in FP32, so weights agree to that precision), and projections
    of msbeam's phantom agree to 2e-3."""
    geom = RayGeometry.msbeam_parallel()
    fan = oracle.fan_from_engine(geom)
    same = total = 0
    for k in range(0, 180, 7):
        for r in range(0, 768, 11):
            line, w = wray(oracle, k, r)
            ind, wgt, _ = oracle.fan_trace(fan, k, r)
            ind = ind[(ind >= 0) & (ind < 512 * 512)]
            total += 1
            m = line.size
            if (m == 0 and ind.size == 0) or (m and ind.size in (m, m + 1) and np.array_equal(ind[:m], line)):
                same += 1
    assert same >= 0.95 * total, (same, total)
    ph = oracle.ms_phantom()
    a = oracle.fan_A(fan, ph.astype(np.float64))
    b = oracle.ms_A(ph)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-3


def test_fan_view_table_equals_uniform_fan(oracle):
    """A fan given by an evenly spaced view table traces exactly the rays of
    the parametric fan geometry."""
    from medimage_gb300.engine import FanGeometry

    g = FanGeometry.covering(96, 1.0, 30, 64)
    rt = RayGeometry.fan_from_view_table(g.n, g.pixel_mm, g.ndets, [g.view0_deg + k * g.view_step_deg
                                                                     for k in range(g.nviews)],
                                         g.sod_mm, g.sdd_mm, g.det_pitch_deg, g.off_center)
    a = oracle.fan_from_engine(g)
    b = oracle.fan_from_engine(rt)
    for v in range(g.nviews):
        for d in range(0, g.ndets, 3):
            assert oracle.fan_endpoints(a, v, d) == oracle.fan_endpoints(b, v, d)
    img = np.random.default_rng(1).random((96, 96))
    np.testing.assert_array_equal(oracle.fan_A(a, img), oracle.fan_A(b, img))


def test_package_phantom_is_msbeam_phantom(gms):
    from medimage_gb300.phantom import msbeam_phantom

    assert digest(msbeam_phantom()) == str(gms["phantom_digest"])

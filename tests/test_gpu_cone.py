"""GPU parity of the 3D cone-beam projectors and the volume solver.

Bars: the traversal (voxel indices and FP32 weight bits) equals the
reference tracer's -- directly against golden traversals made from
industry3d's tracing.cpp, including the C4 geometry -- and the FP32-exact
oracle's; forward and back projection rel-L2 <= 1e-5 against FP64; repeated
projections bitwise equal; two outer solver iterations f and v rel-L2 <= 1e-4
and PSNR within 0.05 dB of the FP64 oracle, with the same exit branches.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import CONE_GEOMS  # noqa: E402


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def small(engine):
    return engine.ConeGeometry(48, 48, 40, 0.5, 72, 36, 44, 0.9, 60.0, 110.0)


def volume(g, seed=0):
    rng = np.random.default_rng(seed)
    z, x, y = np.mgrid[:g.nz, :g.nx, :g.ny].astype(np.float64)
    c = (g.nx - 1) / 2.0
    vol = (((x - c) ** 2 + (y - c) ** 2 + 1.3 * (z - (g.nz - 1) / 2.0) ** 2) < (0.4 * g.nx) ** 2) * 0.02
    for _ in range(6):
        cx, cy, cz = rng.uniform(0.3, 0.7, 3) * np.array([g.nx, g.ny, g.nz])
        r = rng.uniform(2, 5)
        vol += (((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) < r * r) * rng.uniform(-0.008, 0.008)
    return np.clip(vol, 0, None).astype(np.float32)


@pytest.fixture(scope="module")
def splan(engine):
    g = small(engine)
    return g, engine.Plan.cone(g)


@pytest.mark.parametrize("name", ["small", "c4"])
def test_cone_traversal_equals_reference_golden(engine, name):
    gold = np.load(os.path.join(HERE, "golden", "cone.npz"))
    g = CONE_GEOMS[name]
    p = engine.Plan.cone(g)
    off = gold[f"{name}_off"]
    for i, (v, r, c) in enumerate(gold[f"{name}_rays"]):
        pix, w = p.trace_ray(int(v), int(r) * g.ndy + int(c))
        np.testing.assert_array_equal(pix.astype(np.int64), gold[f"{name}_ind"][off[i]:off[i + 1]])
        np.testing.assert_array_equal(w.view(np.uint32), gold[f"{name}_w"][off[i]:off[i + 1]].view(np.uint32))


def test_cone_plan_counts_and_traversal(engine, oracle, splan):
    g, p = splan
    assert p.stats["kind"] == engine.engine.AT_GEOM_CONE and p.stats["nz"] == g.nz
    assert p.stats["segments"] == oracle.cone_segments(g)
    rng = np.random.default_rng(1)
    for _ in range(300):
        v, r, c = int(rng.integers(g.nproj)), int(rng.integers(g.ndx)), int(rng.integers(g.ndy))
        ind, wgt = oracle.cone_trace(g, v, r, c)
        pix, w = p.trace_ray(v, r * g.ndy + c)
        np.testing.assert_array_equal(pix.astype(np.int64), ind)
        np.testing.assert_array_equal(w.view(np.uint32), wgt.view(np.uint32))


def test_cone_projectors_match_fp64(engine, oracle, splan):
    g, p = splan
    vol = volume(g)
    got = p.forward(vol)
    ref = oracle.cone_A(g, vol.astype(np.float64))
    assert rel_l2(got, ref) <= 1e-5, rel_l2(got, ref)
    np.testing.assert_array_equal(got, p.forward(vol))
    sino = np.random.default_rng(2).standard_normal(p.sino_shape).astype(np.float32)
    back = p.back(sino)
    refb = oracle.cone_AT(g, sino.astype(np.float64))
    assert rel_l2(back, refb) <= 1e-5, rel_l2(back, refb)
    np.testing.assert_array_equal(back, p.back(sino))
    x = np.random.default_rng(3).random(p.img_shape).astype(np.float32)
    lhs = float(np.sum(p.forward(x).astype(np.float64) * sino))
    rhs = float(np.sum(x.astype(np.float64) * back))
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + abs(rhs))


def test_cone_larger_volume_matches_oracle(engine, oracle):
    """A 192 x 192 x 160 volume (the small geometry's field of view at a
    quarter of its voxel size, walks of several hundred steps): traversals
    bit-exact against the oracle's, and both projectors within 1e-5 of FP64
    (the back projection of a non-negative sinogram, free of cancellation)."""
    g = engine.ConeGeometry(192, 192, 160, 0.125, 36, 36, 44, 0.9, 60.0, 110.0)
    p = engine.Plan.cone(g)
    assert p.stats["segments"] == oracle.cone_segments(g)
    rng = np.random.default_rng(5)
    for _ in range(200):
        v, r, c = int(rng.integers(g.nproj)), int(rng.integers(g.ndx)), int(rng.integers(g.ndy))
        ind, wgt = oracle.cone_trace(g, v, r, c)
        pix, w = p.trace_ray(v, r * g.ndy + c)
        np.testing.assert_array_equal(pix.astype(np.int64), ind)
        np.testing.assert_array_equal(w.view(np.uint32), wgt.view(np.uint32))
    vol = volume(g, seed=4)
    got = p.forward(vol)
    ref = oracle.cone_A(g, vol.astype(np.float64))
    assert rel_l2(got, ref) <= 1e-5, rel_l2(got, ref)
    sino = np.abs(rng.standard_normal(p.sino_shape)).astype(np.float32)
    back = p.back(sino)
    refb = oracle.cone_AT(g, sino.astype(np.float64))
    assert rel_l2(back, refb) <= 1e-5, rel_l2(back, refb)


def test_cone_solver_matches_oracle(engine, oracle, splan):
    g, p = splan
    vol = volume(g, seed=4)
    sino = oracle.cone_A(g, vol.astype(np.float64))
    prm = engine.Params(iter_alt=2)
    S = engine.Solver([p], prm)
    S.set_sino(0, sino.astype(np.float32))
    S.run()
    f, v = S.get(0)
    fo, vo, tr = oracle.solve(g, sino.astype(np.float32).astype(np.float64), prm.alpha, prm.beta, prm.epsilon,
                              prm.iter_alt, prm.iter_image, prm.iter_edge)
    assert rel_l2(f, fo) <= 1e-4, rel_l2(f, fo)
    assert rel_l2(v, vo) <= 1e-4, rel_l2(v, vo)
    assert abs(engine.phantom.psnr(f, vol) - engine.phantom.psnr(fo, vol)) <= 0.05
    ex_gpu = [(o, s, k, e) for (o, s, k, e, _) in S.trace(0) if e != 0]
    ex_or = [(o, s, k, e) for (o, s, k, _, e) in tr if e != 0]
    assert ex_gpu == ex_or


def test_cone_batch_equals_alone(engine, splan):
    g, p = splan
    a = volume(g, seed=5)
    b = volume(g, seed=6)
    prm = engine.Params(iter_alt=1)
    sa, sb = p.forward(a), p.forward(b)
    S = engine.Solver([p, p], prm)
    S.set_sino(0, sa)
    S.set_sino(1, sb)
    S.run()
    S1 = engine.Solver([p], prm)
    S1.set_sino(0, sb)
    S1.run()
    np.testing.assert_array_equal(S.get(1)[0], S1.get(0)[0])

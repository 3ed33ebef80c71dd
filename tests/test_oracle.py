"""The CPU oracle, pinned: against the golden vectors generated from the
reference's own sources (tests/golden/make_golden.py) and, where the reference
tree is present, against those sources compiled under oracle/_ref."""
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import checksum, ray_digest  # noqa: E402

from medimage_gb300.engine import FanGeometry  # noqa: E402
from medimage_gb300.phantom import ellipse_phantom  # noqa: E402


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(HERE, "golden", "goldnc.npz"))


@pytest.fixture(scope="module")
def gfan():
    return np.load(os.path.join(HERE, "golden", "fan.npz"))


def test_phantom_generator_is_stable(gold):
    np.testing.assert_array_equal(checksum(ellipse_phantom(512, seed=11).astype(np.float64)),
                                  gold["phantom_checksum"])


def test_goldnc_A_golden(oracle, gold):
    a = oracle.gc_A(ellipse_phantom(512, seed=11).astype(np.float64))
    np.testing.assert_array_equal(a[::15], gold["A_rows"])
    np.testing.assert_array_equal(checksum(a), gold["A_checksum"])


def test_goldnc_AStar_golden(oracle, gold):
    sino = np.random.default_rng(13).random((180, 767))
    b = oracle.gc_AStar(sino)
    np.testing.assert_array_equal(b[200:264, 300:364], gold["AStar_crop"])
    np.testing.assert_array_equal(checksum(b), gold["AStar_checksum"])


def test_goldnc_traversal_impulses(oracle, gold):
    """The reference's AStar of a unit bin is that bin's traced pixel set with
    its weights; the oracle's must be identical (set and FP64 weights)."""
    off = gold["impulse_off"]
    for i, (view, det) in enumerate(gold["impulse_bins"]):
        e = np.zeros((180, 767))
        e[view, det] = 1.0
        r = oracle.gc_AStar(e).ravel()
        nz = np.nonzero(r)[0]
        np.testing.assert_array_equal(nz, gold["impulse_pix"][off[i]:off[i + 1]])
        np.testing.assert_array_equal(r[nz], gold["impulse_w"][off[i]:off[i + 1]])


def test_goldnc_solver_golden(oracle, gold):
    ph2 = ellipse_phantom(512, seed=12).astype(np.float64)
    g = oracle.gc_A(ph2)
    f1, tr = oracle.image_step(None, g, np.zeros((512, 512)), np.ones((512, 512)), 1000.0, 1e-4, 10)
    v1, tre = oracle.edge_step(f1, np.ones((512, 512)), 1000.0, 0.002, 1e-4, 10)
    np.testing.assert_array_equal(f1[224:288, 224:288], gold["solver_f_crop"])
    np.testing.assert_array_equal(v1[224:288, 224:288], gold["solver_v_crop"])
    np.testing.assert_array_equal(checksum(f1), gold["solver_f_checksum"])
    np.testing.assert_array_equal(checksum(v1), gold["solver_v_checksum"])
    assert tr[-1][4] == 1  # image step left through maxIt at k == IterImage
    med = oracle.medfilt2(np.random.default_rng(14).random((512, 512)))
    np.testing.assert_array_equal(checksum(med), gold["medfilt_checksum"])


@pytest.mark.parametrize("name,geom", [("c1", FanGeometry.covering(256, 1.0, 360, 512)),
                                       ("c2", FanGeometry.covering(512, 0.75, 720, 888))])
def test_fan_traversal_golden(oracle, gfan, name, geom):
    fan = oracle.fan_from_engine(geom)
    rays, off = gfan[f"{name}_full_rays"], gfan[f"{name}_full_off"]
    for i, (v, d) in enumerate(rays):
        ind, wgt, oob = oracle.fan_trace(fan, int(v), int(d))
        np.testing.assert_array_equal(ind, gfan[f"{name}_full_ind"][off[i]:off[i + 1]])
        np.testing.assert_array_equal(wgt, gfan[f"{name}_full_w"][off[i]:off[i + 1]])
    for (v, d), dig, nb in zip(gfan[f"{name}_digest_rays"], gfan[f"{name}_digest"], gfan[f"{name}_digest_numb"]):
        ind, wgt, _ = oracle.fan_trace(fan, int(v), int(d))
        assert ind.size == nb
        assert ray_digest(ind, wgt) == dig
    assert oracle.fan_segments(fan) == int(gfan[f"{name}_segments"][0])


def test_fan_transpose_and_edges(oracle):
    fan = oracle.fan_from_engine(FanGeometry.covering(48, 1.5, 30, 64))
    rng = np.random.default_rng(1)
    x = rng.random((48, 48))
    y = rng.random((30, 64))
    lhs = float(np.vdot(oracle.fan_A(fan, x), y))
    rhs = float(np.vdot(x, oracle.fan_AT(fan, y)))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # a constant image: every ray's sum equals its traced length
    s = oracle.fan_A(fan, np.ones((48, 48)))
    for (v, d) in [(0, 0), (3, 31), (29, 63)]:
        _, w, _ = oracle.fan_trace(fan, v, d)
        assert math.isclose(s[v, d], w.sum(), rel_tol=1e-14)


def test_median_matches_sort(oracle):
    rng = np.random.default_rng(2)
    img = rng.random((33, 33))
    got = oracle.medfilt2(img)
    pad = np.pad(img, 1)
    win = np.stack([pad[i:i + 33, j:j + 33] for i in range(3) for j in range(3)])
    np.testing.assert_array_equal(got, np.sort(win, axis=0)[4])


ref_only = pytest.mark.skipif(
    not __import__("oracle.pyoracle", fromlist=["Ref"]).Ref.available(),
    reason="the reference's sources are not built on this host (oracle/_ref)")


@ref_only
def test_oracle_equals_reference_goldnc(oracle):
    ref = oracle.Ref()
    rng = np.random.default_rng(9)
    img = rng.random((512, 512))
    np.testing.assert_array_equal(oracle.gc_A(img), ref.A(img))
    sino = rng.random((180, 767))
    np.testing.assert_array_equal(oracle.gc_AStar(sino), ref.AStar(sino))
    np.testing.assert_array_equal(oracle.medfilt2(img), ref.medfilt2(img))


@ref_only
def test_oracle_equals_reference_fan(oracle):
    ref = oracle.Ref()
    rng = np.random.default_rng(10)
    for geom in (FanGeometry.covering(128, 0.5, 64, 96), FanGeometry.covering(300, 1.3, 17, 250, 700.0, 1100.0)):
        fan = oracle.fan_from_engine(geom)
        for _ in range(400):
            v, d = int(rng.integers(geom.nviews)), int(rng.integers(geom.ndets))
            ind, wgt, _ = oracle.fan_trace(fan, v, d)
            ind2, wgt2 = ref.fan_trace_points(geom.n, geom.pixel_mm, *oracle.fan_endpoints(fan, v, d))
            np.testing.assert_array_equal(ind, ind2)
            np.testing.assert_array_equal(wgt, wgt2)
    # near-axis rays (the 1e-4 guard, tracing.cpp:55-56) and end-point cases
    for pts in [(-500.0, 64.0, 700.0, 64.00001), (64.0, -500.0, 64.0, 700.0), (-500.0, 0.0, 700.0, 128.0),
                (-500.0, -500.0, 700.0, 700.0), (-500.0, 64.0, 700.0, 64.0)]:
        ind, wgt = ref.fan_trace_points(128, 1.0, *pts)
        ind2 = np.zeros(1024, np.int32)
        w2 = np.zeros(1024)
        k = oracle.lib().or_fan_trace_points(128, 1.0, *pts, ind2, w2, 1024)
        np.testing.assert_array_equal(ind, ind2[:k])
        np.testing.assert_array_equal(wgt, w2[:k])


@ref_only
def test_oracle_equals_reference_solver_small_iters(oracle):
    ref = oracle.Ref()
    ph = ellipse_phantom(512, seed=19).astype(np.float64)
    g = ref.A(ph)
    f0 = np.zeros((512, 512))
    v0 = np.ones((512, 512))
    f_ref = ref.image_step(g, f0, v0, 1000.0, 1e-4, 3)
    f_or, _ = oracle.image_step(None, g, f0, v0, 1000.0, 1e-4, 3)
    np.testing.assert_array_equal(f_or, f_ref)
    v_ref = ref.edge_step(f_ref, v0, 1000.0, 0.002, 1e-4, 4)
    v_or, _ = oracle.edge_step(f_or, v0, 1000.0, 0.002, 1e-4, 4)
    np.testing.assert_array_equal(v_or, v_ref)

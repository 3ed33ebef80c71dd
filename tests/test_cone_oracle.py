"""The 3D cone-beam restatement (oracle/or_cone.c), pinned: against golden
end points and traversals made from the reference's own industry3d tracer
(tests/golden/make_golden.py), and, where the reference tree is built, against
that tracer directly on random rays (bit-exact indices and FP32 weights)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import CONE_GEOMS  # noqa: E402

from medimage_gb300.engine import ConeGeometry  # noqa: E402


@pytest.fixture(scope="module")
def gcone():
    return np.load(os.path.join(HERE, "golden", "cone.npz"))


@pytest.mark.parametrize("name", ["small", "c4"])
def test_cone_endpoints_and_traversal_golden(oracle, gcone, name):
    g = CONE_GEOMS[name]
    off = gcone[f"{name}_off"]
    for i, (v, r, c) in enumerate(gcone[f"{name}_rays"]):
        s, d = oracle.cone_endpoints(g, int(v), int(r), int(c))
        np.testing.assert_array_equal(np.concatenate([s, d]).view(np.uint32), gcone[f"{name}_ends"][i].view(np.uint32))
        ind, wgt = oracle.cone_trace(g, int(v), int(r), int(c))
        np.testing.assert_array_equal(ind, gcone[f"{name}_ind"][off[i]:off[i + 1]])
        np.testing.assert_array_equal(wgt.view(np.uint32), gcone[f"{name}_w"][off[i]:off[i + 1]].view(np.uint32))


def test_cone_constant_volume_path_lengths(oracle):
    """A central ray through a cube of ones: its line integral is the cube's
    side (in voxels) up to the tracer's dropped final sub-0.05 segment."""
    g = ConeGeometry(32, 32, 32, 1.0, 8, 16, 16, 1.0, 200.0, 400.0)
    ind, wgt = oracle.cone_trace(g, 0, 8, 8, mark_off=True)
    on = ind >= 0
    assert 31.9 < float(wgt[on].astype(np.float64).sum()) <= 32.0 + 1e-4


def test_cone_transpose(oracle):
    g = ConeGeometry(16, 16, 12, 1.0, 10, 10, 12, 1.5, 60.0, 100.0)
    rng = np.random.default_rng(3)
    x = rng.random((12, 16, 16))
    y = rng.random((10, 10, 12))
    lhs = float(np.sum(oracle.cone_A(g, x) * y))
    rhs = float(np.sum(x * oracle.cone_AT(g, y)))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


ref_only = pytest.mark.skipif(
    not __import__("oracle.pyoracle", fromlist=["Ref"]).Ref.available(),
    reason="the reference's sources are not built on this host (oracle/_ref)")


@ref_only
def test_cone_oracle_equals_reference(oracle):
    ref = oracle.Ref()
    rng = np.random.default_rng(5)
    for g in (ConeGeometry(64, 64, 48, 0.4, 90, 64, 64, 0.7, 60.0, 100.0),
              ConeGeometry(40, 40, 40, 0.25, 360, 48, 48, 0.3, 30.0, 70.0)):
        for _ in range(1500):
            v, r, c = int(rng.integers(g.nproj)), int(rng.integers(g.ndx)), int(rng.integers(g.ndy))
            s, d = oracle.cone_endpoints(g, v, r, c)
            s2, d2 = oracle.ref_cone_endpoints(ref, g, v, r, c)
            np.testing.assert_array_equal(np.concatenate([s, d]).view(np.uint32),
                                          np.concatenate([s2, d2]).view(np.uint32))
            i1, w1 = oracle.cone_trace_points(g.nx, g.ny, g.nz, s2, d2)
            i2, w2 = oracle.ref_cone_trace_points(ref, g.nx, g.ny, g.nz, s2, d2)
            np.testing.assert_array_equal(i1, i2)
            np.testing.assert_array_equal(w1.view(np.uint32), w2.view(np.uint32))
    # axis-aligned and near-axis rays (the 1e-4 guard of tracing.cpp:160-162)
    for s, d in [((-50.0, 20.0, 20.0), (90.0, 20.0, 20.0)), ((20.0, -50.0, 20.0), (20.0, 90.0, 20.00001)),
                 ((20.3, 20.7, -50.0), (20.3, 20.7, 90.0)), ((-50.0, -50.0, -50.0), (90.0, 90.0, 90.0))]:
        i1, w1 = oracle.cone_trace_points(40, 40, 40, s, d)
        i2, w2 = oracle.ref_cone_trace_points(ref, 40, 40, 40, s, d)
        np.testing.assert_array_equal(i1, i2)
        np.testing.assert_array_equal(w1.view(np.uint32), w2.view(np.uint32))

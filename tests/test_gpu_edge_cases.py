"""Edge cases of the fan-beam projectors and solver on the GB300.

- The smallest geometries the C-ABI accepts (8 x 8 image), a single view, two
  detectors, and sizes that are not multiples of the kernels' tiles (16 x
  16 pixels, 128-ray blocks, 64-view blocks): traversal bit-exact, projections
  to rel-L2 1e-5 against the FP64 oracle.
- Zero inputs: the forward projection of a zero image and the back projection
  of a zero sinogram are exactly zero, alone and in groups (the back
  projector's fixed-point scale comes from max |r| = 0 there).
- A batch mixing every group form (a group of four, a triple, a pair, a scan
  alone) in one launch per form reconstructs each scan as it does alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def edge_geoms(engine):
    G = engine.FanGeometry.covering
    return [
        G(8, 1.0, 1, 4),       # smallest image, one view
        G(8, 1.0, 5, 2),       # the fewest detectors (an even count, as the fan geometry requires)
        G(9, 0.7, 3, 14),      # odd image: partial 16 x 16 tiles
        G(37, 1.3, 65, 130),   # 65 views (a partial 64-view block), 130 detectors (a partial 128-ray block)
        G(100, 0.9, 128, 258),
    ]


@pytest.mark.parametrize("k", range(5))
def test_small_and_ragged_geometries(engine, oracle, k):
    g = edge_geoms(engine)[k]
    p = engine.Plan.fan(g)
    fan = oracle.fan_from_engine(g)
    assert p.stats["segments"] == oracle.fan_segments(fan)
    for view in sorted({0, g.nviews // 2, g.nviews - 1}):
        for det in sorted({0, g.ndets // 2, g.ndets - 1}):
            ind, _, _ = oracle.fan_trace(fan, view, det)
            pix, _ = p.trace_ray(view, det)
            np.testing.assert_array_equal(pix, ind, err_msg=f"{g} ray ({view},{det})")
    img = engine.phantom.ellipse_phantom(g.n, seed=3, n_random=2)
    ref = oracle.fan_A(fan, img.astype(np.float64))
    if np.linalg.norm(ref) > 0:
        assert rel_l2(p.forward(img), ref) <= TOL
    sino = np.random.default_rng(k).standard_normal((g.nviews, g.ndets)).astype(np.float32)
    refb = oracle.fan_AT(fan, sino.astype(np.float64))
    if np.linalg.norm(refb) > 0:
        assert rel_l2(p.back(sino), refb) <= TOL


def test_zero_inputs_give_zero(engine):
    g = engine.FanGeometry.covering(64, 1.0, 90, 128)
    p = engine.Plan.fan(g)
    assert not np.any(p.forward(np.zeros((64, 64), np.float32)))
    assert not np.any(p.back(np.zeros((90, 128), np.float32)))
    # a group of three: one member's sinogram is zero, the others not
    rng = np.random.default_rng(9)
    sinos = [torch.zeros((90, 128), device="cuda"),
             torch.from_numpy(rng.standard_normal((90, 128)).astype(np.float32)).cuda(),
             torch.from_numpy(rng.standard_normal((90, 128)).astype(np.float32)).cuda()]
    outs = [torch.full((64, 64), 7.0, device="cuda") for _ in range(3)]
    ps = engine.ProjSet([p, p, p])
    ps.back_dev([t.data_ptr() for t in sinos], [t.data_ptr() for t in outs])
    torch.cuda.synchronize()
    assert not torch.any(outs[0])
    for i in (1, 2):
        ref = torch.empty_like(outs[i])
        p.back_dev(sinos[i].data_ptr(), ref.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(outs[i], ref)
    ps.close()


def test_batch_of_every_group_form_equals_alone(engine, oracle):
    geoms = [engine.FanGeometry.covering(48, 2.0, 60, 80),
             engine.FanGeometry.covering(40, 2.4, 50, 70),
             engine.FanGeometry.covering(32, 3.0, 40, 64),
             engine.FanGeometry.covering(56, 1.8, 70, 90)]
    plans = [engine.Plan.fan(g) for g in geoms]
    # plan 0 x4 (a group of four), plan 1 x3, plan 2 x2, plan 3 alone, interleaved
    order = [0, 1, 2, 0, 3, 1, 0, 2, 1, 0]
    sinos = []
    for i, k in enumerate(order):
        ph = engine.phantom.ellipse_phantom(geoms[k].n, seed=200 + i, n_random=3)
        clean = oracle.fan_A(oracle.fan_from_engine(geoms[k]), ph.astype(np.float64))
        sinos.append(engine.phantom.poisson_sinogram(clean, 1e4, 300 + i))
    prm = engine.Params(iter_alt=2)
    B = engine.Solver([plans[k] for k in order], prm)
    for i, s in enumerate(sinos):
        B.set_sino(i, s)
    B.run()
    for i, k in enumerate(order):
        A1 = engine.Solver([plans[k]], prm)
        A1.set_sino(0, sinos[i])
        A1.run()
        fa, va = A1.get(0)
        fb, vb = B.get(i)
        assert rel_l2(fb, fa) <= 1e-6 and rel_l2(vb, va) <= 1e-6, (i, k, rel_l2(fb, fa), rel_l2(vb, va))

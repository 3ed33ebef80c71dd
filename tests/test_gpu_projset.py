"""Projection sets (at_projset_*): several images through their plans in one
launch per kernel, images of the same plan walked together (up to four per
walk).  Every image's projection must equal its own at_forward / at_back
bit for bit, whatever the grouping (groups of four, a group of one, other
plans in between, an off-grid ray-table geometry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


@pytest.mark.parametrize("layout", ["AAAAA", "AABAA", "ABCBA", "A"])
def test_projset_equals_single_calls(engine, layout):
    geoms = {"A": engine.FanGeometry.covering(96, 2.0, 120, 160),
             "B": engine.FanGeometry.covering(64, 3.0, 90, 128),
             "C": engine.RayGeometry.msbeam_parallel(n=64, nproj=30, nray=96)}
    plans = {k: (engine.Plan.rays(g) if k == "C" else engine.Plan.fan(g)) for k, g in geoms.items()}
    pl = [plans[c] for c in layout]
    rng = np.random.default_rng(7)
    imgs = [_dev(engine.phantom.ellipse_phantom(p.n, seed=10 + i, n_random=4)) for i, p in enumerate(pl)]
    sinos = [_dev(rng.standard_normal(p.sino_shape)) for p in pl]
    out_s = [torch.empty(p.sino_shape, device="cuda") for p in pl]
    out_i = [torch.empty(p.img_shape, device="cuda") for p in pl]
    ps = engine.ProjSet(pl)
    for _ in range(2):  # the second call reuses the bound buffers
        ps.forward_dev([t.data_ptr() for t in imgs], [t.data_ptr() for t in out_s])
        ps.back_dev([t.data_ptr() for t in sinos], [t.data_ptr() for t in out_i])
        torch.cuda.synchronize()
        for i, p in enumerate(pl):
            ref_s = torch.empty_like(out_s[i])
            ref_i = torch.empty_like(out_i[i])
            p.forward_dev(imgs[i].data_ptr(), ref_s.data_ptr())
            p.back_dev(sinos[i].data_ptr(), ref_i.data_ptr())
            torch.cuda.synchronize()
            assert torch.equal(out_s[i], ref_s), (layout, i)
            assert torch.equal(out_i[i], ref_i), (layout, i)
    # new buffers re-point the set
    imgs2 = [t * 2 for t in imgs]
    ps.forward_dev([t.data_ptr() for t in imgs2], [t.data_ptr() for t in out_s])
    torch.cuda.synchronize()
    for i, p in enumerate(pl):
        ref_s = torch.empty_like(out_s[i])
        p.forward_dev(imgs2[i].data_ptr(), ref_s.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(out_s[i], ref_s)
    ps.close()


def test_projset_rejects_mixed_families(engine):
    fan = engine.Plan.fan(engine.FanGeometry.covering(64, 3.0, 90, 128))
    gold = engine.Plan.goldnc()
    with pytest.raises(engine.AtError):
        engine.ProjSet([fan, gold])

"""The forward projector's two walks agree bit for bit.

The slab projector (the image staged in shared memory by TMA, slab by slab)
and the walk that gathers through L1 run the same decision bits, crossing
formula, per-word partial sums and Kahan folds, so their sums must be equal
bitwise: for every CTA shape the plan accepts, alone and in every group form
(a pair read as float2, three or four members as float4), and on plans with
rays off the grid (whose CTAs take the L1 path inside the slab kernel).  Shapes
that cannot fit a plan are refused with AT_EINVAL, and a solver built before a
variant change keeps working with the tables it was built with.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(4, 128, 16), (2, 128, 8), (8, 64, 16), (4, 32, 32), (16, 32, 4)]


def geoms(engine):
    G = engine.FanGeometry.covering
    return {
        "c1": G(256, 1.0, 360, 512),
        "c2": G(512, 0.75, 720, 888),
        "ragged": G(100, 0.9, 130, 258),  # partial view groups and detector blocks
        "c3": G(384, 1.0, 540, 768),
    }


def images(engine, n, count, seed):
    return [engine.phantom.ellipse_phantom(n, seed=seed + i, n_random=3 + i) for i in range(count)]


def check_plan(engine, plan, shapes, seed=0):
    imgs = images(engine, plan.n, 4, seed)
    plan.set_forward_variant(0, 0, 0)
    assert plan.stats["slab_views"] == 0
    ref = [plan.forward(im) for im in imgs]
    for shape in shapes:
        try:
            plan.set_forward_variant(*shape)
        except engine.AtError:
            continue  # refused: checked separately below
        assert (plan.stats["slab_views"], plan.stats["slab_rays"], plan.stats["slab_rows"]) == shape
        for im, r in zip(imgs, ref):
            np.testing.assert_array_equal(plan.forward(im), r, err_msg=f"shape {shape}")
        for count in (2, 3, 4):
            ps = engine.ProjSet([plan] * count)
            outs = ps.forward(imgs[:count])
            ps.close()
            for m in range(count):
                np.testing.assert_array_equal(outs[m], ref[m], err_msg=f"shape {shape}, {count} members, #{m}")


@pytest.mark.parametrize("name", ["c1", "c2", "ragged", "c3"])
def test_slab_equals_l1_walk(engine, name):
    plan = engine.Plan.fan(geoms(engine)[name])
    check_plan(engine, plan, SHAPES if name != "c2" else SHAPES[:3], seed=len(name))


def test_slab_on_ray_tables(engine, oracle):
    """msbeam's parallel beam and a non-uniform view table, both as ray
    tables; msbeam's rays along the image's far edge trace segments off the
    grid, so some CTAs take the checked L1 path inside the slab kernel."""
    ms = engine.Plan.rays(engine.RayGeometry.msbeam_parallel())
    ang = np.sort(np.random.default_rng(3).uniform(0.0, 360.0, 97))
    nu = engine.Plan.rays(engine.RayGeometry.fan_from_view_table(160, 1.0, 222, ang, det_pitch_deg=0.19))
    for plan in (ms, nu):
        check_plan(engine, plan, SHAPES[:2], seed=7)


def test_slab_refuses_what_does_not_fit(engine):
    odd = engine.Plan.fan(engine.FanGeometry.covering(37, 1.3, 65, 130))  # rows not 16-byte multiples
    with pytest.raises(engine.AtError):
        odd.set_forward_variant(2, 64, 16)
    assert odd.stats["slab_views"] == 0
    plan = engine.Plan.fan(engine.FanGeometry.covering(64, 1.0, 90, 128))
    for bad in ((1, 100, 16), (8, 128, 16), (1, 32, 0), (1, 32, 300)):  # rays not dividing 128, > 512 threads, rows
        with pytest.raises(engine.AtError):
            plan.set_forward_variant(*bad)
    img = engine.phantom.ellipse_phantom(64, seed=1)
    a = plan.forward(img)
    plan.set_forward_variant(0, 0, 0)
    np.testing.assert_array_equal(plan.forward(img), a)


def test_solver_keeps_its_variant(engine, oracle):
    """A solver made with one variant keeps running after the plan switches to
    another (the plan keeps the tables the solver points at), with bitwise the
    same reconstruction as a solver made after the switch."""
    g = engine.FanGeometry.covering(128, 1.5, 180, 256)
    plan = engine.Plan.fan(g)
    ph = engine.phantom.ellipse_phantom(128, seed=4, n_random=4)
    sino = engine.phantom.poisson_sinogram(oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64)), 1e4, 5)
    prm = engine.Params(iter_alt=2)
    plan.set_forward_variant(2, 128, 16)
    a = engine.Solver([plan, plan], prm)
    plan.set_forward_variant(4, 64, 8)
    b = engine.Solver([plan, plan], prm)
    plan.set_forward_variant(0, 0, 0)
    for s in (a, b):
        s.set_sino(0, sino)
        s.set_sino(1, sino * 0.5)
        s.run()
    for i in range(2):
        fa, va = a.get(i)
        fb, vb = b.get(i)
        np.testing.assert_array_equal(fa, fb)
        np.testing.assert_array_equal(va, vb)
    a.close()
    b.close()

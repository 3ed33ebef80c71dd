"""The back projector's two forms agree bit for bit.

Gathering each pixel's terms from the plan's pixel table and walking the
(ray, 16x16 tile) runs add the same fixed-point terms (the same FP32 segment
weights, residuals and per-scan scale) into exact integer sums, so their
images must be equal bitwise: for single scans and for every group form (a
pair read as float2, three or four members as float4), on fan-beam plans of
the benchmark shapes and ragged ones, on the plain FP32 traversal, on ray
tables, inside solvers whose launches mix plans with and without tables, and
on residuals with a few large outliers (which set the fixed-point quantum).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def geoms(engine):
    G = engine.FanGeometry.covering
    return {
        "c1": G(256, 1.0, 360, 512),
        "c2": G(512, 0.75, 720, 888),
        "ragged": G(100, 0.9, 130, 258),  # tiles cut by the image edge, a partial view block
        "c3": G(384, 1.0, 540, 768),
    }


def residuals(engine, plan, count, seed):
    """Zero-mean noise, a low-count Poisson-like residual with outliers, and
    forward projections of phantoms."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        if i % 3 == 0:
            out.append(rng.standard_normal(plan.sino_shape).astype(np.float32))
        elif i % 3 == 1:
            r = (rng.poisson(3.0, plan.sino_shape) - 3.0).astype(np.float32)
            idx = rng.integers(0, r.size, 5)
            r.reshape(-1)[idx] = rng.choice([-1e4, 1e4], 5).astype(np.float32)
            out.append(r)
        else:
            ph = engine.phantom.ellipse_phantom(plan.n, seed=seed + i, n_random=3)
            out.append(plan.forward(ph))
    return out


def check_plan(engine, plan, seed=0):
    sinos = residuals(engine, plan, 4, seed)
    plan.set_back_variant(0)
    ref = [plan.back(s) for s in sinos]
    refs = {}
    for count in (2, 3, 4):
        ps = engine.ProjSet([plan] * count)
        refs[count] = ps.back(sinos[:count])
        ps.close()
    for count in (2, 3, 4):  # a group is its members' single-scan sums
        for m in range(count):
            np.testing.assert_array_equal(refs[count][m], ref[m])
    plan.set_back_variant(3)
    assert plan.stats["bp_table_use"] == 3 and plan.stats["bp_table_bytes"] > 0
    assert plan.stats["bp_table_weights"] >= plan.stats["segments"] - plan.stats["offgrid"]
    for s, r in zip(sinos, ref):
        np.testing.assert_array_equal(plan.back(s), r)
    for count in (2, 3, 4):
        ps = engine.ProjSet([plan] * count)
        outs = ps.back(sinos[:count])
        ps.close()
        for m in range(count):
            np.testing.assert_array_equal(outs[m], refs[count][m], err_msg=f"{count} members, #{m}")
    plan.set_back_variant(0)


@pytest.mark.parametrize("name", ["c1", "c2", "ragged", "c3"])
def test_table_equals_tile_runs(engine, name):
    check_plan(engine, engine.Plan.fan(geoms(engine)[name]), seed=len(name))


def test_table_on_fp32_traversal(engine):
    check_plan(engine, engine.Plan.fan(geoms(engine)["c1"], alpha="fp32"), seed=11)


def test_table_on_ray_tables(engine):
    """msbeam's parallel beam (rays along the far edge trace off the grid)
    and a non-uniform view table."""
    ms = engine.Plan.rays(engine.RayGeometry.msbeam_parallel())
    ang = np.sort(np.random.default_rng(3).uniform(0.0, 360.0, 97))
    nu = engine.Plan.rays(engine.RayGeometry.fan_from_view_table(160, 1.0, 222, ang, det_pitch_deg=0.19))
    for plan in (ms, nu):
        check_plan(engine, plan, seed=7)


def test_table_refuses_what_does_not_fit(engine):
    """About 90 rays of one view cross each pixel: more than the table's
    6-bit count.  The plan refuses the table and keeps walking tile runs."""
    plan = engine.Plan.fan(engine.FanGeometry.covering(16, 16.0, 24, 2048))
    sino = np.random.default_rng(1).standard_normal(plan.sino_shape).astype(np.float32)
    a = plan.back(sino)
    with pytest.raises(engine.AtError):
        plan.set_back_variant(1)
    assert plan.stats["bp_table_use"] == 0 and plan.stats["bp_table_bytes"] == 0
    np.testing.assert_array_equal(plan.back(sino), a)
    small = engine.Plan.fan(engine.FanGeometry.covering(64, 1.0, 90, 128))
    for bad in (-1, 4):
        with pytest.raises(engine.AtError):
            small.set_back_variant(bad)


def test_solver_with_mixed_launches(engine, oracle):
    """A batch of three plans: four scans of one (a group of four, from its
    table), a pair of another (table for groups only) and one scan of a
    third: without a table, so the launch of pairs and scans alone chooses
    per CTA, then with its table for single scans too, so that launch
    gathers throughout.  Equal bit for bit to the same batch walking tile
    runs, over two runs of the captured graph."""
    G = engine.FanGeometry.covering
    ga, gb, gc = G(96, 2.0, 120, 160), G(64, 3.0, 90, 128), G(80, 2.4, 72, 100)
    pa, pb, pc = engine.Plan.fan(ga), engine.Plan.fan(gb), engine.Plan.fan(gc)
    plans = [pa, pa, pb, pa, pa, pc, pb]
    geo = {id(pa): ga, id(pb): gb, id(pc): gc}
    sinos = []
    for i, p in enumerate(plans):
        g = geo[id(p)]
        ph = engine.phantom.ellipse_phantom(g.n, seed=300 + i, n_random=3)
        clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
        sinos.append(engine.phantom.poisson_sinogram(clean, 1e4, 350 + i))

    def solve():
        s = engine.Solver(plans, engine.Params(iter_alt=2))
        out = []
        for _ in range(2):
            for i, sino in enumerate(sinos):
                s.set_sino(i, sino)
            s.run()
            out.append([s.get(i) for i in range(len(plans))])
        s.close()
        return out

    for p in (pa, pb, pc):
        p.set_back_variant(0)
    ref = solve()
    pa.set_back_variant(3)
    pb.set_back_variant(2)
    got = [solve()]
    pc.set_back_variant(1)
    got.append(solve())
    for g in got:
        for r_run, g_run in zip(ref, g):
            for (fr, vr), (fg, vg) in zip(r_run, g_run):
                np.testing.assert_array_equal(fg, fr)
                np.testing.assert_array_equal(vg, vr)

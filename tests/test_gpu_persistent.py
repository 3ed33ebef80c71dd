"""Persistent projector launches (at_set_batch_launch_mode(1)): a grid of the
resident CTAs pulls work units from a queue instead of one CTA per unit.  Each
unit runs the ordinary kernel body, so a batch of mixed geometries with every
group form (a group of four, a pair, scans alone), and a projection set, give
bitwise the results of the default launches; the queue resets itself, so a
solver's captured graph replays correctly (two runs in a row)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_mode(engine):
    yield
    engine.set_batch_launch_mode(False)


def mixed_batch(engine, oracle):
    G = engine.FanGeometry.covering
    ga, gb, gc = G(96, 2.0, 120, 160), G(64, 3.0, 90, 128), G(80, 2.4, 72, 100)
    pa, pb, pc = engine.Plan.fan(ga), engine.Plan.fan(gb), engine.Plan.fan(gc)
    plans = [pa, pa, pb, pa, pa, pc, pb]  # pa: a group of four; pb: a pair; pc alone
    geoms = {id(pa): ga, id(pb): gb, id(pc): gc}
    sinos = []
    for i, p in enumerate(plans):
        g = geoms[id(p)]
        ph = engine.phantom.ellipse_phantom(g.n, seed=900 + i, n_random=3)
        clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
        sinos.append(engine.phantom.poisson_sinogram(clean, 1e4, 950 + i))
    return plans, sinos


def solve(engine, plans, sinos, runs=2):
    s = engine.Solver(plans, engine.Params(iter_alt=2))
    out = []
    for _ in range(runs):  # the second run replays the captured graph
        for i, sino in enumerate(sinos):
            s.set_sino(i, sino)
        s.run()
        out.append([s.get(i) for i in range(len(plans))])
    s.close()
    return out


def test_persistent_solver_equals_default(engine, oracle, restore_mode):
    plans, sinos = mixed_batch(engine, oracle)
    engine.set_batch_launch_mode(False)
    ref = solve(engine, plans, sinos)
    engine.set_batch_launch_mode(True)
    got = solve(engine, plans, sinos)
    for r_run, g_run in zip(ref, got):
        for (fr, vr), (fg, vg) in zip(r_run, g_run):
            np.testing.assert_array_equal(fg, fr)
            np.testing.assert_array_equal(vg, vr)
    np.testing.assert_array_equal(got[0][0][0], got[1][0][0])


def test_persistent_projection_set_equals_default(engine, oracle, restore_mode):
    plans, sinos = mixed_batch(engine, oracle)
    imgs = [engine.phantom.ellipse_phantom(p.n, seed=40 + i, n_random=2) for i, p in enumerate(plans)]
    engine.set_batch_launch_mode(False)
    ps = engine.ProjSet(plans)
    ref_f, ref_b = ps.forward(imgs), ps.back(sinos)
    ps.close()
    engine.set_batch_launch_mode(True)
    ps = engine.ProjSet(plans)
    for _ in range(2):
        got_f, got_b = ps.forward(imgs), ps.back(sinos)
        for a, b in zip(got_f + got_b, ref_f + ref_b):
            np.testing.assert_array_equal(a, b)
    ps.close()
    with pytest.raises(engine.AtError):
        engine.lib()  # the bindings are loaded
        engine.engine._check("at_set_batch_launch_mode", engine.lib().at_set_batch_launch_mode(2))

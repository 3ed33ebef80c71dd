"""GPU parity of the AT solver against the FP64 oracle restatement of
origin/GoldenC/src/main.c (pinned bit-for-bit to the reference).

Tolerances: final f and v rel-L2 <= 1e-4 and PSNR
within 0.05 dB after the same iteration count; the branch trace (exit reasons
per inner loop) must be identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_case(engine, oracle, n, px, nv, nd, seed, i0=1e4, n_random=5):
    g = engine.FanGeometry.covering(n, px, nv, nd)
    ph = engine.phantom.ellipse_phantom(n, seed=seed, n_random=n_random)
    clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
    sino = engine.phantom.poisson_sinogram(clean, i0, seed + 100)
    return g, ph, sino


def exits(trace_gpu):
    return [(o, s, k, e) for (o, s, k, e, _) in trace_gpu if e != 0]


def exits_oracle(trace_or):
    return [(o, s, k, e) for (o, s, k, _, e) in trace_or if e != 0]


@pytest.mark.parametrize("mode", [0, 1])
def test_fan_solve_matches_oracle(engine, oracle, mode):
    g, ph, sino = make_case(engine, oracle, 96, 2.0, 120, 160, seed=11)
    prm = engine.Params(iter_alt=3, mode=mode)
    plan = engine.Plan.fan(g)
    S = engine.Solver([plan], prm)
    S.set_sino(0, sino)
    S.run()
    f, v = S.get(0)
    fo, vo, tr = oracle.solve(oracle.fan_from_engine(g), sino.astype(np.float64), prm.alpha, prm.beta,
                              prm.epsilon, prm.iter_alt, prm.iter_image, prm.iter_edge)
    assert rel_l2(f, fo) <= TOL, rel_l2(f, fo)
    assert rel_l2(v, vo) <= TOL, rel_l2(v, vo)
    pg = engine.phantom.psnr(f, ph)
    po = engine.phantom.psnr(fo, ph)
    assert abs(pg - po) <= 0.05
    assert exits(S.trace(0)) == exits_oracle(tr)


def test_goldnc_image_and_edge_steps(engine, oracle):
    L = engine.lib()
    ph = engine.phantom.ellipse_phantom(512, seed=21).astype(np.float64)
    g = oracle.gc_A(ph)
    f0 = np.zeros((512, 512))
    v0 = np.ones((512, 512))
    out = np.zeros((512, 512))
    L.minimize_in_IMAGE_variable(out, g, f0, v0, 1000.0, 1e-4, 10)
    assert L.goldnc_status() == 0
    ref, _ = oracle.image_step(None, g, f0, v0, 1000.0, 1e-4, 10)
    assert rel_l2(out, ref) <= TOL, rel_l2(out, ref)
    vout = np.zeros((512, 512))
    L.minimize_in_EDGE_variable(vout, ref, v0, 1000.0, 0.002, 1e-4, 10)
    assert L.goldnc_status() == 0
    vref, _ = oracle.edge_step(ref, v0, 1000.0, 0.002, 1e-4, 10)
    assert rel_l2(vout, vref) <= TOL, rel_l2(vout, vref)


def test_batch_equals_alone(engine, oracle):
    cases = [make_case(engine, oracle, n, px, nv, nd, seed=s)
             for (n, px, nv, nd, s) in [(64, 3.0, 90, 128, 31), (96, 2.0, 120, 160, 32), (80, 2.4, 72, 100, 33)]]
    prm = engine.Params(iter_alt=2)
    plans = [engine.Plan.fan(g) for g, _, _ in cases]
    B = engine.Solver(plans, prm)
    for i, (_, _, sino) in enumerate(cases):
        B.set_sino(i, sino)
    B.run()
    for i, (g, _, sino) in enumerate(cases):
        A1 = engine.Solver([plans[i]], prm)
        A1.set_sino(0, sino)
        A1.run()
        fa, va = A1.get(0)
        fb, vb = B.get(i)
        assert rel_l2(fb, fa) <= 1e-6 and rel_l2(vb, va) <= 1e-6


def test_shared_plan_groups_equal_alone(engine, oracle):
    """Scans of one plan are projected together (up to four per walk); a fifth
    scan of that plan starts a second group, and a scan of another plan sits
    between them.  Each must still reconstruct as it does alone."""
    gA, _, _ = make_case(engine, oracle, 96, 2.0, 120, 160, seed=51)
    gB, _, sB = make_case(engine, oracle, 64, 3.0, 90, 128, seed=52)
    pA, pB = engine.Plan.fan(gA), engine.Plan.fan(gB)
    sinos = []
    for s in range(5):
        ph = engine.phantom.ellipse_phantom(96, seed=60 + s, n_random=3 + s)
        clean = oracle.fan_A(oracle.fan_from_engine(gA), ph.astype(np.float64))
        sinos.append(engine.phantom.poisson_sinogram(clean, 1e4 * (s + 1), 160 + s))
    plans = [pA, pA, pB, pA, pA, pA]
    data = [sinos[0], sinos[1], sB, sinos[2], sinos[3], sinos[4]]
    prm = engine.Params(iter_alt=2)
    B = engine.Solver(plans, prm)
    for i, d in enumerate(data):
        B.set_sino(i, d)
    B.run()
    for i, (p, d) in enumerate(zip(plans, data)):
        A1 = engine.Solver([p], prm)
        A1.set_sino(0, d)
        A1.run()
        fa, va = A1.get(0)
        fb, vb = B.get(i)
        assert rel_l2(fb, fa) <= 1e-6 and rel_l2(vb, va) <= 1e-6, (i, rel_l2(fb, fa), rel_l2(vb, va))
        assert exits(B.trace(i)) == exits(A1.trace(0))


def test_reconstruct_host_matches_solver(engine, oracle):
    g, ph, sino = make_case(engine, oracle, 64, 3.0, 90, 128, seed=41)
    prm = engine.Params(iter_alt=2)
    plan = engine.Plan.fan(g)
    f1, v1 = engine.reconstruct(plan, prm, sino)
    S = engine.Solver([plan], prm)
    S.set_sino(0, sino)
    S.run()
    f2, v2 = S.get(0)
    np.testing.assert_array_equal(f1, f2)
    np.testing.assert_array_equal(v1, v2)

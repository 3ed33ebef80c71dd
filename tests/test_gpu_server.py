"""The continuous-batching server: requests arriving while others run join the
batch as slots and budget free up; every result must equal the same request
served alone (bitwise: a request's arithmetic does not depend on the mix) and
the fixed-batch solver's result within 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_requests(engine, oracle):
    G = engine.FanGeometry.covering
    geoms = [G(64, 3.0, 90, 128), G(96, 2.0, 120, 160), G(80, 2.4, 72, 100)]
    plans = [engine.Plan.fan(g) for g in geoms]
    reqs = []
    for i in range(7):
        g, p = geoms[i % 3], plans[i % 3]
        ph = engine.phantom.ellipse_phantom(g.n, seed=300 + i, n_random=3)
        clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
        sino = engine.phantom.poisson_sinogram(clean, 1e4, 400 + i)
        reqs.append((p, sino, 2 + (i % 3), 0.002 * i))
    return plans, reqs


def test_server_mix_equals_alone(engine, oracle):
    plans, reqs = make_requests(engine, oracle)
    srv = engine.Server(hbm_budget_bytes=1 << 34, max_active=3)
    ids = [srv.submit(p, s, it, arr) for (p, s, it, arr) in reqs]
    srv.run()
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["p99_latency_s"] >= st["p50_latency_s"] > 0
    for rid, (p, s, it, _) in zip(ids, reqs):
        f_mix, v_mix, lat, wait = srv.result(rid)
        assert lat > 0 and wait >= 0
        alone = engine.Server(hbm_budget_bytes=1 << 34, max_active=1)
        a = alone.submit(p, s, it, 0.0)
        alone.run()
        f_one, v_one, _, _ = alone.result(a)
        np.testing.assert_array_equal(f_mix, f_one)
        np.testing.assert_array_equal(v_mix, v_one)
        solver = engine.Solver([p], engine.Params(iter_alt=it))
        solver.set_sino(0, s)
        solver.run()
        f_s, v_s = solver.get(0)
        assert np.linalg.norm(f_mix - f_s) <= 1e-6 * np.linalg.norm(f_s)
        assert np.linalg.norm(v_mix - v_s) <= 1e-6 * np.linalg.norm(v_s)


def test_server_admission_respects_budget(engine, oracle):
    plans, reqs = make_requests(engine, oracle)
    one = engine.Solver.footprint([plans[1]])  # largest of the three geometries
    srv = engine.Server(hbm_budget_bytes=int(2.2 * one), max_active=8)
    for (p, s, it, arr) in reqs:
        srv.submit(p, s, it, 0.0)
    srv.run()
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["peak_state_bytes"] <= int(2.2 * one)
    tiny = engine.Server(hbm_budget_bytes=1024, max_active=2)
    with pytest.raises(engine.AtError) as ei:
        tiny.submit(plans[0], reqs[0][1], 2, 0.0)
    assert ei.value.code == -5


def test_server_mixes_slices_and_cone_volumes(engine, oracle):
    """Cone-beam volumes run in the same rounds as fan-beam slices (a second
    batch); each result equals the request served alone, bitwise."""
    plans, reqs = make_requests(engine, oracle)
    cg = engine.ConeGeometry(32, 32, 24, 1.0, 40, 28, 36, 1.6, 80.0, 150.0)
    cp = engine.Plan.cone(cg)
    for i in range(2):
        vol = engine.phantom.csg_phantom(32, 24, seed=70 + i, n_parts=5, n_voids=4)
        reqs.insert(2 * i + 1, (cp, cp.forward(vol), 2 + i, 0.001 * (2 * i + 1)))
    srv = engine.Server(hbm_budget_bytes=1 << 34, max_active=4)
    ids = [srv.submit(p, s, it, arr) for (p, s, it, arr) in reqs]
    srv.run()
    assert srv.stats()["completed"] == len(reqs)
    for rid, (p, s, it, _) in zip(ids, reqs):
        f_mix, v_mix, _, _ = srv.result(rid)
        alone = engine.Server(hbm_budget_bytes=1 << 34, max_active=1)
        a = alone.submit(p, s, it, 0.0)
        alone.run()
        f_one, v_one, _, _ = alone.result(a)
        assert f_mix.shape == p.img_shape
        np.testing.assert_array_equal(f_mix, f_one)
        np.testing.assert_array_equal(v_mix, v_one)


def test_server_quality_stop(engine, oracle):
    """Requests with a PSNR target (measured on the GPU after every outer
    iteration against the request's reference image) stop at the first
    iteration that reaches it; a request stops at the same iteration and with
    the same image alone and in a mix (bitwise), within 1e-6 of a solver run of
    that many iterations, and the measured PSNR agrees with numpy's.  Each
    target is set from the request's own PSNR trajectory (a solver stepped one
    outer iteration at a time), so the expected stop iteration is known."""
    G = engine.FanGeometry.covering
    geoms = [G(64, 3.0, 90, 128), G(96, 2.0, 120, 160)]
    plans = [engine.Plan.fan(g) for g in geoms]
    iters = 8
    reqs, expect = [], []
    for i in range(6):
        g, p = geoms[i % 2], plans[i % 2]
        ph = engine.phantom.ellipse_phantom(g.n, seed=500 + i, n_random=3)
        clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
        sino = engine.phantom.poisson_sinogram(clean, 1e4, 600 + i)
        sv = engine.Solver([p], engine.Params(iter_alt=iters))
        sv.set_sino(0, sino)
        sv.reset()
        traj = []
        for _ in range(iters):
            sv.step(1)
            traj.append(engine.phantom.psnr(sv.get(0)[0], ph))
        sv.close()
        if i < 4:  # halfway between the PSNR after 3 and after 4 outer iterations
            target = 0.5 * (traj[2] + traj[3]) if traj[3] > traj[2] else traj[3] - 1e-3
            stop = next(k + 1 for k, t in enumerate(traj) if t >= target)
        else:  # unreachable: iter_alt ends the request
            target, stop = max(traj) + 5.0, iters
        reqs.append((p, sino, iters, ph, target, 0.001 * i))
        expect.append(stop)

    def serve(subset, slots):
        srv = engine.Server(hbm_budget_bytes=1 << 34, max_active=slots)
        ids = [srv.submit_psnr(p, s, it, ph, tgt, arr) for (p, s, it, ph, tgt, arr) in subset]
        srv.run()
        out = [(srv.result(i)[:2], srv.result_info(i)) for i in ids]
        st = srv.stats()
        srv.close()
        return out, st

    mix, st = serve(reqs, 4)
    assert st["completed"] == len(reqs)
    assert st["psnr_stops"] == sum(1 for _, info in mix if info["stopped_by_psnr"])
    for req, stop, ((f, v), info) in zip(reqs, expect, mix):
        p, s, it, ph, tgt, _ = req
        assert info["iterations"] == stop
        assert info["stopped_by_psnr"] == (stop < it)
        assert abs(info["psnr_db"] - engine.phantom.psnr(f, ph)) < 1e-6
        assert (info["psnr_db"] >= tgt) == info["stopped_by_psnr"] or stop == it
        (fa, va), ia = serve([req], 1)[0][0]
        assert ia == info
        np.testing.assert_array_equal(fa, f)
        np.testing.assert_array_equal(va, v)
        solver = engine.Solver([p], engine.Params(iter_alt=info["iterations"]))
        solver.set_sino(0, s)
        solver.run()
        fs, vs = solver.get(0)
        solver.close()
        assert np.linalg.norm(fs - f) <= 1e-6 * np.linalg.norm(fs)
        assert np.linalg.norm(vs - v) <= 1e-6 * np.linalg.norm(vs)

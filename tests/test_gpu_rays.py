"""GPU parity of ray-table plans (at_plan_create_rays): any 2D geometry given
ray by ray through the arguments of the reference tracer forward_proj
(helical/rebin/src/tracing.cpp:22-147).  Same bars as the fan plans:
traversal bit-exact against the FP64 oracle, projections rel-L2 <= 1e-5,
solver f and v rel-L2 <= 1e-4 and PSNR within 0.05 dB.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def msplan(engine):
    g = engine.RayGeometry.msbeam_parallel()
    return g, engine.Plan.rays(g)


def test_uniform_view_table_equals_fan_plan(engine, oracle):
    fg = engine.FanGeometry.covering(128, 0.5, 120, 190)
    rg = engine.RayGeometry.fan_from_view_table(fg.n, fg.pixel_mm, fg.ndets,
                                                [fg.view0_deg + k * fg.view_step_deg for k in range(fg.nviews)],
                                                fg.sod_mm, fg.sdd_mm, fg.det_pitch_deg, fg.off_center)
    pf, pr = engine.Plan.fan(fg), engine.Plan.rays(rg)
    assert pr.stats["kind"] == engine.engine.AT_GEOM_RAYS
    assert pr.stats["segments"] == pf.stats["segments"]
    for v, d in [(0, 0), (7, 95), (60, 189), (119, 3)]:
        a, b = pf.trace_ray(v, d), pr.trace_ray(v, d)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    img = engine.phantom.ellipse_phantom(fg.n, seed=3, n_random=5)
    np.testing.assert_array_equal(pf.forward(img), pr.forward(img))
    sino = np.random.default_rng(2).standard_normal((fg.nviews, fg.ndets)).astype(np.float32)
    ref = oracle.fan_AT(oracle.fan_from_engine(fg), sino.astype(np.float64))
    assert rel_l2(pr.back(sino), ref) <= 1e-5


def test_nonuniform_view_table(engine, oracle):
    rng = np.random.default_rng(5)
    angles = np.sort(rng.uniform(0.0, 360.0, 97))
    g = engine.RayGeometry.fan_from_view_table(160, 1.0, 222, angles, det_pitch_deg=0.19)
    p = engine.Plan.rays(g)
    fan = oracle.fan_from_engine(g)
    assert p.stats["segments"] == oracle.fan_segments(fan)
    for _ in range(200):
        v, d = int(rng.integers(g.nviews)), int(rng.integers(g.ndets))
        ind, wgt, _ = oracle.fan_trace(fan, v, d)
        pix, w = p.trace_ray(v, d)
        np.testing.assert_array_equal(pix, ind)
        np.testing.assert_allclose(w, wgt, atol=2e-4, rtol=0)
    img = engine.phantom.ellipse_phantom(160, seed=8, n_random=6)
    assert rel_l2(p.forward(img), oracle.fan_A(fan, img.astype(np.float64))) <= 1e-5
    sino = rng.standard_normal((g.nviews, g.ndets)).astype(np.float32)
    assert rel_l2(p.back(sino), oracle.fan_AT(fan, sino.astype(np.float64))) <= 1e-5


def test_msbeam_geometry_projectors(engine, oracle, msplan):
    g, p = msplan
    fan = oracle.fan_from_engine(g)
    assert p.stats["segments"] == oracle.fan_segments(fan)
    rng = np.random.default_rng(6)
    rays = [(0, 0), (0, 384), (0, 640), (45, 384), (90, 384), (90, 767), (179, 1)]
    rays += [(int(rng.integers(180)), int(rng.integers(768))) for _ in range(300)]
    for v, d in rays:
        ind, wgt, _ = oracle.fan_trace(fan, v, d)
        pix, w = p.trace_ray(v, d)
        np.testing.assert_array_equal(pix, ind, err_msg=f"ray ({v},{d})")
        np.testing.assert_allclose(w, wgt, atol=2e-4, rtol=0)
    ph = oracle.ms_phantom()
    assert rel_l2(p.forward(ph), oracle.fan_A(fan, ph.astype(np.float64))) <= 1e-5
    sino = rng.random((180, 768)).astype(np.float32)
    got = p.back(sino)
    assert rel_l2(got, oracle.fan_AT(fan, sino.astype(np.float64))) <= 1e-5
    np.testing.assert_array_equal(got, p.back(sino))  # deterministic


def test_msbeam_geometry_solver(engine, oracle, msplan):
    """Two outer iterations of the AT solver on msbeam's phantom and geometry
    (the count that passes msbeam's own PSNR), against the FP64 oracle."""
    g, p = msplan
    fan = oracle.fan_from_engine(g)
    ph = oracle.ms_phantom()
    sino = p.forward(ph)
    prm = engine.Params(iter_alt=2)
    S = engine.Solver([p], prm)
    S.set_sino(0, sino)
    S.run()
    f, v = S.get(0)
    fo, vo, _ = oracle.solve(fan, sino.astype(np.float64), prm.alpha, prm.beta, prm.epsilon, prm.iter_alt,
                             prm.iter_image, prm.iter_edge)
    assert rel_l2(f, fo) <= 1e-4, rel_l2(f, fo)
    assert rel_l2(v, vo) <= 1e-4, rel_l2(v, vo)
    peak = float(ph.max())
    assert abs(engine.phantom.psnr(f, ph, peak) - engine.phantom.psnr(fo, ph, peak)) <= 0.05


def test_server_accepts_ray_tables(engine, msplan):
    g, p = msplan
    ph = engine.phantom.ellipse_phantom(512, seed=4, n_random=4)
    sino = p.forward(ph)
    prm = engine.Params(iter_alt=1)
    S = engine.Solver([p], prm)
    S.set_sino(0, sino)
    S.run()
    f_alone, _ = S.get(0)
    srv = engine.Server(8 << 30, 4, prm, fp_rays_per_thread=p.stats["fp_rays_per_thread"])
    rid = srv.submit(p, sino, prm.iter_alt, arrival_s=0.0)
    srv.run()
    f_srv = srv.result(rid)[0]
    np.testing.assert_array_equal(f_srv, f_alone)

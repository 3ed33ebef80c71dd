"""GPU parity at the benchmark configurations' own sizes, against the FP64
oracle restatement of origin/GoldenC/src/main.c:35-360 with the fan tracer of
helical/rebin/src/tracing.cpp:22-147 (the oracle is pinned bit for bit to the
reference's sources by test_oracle.py and the golden vectors).

  C1  256^2 (1 mm), 360 views x 512 detectors, Poisson I0 = 1e4, 20 outer
      iterations: the whole reconstruction.  f and v rel-L2 <= 1e-4, PSNR within
      0.05 dB of the oracle's, identical exit branches.
  C2  512^2 (0.75 mm), 720 views x 888 detectors: the projectors at full size
      (forward rel-L2 <= 1e-5; back projection of a sinogram <= 1e-5, of
      zero-mean noise within 1e-5 of the back projection of its magnitude;
      segment count and sampled traversals exact); and the
      50-iteration reconstruction, bounded by the problem's own conditioning
      (below).
  C3  the uneven slice shapes (grids 256/384/512 over a 384 mm field, 360/540/
      720 views, 512/768/888 detectors): projectors at full size and a short
      reconstruction.

The C2 reconstruction after 50 outer iterations is not stable to 1e-4 in any
arithmetic: the oracle itself, run in FP64 on the sinogram perturbed by 1e-7
relative (below FP32 resolution), moves by 3e-4 .. 3e-3 from the 10th outer
iteration on, where the median filter and the 1.1x instability revert make
discontinuous choices.  So the test holds the engine to that yardstick: at
every checkpoint its distance from the FP64 run must stay within K_COND times
the FP64-vs-perturbed-FP64 distance (and within 1e-4 while that distance is
below 1e-6), its PSNR within 0.05 dB of the FP64 run's, and its exit branches
identical.
"""
import dataclasses

import numpy as np
import pytest

from medimage_gb300 import configs

pytestmark = pytest.mark.gpu

FP_TOL = 1e-5     # one projection against FP64
SOLVE_TOL = 1e-4  # final f and v against FP64
PSNR_TOL = 0.05   # dB
K_COND = 10.0     # engine gap / FP64 perturbation gap, C2 after the median steps


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def exits(trace_gpu):
    return [(o, s, k, e) for (o, s, k, e, _) in trace_gpu if e != 0]


def exits_oracle(trace_or):
    return [(o, s, k, e) for (o, s, k, _, e) in trace_or if e != 0]


def spec_data(engine, oracle, spec):
    """The configuration's seeded phantom and its noisy sinogram (the oracle's
    FP64 projection, Poisson noise, -log), as the benchmark builds them."""
    g = spec.geom
    ph = engine.phantom.ellipse_phantom(g.n, seed=spec.seed, n_random=spec.n_random)
    clean = oracle.fan_A(oracle.fan_from_engine(g), ph.astype(np.float64))
    sino = engine.phantom.poisson_sinogram(clean, spec.i0, spec.seed + 1000)
    return ph, sino


def check_projectors(engine, oracle, g, plan, n_sample=400, seed=0):
    fan = oracle.fan_from_engine(g)
    assert plan.stats["segments"] == oracle.fan_segments(fan)
    rng = np.random.default_rng(seed)
    rays = [(v, d) for v in (0, g.nviews // 8, g.nviews // 4, g.nviews // 2, g.nviews - 1)
            for d in (0, 1, g.ndets // 2 - 1, g.ndets // 2, g.ndets - 1)]
    rays += [(int(rng.integers(g.nviews)), int(rng.integers(g.ndets))) for _ in range(n_sample)]
    for v, d in rays:
        ind, _, _ = oracle.fan_trace(fan, v, d)
        pix, _ = plan.trace_ray(v, d)
        np.testing.assert_array_equal(pix, ind, err_msg=f"ray ({v},{d})")
    img = engine.phantom.ellipse_phantom(g.n, seed=seed + 7, n_random=10)
    got = plan.forward(img)
    ref = oracle.fan_A(fan, img.astype(np.float64))
    assert rel_l2(got, ref) <= FP_TOL, rel_l2(got, ref)
    # back projection of a sinogram (the first back projection of a
    # reconstruction, r = g): 1e-5
    sino = ref.astype(np.float32)
    got = plan.back(sino)
    assert rel_l2(got, oracle.fan_AT(fan, sino.astype(np.float64))) <= FP_TOL
    # of zero-mean noise: the pixel sums cancel, so the error is measured
    # against the back projection of |r|, the size of the terms summed.  Each
    # FP32 weight carries about half an ulp of its crossing parameter (3e-5 mm
    # at 500 mm along the ray); a cancelling sum of ~1000 terms keeps that
    # error while its value shrinks (rel-L2 1.2e-5 to 1.5e-5 at C2 and C3)
    sino = rng.standard_normal((g.nviews, g.ndets)).astype(np.float32)
    got = plan.back(sino)
    ref = oracle.fan_AT(fan, sino.astype(np.float64))
    scale = np.linalg.norm(oracle.fan_AT(fan, np.abs(sino).astype(np.float64)))
    assert np.linalg.norm(got - ref) <= FP_TOL * scale, (rel_l2(got, ref), np.linalg.norm(got - ref) / scale)


@pytest.mark.parametrize("mode", [0, 1])
def test_c1_reconstruction_matches_fp64(engine, oracle, mode):
    """Exact mode (GoldenC's projection count) and linear mode (the CG's
    sinograms updated by linearity, A(f + c p) = Af + c Ap: 12 forward
    projections per outer iteration instead of 29) against the same FP64
    solve of GoldenC's algorithm."""
    spec = configs.c1()
    ph, sino = spec_data(engine, oracle, spec)
    prm = dataclasses.replace(configs.params_for(spec), mode=mode)
    plan = engine.Plan.fan(spec.geom)
    S = engine.Solver([plan], prm)
    S.set_sino(0, sino)
    S.run()
    f, v = S.get(0)
    fo, vo, tr = oracle.solve(oracle.fan_from_engine(spec.geom), sino.astype(np.float64), prm.alpha, prm.beta,
                              prm.epsilon, prm.iter_alt, prm.iter_image, prm.iter_edge)
    assert rel_l2(f, fo) <= SOLVE_TOL, rel_l2(f, fo)
    assert rel_l2(v, vo) <= SOLVE_TOL, rel_l2(v, vo)
    assert abs(engine.phantom.psnr(f, ph) - engine.phantom.psnr(fo, ph)) <= PSNR_TOL
    assert exits(S.trace(0)) == exits_oracle(tr)
    S.close()


def test_c2_projectors_match_fp64(engine, oracle):
    g = configs.c2().geom
    plan = engine.Plan.fan(g)
    check_projectors(engine, oracle, g, plan, n_sample=600, seed=2)


def test_c2_back_projection_of_low_count_residuals(engine, oracle):
    """The back projector rounds every term w*r to a multiple of one quantum per
    call, q = 2^(e - b) with 2^(e-1) <= 1.5 pixel max|r| < 2^e and b = 22 bits
    at C2, so the sinogram's largest |r| sets the precision of every term.  The
    residual of a low-count scan (Poisson I0 = 200: photon-starved rays clamp to
    one count) must back project within 1e-5 of FP64; with planted outliers
    1e4 times its largest value (far beyond what the solver meets), each pixel
    must stay within the worst-case bound T q / 2, T the most terms a pixel can
    receive (at most 5 rays per view cross a C2 pixel, 720 views)."""
    spec = configs.c2()
    g = spec.geom
    fan = oracle.fan_from_engine(g)
    plan = engine.Plan.fan(g)
    ph = engine.phantom.ellipse_phantom(g.n, seed=9, n_random=20)
    clean = oracle.fan_A(fan, ph.astype(np.float64))
    noisy = engine.phantom.poisson_sinogram(clean, 200.0, 77).astype(np.float64)
    r32 = (noisy - clean).astype(np.float32)
    got = plan.back(r32)
    ref = oracle.fan_AT(fan, r32.astype(np.float64))
    assert rel_l2(got, ref) <= FP_TOL, rel_l2(got, ref)
    rng = np.random.default_rng(8)
    out = r32.copy()
    idx = rng.choice(out.size, 20, replace=False)
    out.ravel()[idx] = np.abs(r32).max() * 1e4 * rng.choice([-1.0, 1.0], 20)
    got = plan.back(out).astype(np.float64)
    ref = oracle.fan_AT(fan, out.astype(np.float64))
    _, e = np.frexp(1.5 * g.pixel_mm * float(np.abs(out).max()))
    q = np.ldexp(1.0, int(e) - 22)
    assert np.abs(got - ref).max() <= 5 * g.nviews * q / 2 + 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("n,nv,nd", [(384, 540, 768), (384, 720, 512), (256, 540, 888), (512, 360, 768)])
def test_c3_shapes_projectors_match_fp64(engine, oracle, n, nv, nd):
    g = engine.FanGeometry.covering(n, 384.0 / n, nv, nd)
    plan = engine.Plan.fan(g)
    check_projectors(engine, oracle, g, plan, n_sample=200, seed=n + nv + nd)


def test_c3_shape_reconstruction_matches_fp64(engine, oracle):
    """A C3 slice (384^2, 540 views x 768 detectors) for 4 outer iterations."""
    spec = configs.SliceSpec(engine.FanGeometry.covering(384, 1.0, 540, 768), 7e3, 1033, 0, 4)
    ph, sino = spec_data(engine, oracle, spec)
    prm = configs.params_for(spec)
    plan = engine.Plan.fan(spec.geom)
    S = engine.Solver([plan], prm)
    S.set_sino(0, sino)
    S.run()
    f, v = S.get(0)
    fo, vo, tr = oracle.solve(oracle.fan_from_engine(spec.geom), sino.astype(np.float64), prm.alpha, prm.beta,
                              prm.epsilon, prm.iter_alt, prm.iter_image, prm.iter_edge)
    assert rel_l2(f, fo) <= SOLVE_TOL, rel_l2(f, fo)
    assert rel_l2(v, vo) <= SOLVE_TOL, rel_l2(v, vo)
    assert abs(engine.phantom.psnr(f, ph) - engine.phantom.psnr(fo, ph)) <= PSNR_TOL
    assert exits(S.trace(0)) == exits_oracle(tr)
    S.close()


def test_c2_reconstruction_within_its_conditioning(engine, oracle):
    spec = configs.c2()
    g = spec.geom
    fan = oracle.fan_from_engine(g)
    ph, sino32 = spec_data(engine, oracle, spec)
    sino = sino32.astype(np.float64)
    pert = sino * (1.0 + 1e-7 * np.random.default_rng(0).standard_normal(sino.shape))
    prm = configs.params_for(spec)
    marks = [1, 2, 3, 5] + list(range(10, spec.iters + 1, 10))

    def oracle_run(s):
        f, v, snaps, trace = np.zeros((g.n, g.n)), np.ones((g.n, g.n)), {}, []
        for it in range(1, spec.iters + 1):
            f, ti = oracle.image_step(fan, s, f, v, prm.alpha, prm.epsilon, prm.iter_image)
            v, te = oracle.edge_step(f, v, prm.alpha, prm.beta, prm.epsilon, prm.iter_edge)
            trace += [(it,) + tuple(t[1:]) for t in ti] + [(it,) + tuple(t[1:]) for t in te]
            if it in marks:
                snaps[it] = (f.copy(), v.copy())
        return snaps, trace

    ref, ref_trace = oracle_run(sino)
    alt, _ = oracle_run(pert)
    plan = engine.Plan.fan(g)
    S = engine.Solver([plan], prm)
    S.set_sino(0, sino32)
    S.reset()
    report = []
    for it in range(1, spec.iters + 1):
        S.step(1)
        if it not in marks:
            continue
        f, v = S.get(0)
        for name, got, a, b in (("f", f, ref[it][0], alt[it][0]), ("v", v, ref[it][1], alt[it][1])):
            gap, cond = rel_l2(got, a), rel_l2(b, a)
            bar = SOLVE_TOL if cond < 1e-6 else K_COND * cond
            report.append((it, name, gap, cond))
            assert gap <= max(bar, SOLVE_TOL), (it, name, gap, cond)
    f, v = S.get(0)
    assert abs(engine.phantom.psnr(f, ph) - engine.phantom.psnr(ref[spec.iters][0], ph)) <= PSNR_TOL
    assert exits(S.trace(0)) == exits_oracle(ref_trace)
    S.close()


def test_c2_plain_fp32_alpha_plan(engine, oracle):
    """The plain form (the traversal's lambda arithmetic in FP32, no FP64 on the
    GPU) at C2: it builds, both projectors run, and its departures from the
    reference's traversal stay small; the FP64-alpha plan is the exact one."""
    g = configs.c2().geom
    fan = oracle.fan_from_engine(g)
    p32 = engine.Plan.fan(g, alpha="fp32")
    s_ref = oracle.fan_segments(fan)
    assert abs(p32.stats["segments"] - s_ref) <= 1e-4 * s_ref
    img = engine.phantom.ellipse_phantom(g.n, seed=12, n_random=20)
    ref = oracle.fan_A(fan, img.astype(np.float64))
    assert rel_l2(p32.forward(img), ref) <= 1e-3
    sino = np.random.default_rng(12).standard_normal((g.nviews, g.ndets)).astype(np.float32)
    assert rel_l2(p32.back(sino), oracle.fan_AT(fan, sino.astype(np.float64))) <= 1e-3
    with pytest.raises(ValueError):
        engine.Plan.fan(g, alpha="fp16")

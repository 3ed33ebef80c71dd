"""PSNR and SSIM on the GPU against numpy restatements of the same formulas
(PSNR.m; Wang et al. 2004 SSIM with ssim_index.m's defaults)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ssim_numpy(x, y, L):
    from scipy.signal import correlate2d

    ax = np.arange(11) - 5.0
    g = np.exp(-(ax[:, None] ** 2 + ax[None, :] ** 2) / (2 * 1.5 ** 2))
    g /= g.sum()
    x = x.astype(np.float64)
    y = y.astype(np.float64)
    f = lambda a: correlate2d(a, g, mode="valid")  # noqa: E731
    mx, my = f(x), f(y)
    vx, vy, cxy = f(x * x) - mx * mx, f(y * y) - my * my, f(x * y) - mx * my
    c1, c2 = (0.01 * L) ** 2, (0.03 * L) ** 2
    return float(np.mean((2 * mx * my + c1) * (2 * cxy + c2) / ((mx * mx + my * my + c1) * (vx + vy + c2))))


def test_psnr_and_ssim_match_numpy(engine):
    rng = np.random.default_rng(8)
    ref = engine.phantom.ellipse_phantom(128, seed=4, n_random=6)
    x = (ref + rng.normal(0, 0.001, ref.shape)).astype(np.float32)
    q = engine.quality(x, ref, dynamic_range=0.02)
    assert abs(q["psnr_db"] - engine.phantom.psnr(x, ref)) < 1e-9
    assert abs(q["ssim"] - ssim_numpy(x, ref, 0.02)) < 1e-9
    q256 = engine.quality(x, ref, peak=256.0, dynamic_range=255.0)
    assert abs(q256["psnr_db"] - engine.phantom.psnr(x, ref, peak=256.0)) < 1e-9
    assert abs(engine.quality(ref, ref, dynamic_range=0.02)["ssim"] - 1.0) < 1e-12

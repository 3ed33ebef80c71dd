"""Seeded synthetic inputs: ellipse phantoms and Poisson-noisy sinograms.

The reference ships no phantom or noise model for this path (GoldenC reads a
missing phantom.dat and projects it without noise), so these generators define
the workloads:

* modified Shepp-Logan (Toft's ten-ellipse table, intensities 0..1) scaled to
  attenuation 0..0.02 /mm, each centre jittered by up to +-2 pixels;
* optional small random ellipses (semi-axes 2..8 px, contrast +-0.002 /mm);
* data: line integrals of the pixel image through the engine's own projector,
  Poisson counts N ~ Poisson(I0 exp(-p)), sinogram -log(max(N, 1) / I0).

Coordinates: pixel (x, y) (x = first, slow index) has its centre at normalised
((x + 0.5 - n/2) / (n/2), (y + 0.5 - n/2) / (n/2)).
"""
from __future__ import annotations

import numpy as np

# Modified Shepp-Logan (Toft 1996): intensity, semi-axis a, semi-axis b,
# centre x0, centre y0, rotation (degrees)
MODIFIED_SHEPP_LOGAN = (
    (1.0, 0.69, 0.92, 0.0, 0.0, 0.0),
    (-0.8, 0.6624, 0.8740, 0.0, -0.0184, 0.0),
    (-0.2, 0.1100, 0.3100, 0.22, 0.0, -18.0),
    (-0.2, 0.1600, 0.4100, -0.22, 0.0, 18.0),
    (0.1, 0.2100, 0.2500, 0.0, 0.35, 0.0),
    (0.1, 0.0460, 0.0460, 0.0, 0.1, 0.0),
    (0.1, 0.0460, 0.0460, 0.0, -0.1, 0.0),
    (0.1, 0.0460, 0.0230, -0.08, -0.605, 0.0),
    (0.1, 0.0230, 0.0230, 0.0, -0.606, 0.0),
    (0.1, 0.0230, 0.0460, 0.06, -0.605, 0.0),
)


def _ellipses(n: int, rng: np.random.Generator, scale: float, jitter_px: float, n_random: int,
              radius_px=(2.0, 8.0), contrast: float = 0.002):
    half = n / 2.0
    out = []
    for (A, a, b, x0, y0, phi) in MODIFIED_SHEPP_LOGAN:
        jx, jy = rng.uniform(-jitter_px, jitter_px, size=2) / half
        out.append((A * scale, a, b, x0 + jx, y0 + jy, phi))
    for _ in range(n_random):
        a, b = rng.uniform(radius_px[0], radius_px[1], size=2) / half
        r = 0.55 * np.sqrt(rng.uniform())
        t = rng.uniform(0, 2 * np.pi)
        phi = rng.uniform(0, 180)
        sign = 1.0 if rng.uniform() < 0.5 else -1.0
        out.append((sign * contrast, a, b, r * np.cos(t), r * np.sin(t), phi))
    return out


def ellipse_phantom(n: int, seed: int, *, scale: float = 0.02, jitter_px: float = 2.0, n_random: int = 0,
                    radius_px=(2.0, 8.0), contrast: float = 0.002) -> np.ndarray:
    """n x n FP32 attenuation image (1/mm) with the seeded ellipse table."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    half = n / 2.0
    c = (np.arange(n, dtype=np.float64) + 0.5 - half) / half
    X, Y = np.meshgrid(c, c, indexing="ij")
    img = np.zeros((n, n), np.float64)
    for (A, a, b, x0, y0, phi) in _ellipses(n, rng, scale, jitter_px, n_random, radius_px, contrast):
        th = np.deg2rad(phi)
        xr = (X - x0) * np.cos(th) + (Y - y0) * np.sin(th)
        yr = -(X - x0) * np.sin(th) + (Y - y0) * np.cos(th)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += A
    return np.maximum(img, 0.0).astype(np.float32)


def poisson_sinogram(clean: np.ndarray, i0: float, seed: int) -> np.ndarray:
    """-log(max(N,1)/I0) with N ~ Poisson(I0 exp(-p)), FP32."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    lam = i0 * np.exp(-np.asarray(clean, np.float64))
    counts = rng.poisson(lam)
    return (-np.log(np.maximum(counts, 1) / i0)).astype(np.float32)


def psnr(x: np.ndarray, ref: np.ndarray, peak: float | None = None) -> float:
    """10 log10(peak^2 / MSE); peak defaults to max(ref) (the phantom maximum)."""
    ref = np.asarray(ref, np.float64)
    mse = float(np.mean((np.asarray(x, np.float64) - ref) ** 2))
    peak = float(ref.max()) if peak is None else peak
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def msbeam_phantom() -> np.ndarray:
    """The built-in test image of msbeam/CPU_OpenMP (main.c:92-181): 512 x 512
    unit pixels, a disc of 1 (radius 180), four discs of 2, 2.5, 2.25 and 3
    (radius 30, centres +-80), a ring of 1.25 and two bar patterns of 2.
    Distances are evaluated in FP32 as there, so the image is bit-identical to
    the one that program reconstructs."""
    n = 512
    f = np.zeros((n, n), np.float32)
    x = (np.arange(n, dtype=np.float64) - 255.5).astype(np.float32)[:, None]
    y = (np.arange(n, dtype=np.float64) - 255.5).astype(np.float32)[None, :]

    def dist(cx: float, cy: float) -> np.ndarray:
        dx = (x - np.float32(cx)).astype(np.float32)
        dy = (y - np.float32(cy)).astype(np.float32)
        s = (dx * dx).astype(np.float32) + (dy * dy).astype(np.float32)
        return np.sqrt(s.astype(np.float64)).astype(np.float32).astype(np.float64)

    for cx, cy, r, val in ((0, 0, 180.0, 1.0), (80, 80, 30.0, 2.0), (-80, 80, 30.0, 2.5), (80, -80, 30.0, 2.25),
                           (-80, -80, 30.0, 3.0)):
        f[dist(cx, cy) <= r] = val
    d = dist(0, 120)
    f[(d >= 29.0) & (d <= 30.0)] = 1.25
    for r0 in (165, 340):
        for p in range(7):
            c0, c1 = (238, 256) if p % 2 == 0 else (256, 274)
            f[r0 + 2 * p:r0 + 2 * p + 2, c0:c1] = 2.0
    return f


def csg_phantom(n: int, nz: int, seed: int = 0, n_parts: int | None = None, n_voids: int = 50,
                mu: float = 0.02) -> np.ndarray:
    """Seeded industrial-CT volume (nz, n, n): a part built from 8-16 solid
    ellipsoids and z-axis cylinders (attenuation mu..1.5 mu per voxel) inside
    the inscribed cylinder, with `n_voids` small spherical voids.  Each
    primitive is evaluated inside its bounding box only."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    vol = np.zeros((nz, n, n), np.float32)
    parts = int(rng.integers(8, 17)) if n_parts is None else n_parts
    c, cz = (n - 1) / 2.0, (nz - 1) / 2.0

    def box(center, radii):
        lo = [max(0, int(np.floor(center[k] - radii[k]))) for k in range(3)]
        hi = [min(s, int(np.ceil(center[k] + radii[k])) + 1) for k, s in enumerate((nz, n, n))]
        z, x, y = np.ogrid[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        return (slice(lo[0], hi[0]), slice(lo[1], hi[1]), slice(lo[2], hi[2])), z, x, y

    for _ in range(parts):
        rz = rng.uniform(0.1, 0.35) * nz
        rx, ry = rng.uniform(0.06, 0.22, 2) * n
        cen = (cz + rng.uniform(-0.2, 0.2) * nz, c + rng.uniform(-0.2, 0.2) * n, c + rng.uniform(-0.2, 0.2) * n)
        val = np.float32(mu * rng.uniform(1.0, 1.5))
        sl, z, x, y = box(cen, (rz, rx, ry))
        if rng.uniform() < 0.5:  # ellipsoid
            m = ((z - cen[0]) / rz) ** 2 + ((x - cen[1]) / rx) ** 2 + ((y - cen[2]) / ry) ** 2 <= 1.0
        else:  # cylinder along z
            m = (((x - cen[1]) / rx) ** 2 + ((y - cen[2]) / ry) ** 2 <= 1.0) & (np.abs(z - cen[0]) <= rz)
        sub = vol[sl]
        sub[np.broadcast_to(m, sub.shape)] = val
    for _ in range(n_voids):
        r = rng.uniform(0.005, 0.02) * n
        cen = (cz + rng.uniform(-0.3, 0.3) * nz, c + rng.uniform(-0.25, 0.25) * n, c + rng.uniform(-0.25, 0.25) * n)
        sl, z, x, y = box(cen, (r, r, r))
        m = (z - cen[0]) ** 2 + (x - cen[1]) ** 2 + (y - cen[2]) ** 2 <= r * r
        sub = vol[sl]
        sub[np.broadcast_to(m, sub.shape)] = 0.0
    return vol

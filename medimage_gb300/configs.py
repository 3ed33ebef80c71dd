"""The benchmark workloads as geometry + parameters.

C1  256^2 (1 mm), 360 views x 512 detectors, I0 1e4, 20 AT iterations
C2  512^2 (0.75 mm), 720 views x 888 detectors, I0 5e3, 50 AT iterations,
    ten Shepp-Logan ellipses plus 20 random small ellipses
C3  64 uneven slices: grid {256,384,512}^2 over a 384 mm field, views
    {360,540,720}, detectors {512,768,888}, I0 in [2e3, 2e4], 30 iterations
C4  512^3 cone beam (0.2 mm voxels), 720 views of a 768 x 1024 detector
    (0.4 mm), SOD 600 / SDD 1000 mm, CSG part of 8-16 ellipsoids/cylinders
    with 50 voids, I0 2e4, 10 AT iterations
Fan: SOD 541 mm, SDD 949 mm, equiangular detector just covering the image's
circumscribed circle, views evenly over 360 degrees.  AT weights are GoldenC's
defaults (alpha 1000, beta 0.002, epsilon 1e-4, 10 image and 10 edge
iterations per outer iteration).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .engine import ConeGeometry, FanGeometry, Params


@dataclass
class SliceSpec:
    geom: FanGeometry
    i0: float
    seed: int
    n_random: int
    iters: int


def c1(seed: int = 1) -> SliceSpec:
    return SliceSpec(FanGeometry.covering(256, 1.0, 360, 512), 1e4, seed, 0, 20)


def c2(seed: int = 2) -> SliceSpec:
    return SliceSpec(FanGeometry.covering(512, 0.75, 720, 888), 5e3, seed, 20, 50)


def c3(count: int = 64, seed: int = 3) -> list[SliceSpec]:
    rng = np.random.default_rng(np.random.PCG64(seed))
    out = []
    for i in range(count):
        n = int(rng.choice([256, 384, 512]))
        nv = int(rng.choice([360, 540, 720]))
        nd = int(rng.choice([512, 768, 888]))
        i0 = float(rng.uniform(2e3, 2e4))
        out.append(SliceSpec(FanGeometry.covering(n, 384.0 / n, nv, nd), i0, 1000 + i, 0, 30))
    return out


@dataclass
class VolumeSpec:
    geom: ConeGeometry
    i0: float
    seed: int
    iters: int


def c4(seed: int = 4, n: int = 512, nz: int = 512) -> VolumeSpec:
    """C4; smaller volumes keep the field of view (voxel 0.2 * 512 / n mm)."""
    return VolumeSpec(ConeGeometry(n, n, nz, 0.2 * 512 / n, 720, 768, 1024, 0.4, 600.0, 1000.0), 2e4, seed, 10)


def params_for(spec, mode: int = 0) -> Params:
    return Params(iter_alt=spec.iters, mode=mode)

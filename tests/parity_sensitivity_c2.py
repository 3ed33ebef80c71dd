"""How well-conditioned is the C2 reconstruction itself?  (A measurement
script, not a test: it needs a GPU and about four minutes of CPU time.)

At the C2 configuration (512^2, 720 x 888 fan, I0 = 5e3, 50 outer iterations)
the engine's f differs from the FP64 oracle's by ~1.7e-3 rel-L2 (v: ~1e-6),
with PSNR within 0.001 dB and the same exit branches.  This script shows where
that comes from: it runs the FP64 oracle twice, once on the sinogram and once
on the sinogram perturbed by 1e-7 relative (below FP32 rounding), and prints,
every few outer iterations, the engine-vs-FP64 gap next to the
FP64-vs-perturbed-FP64 gap.

    python tests/parity_sensitivity_c2.py
"""
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import medimage_gb300 as mg  # noqa: E402
from medimage_gb300 import configs  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def rel(x, y):
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def main():
    spec = configs.c2()
    g = spec.geom
    fan = po.fan_from_engine(g)
    ph = mg.phantom.ellipse_phantom(g.n, seed=spec.seed, n_random=spec.n_random)
    clean = po.fan_A(fan, ph.astype(np.float64))
    sino = mg.phantom.poisson_sinogram(clean, spec.i0, spec.seed + 1000).astype(np.float64)
    pert = sino * (1 + 1e-7 * np.random.default_rng(0).standard_normal(sino.shape))
    plan = mg.Plan.fan(g)
    S = mg.Solver([plan], mg.Params(iter_alt=spec.iters))
    S.set_sino(0, sino.astype(np.float32))
    S.reset()
    marks = [1, 2, 3] + list(range(5, spec.iters + 1, 5))

    def oracle_run(s):
        f, v, snaps = np.zeros((g.n, g.n)), np.ones((g.n, g.n)), {}
        for it in range(1, spec.iters + 1):
            f, _ = po.image_step(fan, s, f, v, 1000.0, 1e-4, 10)
            v, _ = po.edge_step(f, v, 1000.0, 0.002, 1e-4, 10)
            if it in marks:
                snaps[it] = (f.copy(), v.copy())
        return snaps

    t = time.time()
    a, b = oracle_run(sino), oracle_run(pert)
    for it in range(1, spec.iters + 1):
        S.step(1)
        if it in marks:
            f, v = S.get(0)
            print(json.dumps({"it": it, "gpu_vs_fp64_f": rel(f, a[it][0]), "fp64_pert_vs_fp64_f": rel(b[it][0], a[it][0]),
                              "gpu_vs_fp64_v": rel(v, a[it][1]), "fp64_pert_vs_fp64_v": rel(b[it][1], a[it][1])}),
                  flush=True)
    print("oracle seconds", round(time.time() - t, 1))


if __name__ == "__main__":
    main()

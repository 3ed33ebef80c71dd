"""Time the forward and back projectors alone on one workload geometry.

    python -m medimage_gb300.projbench [--config c1|c2|c4] [--n N] [--reps N] [--which fp,bp]

Prints one JSON line per projector: average launch time (CUDA events on the
launching stream), algorithmic bytes per launch (forward 4 S + 4 R, back
4 S + 4 P; S segments, R rays, P pixels or voxels) and the resulting GB/s.
Used as the command under the profiler as well.  c4 is the 512^3 cone beam
(--n shrinks the volume, same field of view).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np

from . import configs, engine, phantom


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c4"])
    ap.add_argument("--n", type=int, default=512, help="c4 volume edge (voxels)")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--which", default="fp,bp")
    args = ap.parse_args()
    if args.config == "c4":
        spec = configs.c4(n=args.n, nz=args.n)
        plan = engine.Plan.cone(spec.geom)
        img = phantom.csg_phantom(args.n, args.n, seed=spec.seed)
        names = ("cone_fp_kernel", "cone_bp_kernel")
    else:
        spec = getattr(configs, args.config)()
        plan = engine.Plan.fan(spec.geom)
        img = phantom.ellipse_phantom(plan.n, seed=spec.seed, n_random=spec.n_random)
        names = ("fan_fp_kernel", "fan_bp_kernel")
    L = engine.lib()
    st = C.c_void_p()
    engine._check("at_stream_create", L.at_stream_create(C.byref(st)))
    sino = np.random.default_rng(0).standard_normal(plan.sino_shape).astype(np.float32)
    bufs = {}
    for name, arr in (("img", img), ("sino", sino), ("img_out", img), ("sino_out", sino)):
        p = C.c_void_p()
        engine._check("at_dev_alloc", L.at_dev_alloc(C.byref(p), arr.nbytes))
        engine._check("h2d", L.at_memcpy_h2d(p, arr.ctypes.data, arr.nbytes, st))
        bufs[name] = p.value
    import torch

    ts = torch.cuda.ExternalStream(st.value)
    S, R, P = plan.stats["segments"], plan.stats["rays"], int(np.prod(plan.img_shape))
    jobs = {
        "fp": (names[0], lambda: plan.forward_dev(bufs["img"], bufs["sino_out"], st.value), 4 * S + 4 * R),
        "bp": (names[1], lambda: plan.back_dev(bufs["sino"], bufs["img_out"], st.value), 4 * S + 4 * P),
    }
    for key in args.which.split(","):
        kname, fn, nbytes = jobs[key]
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ts)
        for _ in range(args.reps):
            fn()
        e1.record(ts)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.reps
        print(json.dumps({"kernel": kname, "config": args.config, "shape": list(plan.img_shape),
                          "launch_ms": round(ms, 5), "gsegs_per_s": round(S / (ms / 1e3) / 1e9, 2),
                          "algorithmic_bytes": nbytes, "gbs": round(nbytes / (ms / 1e3) / 1e9, 1),
                          "segments": S, "rays": R, "pixels": P}))
    for p in bufs.values():
        L.at_dev_free(C.c_void_p(p))


if __name__ == "__main__":
    main()

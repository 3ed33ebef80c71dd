"""Time the forward and back projectors alone on one workload geometry.

    python -m medimage_gb300.projbench [--config c1|c2] [--reps N] [--which fp,bp]

Prints one JSON line per projector: average launch time (CUDA events on the
launching stream), algorithmic bytes per launch (forward 4 S + 4 R, back
4 S + 4 P; S segments, R rays, P pixels) and the resulting GB/s.  Used as the
command under the profiler as well.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np

from . import configs, engine, phantom


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2", choices=["c1", "c2"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--which", default="fp,bp")
    args = ap.parse_args()
    spec = getattr(configs, args.config)()
    plan = engine.Plan.fan(spec.geom)
    L = engine.lib()
    st = C.c_void_p()
    engine._check("at_stream_create", L.at_stream_create(C.byref(st)))
    n, nv, nd = plan.n, plan.nviews, plan.ndets
    img = phantom.ellipse_phantom(n, seed=spec.seed, n_random=spec.n_random)
    sino = np.random.default_rng(0).standard_normal((nv, nd)).astype(np.float32)
    bufs = {}
    for name, arr in (("img", img), ("sino", sino), ("img_out", img), ("sino_out", sino)):
        p = C.c_void_p()
        engine._check("at_dev_alloc", L.at_dev_alloc(C.byref(p), arr.nbytes))
        engine._check("h2d", L.at_memcpy_h2d(p, arr.ctypes.data, arr.nbytes, st))
        bufs[name] = p.value
    import torch

    ts = torch.cuda.ExternalStream(st.value)
    S, R, P = plan.stats["segments"], plan.stats["rays"], n * n
    jobs = {
        "fp": ("fan_fp_kernel", lambda: plan.forward_dev(bufs["img"], bufs["sino_out"], st.value), 4 * S + 4 * R),
        "bp": ("fan_bp_kernel", lambda: plan.back_dev(bufs["sino"], bufs["img_out"], st.value), 4 * S + 4 * P),
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
        print(json.dumps({"kernel": kname, "config": args.config, "launch_ms": round(ms, 5),
                          "algorithmic_bytes": nbytes, "gbs": round(nbytes / (ms / 1e3) / 1e9, 1),
                          "segments": S, "rays": R, "pixels": P}))
    for p in bufs.values():
        L.at_dev_free(C.c_void_p(p))


if __name__ == "__main__":
    main()

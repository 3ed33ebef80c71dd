"""Time the forward and back projectors alone on one workload geometry.

    python -m medimage_gb300.projbench [--config c1|c2|c4] [--n N] [--reps N] [--which fp,bp] [--group G]
                                       [--variant l1|views,rays,rows] [--bp runs|table]

Prints one JSON line per projector: average launch time (CUDA events on the
launching stream around each launch, L2 flushed before each unless --warm), algorithmic bytes per launch (forward 4 S + 4 R, back
4 S + 4 P; S segments, R rays, P pixels or voxels) and the resulting GB/s.
Used as the command under the profiler as well.  c4 is the 512^3 cone beam
(--n shrinks the volume, same field of view).  --group G (2D) projects G
images of the plan together through a projection set, the grouped kernels
(one walk of the plan for up to four images); bytes are then G times one
image's.
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
    ap.add_argument("--group", type=int, default=1, help="images projected together (2D plans)")
    ap.add_argument("--warm", action="store_true", help="no L2 flush between timed launches")
    ap.add_argument("--variant", default="",
                    help="forward projector of 2D plans: 'l1', or views,rays,rows of the slab projector "
                         "(default: the autotuner's choice)")
    ap.add_argument("--bp", default="", choices=["", "runs", "table"],
                    help="back projector of 2D plans: walk tile runs, or gather from the pixel table "
                         "(default: the plan's choice)")
    args = ap.parse_args()
    if args.config == "c4":
        spec = configs.c4(n=args.n, nz=args.n)
        plan = engine.Plan.cone(spec.geom)
        img = phantom.csg_phantom(args.n, args.n, seed=spec.seed)
        names = ("cone_fp_kernel", "cone_bp_kernel")
    else:
        spec = getattr(configs, args.config)()
        plan = engine.Plan.fan(spec.geom)
        if args.variant:
            plan.set_forward_variant(*([0, 0, 0] if args.variant == "l1" else
                                       [int(x) for x in args.variant.split(",")]))
        if args.bp:
            plan.set_back_variant(3 if args.bp == "table" else 0)
        img = phantom.ellipse_phantom(plan.n, seed=spec.seed, n_random=spec.n_random)
        names = ("fan_fp_kernel", "fan_bp_kernel")
    L = engine.lib()
    st = C.c_void_p()
    engine._check("at_stream_create", L.at_stream_create(C.byref(st)))
    sino = np.random.default_rng(0).standard_normal(plan.sino_shape).astype(np.float32)
    bufs = {}
    G = max(1, args.group) if args.config != "c4" else 1
    for g in range(G):
        for name, arr in (("img", img), ("sino", sino), ("img_out", img), ("sino_out", sino)):
            p = C.c_void_p()
            engine._check("at_dev_alloc", L.at_dev_alloc(C.byref(p), arr.nbytes))
            engine._check("h2d", L.at_memcpy_h2d(p, arr.ctypes.data, arr.nbytes, st))
            bufs[name if g == 0 else f"{name}{g}"] = p.value
    import torch

    ts = torch.cuda.ExternalStream(st.value)
    S, R, P = plan.stats["segments"], plan.stats["rays"], int(np.prod(plan.img_shape))
    jobs = {
        "fp": (names[0], lambda: plan.forward_dev(bufs["img"], bufs["sino_out"], st.value), 4 * S + 4 * R),
        "bp": (names[1], lambda: plan.back_dev(bufs["sino"], bufs["img_out"], st.value), 4 * S + 4 * P),
    }
    pset = None
    if G > 1:
        pset = engine.ProjSet([plan] * G)
        sel = lambda key: [bufs[key if g == 0 else f"{key}{g}"] for g in range(G)]  # noqa: E731
        jobs = {
            "fp": ("fan_fp_kernel<group>", lambda: pset.forward_dev(sel("img"), sel("sino_out"), st.value),
                   G * (4 * S + 4 * R)),
            "bp": ("fan_bp_group_kernel", lambda: pset.back_dev(sel("sino"), sel("img_out"), st.value),
                   G * (4 * S + 4 * P)),
        }
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for key in args.which.split(","):
        kname, fn, nbytes = jobs[key]
        for _ in range(2):
            fn()
        # each timed launch has its own events; L2 (129 MB) is flushed before
        # it by a 256 MiB write unless --warm
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.reps)]
        for e0, e1 in evs:
            if not args.warm:
                with torch.cuda.stream(ts):
                    flush.zero_()
            e0.record(ts)
            fn()
            e1.record(ts)
        torch.cuda.synchronize()
        ms = sum(e0.elapsed_time(e1) for e0, e1 in evs) / args.reps
        print(json.dumps({"kernel": kname, "config": args.config, "shape": list(plan.img_shape), "images": G,
                          "l2": "warm" if args.warm else "flushed",
                          "launch_ms": round(ms, 5), "gsegs_per_s": round(G * S / (ms / 1e3) / 1e9, 2),
                          "algorithmic_bytes": nbytes, "gbs": round(nbytes / (ms / 1e3) / 1e9, 1),
                          "segments": S, "rays": R, "pixels": P,
                          "variant": {k: plan.stats[k] for k in ("fp_rays_per_thread", "slab_views", "slab_rays",
                                                                 "slab_rows", "slab_wbox", "slab_fallback_ctas",
                                                                 "bp_table_use", "bp_table_bytes")
                                      if k in plan.stats}}))
    if pset is not None:
        pset.close()
    for p in bufs.values():
        L.at_dev_free(C.c_void_p(p))


if __name__ == "__main__":
    main()

"""Benchmark: 512^2 AT reconstruction slices/s on one GB300 (the C2 workload).

Workload (C2): 512x512 FP32 slices, 0.75 mm pixels, fan beam (SOD 541 mm,
SDD 949 mm) with 720 views x 888 equiangular detectors, seeded Shepp-Logan +
20 random ellipses, Poisson noise at I0 = 5e3, 50 AT outer iterations with
GoldenC's defaults (alpha 1000, beta 0.002, epsilon 1e-4, 10 image + 10 edge
iterations each).  A step reconstructs a batch of slices (16 by default)
from scratch (f = 0, v = 1) in one batched, graph-captured solver; the
slices share one plan, so their projections run grouped.  The plain form
(one slice per solver, one after another) is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  : slices/s with the sinograms resident in HBM, CUDA-event timed over K
         steps on the solver's stream, L2 flushed (256 MiB write) before every
         step.
e2e    : the same through the C-ABI with host buffers: every step copies the
         sinograms in from pinned host memory and f, v back out.
roofline: the dominant kernel timed alone with CUDA events on its stream, at
         the same workload, against the measured HBM copy bandwidth.  The
         step's slices share a plan, so it runs the grouped projectors (one
         walk of the plan for up to four slices); those are timed through a
         projection set, their algorithmic bytes the sum over their slices (an
         effective bandwidth: images and sinograms stay in L2).
--impl reference: the reference algorithm on the host cores (the FP64 oracle
         restatement of GoldenC's solver with the fan tracer, all threads), each
         step one outer iteration of one slice, scaled to slices/s.
N > 1 (torchrun): independent replicas, one per GPU ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "512^2 AT recon slices/s"
UNIT = "slices/s"
WORKLOAD = ("C2 512x512 0.75mm fan-beam AT reconstruction: 720 views x 888 dets, SOD 541 / SDD 949 mm, "
            "Shepp-Logan + 20 random ellipses, Poisson I0=5e3, 50 outer x (10 image CG + 10 edge) iterations")


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def reduce_max(x: float, device="cpu") -> float:
    """Max over ranks (the slowest replica sets the whole-job time)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds: float, world: int) -> float:
    """Replicas only: every rank processes its own units; the job's rate is all
    units over the slowest rank's time."""
    return units_per_rank * world / seconds


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_counters(kernel: str) -> dict:
    """ncu counters of `kernel` from the committed profile summary
    (profiles/traffic.json): DRAM bytes per launch, the limiting unit and its
    throughput, sectors per request."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            ent = json.load(fh).get(kernel)
    except (OSError, ValueError):
        return {}
    if ent is None:
        return {}
    return ent if isinstance(ent, dict) else {"dram_bytes": ent}


class OracleSolve:
    """The FP64 oracle's whole C2 reconstruction (50 outer iterations, the
    reference algorithm) in a background thread: the ctypes call releases the
    GIL, so GPU-bound side samples proceed meanwhile.  Its f and v are the
    reference of the C2 parity block."""

    def __init__(self, spec, sino, nthreads: int):
        from oracle import pyoracle as po

        self.po, self.spec, self.sino, self.nthreads = po, spec, sino.astype(np.float64), nthreads
        self.result, self.seconds, self.error = None, None, None
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _run(self):
        try:
            fan = self.po.fan_from_engine(self.spec.geom)
            t0 = time.perf_counter()
            self.result = self.po.solve(fan, self.sino, 1000.0, 0.002, 1e-4, self.spec.iters, 10, 10,
                                        nthreads=self.nthreads)
            self.seconds = time.perf_counter() - t0
        except Exception as e:  # reported in the parity block, never fatal to the bench line
            self.error = f"{type(e).__name__}: {e}"

    def join(self):
        self.thread.join()
        return self.result


def make_inputs(mg, spec, batch: int):
    """Seeded phantoms and noisy sinograms (projected by the engine itself)."""
    plan = mg.Plan.fan(spec.geom)
    phantoms, sinos = [], []
    for b in range(batch):
        ph = mg.phantom.ellipse_phantom(spec.geom.n, seed=spec.seed + b, n_random=spec.n_random)
        clean = plan.forward(ph)
        sinos.append(mg.phantom.poisson_sinogram(clean, spec.i0, spec.seed + 1000 + b))
        phantoms.append(ph)
    return plan, phantoms, sinos


def run_ours(args):
    import torch

    import medimage_gb300 as mg
    from medimage_gb300 import configs

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    spec = configs.c2()
    B = args.batch
    plan, phantoms, sinos = make_inputs(mg, spec, B)
    S_seg = plan.stats["segments"]
    R = plan.stats["rays"]
    P = spec.geom.n * spec.geom.n
    prm = configs.params_for(spec, mode=args.mode)
    solver = mg.Solver([plan] * B, prm)
    for b in range(B):
        solver.set_sino(b, sinos[b])
    import ctypes as C

    stream_ptr = C.c_void_p()
    mg.engine._check("at_stream_create", mg.lib().at_stream_create(C.byref(stream_ptr)))
    st = stream_ptr.value
    tstream = torch.cuda.ExternalStream(st)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        with torch.cuda.stream(tstream):
            flush.zero_()
        solver.run(stream=st, sync=False)

    for _ in range(args.warmup):
        step()
    solver.sync(st)
    launches_outer = solver.launches_per_outer
    # ---- value: device-resident inputs
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(tstream)
        for _ in range(args.steps):
            step()
        ev1.record(tstream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = reduce_max(ev0.elapsed_time(ev1), device="cuda")
    slices = args.steps * B * world
    value = whole_job_rate(args.steps * B, ms / 1e3, world)
    f0, v0 = solver.get(0, stream=st)
    psnr = mg.phantom.psnr(f0, phantoms[0])
    quality = mg.quality(f0, phantoms[0], dynamic_range=float(phantoms[0].max()))  # on the GPU
    tr = solver.trace(0)

    # ---- e2e: host buffers through the C-ABI, copies inside the timed region
    pinned_in = [torch.empty(sinos[0].shape, dtype=torch.float32, pin_memory=True) for _ in range(B)]
    for b in range(B):
        pinned_in[b].numpy()[...] = sinos[b]
    pin_f = [torch.empty((spec.geom.n, spec.geom.n), dtype=torch.float32, pin_memory=True) for _ in range(B)]
    pin_v = [torch.empty((spec.geom.n, spec.geom.n), dtype=torch.float32, pin_memory=True) for _ in range(B)]
    L = mg.lib()
    fp32 = C.POINTER(C.c_float)

    def e2e_step():
        for b in range(B):
            mg.engine._check("set_sino_host", L.at_solver_set_sino_host(
                solver.handle, b, pinned_in[b].numpy(), C.c_void_p(st)))
        solver.run(stream=st, sync=False)
        for b in range(B):
            mg.engine._check("get_host", L.at_solver_get_host(
                solver.handle, b, pin_f[b].numpy(), pin_v[b].numpy(), C.c_void_p(st)))

    e2e_step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t0, device="cuda")
    e2e_value = whole_job_rate(args.steps * B, e2e_s, world)
    del fp32

    # ---- linear-mode variant (same slices, redundant forward projections replaced)
    variants = {}
    if args.variants and prm.mode == 0:
        prm_lin = configs.params_for(spec, mode=1)
        lin = mg.Solver([plan] * B, prm_lin)
        for b in range(B):
            lin.set_sino(b, sinos[b])
        lin.run(stream=st)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(tstream)
        for _ in range(args.steps):
            with torch.cuda.stream(tstream):
                flush.zero_()
            lin.run(stream=st, sync=False)
        e1.record(tstream)
        torch.cuda.synchronize()
        fl, _ = lin.get(0, stream=st)
        variants["linear"] = {"value": round(args.steps * B / (e0.elapsed_time(e1) / 1e3), 4), "unit": UNIT,
                              "psnr_db": round(mg.phantom.psnr(fl, phantoms[0]), 3),
                              "f_rel_l2_vs_exact": float(np.linalg.norm(fl - f0) / np.linalg.norm(f0))}
        lin.close()
        # the plain per-slice form: one slice per solver, slices one after another
        one = mg.Solver([plan], prm)
        nplain = 2
        one.set_sino(0, sinos[0])
        one.run(stream=st)
        torch.cuda.synchronize()
        plain_ms = 0.0
        for b in range(nplain):
            one.set_sino(0, sinos[b])
            with torch.cuda.stream(tstream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(tstream)
            one.run(stream=st, sync=False)
            e1.record(tstream)
            torch.cuda.synchronize()
            plain_ms += e0.elapsed_time(e1)
            if b == 0:
                fp, _ = one.get(0, stream=st)
        plain = nplain / (plain_ms / 1e3)
        variants["plain_one_slice_per_solver"] = {
            "value": round(plain, 4), "unit": UNIT, "slices": nplain,
            "batched_over_plain": round(value / plain, 2),
            "f_rel_l2_batched_vs_plain": float(np.linalg.norm(fp - f0) / np.linalg.norm(f0))}
        one.close()

    # ---- roofline: the dominant kernel alone, same workload, CUDA events.
    # The step's slices share one plan, so its projections run grouped (up to
    # four slices per walk of the plan): the grouped launches are timed through
    # a projection set over the step's slices, the single-slice kernels beside
    # them.  A grouped launch's algorithmic bytes are its slices' sum.
    G = B
    d_img = [torch.from_numpy(phantoms[b]).cuda() for b in range(G)]
    d_sino = [torch.from_numpy(sinos[b]).cuda() for b in range(G)]
    d_out_s = [torch.empty_like(t) for t in d_sino]
    d_out_i = [torch.empty_like(t) for t in d_img]
    pset = mg.ProjSet([plan] * G)
    ptr = lambda ts: [t.data_ptr() for t in ts]  # noqa: E731
    kern = {}
    cases = [
        ("fan_fp_kernel", lambda: plan.forward_dev(d_img[0].data_ptr(), d_out_s[0].data_ptr(), st), 4 * S_seg + 4 * R),
        ("fan_bp_kernel", lambda: plan.back_dev(d_sino[0].data_ptr(), d_out_i[0].data_ptr(), st), 4 * S_seg + 4 * P)]
    if G > 1:
        cases += [
            ("fan_fp_kernel<group>", lambda: pset.forward_dev(ptr(d_img), ptr(d_out_s), st), G * (4 * S_seg + 4 * R)),
            ("fan_bp_group_kernel", lambda: pset.back_dev(ptr(d_sino), ptr(d_out_i), st), G * (4 * S_seg + 4 * P))]
    for name, fn, nbytes in cases:
        for _ in range(3):
            fn()
        # L2 flushed before every timed launch (as in the step, where the back
        # projector's run list evicts the forward projector's plan)
        reps = 20
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in evs:
            with torch.cuda.stream(tstream):
                flush.zero_()
            e0.record(tstream)
            fn()
            e1.record(tstream)
        torch.cuda.synchronize()
        kern[name] = {"ms": sum(e0.elapsed_time(e1) for e0, e1 in evs) / reps, "bytes": nbytes}
    # calls per slice in the timed workload
    K, KI = prm.iter_alt, prm.iter_image
    fp_calls = K * (3 * KI - 1) if prm.mode == 0 else None
    bp_calls = K * KI
    if fp_calls is None:
        fp_calls = K * (KI + 2)
    # the kernels the step runs: grouped when the step holds several slices
    ran = [n for n in kern if ("group" in n) == (G > 1)]
    share = {n: kern[n]["ms"] * (fp_calls if "fp" in n else bp_calls) for n in ran}
    dom = max(share, key=share.get)
    pset.close()
    peak, peak_kind = measured_peak_hbm()
    achieved = kern[dom]["bytes"] / (kern[dom]["ms"] / 1e3) / 1e9
    prof = profile_counters(dom)
    traffic = prof.get("dram_bytes")
    if traffic is not None and "group" in dom:
        # captured on one group of four slices; each group of a launch streams
        # the plan once, so DRAM traffic scales with the groups in the launch
        traffic = int(traffic * ((G + 3) // 4))
    dram_frac = None if traffic is None else traffic / (kern[dom]["ms"] / 1e3) / 1e9 / peak
    gsegs = S_seg * (fp_calls + bp_calls) * slices / (ms / 1e3) / 1e9
    clocks = clk.summary()

    out = None
    if rank == 0:
        # the FP64 oracle's whole C2 reconstruction runs on the host cores
        # (leaving four to the GPU-driving thread) while the GPU-bound side
        # samples run; the CPU timings and the serving loop come after it
        ora = OracleSolve(spec, sinos[0], max(1, (os.cpu_count() or 1) - 4)) if args.parity else None
        par_gpu = run_parity_gpu(mg, spec, plan, phantoms[0], sinos[0], st) if args.parity else None
        cone = run_cone_c4(mg, st, tstream) if args.cone else None
        c3 = run_batched_c3(mg, st, tstream) if args.c3 else None
        parity = finish_parity(mg, spec, par_gpu, ora, phantoms[0], sinos[0]) if args.parity else None
        serving = run_serving(mg, args.serve_requests, target_db=args.serve_psnr) if args.serve_requests > 0 else None
        cpu = cpu_baseline(spec, sinos[0], args.cpu_outer) if not args.no_cpu else None
        openmp = run_openmp_equal_psnr(mg, st, tstream, batch=8) if not args.no_cpu else None
        goldnc = run_goldnc_native(mg) if not args.no_cpu else None
        out = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantoms, Poisson noise)",
            "config": {"workload": WORKLOAD, "slices_per_step": B, "mode": "exact" if prm.mode == 0 else "linear",
                       "parallelism": f"replicas{world}", "l2": "flushed (256 MiB write) before every step",
                       "segments_per_projection": S_seg, "projections_per_slice": {"forward": fp_calls, "back": bp_calls}},
            "gsegs_per_s": round(gsegs, 3),
            "psnr_db": round(psnr, 3),
            "ssim": round(quality["ssim"], 4),
            "exits": [t[:4] for t in tr if t[3] != 0][:6],
            "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": int(B * sinos[0].nbytes),
                    "d2h_bytes_per_step": int(B * 2 * phantoms[0].nbytes)},
            "roofline": {"kernel": dom, "bound": prof.get("bound", "hbm"), "achieved": round(achieved, 1),
                         "peak": peak, "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": traffic, "algorithmic_bytes_per_launch": kern[dom]["bytes"],
                         "launch_ms": round(kern[dom]["ms"], 5),
                         "dram_frac": None if dram_frac is None else round(dram_frac, 4),
                         "limiter": {k: prof[k] for k in ("unit", "throughput_pct", "sectors_per_request",
                                                          "issue_active_pct", "source") if k in prof},
                         "note": ("achieved = algorithmic bytes (4 S + 4 R per slice) / CUDA-event time: an "
                                  "effective gather rate, not DRAM traffic.  The images, sinograms and most of "
                                  "the plan stay in the 129 MB L2, so the kernel is bound by the SM's load path "
                                  "(the 'limiter' unit, from ncu), and its DRAM traffic ('traffic', ncu) is "
                                  "dram_frac of the measured HBM peak") if prof.get("bound", "hbm") != "hbm"
                         else None,
                         "kernels": {k: {"launch_ms": round(v["ms"], 5),
                                         "achieved_gbs": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)}
                                     for k, v in kern.items()}},
            "cpu_baseline": cpu,
            "parity_c2": parity,
            "openmp_equal_psnr": openmp,
            "goldnc_native": goldnc,
            "cone_c4": cone,
            "batched_c3": c3,
            "variants": variants,
            "serving": serving,
            "clocks": clocks,
            "gpu_launches": int(args.steps * (1 + prm.iter_alt * launches_outer)),
        }
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def run_parity_gpu(mg, spec, plan, phantom, sino, st):
    """The engine's half of the C2 parity block, for both traversal forms: the
    FP64-alpha plan (the reference's traversal, the form the bench times) and
    the plain FP32-alpha plan.  Per form: a forward projection of the phantom,
    a back projection of the sinogram (the first back projection of the
    reconstruction, r = g - A 0), and the 50-outer-iteration reconstruction of
    one slice."""
    from medimage_gb300 import configs

    prm = configs.params_for(spec)
    out = {}
    for form, pl in (("fp64_alpha", plan), ("fp32_alpha", mg.Plan.fan(spec.geom, alpha="fp32"))):
        sv = mg.Solver([pl], prm)
        sv.set_sino(0, sino, stream=st)
        sv.run(stream=st)
        f, v = sv.get(0, stream=st)
        out[form] = {"fp": pl.forward(phantom), "bp": pl.back(sino), "f": f, "v": v, "trace": sv.trace(0),
                     "segments": pl.stats["segments"]}
        sv.close()
    return out


def finish_parity(mg, spec, gpu, ora, phantom, sino):
    """C2 parity block: rel-L2 of each form's forward projection, back
    projection, final f and final v against the FP64 oracle (GoldenC's
    algorithm with the reference fan tracer, main.c:35-360 and
    tracing.cpp:22-147), the PSNR of each, and whether the exit branches of
    every inner loop agree."""
    from oracle import pyoracle as po

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    fan = po.fan_from_engine(spec.geom)
    cores = os.cpu_count() or 1
    fp_ref = po.fan_A(fan, phantom.astype(np.float64), cores)
    bp_ref = po.fan_AT(fan, sino.astype(np.float64), cores)
    res = ora.join() if ora is not None else None
    block = {"workload": "C2 slice (seed 2): forward projection of the phantom, back projection of the noisy "
                         "sinogram, and the 50-outer-iteration reconstruction, each against FP64",
             "oracle": "FP64 restatement of GoldenC main.c:35-360 with the helical/rebin fan tracer "
                       "(pinned bit for bit to the reference's sources)",
             "psnr_peak": "phantom max", "segments_fp64_oracle": po.fan_segments(fan, cores)}
    if res is None:
        block["error"] = ora.error if ora is not None else "oracle solve skipped"
    else:
        fo, vo, tr = res
        block["oracle_solve_s"] = round(ora.seconds, 1)
        block["oracle_threads"] = ora.nthreads
        block["psnr_db_fp64"] = round(mg.phantom.psnr(fo, phantom), 4)
        ex_or = [(o, s_, k, e) for (o, s_, k, _, e) in tr if e != 0]
    for form, d in gpu.items():
        ent = {"forward_rel_l2": rel(d["fp"], fp_ref), "back_rel_l2": rel(d["bp"], bp_ref),
               "segments": d["segments"]}
        if res is not None:
            ex = [(o, s_, k, e) for (o, s_, k, e, _) in d["trace"] if e != 0]
            ent.update({"f_rel_l2": rel(d["f"], fo), "v_rel_l2": rel(d["v"], vo),
                        "psnr_db": round(mg.phantom.psnr(d["f"], phantom), 4),
                        "psnr_minus_fp64_db": round(mg.phantom.psnr(d["f"], phantom) -
                                                    mg.phantom.psnr(fo, phantom), 4),
                        "exit_branches_identical": ex == ex_or})
        block[form] = ent
    return block


def run_serving(mg, n_requests: int, seed: int = 5, target_db: float = 0.0):
    """C5-style serving sample: seeded requests with Poisson arrivals, served by
    the continuous-batching server and again one request at a time.  The mix is
    C5's: 256^2/512^2 slices with 360-720 views and 512-888 detectors, 1024^2
    slices with 1440 views x 1536 detectors (about 22 %), and every tenth
    request a 256^3 cone-beam volume with 360 projections of 384 x 512 cells;
    20-50 outer iterations each.  With target_db > 0 every request carries a
    quality stop (its phantom as reference, PSNR measured on the GPU after each
    outer iteration): it finishes at the first iteration reaching target_db,
    or after its iteration count.  Both forms stop each request at the same
    iteration with the same image (equal PSNR by construction)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    G = mg.FanGeometry.covering
    small = [G(256, 1.0, 360, 512), G(256, 1.0, 720, 888), G(512, 0.75, 720, 888), G(512, 0.75, 360, 512)]
    large = G(1024, 0.375, 1440, 1536)
    cone = mg.ConeGeometry(256, 256, 256, 0.4, 360, 384, 512, 0.8, 600.0, 1000.0)
    plans = {}

    def plan_of(g):
        key = repr(g)
        if key not in plans:
            plans[key] = mg.Plan.cone(g) if isinstance(g, mg.ConeGeometry) else mg.Plan.fan(g)
        return plans[key]

    reqs = []
    for i in range(n_requests):
        u = rng.uniform()
        if i % 10 == 5:
            g = cone
            p = plan_of(g)
            ph = mg.phantom.csg_phantom(256, 256, seed=7000 + i)
        else:
            g = large if u < 0.22 else small[int(rng.integers(len(small)))]
            p = plan_of(g)
            ph = mg.phantom.ellipse_phantom(g.n, seed=7000 + i, n_random=int(rng.integers(0, 20)))
        sino = mg.phantom.poisson_sinogram(p.forward(ph), float(rng.uniform(2e3, 2e4)), 8000 + i)
        reqs.append((p, sino, int(rng.integers(20, 51)), ph))
    # arrivals: Poisson, mean gap a third of the mean request time alone
    alone = mg.Server(hbm_budget_bytes=150 << 30, max_active=1)
    t0 = time.perf_counter()
    rid = alone.submit(reqs[0][0], reqs[0][1], 1, 0.0)
    alone.run()
    one_iter = time.perf_counter() - t0
    mean_service = one_iter * np.mean([r[2] for r in reqs]) * 1.5
    gaps = rng.exponential(mean_service / 3.0, size=n_requests)
    arrivals = np.concatenate([[0.0], np.cumsum(gaps[:-1])])
    out = {}
    results = {}
    infos = {}
    for name, slots in (("continuous", 64), ("one_at_a_time", 1)):
        srv = mg.Server(hbm_budget_bytes=150 << 30, max_active=slots)
        if target_db > 0:
            ids = [srv.submit_psnr(p, s, it, ph, target_db, float(a)) for (p, s, it, ph), a in zip(reqs, arrivals)]
        else:
            ids = [srv.submit(p, s, it, float(a)) for (p, s, it, _), a in zip(reqs, arrivals)]
        srv.run()
        st = srv.stats()
        res = [srv.result(i) for i in ids]
        infos[name] = [srv.result_info(i) for i in ids]
        results[name] = res
        out[name] = {"p50_latency_s": round(st["p50_latency_s"], 4), "p99_latency_s": round(st["p99_latency_s"], 4),
                     "slices_per_s": round(st["slices_per_s"], 4), "rounds": st["rounds"],
                     "peak_state_gb": round(st["peak_state_bytes"] / 1e9, 3), "psnr_stops": st["psnr_stops"]}
        srv.close()
    same = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
               for a, b in zip(results["continuous"], results["one_at_a_time"]))
    same_iters = [a["iterations"] for a in infos["continuous"]] == [b["iterations"] for b in infos["one_at_a_time"]]
    psnr = [mg.phantom.psnr(r[0], q[3]) for r, q in zip(results["continuous"], reqs)]
    out.update({"requests": n_requests, "mix": "C5: 256^2/512^2 slices, ~22% 1024^2 (1440x1536), every tenth a "
                                                "256^3 cone volume (360 x 384 x 512)",
                "iterations": "20-50 outer per request", "budget_gb": 150,
                "quality_stop_psnr_db": target_db if target_db > 0 else None,
                "iterations_run_median": float(np.median([a["iterations"] for a in infos["continuous"]])),
                "same_stop_iteration_alone_vs_mix": bool(same_iters),
                "results_identical_alone_vs_mix": bool(same), "psnr_db_median": round(float(np.median(psnr)), 3),
                "speedup_slices_per_s": round(out["continuous"]["slices_per_s"] /
                                              max(out["one_at_a_time"]["slices_per_s"], 1e-12), 3)})
    return out


def run_batched_c3(mg, st, tstream):
    """C3, 64 uneven slices ({256,384,512}^2, {360,540,720} views, {512,768,888}
    detectors, 30 outer iterations): all 64 in one batch (one launch per kernel
    for the whole set, uneven early exits handled per scan) against the plain
    form, one slice after another, each with its own solver.  L2 is flushed
    before each form; CUDA events on the launching stream."""
    import torch

    from medimage_gb300 import configs

    specs = configs.c3()
    plans = {}
    items = []
    for sp in specs:
        key = (sp.geom.n, sp.geom.nviews, sp.geom.ndets)
        if key not in plans:
            plans[key] = mg.Plan.fan(sp.geom)
        p = plans[key]
        ph = mg.phantom.ellipse_phantom(sp.geom.n, seed=sp.seed, n_random=sp.n_random)
        items.append((p, mg.phantom.poisson_sinogram(p.forward(ph), sp.i0, sp.seed + 500), ph))
    prm = mg.Params(iter_alt=specs[0].iters)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    batched = mg.Solver([it[0] for it in items], prm)
    for k, it in enumerate(items):
        batched.set_sino(k, it[1])
    singles = []
    for it in items:
        sv = mg.Solver([it[0]], prm)
        sv.set_sino(0, it[1])
        singles.append(sv)
    # warm up (graph capture) both forms
    batched.run(stream=st)
    for sv in singles:
        sv.run(stream=st)
    out = {"workload": "C3: 64 uneven fan-beam slices, 30 outer iterations each", "slices": len(items)}
    for name, fn in (("batched", lambda: batched.run(stream=st, sync=False)),
                     ("plain", lambda: [sv.run(stream=st, sync=False) for sv in singles])):
        with torch.cuda.stream(tstream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(tstream)
        fn()
        e1.record(tstream)
        torch.cuda.synchronize()
        out[f"slices_per_s_{name}"] = round(len(items) / (e0.elapsed_time(e1) / 1e3), 3)
    # slices of one geometry are projected together in the batch (one walk of the
    # plan for up to four), which changes the order of FP64 energy sums only
    dev = 0.0
    for k in range(len(items)):
        fb, fs = batched.get(k, stream=st)[0].astype(np.float64), singles[k].get(0, stream=st)[0].astype(np.float64)
        dev = max(dev, float(np.linalg.norm(fb - fs) / max(np.linalg.norm(fs), 1e-300)))
    out["batched_over_plain"] = round(out["slices_per_s_batched"] / out["slices_per_s_plain"], 2)
    out["max_rel_l2_batched_vs_plain"] = dev
    out["psnr_db_median"] = round(float(np.median([mg.phantom.psnr(batched.get(k, stream=st)[0], it[2])
                                                   for k, it in enumerate(items)])), 3)
    batched.close()
    for sv in singles:
        sv.close()
    return out


def run_cone_c4(mg, st, tstream, reps: int = 2):
    """C4, the 512^3 cone beam (720 views of 768 x 1024 cells): forward and back
    projection at full size, timed with CUDA events on the launching stream;
    one outer iteration of the exact-mode volume solver (29 forward + 10 back
    projections and the volume passes) timed on the phantom's projection, and
    a 10-iteration reconstruction estimated from it."""
    import torch

    from medimage_gb300 import configs

    spec = configs.c4()
    plan = mg.Plan.cone(spec.geom)
    vol = mg.phantom.csg_phantom(512, 512, seed=spec.seed)
    nvox, nbins = vol.size, int(np.prod(plan.sino_shape))
    d_vol = torch.from_numpy(vol).cuda()
    d_sino = torch.empty(nbins, dtype=torch.float32, device="cuda")
    d_back = torch.empty(nvox, dtype=torch.float32, device="cuda")
    S, R = plan.stats["segments"], plan.stats["rays"]
    peak, _ = measured_peak_hbm()
    out = {"workload": "C4: 512^3 voxels of 0.2 mm, 720 views x 768 x 1024 cells of 0.4 mm, SOD 600 / SDD 1000 mm, "
                       "CSG part", "segments_per_projection": S, "rays": R}
    for name, fn, nbytes in (("forward", lambda: plan.forward_dev(d_vol.data_ptr(), d_sino.data_ptr(), st),
                              4 * S + 4 * R),
                             ("back", lambda: plan.back_dev(d_sino.data_ptr(), d_back.data_ptr(), st),
                              4 * S + 4 * nvox)):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(tstream)
        for _ in range(reps):
            fn()
        e1.record(tstream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        gbs = nbytes / (ms / 1e3) / 1e9
        out[name] = {"launch_ms": round(ms, 2), "gsegs_per_s": round(S / (ms / 1e3) / 1e9, 1),
                     "algorithmic_gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 3)}
    plan.forward_dev(d_vol.data_ptr(), d_sino.data_ptr(), st)  # the phantom's projection as data
    solver = mg.Solver([plan], configs.params_for(spec))
    solver.set_sino_dev(0, d_sino.data_ptr(), stream=st)
    solver.reset(stream=st)
    solver.step(1, stream=st)  # the graph is captured on the first step
    solver.reset(stream=st)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(tstream)
    solver.step(1, stream=st, sync=False)
    e1.record(tstream)
    torch.cuda.synchronize()
    outer_s = e0.elapsed_time(e1) / 1e3
    out["seconds_per_outer_iteration"] = round(outer_s, 2)
    out["est_seconds_per_volume_10_iterations"] = round(10 * outer_s, 1)
    solver.close()
    del d_vol, d_sino, d_back, plan
    torch.cuda.empty_cache()
    return out


def run_openmp_equal_psnr(mg, st, tstream, batch: int, reps: int = 3):
    """The reference's OpenMP path (msbeam/CPU_OpenMP: row-action AT, its own
    512^2 phantom, 180 x 768 parallel beam, 10 sweeps) on all host cores,
    against this engine on the same phantom and ray geometry (a ray table of
    msbeam's rays), run with the cheapest iteration schedule (outer x inner
    CG iterations, exact or linear mode) whose PSNR reaches msbeam's.  PSNR peak: the phantom maximum (3.0).  Data: noiseless, each
    side projecting the phantom with its own projector (msbeam's A of
    proj.c:14-32 for msbeam, the engine's forward projector for the engine)."""
    import torch

    from oracle import pyoracle as po

    geom = mg.RayGeometry.msbeam_parallel()
    plan = mg.Plan.rays(geom)
    ph = mg.phantom.msbeam_phantom()
    peak = float(ph.max())
    sino = plan.forward(ph)
    # CPU: msbeam port (bit-identical to the reference with one thread; racy
    # over views like the reference with several)
    cores = os.cpu_count() or 1
    g_ms = po.ms_A(ph)
    t0 = time.perf_counter()
    f_cpu, _ = po.ms_solve(g_ms, 10, cores)
    cpu_s = time.perf_counter() - t0
    cpu_psnr = mg.phantom.psnr(f_cpu, ph, peak)
    # GPU: the cheapest schedule (outer x inner iterations, exact or linear
    # mode) whose PSNR reaches msbeam's; PSNR computed on the GPU
    cands = [(1, ii) for ii in (10, 12, 14, 16, 20)] + [(k, 10) for k in range(2, 11)]
    sched = []
    for mode in (1, 0):
        for K, II in cands:
            fps = K * (II + 2) if mode == 1 else K * (3 * II - 1)
            sched.append((fps + K * II, K, II, mode))
    sched.sort()
    tried = []
    prm = None
    for _, K, II, mode in sched:
        cand = mg.Params(iter_alt=K, iter_image=II, mode=mode)
        S = mg.Solver([plan], cand)
        S.set_sino(0, sino)
        S.run()
        q = mg.quality(S.get(0)[0], ph, peak)["psnr_db"]
        S.close()
        tried.append([K, II, mode, round(q, 3)])
        if q >= cpu_psnr:
            prm = cand
            break
    if prm is None:
        return {"unavailable": "no schedule up to 10 outer iterations reached msbeam's PSNR", "tried": tried}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    rates = {}
    for name, B in (("plain", 1), ("batched", batch)):
        sv = mg.Solver([plan] * B, prm)
        for b in range(B):
            sv.set_sino(b, sino)
        sv.run(stream=st)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ms = 0.0
        for _ in range(reps):
            with torch.cuda.stream(tstream):
                flush.zero_()
            e0.record(tstream)
            sv.run(stream=st, sync=False)
            e1.record(tstream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        rates[name] = B * reps / (ms / 1e3)
        f_gpu = sv.get(0)[0]
        sv.close()
    # end to end: one call with host buffers (at_reconstruct_host)
    mg.reconstruct(plan, prm, sino)
    t0 = time.perf_counter()
    for _ in range(reps):
        f_e2e, _ = mg.reconstruct(plan, prm, sino)
    e2e = reps / (time.perf_counter() - t0)
    # the same algorithm as msbeam on the GPU (row-action mode, 10 sweeps, data
    # from msbeam's projection on the GPU), alone and in batches of `batch`
    ra = mg.RowAction()
    ra_rate, ra_psnr = {}, None
    d_ph = torch.from_numpy(ph).cuda()
    d_g1 = torch.empty((1, 180, 768), dtype=torch.float32, device="cuda")
    ra.forward_dev(1, d_ph.data_ptr(), d_g1.data_ptr(), stream=st)
    torch.cuda.synchronize()
    for B in (1, batch):
        d_g = d_g1.repeat(B, 1, 1).contiguous()
        d_f = torch.empty((B, 512, 512), dtype=torch.float32, device="cuda")
        d_v = torch.empty_like(d_f)
        ra.run_dev(B, d_g.data_ptr(), d_f.data_ptr(), d_v.data_ptr(), stream=st)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(tstream)
        ra.run_dev(B, d_g.data_ptr(), d_f.data_ptr(), d_v.data_ptr(), stream=st)
        e1.record(tstream)
        torch.cuda.synchronize()
        ra_rate[B] = B / (e0.elapsed_time(e1) / 1e3)
        if B == 1:
            ra_psnr = mg.phantom.psnr(d_f[0].cpu().numpy(), ph, peak)
    ra.close()
    cpu_rate = 1.0 / cpu_s
    return {
        "reference": f"msbeam/CPU_OpenMP restated (oracle/or_msbeam.c), OpenMP {cores} threads, 10 sweeps",
        "workload": "msbeam phantom 512^2, parallel beam 180 views x 768 rays, noiseless",
        "psnr_peak": "phantom max (3.0)",
        "cpu": {"seconds_per_slice": round(cpu_s, 3), "slices_per_s": round(cpu_rate, 4),
                "psnr_db": round(cpu_psnr, 3), "cores": cores, "kind": "port"},
        "gpu": {"outer_iterations": prm.iter_alt, "image_iterations": prm.iter_image,
                "mode": "linear" if prm.mode == 1 else "exact", "schedules_tried": tried,
                "psnr_db": round(mg.phantom.psnr(f_gpu, ph, peak), 3),
                "slices_per_s_plain": round(rates["plain"], 2),
                f"slices_per_s_batch{batch}": round(rates["batched"], 2),
                "slices_per_s_e2e_host_call": round(e2e, 2),
                "l2": "flushed before every timed run"},
        "gpu_row_action": {"algorithm": "msbeam's row-action AT on the GPU (at_rowaction_run), 10 sweeps, rays of a "
                                         "view in 4 interleaved groups",
                           "psnr_db": round(float(ra_psnr), 3), "slices_per_s_plain": round(ra_rate[1], 2),
                           f"slices_per_s_batch{batch}": round(ra_rate[batch], 2),
                           "speedup_plain": round(ra_rate[1] / cpu_rate, 1),
                           "speedup_batched": round(ra_rate[batch] / cpu_rate, 1)},
        "speedup_plain": round(rates["plain"] / cpu_rate, 1),
        "speedup_batched": round(rates["batched"] / cpu_rate, 1),
        "speedup_e2e": round(e2e / cpu_rate, 1),
    }


def run_goldnc_native(mg, reps: int = 3):
    """GoldenC as shipped against the engine's drop-in entry points, at
    GoldenC's own geometry (512 x 512 parallel beam, 180 views x 767 bins,
    origin/GoldenC/src/config.h:10-13) and defaults (alpha 1000, beta 0.002,
    epsilon 1e-4, 10 + 10 inner iterations): one outer iteration (image step,
    then edge step, main.c:43-47) from f = 0, v = 1.

    The CPU leg is the FP64 oracle restatement of GoldenC with GoldenC's own
    projector on one thread (the reference has no threading).  The engine leg
    calls minimize_in_IMAGE_variable and minimize_in_EDGE_variable with host
    FP64 arrays, so its time includes every host/device copy the drop-in
    makes."""
    try:
        from oracle import pyoracle as po

        L = mg.lib()
        n = 512
        ph = np.ascontiguousarray(mg.phantom.ellipse_phantom(n, seed=61), np.float64)
        g = np.zeros((180, 767), np.float64)
        L.A(g, ph)  # the data, as GoldenC's main makes it (main.c:56)
        f0, v0 = np.zeros((n, n), np.float64), np.ones((n, n), np.float64)
        f1, v1 = np.zeros((n, n), np.float64), np.zeros((n, n), np.float64)

        def outer():
            L.minimize_in_IMAGE_variable(f1, g, f0, v0, 1000.0, 1e-4, 10)
            L.minimize_in_EDGE_variable(v1, f1, v0, 1000.0, 0.002, 1e-4, 10)

        outer()  # warm-up
        times = []
        for _ in range(reps):
            t0 = time.perf_counter()
            outer()
            times.append(time.perf_counter() - t0)
        status = int(L.goldnc_status())
        t0 = time.perf_counter()
        fo, vo, _ = po.solve(None, g, 1000.0, 0.002, 1e-4, 1, 10, 10, nthreads=1)
        cpu_s = time.perf_counter() - t0
        eng_s = statistics.median(times)
        return {
            "geometry": "GoldenC's own: 512^2 parallel beam, 180 views x 767 bins",
            "sample": "one outer iteration (10 image CG + 10 edge) from f = 0, v = 1",
            "engine_dropin_s": round(eng_s, 5), "goldnc_cpu_s": round(cpu_s, 3),
            "goldnc_cpu": {"cores": 1, "kind": "port"},
            "speedup": round(cpu_s / eng_s, 1),
            "status": status,
            "rel_l2_f": float(np.linalg.norm(f1 - fo) / max(np.linalg.norm(fo), 1e-300)),
            "rel_l2_v": float(np.linalg.norm(v1 - vo) / max(np.linalg.norm(vo), 1e-300)),
        }
    except Exception as e:  # a side sample: report, never lose the bench line
        return {"error": f"{type(e).__name__}: {e}"}


def cpu_baseline(spec, sino, outer: int):
    """The FP64 oracle (reference algorithm) on all host cores: `outer` outer
    iterations of one slice, scaled to slices/s."""
    from oracle import pyoracle as po

    cores = os.cpu_count() or 1
    fan = po.fan_from_engine(spec.geom)
    t0 = time.perf_counter()
    po.solve(fan, sino.astype(np.float64), 1000.0, 0.002, 1e-4, outer, 10, 10, nthreads=cores)
    dt = time.perf_counter() - t0
    per_slice = dt / outer * spec.iters
    return {"value": round(1.0 / per_slice, 6), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{outer} of {spec.iters} outer iterations of one C2 slice (FP64 oracle restatement of "
                      f"GoldenC main.c with the helical/rebin fan tracer, OpenMP {cores} threads), "
                      f"{dt:.2f} s, scaled x{spec.iters / outer:g}"}


def run_reference(args):
    """--impl reference: the reference algorithm on the host cores."""
    rank, world, _ = env_rank()
    if rank != 0:
        return None
    import medimage_gb300.configs as configs
    from medimage_gb300.phantom import ellipse_phantom, poisson_sinogram
    from oracle import pyoracle as po

    spec = configs.c2()
    fan = po.fan_from_engine(spec.geom)
    cores = os.cpu_count() or 1
    ph = ellipse_phantom(spec.geom.n, seed=spec.seed, n_random=spec.n_random)
    clean = po.fan_A(fan, ph.astype(np.float64), cores)
    sino = poisson_sinogram(clean, spec.i0, spec.seed + 1000).astype(np.float64)
    for _ in range(args.warmup):
        po.solve(fan, sino, 1000.0, 0.002, 1e-4, 1, 10, 10, nthreads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        po.solve(fan, sino, 1000.0, 0.002, 1e-4, 1, 10, 10, nthreads=cores)
    dt = time.perf_counter() - t0
    per_outer = dt / args.steps
    value = 1.0 / (per_outer * spec.iters)
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(per_outer * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded phantoms, Poisson noise)",
        "config": {"workload": WORKLOAD, "slices_per_step": 1, "sample": "one outer iteration per step"},
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "each step = 1 of 50 outer iterations of one C2 slice, FP64 oracle restatement "
                                   "of GoldenC main.c + helical/rebin fan tracer, OpenMP; scaled x50"},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--batch", type=int, default=16, help="slices reconstructed together per step")
    ap.add_argument("--mode", type=int, default=0, help="0 exact projection count, 1 linear-mode updates")
    ap.add_argument("--cpu-outer", type=int, default=1, help="outer iterations in the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--serve-requests", type=int, default=12, help="requests in the serving sample (0 = skip)")
    ap.add_argument("--serve-psnr", type=float, default=26.0,
                    help="quality stop of every serving request (dB against its phantom; 0 = none)")
    ap.add_argument("--serve-only", action="store_true",
                    help="only the serving sample (its own JSON line; for long C5 runs)")
    ap.add_argument("--no-variants", dest="variants", action="store_false", help="skip the linear-mode variant")
    ap.add_argument("--no-cone", dest="cone", action="store_false", help="skip the C4 cone-beam projector sample")
    ap.add_argument("--no-c3", dest="c3", action="store_false", help="skip the C3 batched-versus-plain sample")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the C2 parity block (FP64 oracle reconstruction on the host cores)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.serve_only:
        import medimage_gb300 as mg

        print(json.dumps({"serving": run_serving(mg, args.serve_requests, target_db=args.serve_psnr)}))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Generate the golden vectors under tests/golden/ from the reference's own
sources (compiled by oracle/ref.mk into oracle/_ref/).  Run where the reference
tree is present:

    make -f oracle/ref.mk REF=<reference tree> && python tests/golden/make_golden.py

Fixtures (all inputs are seeded and regenerated by the tests):
  goldnc.npz  GoldenC proj.c A / AStar outputs (checksums + crops), sparse
              AStar impulse responses (the exact pixel sets and weights of
              sampled bins), one outer iteration of main.c's image and edge
              steps (checksums + crops)
  fan.npz     helical/rebin tracing.cpp ray traversals at the C1 and C2 fan
              geometries: full (pixel, weight) lists for sampled rays and
              per-ray digests for many more
  cone.npz    industry3d cone() end points and forward_proj traversals
              (voxel indices and FP32 weights, bit patterns) for sampled
              rays of a small cone geometry and of the C4 geometry
  msbeam.npz  msbeam/CPU_OpenMP: the built-in phantom (from the std.dat the
              program writes), wray traversals of sampled rays, rows of
              A(phantom), and digests + crops of f and v after the program's
              10 sweeps with one thread (deterministic then)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import math
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from medimage_gb300.engine import ConeGeometry, FanGeometry  # noqa: E402
from medimage_gb300.phantom import ellipse_phantom  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def checksum(x: np.ndarray) -> np.ndarray:
    """[sum, sum of squares, weighted sum] with exactly rounded sums (fsum)."""
    x = np.asarray(x, np.float64).ravel()
    w = np.random.default_rng(12345).random(x.size)
    return np.array([math.fsum(x), math.fsum(x * x), math.fsum(x * w)])


def ray_digest(ind: np.ndarray, wgt: np.ndarray) -> str:
    h = hashlib.sha1()
    h.update(np.ascontiguousarray(ind, np.int32).tobytes())
    h.update(np.ascontiguousarray(wgt, np.float64).tobytes())
    return h.hexdigest()


def goldnc(ref: po.Ref) -> dict:
    out = {}
    ph = ellipse_phantom(512, seed=11).astype(np.float64)
    out["phantom_checksum"] = checksum(ph)
    a = ref.A(ph)
    out["A_checksum"] = checksum(a)
    out["A_rows"] = a[::15].copy()  # 12 views, full detector rows
    rng = np.random.default_rng(13)
    sino = rng.random((180, 767))
    b = ref.AStar(sino)
    out["AStar_checksum"] = checksum(b)
    out["AStar_crop"] = b[200:264, 300:364].copy()
    # impulse responses: AStar(e_bin) is the bin's traversal (pixel set + weights)
    bins = [(1, 0), (1, 383), (1, 700), (23, 250), (44, 600), (45, 383), (46, 10), (89, 500), (91, 383),
            (120, 77), (135, 300), (150, 766), (179, 383), (0, 300), (90, 300)]
    imp_pix, imp_w, imp_off = [], [], [0]
    for (view, det) in bins:
        e = np.zeros((180, 767))
        e[view, det] = 1.0
        r = ref.AStar(e).ravel()
        nz = np.nonzero(r)[0]
        imp_pix.append(nz.astype(np.int32))
        imp_w.append(r[nz])
        imp_off.append(imp_off[-1] + nz.size)
    out["impulse_bins"] = np.array(bins, np.int32)
    out["impulse_pix"] = np.concatenate(imp_pix)
    out["impulse_w"] = np.concatenate(imp_w)
    out["impulse_off"] = np.array(imp_off, np.int64)
    # one outer iteration of the solver on noiseless data g = A(phantom) (main.c:60)
    ph2 = ellipse_phantom(512, seed=12).astype(np.float64)
    g = ref.A(ph2)
    f0 = np.zeros((512, 512))
    v0 = np.ones((512, 512))
    f1 = ref.image_step(g, f0, v0, 1000.0, 1e-4, 10)
    v1 = ref.edge_step(f1, v0, 1000.0, 0.002, 1e-4, 10)
    out["solver_f_checksum"] = checksum(f1)
    out["solver_v_checksum"] = checksum(v1)
    out["solver_f_crop"] = f1[224:288, 224:288].copy()
    out["solver_v_crop"] = v1[224:288, 224:288].copy()
    out["medfilt_checksum"] = checksum(ref.medfilt2(np.random.default_rng(14).random((512, 512))))
    return out


def fan(ref: po.Ref) -> dict:
    out = {}
    for name, geom in (("c1", FanGeometry.covering(256, 1.0, 360, 512)),
                       ("c2", FanGeometry.covering(512, 0.75, 720, 888))):
        f = po.fan_from_engine(geom)
        rng = np.random.default_rng(17)
        full = [(v, d) for v in (0, 45, 90, 137, geom.nviews - 1) for d in (0, geom.ndets // 2, geom.ndets - 1)]
        full += [(int(rng.integers(geom.nviews)), int(rng.integers(geom.ndets))) for _ in range(25)]
        ind_all, w_all, off = [], [], [0]
        for (v, d) in full:
            sx, sy, dx, dy = po.fan_endpoints(f, v, d)
            ind, wgt = ref.fan_trace_points(geom.n, geom.pixel_mm, sx, sy, dx, dy)
            ind_all.append(ind)
            w_all.append(wgt)
            off.append(off[-1] + ind.size)
        out[f"{name}_full_rays"] = np.array(full, np.int32)
        out[f"{name}_full_ind"] = np.concatenate(ind_all).astype(np.int32)
        out[f"{name}_full_w"] = np.concatenate(w_all)
        out[f"{name}_full_off"] = np.array(off, np.int64)
        dig_rays = [(int(rng.integers(geom.nviews)), int(rng.integers(geom.ndets))) for _ in range(1500)]
        digests, counts = [], []
        for (v, d) in dig_rays:
            sx, sy, dx, dy = po.fan_endpoints(f, v, d)
            ind, wgt = ref.fan_trace_points(geom.n, geom.pixel_mm, sx, sy, dx, dy)
            digests.append(ray_digest(ind, wgt))
            counts.append(ind.size)
        out[f"{name}_digest_rays"] = np.array(dig_rays, np.int32)
        out[f"{name}_digest"] = np.array(digests)
        out[f"{name}_digest_numb"] = np.array(counts, np.int32)
        out[f"{name}_segments"] = np.array([po.fan_segments(f)], np.int64)
    return out


def float_digest(x: np.ndarray) -> str:
    return hashlib.sha1(np.ascontiguousarray(x, np.float32).tobytes()).hexdigest()


MS_RAYS = [(0, 0), (0, 384), (0, 767), (1, 200), (29, 500), (44, 384), (45, 100), (45, 700), (60, 300),
           (89, 383), (90, 384), (91, 12), (120, 400), (134, 650), (135, 384), (150, 90), (179, 384), (179, 767)]


def msbeam(ref: po.Ref) -> dict:
    out = {}
    ms = ref.ms
    ms.wray.argtypes = [C.c_int, C.c_int, po._ip, po._fp32, C.POINTER(C.c_int), C.POINTER(C.c_float)]
    ms.omp_set_num_threads.argtypes = [C.c_int]
    ind_all, w_all, off = [], [], [0]
    for (k, r) in MS_RAYS:
        line = np.zeros(2048, np.int32)
        w = np.zeros(2048, np.float32)
        nb, sn = C.c_int(), C.c_float()
        ms.wray(k, r, line, w, C.byref(nb), C.byref(sn))
        ind_all.append(line[: nb.value].copy())
        w_all.append(w[: nb.value].copy())
        off.append(off[-1] + nb.value)
    out["wray_rays"] = np.array(MS_RAYS, np.int32)
    out["wray_ind"] = np.concatenate(ind_all)
    out["wray_w"] = np.concatenate(w_all)
    out["wray_off"] = np.array(off, np.int64)
    with tempfile.TemporaryDirectory() as tmp:
        f, v = po.ref_msbeam_run(ref, 1, tmp)
        ph = np.loadtxt(os.path.join(tmp, "std.dat"), dtype=np.float64).astype(np.float32)
    out["phantom_digest"] = np.array(float_digest(ph))
    g = np.zeros(180 * 768, np.float32)
    ms.A(g, np.ascontiguousarray(ph.ravel()))
    out["A_rows"] = g.reshape(180, 768)[::15].copy()
    out["A_digest"] = np.array(float_digest(g))
    out["f_digest"] = np.array(float_digest(f))
    out["v_digest"] = np.array(float_digest(v))
    out["f_crop"] = f[216:296, 216:296].copy()
    out["v_crop"] = v[216:296, 216:296].copy()
    return out


CONE_GEOMS = {
    "small": ConeGeometry(64, 64, 48, 0.4, 90, 64, 64, 0.7, 60.0, 100.0),
    "c4": ConeGeometry(512, 512, 512, 0.2, 720, 768, 1024, 0.4, 600.0, 1000.0, 384, 384),
}


def cone(ref: po.Ref) -> dict:
    """Reference end points and traversals.  The reference centres both
    detector axes at NDX/2 (ct3d.cpp:90), so the C4 entry, whose detector is
    not square (768 rows x 1024 columns), uses NDX/2 = 384 on both axes."""
    out = {}
    for name, g in CONE_GEOMS.items():
        rng = np.random.default_rng(31)
        rays = [(0, g.ndx // 2, g.ndy // 2), (g.nproj // 4, 0, 0), (g.nproj // 2, g.ndx - 1, g.ndy - 1)]
        rays += [(int(rng.integers(g.nproj)), int(rng.integers(g.ndx)), int(rng.integers(g.ndy))) for _ in range(60)]
        ends, ind_all, w_all, off = [], [], [], [0]
        for (v, r, c) in rays:
            s, d = po.ref_cone_endpoints(ref, g, v, r, c)
            ind, wgt = po.ref_cone_trace_points(ref, g.nx, g.ny, g.nz, s, d)
            ends.append(np.concatenate([s, d]))
            ind_all.append(ind)
            w_all.append(wgt)
            off.append(off[-1] + ind.size)
        out[f"{name}_rays"] = np.array(rays, np.int32)
        out[f"{name}_ends"] = np.array(ends, np.float32)
        out[f"{name}_ind"] = np.concatenate(ind_all).astype(np.int64)
        out[f"{name}_w"] = np.concatenate(w_all).astype(np.float32)
        out[f"{name}_off"] = np.array(off, np.int64)
    return out


def main() -> None:
    if not po.Ref.available():
        raise SystemExit("oracle/_ref is not built: run make -f oracle/ref.mk REF=<reference root>")
    ref = po.Ref()
    np.savez_compressed(os.path.join(OUT, "goldnc.npz"), **goldnc(ref))
    np.savez_compressed(os.path.join(OUT, "fan.npz"), **fan(ref))
    np.savez_compressed(os.path.join(OUT, "msbeam.npz"), **msbeam(ref))
    np.savez_compressed(os.path.join(OUT, "cone.npz"), **cone(ref))
    for fn in ("goldnc.npz", "fan.npz", "msbeam.npz", "cone.npz"):
        print(fn, os.path.getsize(os.path.join(OUT, fn)))


if __name__ == "__main__":
    main()

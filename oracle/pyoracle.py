"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py as the checker.  The engine package never imports this module.

Also binds the reference's own sources compiled under ``oracle/_ref`` (built by
``oracle/ref.mk`` where the reference tree is present) so tests can pin the
restatement against them.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

GC_N, GC_DETS, GC_VIEWS = 512, 767, 180

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_fp32 = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class FanGeom(C.Structure):
    """Mirror of ``or_fan_geom`` (oracle/at_oracle.h)."""

    _fields_ = [
        ("n", C.c_int),
        ("pixel_mm", C.c_double),
        ("nviews", C.c_int),
        ("ndets", C.c_int),
        ("sod_mm", C.c_double),
        ("sdd_mm", C.c_double),
        ("det_pitch_deg", C.c_double),
        ("off_center", C.c_double),
        ("view0_deg", C.c_double),
        ("view_step_deg", C.c_double),
        ("ends", C.c_void_p),
    ]


class ConeGeom(C.Structure):
    """Mirror of ``or_cone_geom`` (oracle/at_oracle.h)."""

    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("voxel", C.c_float), ("nproj", C.c_int),
                ("ndx", C.c_int), ("ndy", C.c_int), ("pitch", C.c_float), ("sod", C.c_float), ("sdd", C.c_float),
                ("half_rows", C.c_int), ("half_cols", C.c_int)]


class Projector(C.Structure):
    _fields_ = [("kind", C.c_int), ("fan", FanGeom), ("nthreads", C.c_int), ("cone", ConeGeom)]


class TraceRec(C.Structure):
    _fields_ = [
        ("outer", C.c_int),
        ("step", C.c_int),
        ("k", C.c_int),
        ("s", C.c_double * 6),
        ("exit_reason", C.c_int),
    ]


class Trace(C.Structure):
    _fields_ = [("recs", C.POINTER(TraceRec)), ("cap", C.c_int), ("count", C.c_int)]


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_gc_A.argtypes = [_dp, _dp]
        L.or_gc_AStar.argtypes = [_dp, _dp]
        L.or_gc_walk.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, C.c_int]
        L.or_gc_walk.restype = C.c_int
        L.or_fan_endpoints.argtypes = [C.POINTER(FanGeom), C.c_int, C.c_int] + [C.POINTER(C.c_double)] * 4
        L.or_fan_trace.argtypes = [C.POINTER(FanGeom), C.c_int, C.c_int, _ip, _dp, C.c_int, C.POINTER(C.c_int)]
        L.or_fan_trace.restype = C.c_int
        L.or_fan_trace_points.argtypes = [C.c_int, C.c_double] + [C.c_double] * 4 + [_ip, _dp, C.c_int]
        L.or_fan_trace_points.restype = C.c_int
        L.or_fan_count_segments.argtypes = [C.POINTER(FanGeom), C.c_int]
        L.or_fan_count_segments.restype = C.c_int64
        L.or_fan_A.argtypes = [C.POINTER(FanGeom), _dp, _dp, C.c_int]
        L.or_fan_AT.argtypes = [C.POINTER(FanGeom), _dp, _dp, C.c_int]
        L.or_medfilt2.argtypes = [C.c_int, _dp]
        L.or_image_step.argtypes = [C.POINTER(Projector), _dp, _dp, _dp, _dp, C.c_double, C.c_double,
                                    C.c_int, C.POINTER(Trace), C.c_int]
        L.or_edge_step.argtypes = [C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_int,
                                   C.POINTER(Trace), C.c_int]
        L.or_solve.argtypes = [C.POINTER(Projector), _dp, _dp, _dp, C.c_double, C.c_double, C.c_double,
                               C.c_int, C.c_int, C.c_int, C.POINTER(Trace)]
        L.or_ms_wray.argtypes = [C.c_int, C.c_int, _ip, _fp32]
        L.or_ms_wray.restype = C.c_int
        L.or_ms_A.argtypes = [_fp32, _fp32]
        L.or_ms_solve.argtypes = [_fp32, _fp32, _fp32, C.c_int, C.c_int]
        L.or_ms_phantom.argtypes = [_fp32]
        L.or_ms_solve_phased.argtypes = [_fp32, _fp32, _fp32, C.c_int, C.c_int]
        L.or_cone_theta.argtypes = [C.POINTER(ConeGeom), C.c_int]
        L.or_cone_theta.restype = C.c_float
        L.or_cone_endpoints.argtypes = [C.POINTER(ConeGeom), C.c_int, C.c_int, C.c_int, _fp32, _fp32]
        L.or_cone_trace_points.argtypes = [C.c_int] * 3 + [C.c_float] * 6 + [_i64, _fp32, C.c_int, C.c_int]
        L.or_cone_trace_points.restype = C.c_int
        L.or_cone_trace.argtypes = [C.POINTER(ConeGeom), C.c_int, C.c_int, C.c_int, _i64, _fp32, C.c_int, C.c_int]
        L.or_cone_trace.restype = C.c_int
        L.or_cone_count_segments.argtypes = [C.POINTER(ConeGeom), C.c_int]
        L.or_cone_count_segments.restype = C.c_int64
        L.or_cone_A.argtypes = [C.POINTER(ConeGeom), _dp, _dp, C.c_int]
        L.or_cone_AT.argtypes = [C.POINTER(ConeGeom), _dp, _dp, C.c_int]
        L.or_edge_step_vol.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_int,
                                       C.POINTER(Trace), C.c_int]
        L.or_proj_A.argtypes = [C.POINTER(Projector), _dp, _dp]
        L.or_proj_AT.argtypes = [C.POINTER(Projector), _dp, _dp]
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# geometry helpers
# --------------------------------------------------------------------------
@dataclass
class Fan:
    n: int
    pixel_mm: float
    nviews: int
    ndets: int
    sod_mm: float = 541.0
    sdd_mm: float = 949.0
    det_pitch_deg: float = 0.0
    off_center: float = 0.5
    view0_deg: float = 0.0
    view_step_deg: float = 0.0
    ends: np.ndarray | None = None  # [nviews*ndets, 4] ray table (sx, sy, dx, dy)

    def c(self) -> FanGeom:
        ptr = None
        if self.ends is not None:
            self.ends = np.ascontiguousarray(self.ends, np.float64)
            assert self.ends.shape == (self.nviews * self.ndets, 4)
            ptr = self.ends.ctypes.data
        return FanGeom(self.n, self.pixel_mm, self.nviews, self.ndets, self.sod_mm, self.sdd_mm,
                       self.det_pitch_deg, self.off_center, self.view0_deg, self.view_step_deg, ptr)


def fan_from_engine(geom) -> Fan:
    """Build the oracle's fan description from an engine-side geometry object
    that has the same field names (n, pixel_mm, nviews, ndets, ...), or from a
    ray table (an object with an `endpoints` array)."""
    if getattr(geom, "endpoints", None) is not None:
        return Fan(geom.n, geom.pixel_mm, geom.nviews, geom.ndets, ends=geom.endpoints)
    return Fan(geom.n, geom.pixel_mm, geom.nviews, geom.ndets, geom.sod_mm, geom.sdd_mm,
               geom.det_pitch_deg, geom.off_center, geom.view0_deg, geom.view_step_deg)


def projector(geom, nthreads: int = 0) -> Projector:
    """GoldenC (None), fan beam / ray table (Fan) or cone beam (an object
    with the cone-geometry fields, e.g. ConeGeometry)."""
    if geom is None:
        return Projector(0, FanGeom(), nthreads)
    if hasattr(geom, "ndx"):
        return Projector(2, FanGeom(), nthreads, cone_c(geom))
    return Projector(1, geom.c(), nthreads)


def _image_shape(geom):
    if geom is None:
        return (GC_N, GC_N)
    if hasattr(geom, "ndx"):
        return (geom.nz, geom.nx, geom.ny)
    return (geom.n, geom.n)


# --------------------------------------------------------------------------
# GoldenC projector
# --------------------------------------------------------------------------
def gc_A(img: np.ndarray) -> np.ndarray:
    out = np.zeros((GC_VIEWS, GC_DETS), np.float64)
    lib().or_gc_A(out, np.ascontiguousarray(img, np.float64))
    return out


def gc_AStar(sino: np.ndarray) -> np.ndarray:
    out = np.zeros((GC_N, GC_N), np.float64)
    lib().or_gc_AStar(out, np.ascontiguousarray(sino, np.float64))
    return out


def gc_walk(alpha: int, tile: int, raynum: int):
    ix = np.zeros(1024, np.int32)
    iy = np.zeros(1024, np.int32)
    w = np.zeros(1024, np.float64)
    n = lib().or_gc_walk(alpha, tile, raynum, ix, iy, w, 1024)
    return ix[:n].copy(), iy[:n].copy(), w[:n].copy()


# --------------------------------------------------------------------------
# fan projector
# --------------------------------------------------------------------------
def fan_trace(fan: Fan, view: int, det: int):
    cap = 2 * fan.n + 8
    ind = np.zeros(cap, np.int32)
    wgt = np.zeros(cap, np.float64)
    oob = C.c_int(0)
    g = fan.c()
    n = lib().or_fan_trace(C.byref(g), view, det, ind, wgt, cap, C.byref(oob))
    return ind[:n].copy(), wgt[:n].copy(), oob.value


def fan_endpoints(fan: Fan, view: int, det: int):
    vals = [C.c_double() for _ in range(4)]
    g = fan.c()
    lib().or_fan_endpoints(C.byref(g), view, det, *[C.byref(v) for v in vals])
    return tuple(v.value for v in vals)


def fan_segments(fan: Fan, nthreads: int = 0) -> int:
    g = fan.c()
    return int(lib().or_fan_count_segments(C.byref(g), nthreads))


def fan_A(fan: Fan, img: np.ndarray, nthreads: int = 0) -> np.ndarray:
    out = np.zeros((fan.nviews, fan.ndets), np.float64)
    g = fan.c()
    lib().or_fan_A(C.byref(g), out, np.ascontiguousarray(img, np.float64), nthreads)
    return out


def fan_AT(fan: Fan, sino: np.ndarray, nthreads: int = 0) -> np.ndarray:
    out = np.zeros((fan.n, fan.n), np.float64)
    g = fan.c()
    lib().or_fan_AT(C.byref(g), out, np.ascontiguousarray(sino, np.float64), nthreads)
    return out


# --------------------------------------------------------------------------
# solver
# --------------------------------------------------------------------------
def _new_trace(cap: int = 4096):
    recs = (TraceRec * cap)()
    tr = Trace(C.cast(recs, C.POINTER(TraceRec)), cap, 0)
    return tr, recs


def _trace_list(tr: Trace, recs):
    return [(r.outer, r.step, r.k, tuple(r.s), r.exit_reason) for r in recs[: tr.count]]


def solve(fan: Fan | None, g: np.ndarray, alpha: float, beta: float, epsilon: float,
          iter_alt: int, iter_image: int = 10, iter_edge: int = 10, nthreads: int = 0):
    """FP64 AT reconstruction (GoldenC main.c:35-49) with the GoldenC projector
    (fan=None) or the fan-beam projector.  Returns (f, v, trace)."""
    P = projector(fan, nthreads)
    f = np.zeros(_image_shape(fan), np.float64)
    v = np.ones(_image_shape(fan), np.float64)
    tr, recs = _new_trace()
    lib().or_solve(C.byref(P), np.ascontiguousarray(g, np.float64), f, v, alpha, beta, epsilon,
                   iter_alt, iter_image, iter_edge, C.byref(tr))
    return f, v, _trace_list(tr, recs)


def image_step(fan: Fan | None, g, f, v, alpha, epsilon, iter_image, nthreads: int = 0):
    P = projector(fan, nthreads)
    out = np.zeros_like(f, dtype=np.float64)
    tr, recs = _new_trace()
    lib().or_image_step(C.byref(P), out, np.ascontiguousarray(g, np.float64),
                        np.ascontiguousarray(f, np.float64), np.ascontiguousarray(v, np.float64),
                        alpha, epsilon, iter_image, C.byref(tr), 1)
    return out, _trace_list(tr, recs)


def edge_step(f, v, alpha, beta, epsilon, iter_edge):
    """GoldenC's edge step on an image (n, n) or a volume (nz, n, n)."""
    f = np.ascontiguousarray(f, np.float64)
    nz, n = (1, f.shape[0]) if f.ndim == 2 else (f.shape[0], f.shape[1])
    out = np.zeros(f.shape, np.float64)
    tr, recs = _new_trace()
    lib().or_edge_step_vol(n, nz, out, f, np.ascontiguousarray(v, np.float64), alpha, beta, epsilon, iter_edge,
                           C.byref(tr), 1)
    return out, _trace_list(tr, recs)


def medfilt2(img: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(img, np.float64).copy()
    lib().or_medfilt2(out.shape[0], out)
    return out


# --------------------------------------------------------------------------
# 3D cone beam (industry3d/src/tracing.cpp restated)
# --------------------------------------------------------------------------
def cone_c(geom) -> ConeGeom:
    """ConeGeom from an object with the fields nx, ny, nz, voxel_mm, nproj,
    ndx, ndy, pitch_mm, sod_mm, sdd_mm, half_rows, half_cols."""
    return ConeGeom(geom.nx, geom.ny, geom.nz, geom.voxel_mm, geom.nproj, geom.ndx, geom.ndy, geom.pitch_mm,
                    geom.sod_mm, geom.sdd_mm, geom.half_rows, geom.half_cols)


def cone_endpoints(geom, view: int, row: int, col: int):
    s = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    g = cone_c(geom)
    lib().or_cone_endpoints(C.byref(g), view, row, col, s, d)
    return s, d


def cone_trace(geom, view: int, row: int, col: int, mark_off: bool = False):
    """(voxel index, FP32 weight) of every segment; with mark_off, segments
    whose voxel lies off the grid have index -1."""
    cap = 2 * (geom.nx + geom.ny + geom.nz) + 16
    ind = np.zeros(cap, np.int64)
    wgt = np.zeros(cap, np.float32)
    g = cone_c(geom)
    n = lib().or_cone_trace(C.byref(g), view, row, col, ind, wgt, cap, int(mark_off))
    return ind[:n].copy(), wgt[:n].copy()


def cone_trace_points(nx, ny, nz, s, d):
    cap = 2 * (nx + ny + nz) + 16
    ind = np.zeros(cap, np.int64)
    wgt = np.zeros(cap, np.float32)
    n = lib().or_cone_trace_points(nx, ny, nz, *[float(x) for x in s], *[float(x) for x in d], ind, wgt, cap, 0)
    return ind[:n].copy(), wgt[:n].copy()


def cone_segments(geom, nthreads: int = 0) -> int:
    g = cone_c(geom)
    return int(lib().or_cone_count_segments(C.byref(g), nthreads))


def cone_A(geom, vol: np.ndarray, nthreads: int = 0) -> np.ndarray:
    out = np.zeros((geom.nproj, geom.ndx, geom.ndy), np.float64)
    g = cone_c(geom)
    lib().or_cone_A(C.byref(g), out, np.ascontiguousarray(vol, np.float64), nthreads)
    return out


def cone_AT(geom, sino: np.ndarray, nthreads: int = 0) -> np.ndarray:
    out = np.zeros((geom.nz, geom.nx, geom.ny), np.float64)
    g = cone_c(geom)
    lib().or_cone_AT(C.byref(g), out, np.ascontiguousarray(sino, np.float64), nthreads)
    return out


# --------------------------------------------------------------------------
# msbeam/CPU_OpenMP restatement (row-action AT, the OpenMP CPU comparator)
# --------------------------------------------------------------------------
MS_N, MS_NPROJ, MS_NRAY = 512, 180, 768


def ms_phantom() -> np.ndarray:
    f = np.zeros((MS_N, MS_N), np.float32)
    lib().or_ms_phantom(f)
    return f


def ms_A(img: np.ndarray) -> np.ndarray:
    g = np.zeros((MS_NPROJ, MS_NRAY), np.float32)
    lib().or_ms_A(g, np.ascontiguousarray(img, np.float32))
    return g


def ms_solve_phased(g: np.ndarray, iters: int = 10, phases: int = 4):
    """One thread, rays of each view in `phases` interleaved groups (the GPU
    row-action order); phases = 1 is msbeam's own one-thread order."""
    f = np.zeros((MS_N, MS_N), np.float32)
    v = np.ones((MS_N, MS_N), np.float32)
    lib().or_ms_solve_phased(np.ascontiguousarray(g, np.float32), f, v, iters, phases)
    return f, v


def ms_solve(g: np.ndarray, iters: int = 10, nthreads: int = 0):
    f = np.zeros((MS_N, MS_N), np.float32)
    v = np.ones((MS_N, MS_N), np.float32)
    lib().or_ms_solve(np.ascontiguousarray(g, np.float32), f, v, iters, nthreads)
    return f, v


# --------------------------------------------------------------------------
# the reference's own sources (oracle/_ref), only where they were built
# --------------------------------------------------------------------------
class Ref:
    """The reference's GoldenC main.c/proj.c and helical tracer, compiled by
    oracle/ref.mk.  ``Ref.available()`` is False on hosts without them."""

    @staticmethod
    def available() -> bool:
        return all(os.path.exists(os.path.join(REF_DIR, f))
                   for f in ("libgoldnc_ref.so", "libfan_ref.so", "libmsbeam_ref.so", "libcone_ref.so"))

    def __init__(self):
        self.gc = C.CDLL(os.path.join(REF_DIR, "libgoldnc_ref.so"))
        self.fan = C.CDLL(os.path.join(REF_DIR, "libfan_ref.so"))
        self.gc.A.argtypes = [_dp, _dp]
        self.gc.AStar.argtypes = [_dp, _dp]
        self.gc.medfilt2.argtypes = [_dp]
        self.gc.minimize_in_IMAGE_variable.argtypes = [_dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int]
        self.gc.minimize_in_EDGE_variable.argtypes = [_dp, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                                      C.c_int]
        self.fan.fanref_trace.argtypes = [C.c_int, C.c_double] + [C.c_double] * 4 + [_ip, _dp]
        self.fan.fanref_trace.restype = C.c_int
        self.cone = C.CDLL(os.path.join(REF_DIR, "libcone_ref.so"))
        self.cone.coneref_endpoints.argtypes = [C.c_int] * 3 + [C.c_float] + [C.c_int] * 3 + [C.c_float] * 3 + \
            [C.c_int] * 3 + [_fp32, _fp32]
        self.cone.coneref_trace.argtypes = [C.c_int] * 3 + [C.c_float] * 6 + [_i64, _fp32]
        self.cone.coneref_trace.restype = C.c_int
        self.ms = C.CDLL(os.path.join(REF_DIR, "libmsbeam_ref.so"))
        self.ms.msbeam_ref_main.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        self.ms.A.argtypes = [_fp32, _fp32]

    def A(self, img):
        out = np.zeros((GC_VIEWS, GC_DETS), np.float64)
        self.gc.A(out, np.ascontiguousarray(img, np.float64))
        return out

    def AStar(self, sino):
        out = np.zeros((GC_N, GC_N), np.float64)
        self.gc.AStar(out, np.ascontiguousarray(sino, np.float64))
        return out

    def medfilt2(self, img):
        out = np.ascontiguousarray(img, np.float64).copy()
        self.gc.medfilt2(out)
        return out

    def image_step(self, g, f, v, alpha, epsilon, iters):
        out = np.zeros((GC_N, GC_N), np.float64)
        self.gc.minimize_in_IMAGE_variable(out, np.ascontiguousarray(g, np.float64),
                                           np.ascontiguousarray(f, np.float64),
                                           np.ascontiguousarray(v, np.float64), alpha, epsilon, iters)
        return out

    def edge_step(self, f, v, alpha, beta, epsilon, iters):
        out = np.zeros((GC_N, GC_N), np.float64)
        self.gc.minimize_in_EDGE_variable(out, np.ascontiguousarray(f, np.float64),
                                          np.ascontiguousarray(v, np.float64), alpha, beta, epsilon, iters)
        return out

    def fan_trace_points(self, n, px, sx, sy, dx, dy):
        ind = np.zeros(4 * n + 64, np.int32)
        wgt = np.zeros(4 * n + 64, np.float64)
        k = self.fan.fanref_trace(n, px, sx, sy, dx, dy, ind, wgt)
        return ind[:k].copy(), wgt[:k].copy()


def ref_msbeam_run(ref: "Ref", nthreads: int, workdir: str):
    """Runs the reference msbeam program (its own phantom, data and 10 sweeps)
    in `workdir` (it writes std.dat, g.dat, img.dat, edge.dat there) and
    returns its final f and v from the library's globals."""
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        argv = (C.c_char_p * 2)(b"msbeam", str(nthreads).encode())
        ref.ms.msbeam_ref_main(2, argv)
    finally:
        os.chdir(cwd)
    f = np.ctypeslib.as_array((C.c_float * (MS_N * MS_N)).in_dll(ref.ms, "f")).reshape(MS_N, MS_N).copy()
    v = np.ctypeslib.as_array((C.c_float * (MS_N * MS_N)).in_dll(ref.ms, "v")).reshape(MS_N, MS_N).copy()
    return f, v


def ref_cone_endpoints(ref: "Ref", geom, view: int, row: int, col: int):
    s = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    ref.cone.coneref_endpoints(geom.nx, geom.ny, geom.nz, geom.voxel_mm, geom.nproj, geom.ndx, geom.ndy,
                               geom.pitch_mm, geom.sod_mm, geom.sdd_mm, view, row, col, s, d)
    return s, d


def ref_cone_trace_points(ref: "Ref", nx, ny, nz, s, d):
    cap = 4 * (nx + ny + nz) + 16  # the reference writes without a bound
    ind = np.zeros(cap, np.int64)
    wgt = np.zeros(cap, np.float32)
    n = ref.cone.coneref_trace(nx, ny, nz, *[float(x) for x in s], *[float(x) for x in d], ind, wgt)
    return ind[:n].copy(), wgt[:n].copy()

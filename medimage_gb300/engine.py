"""ctypes bindings of libat_engine.so (include/at_engine.h, include/goldnc.h)."""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libat_engine.so")

AT_GEOM_GOLDNC, AT_GEOM_FAN, AT_GEOM_RAYS, AT_GEOM_CONE = 0, 1, 2, 3
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class AtError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, call: str, code: int, msg: str):
        super().__init__(f"{call} failed ({code}): {msg}")
        self.code = code


class _FanGeom(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("pixel_mm", C.c_double),
        ("nviews", C.c_int32),
        ("ndets", C.c_int32),
        ("sod_mm", C.c_double),
        ("sdd_mm", C.c_double),
        ("det_pitch_deg", C.c_double),
        ("off_center", C.c_double),
        ("view0_deg", C.c_double),
        ("view_step_deg", C.c_double),
    ]


class _ConeGeom(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("voxel_mm", C.c_float),
                ("nproj", C.c_int32), ("ndx", C.c_int32), ("ndy", C.c_int32), ("pitch_mm", C.c_float),
                ("sod_mm", C.c_float), ("sdd_mm", C.c_float), ("half_rows", C.c_int32), ("half_cols", C.c_int32)]


class _RowActionParams(C.Structure):
    _fields_ = [("alpha", C.c_float), ("beta", C.c_double), ("epsilon", C.c_double), ("lambda0", C.c_float),
                ("lambda_decay", C.c_float), ("sweeps", C.c_int32), ("phases", C.c_int32)]


class _Params(C.Structure):
    _fields_ = [
        ("alpha", C.c_double),
        ("beta", C.c_double),
        ("epsilon", C.c_double),
        ("iter_alt", C.c_int32),
        ("iter_image", C.c_int32),
        ("iter_edge", C.c_int32),
        ("mode", C.c_int32),
    ]


class _PlanStats(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n", C.c_int32),
        ("nviews", C.c_int32),
        ("ndets", C.c_int32),
        ("rays", C.c_int64),
        ("segments", C.c_int64),
        ("offgrid", C.c_int64),
        ("device_bytes", C.c_int64),
        ("max_segments", C.c_int32),
        ("fp_rays_per_thread", C.c_int32),
        ("bp_runs", C.c_int64),
        ("nz", C.c_int32),
        ("slab_views", C.c_int32),
        ("slab_rays", C.c_int32),
        ("slab_rows", C.c_int32),
        ("slab_wbox", C.c_int32),
        ("slab_fallback_ctas", C.c_int32),
        ("bp_table_use", C.c_int32),
        ("bp_table_bytes", C.c_int64),
        ("bp_table_weights", C.c_int64),
    ]


class _ServerConfig(C.Structure):
    _fields_ = [
        ("hbm_budget_bytes", C.c_size_t),
        ("max_active", C.c_int32),
        ("alpha", C.c_double),
        ("beta", C.c_double),
        ("epsilon", C.c_double),
        ("iter_image", C.c_int32),
        ("iter_edge", C.c_int32),
        ("mode", C.c_int32),
        ("fp_rays_per_thread", C.c_int32),
    ]


class _ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64),
        ("completed", C.c_int64),
        ("rounds", C.c_int64),
        ("p50_latency_s", C.c_double),
        ("p99_latency_s", C.c_double),
        ("max_latency_s", C.c_double),
        ("slices_per_s", C.c_double),
        ("busy_s", C.c_double),
        ("peak_state_bytes", C.c_size_t),
        ("psnr_stops", C.c_int64),
    ]


# exported symbol -> (argtypes, restype); the table doubles as the ABI list the
# CPU tests compare with include/*.h
SIGNATURES = {
    "at_last_error": ([], C.c_char_p),
    "at_device_info": ([C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_size_t)], C.c_int),
    "at_plan_create_fan": ([C.POINTER(_FanGeom), C.POINTER(C.c_void_p)], C.c_int),
    "at_plan_create_fan_ex": ([C.POINTER(_FanGeom), C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "at_plan_create_goldnc": ([C.POINTER(C.c_void_p)], C.c_int),
    "at_plan_set_forward_variant": ([C.c_void_p, C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "at_plan_set_back_variant": ([C.c_void_p, C.c_int32], C.c_int),
    "at_set_batch_launch_mode": ([C.c_int32], C.c_int),
    "at_rowaction_create": ([C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "at_rowaction_destroy": ([C.c_void_p], None),
    "at_rowaction_segments": ([C.c_void_p, C.POINTER(C.c_int64)], C.c_int),
    "at_rowaction_trace": ([C.c_void_p, C.c_int32, C.c_int32, _ip, _fp, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "at_rowaction_forward": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "at_rowaction_run": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(_RowActionParams),
                          C.c_void_p], C.c_int),
    "at_plan_create_cone": ([C.POINTER(_ConeGeom), C.POINTER(C.c_void_p)], C.c_int),
    "at_plan_create_rays": ([C.c_int32, C.c_double, C.c_int32, C.c_int32, _dp, C.POINTER(C.c_void_p)], C.c_int),
    "at_plan_destroy": ([C.c_void_p], None),
    "at_plan_get_stats": ([C.c_void_p, C.POINTER(_PlanStats)], C.c_int),
    "at_plan_trace_ray": ([C.c_void_p, C.c_int32, C.c_int32, _ip, _fp, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "at_forward": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "at_back": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "at_forward_host": ([C.c_void_p, _fp, _fp], C.c_int),
    "at_back_host": ([C.c_void_p, _fp, _fp], C.c_int),
    "at_dev_alloc": ([C.POINTER(C.c_void_p), C.c_size_t], C.c_int),
    "at_dev_free": ([C.c_void_p], C.c_int),
    "at_memcpy_h2d": ([C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p], C.c_int),
    "at_memcpy_d2h": ([C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p], C.c_int),
    "at_stream_create": ([C.POINTER(C.c_void_p)], C.c_int),
    "at_stream_destroy": ([C.c_void_p], C.c_int),
    "at_stream_sync": ([C.c_void_p], C.c_int),
    "at_solver_create": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(_Params), C.POINTER(C.c_void_p)], C.c_int),
    "at_solver_destroy": ([C.c_void_p], None),
    "at_projset_create": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)], C.c_int),
    "at_projset_destroy": ([C.c_void_p], None),
    "at_projset_forward": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_void_p], C.c_int),
    "at_projset_back": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_void_p], C.c_int),
    "at_solver_footprint": ([C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_size_t)], C.c_int),
    "at_solver_set_sino": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "at_solver_set_sino_host": ([C.c_void_p, C.c_int32, _fp, C.c_void_p], C.c_int),
    "at_solver_reset": ([C.c_void_p, C.c_void_p], C.c_int),
    "at_solver_run": ([C.c_void_p, C.c_void_p], C.c_int),
    "at_solver_step": ([C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "at_solver_get": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "at_solver_get_host": ([C.c_void_p, C.c_int32, _fp, _fp, C.c_void_p], C.c_int),
    "at_solver_set_fv_host": ([C.c_void_p, C.c_int32, _fp, _fp, C.c_void_p], C.c_int),
    "at_solver_trace": ([C.c_void_p, C.c_int32, _dp, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "at_solver_launches_per_outer": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "at_reconstruct_host": ([C.c_void_p, C.POINTER(_Params), _fp, _fp, _fp], C.c_int),
    "at_forward_residual_noalloc": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
                                    C.c_int),
    "at_psnr": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_double), C.c_void_p], C.c_int),
    "at_ssim": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.POINTER(C.c_double), C.c_void_p],
                C.c_int),
    "at_server_create": ([C.POINTER(_ServerConfig), C.POINTER(C.c_void_p)], C.c_int),
    "at_server_destroy": ([C.c_void_p], None),
    "at_server_submit": ([C.c_void_p, C.c_void_p, _fp, C.c_int32, C.c_double, C.POINTER(C.c_int64)], C.c_int),
    "at_server_run": ([C.c_void_p, C.c_double], C.c_int),
    "at_server_submit_psnr": ([C.c_void_p, C.c_void_p, _fp, C.c_int32, C.c_double, _fp, C.c_double, C.c_double,
                               C.POINTER(C.c_int64)], C.c_int),
    "at_server_result_info": ([C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                               C.POINTER(C.c_int32)], C.c_int),
    "at_server_result": ([C.c_void_p, C.c_int64, _fp, _fp, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    "at_server_get_stats": ([C.c_void_p, C.POINTER(_ServerStats)], C.c_int),
    # GoldenC drop-in (include/goldnc.h)
    "A": ([_dp, _dp], None),
    "AStar": ([_dp, _dp], None),
    "minimize_in_IMAGE_variable": ([_dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int], None),
    "minimize_in_EDGE_variable": ([_dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_int], None),
    "medfilt2": ([_dp], None),
    "MumfordShah": ([C.c_double, C.c_double, C.c_double], None),
    "goldnc_status": ([], C.c_int),
    "goldnc_set_iterations": ([C.c_int, C.c_int, C.c_int], None),
}

_lib = None


def lib() -> C.CDLL:
    """Load libat_engine.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m medimage_gb300.build` "
                "(the engine has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(call: str, rc: int) -> None:
    if rc != 0:
        raise AtError(call, rc, lib().at_last_error().decode(errors="replace"))


def device_info():
    name = C.create_string_buffer(256)
    sms = C.c_int()
    mem = C.c_size_t()
    _check("at_device_info", lib().at_device_info(name, 256, C.byref(sms), C.byref(mem)))
    return {"name": name.value.decode(), "sm_count": sms.value, "hbm_bytes": mem.value}


@dataclass
class FanGeometry:
    """2D fan-beam geometry with the parameters of the reference's fan tracer
    (helical/rebin/src/main.h:16-47, ms2d.cpp:30-62,172-183)."""

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

    @classmethod
    def covering(cls, n: int, pixel_mm: float, nviews: int, ndets: int, sod_mm: float = 541.0,
                 sdd_mm: float = 949.0, arc_deg: float = 360.0) -> "FanGeometry":
        """Equiangular detector whose fan just covers the image's circumscribed
        circle (fan = 2 asin(r / SOD), r = n * pixel * sqrt(2) / 2), views evenly
        over `arc_deg`."""
        r = n * pixel_mm * math.sqrt(2.0) / 2.0
        fan_deg = 2.0 * math.degrees(math.asin(r / sod_mm))
        return cls(n, pixel_mm, nviews, ndets, sod_mm, sdd_mm, fan_deg / ndets, 0.5, 0.0, arc_deg / nviews)

    def c(self) -> _FanGeom:
        return _FanGeom(self.n, self.pixel_mm, self.nviews, self.ndets, self.sod_mm, self.sdd_mm,
                        self.det_pitch_deg, self.off_center, self.view0_deg, self.view_step_deg)


@dataclass
class RayGeometry:
    """Any 2D geometry as a table of rays: endpoints[view*ndets + det] =
    (sx, sy, dx, dy) in mm, the arguments of the reference tracer
    forward_proj (helical/rebin/src/tracing.cpp:22-147), in the frame of
    FanGeometry (pixel index x*n + y, image on [0, n*pixel_mm]^2)."""

    n: int
    pixel_mm: float
    nviews: int
    ndets: int
    endpoints: np.ndarray = field(repr=False, default=None)

    def __post_init__(self):
        self.endpoints = np.ascontiguousarray(self.endpoints, np.float64).reshape(self.nviews * self.ndets, 4)

    @classmethod
    def fan_from_view_table(cls, n: int, pixel_mm: float, ndets: int, angle_deg, sod_mm: float = 541.0,
                            sdd_mm: float = 949.0, det_pitch_deg: float = 0.0,
                            off_center: float = 0.5) -> "RayGeometry":
        """Fan beam whose source angles come from a view table (one angle per
        projection, any spacing), as helical/rebin reads them
        (ms2d.cpp:30-62) and places source and detector (ms2d.cpp:172-183).
        The trig goes through the C library like the reference's."""
        ang = [float(a) for a in np.asarray(angle_deg, np.float64).ravel()]
        per_rad = det_pitch_deg * math.pi / 180.0
        half = ndets // 2
        dets = [((j + off_center) * per_rad + math.pi) for j in range(-half, ndets - half)]
        dcos = [math.cos(a) for a in dets]
        dsin = [math.sin(a) for a in dets]
        out = np.empty((len(ang), ndets, 4), np.float64)
        for v, a in enumerate(ang):
            scos, ssin = math.cos(a / 180.0 * math.pi), math.sin(a / 180.0 * math.pi)
            sx = sod_mm * scos + n * pixel_mm / 2.0
            sy = sod_mm * ssin + n * pixel_mm / 2.0
            for j in range(ndets):
                out[v, j, 0] = sx
                out[v, j, 1] = sy
                out[v, j, 2] = sdd_mm * (dcos[j] * scos - dsin[j] * ssin) + sx
                out[v, j, 3] = sdd_mm * (dsin[j] * scos + dcos[j] * ssin) + sy
        return cls(n, pixel_mm, len(ang), ndets, out.reshape(-1, 4))

    @classmethod
    def msbeam_parallel(cls, n: int = 512, nproj: int = 180, nray: int = 768) -> "RayGeometry":
        """The parallel beam of msbeam/CPU_OpenMP (proj.c:53-65, proto.h:4-6):
        unit pixels, view k at angle pi*k/nproj (sin and cos rounded to float
        as there), ray r on the line through t*(-sin, cos), t = r - nray/2,
        along (cos, sin).  msbeam addresses pixel (ix, iy) as iy*n + ix, so its
        (x, y) is (y, x) here; each ray is given by two points n units either
        side of its closest approach to the centre."""
        out = np.empty((nproj, nray, 4), np.float64)
        half = n / 2.0
        for k in range(nproj):
            sin_t = float(np.float32(math.sin(3.14159265359 / nproj * k)))
            cos_t = float(np.float32(math.cos(3.14159265359 / nproj * k)))
            for r in range(nray):
                t = float(r - nray // 2)
                mx, my = -sin_t * t + half, cos_t * t + half  # msbeam (x, y) of the closest point
                px, py = my, mx                                # this frame
                ux, uy = sin_t, cos_t                          # direction (cos, sin) swapped
                out[k, r] = (px - n * ux, py - n * uy, px + n * ux, py + n * uy)
        return cls(n, 1.0, nproj, nray, out.reshape(-1, 4))


@dataclass
class ConeGeometry:
    """3D cone beam with a flat detector: the parameters of industry3d
    (ct3d.h:17-56, tracing.cpp:51-81).  Volume nz x nx x ny voxels
    (index z*nx*ny + x*ny + y), sinogram [nproj][ndx][ndy].  half_rows and
    half_cols centre the detector; the reference uses NDX/2 for both."""

    nx: int
    ny: int
    nz: int
    voxel_mm: float
    nproj: int
    ndx: int
    ndy: int
    pitch_mm: float
    sod_mm: float
    sdd_mm: float
    half_rows: int = -1
    half_cols: int = -1

    def __post_init__(self):
        if self.half_rows < 0:
            self.half_rows = self.ndx // 2
        if self.half_cols < 0:
            self.half_cols = self.ndy // 2

    def c(self) -> _ConeGeom:
        return _ConeGeom(self.nx, self.ny, self.nz, self.voxel_mm, self.nproj, self.ndx, self.ndy, self.pitch_mm,
                         self.sod_mm, self.sdd_mm, self.half_rows, self.half_cols)


@dataclass
class Params:
    """AT weights and iteration counts; defaults are GoldenC's config.h:6-17."""

    alpha: float = 1000.0
    beta: float = 0.002
    epsilon: float = 0.0001
    iter_alt: int = 10
    iter_image: int = 10
    iter_edge: int = 10
    mode: int = 0  # 0 exact projection count, 1 linear-mode sinogram updates

    def c(self) -> _Params:
        return _Params(self.alpha, self.beta, self.epsilon, self.iter_alt, self.iter_image, self.iter_edge,
                       self.mode)


class Plan:
    """Device-resident projector plan of one geometry."""

    def __init__(self, handle: C.c_void_p, geom):
        self._h = handle
        self.geom = geom
        st = _PlanStats()
        _check("at_plan_get_stats", lib().at_plan_get_stats(self._h, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in _PlanStats._fields_}
        self.n, self.nviews, self.ndets, self.nz = st.n, st.nviews, st.ndets, st.nz
        if st.kind == AT_GEOM_CONE:
            self.img_shape = (st.nz, st.n, st.n)
            self.sino_shape = (geom.nproj, geom.ndx, geom.ndy)
        else:
            self.img_shape = (st.n, st.n)
            self.sino_shape = (st.nviews, st.ndets)

    @classmethod
    def fan(cls, geom: FanGeometry, alpha: str = "fp64") -> "Plan":
        """alpha="fp64": the reference's FP64 traversal (bit-identical pixel
        sequences); "fp32": the same steps in FP32 (the plain form, kept to
        measure the precision each form reaches)."""
        if alpha not in ("fp64", "fp32"):
            raise ValueError(f"alpha must be 'fp64' or 'fp32', not {alpha!r}")
        h = C.c_void_p()
        g = geom.c()
        _check("at_plan_create_fan_ex", lib().at_plan_create_fan_ex(C.byref(g), 0 if alpha == "fp64" else 1,
                                                                    C.byref(h)))
        return cls(h, geom)

    @classmethod
    def rays(cls, geom: RayGeometry) -> "Plan":
        h = C.c_void_p()
        _check("at_plan_create_rays", lib().at_plan_create_rays(geom.n, geom.pixel_mm, geom.nviews, geom.ndets,
                                                                geom.endpoints, C.byref(h)))
        return cls(h, geom)

    @classmethod
    def cone(cls, geom: ConeGeometry) -> "Plan":
        h = C.c_void_p()
        g = geom.c()
        _check("at_plan_create_cone", lib().at_plan_create_cone(C.byref(g), C.byref(h)))
        return cls(h, geom)

    @classmethod
    def goldnc(cls) -> "Plan":
        h = C.c_void_p()
        _check("at_plan_create_goldnc", lib().at_plan_create_goldnc(C.byref(h)))
        return cls(h, None)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib().at_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_forward_variant(self, views: int = 0, rays: int = 0, rows: int = 0) -> None:
        """Pin the forward projector: (0, 0, 0) the L1 walk, else the slab
        projector with that CTA shape and slab height (bitwise the same sums)."""
        _check("at_plan_set_forward_variant", lib().at_plan_set_forward_variant(self._h, views, rays, rows))
        st = _PlanStats()
        _check("at_plan_get_stats", lib().at_plan_get_stats(self._h, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in _PlanStats._fields_}

    def set_back_variant(self, use: int) -> None:
        """Back projector of later batches: bit0 single scans, bit1 groups of
        scans sharing the plan gather from the pixel table (built on first
        use); a clear bit walks tile runs.  Bitwise the same sums."""
        _check("at_plan_set_back_variant", lib().at_plan_set_back_variant(self._h, use))
        st = _PlanStats()
        _check("at_plan_get_stats", lib().at_plan_get_stats(self._h, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in _PlanStats._fields_}

    def trace_ray(self, view: int, det: int):
        cap = 4 * 8192
        pix = np.zeros(cap, np.int32)
        w = np.zeros(cap, np.float32)
        n = C.c_int32()
        _check("at_plan_trace_ray", lib().at_plan_trace_ray(self._h, view, det, pix, w, cap, C.byref(n)))
        return pix[: n.value].copy(), w[: n.value].copy()

    def forward(self, img: np.ndarray) -> np.ndarray:
        img = np.ascontiguousarray(img, np.float32)
        if img.shape != self.img_shape:
            raise ValueError(f"image shape {img.shape}, plan expects {self.img_shape}")
        out = np.zeros(self.sino_shape, np.float32)
        _check("at_forward_host", lib().at_forward_host(self._h, img, out))
        return out

    def back(self, sino: np.ndarray) -> np.ndarray:
        sino = np.ascontiguousarray(sino, np.float32)
        if sino.shape != self.sino_shape:
            raise ValueError(f"sinogram shape {sino.shape}, plan expects {self.sino_shape}")
        out = np.zeros(self.img_shape, np.float32)
        _check("at_back_host", lib().at_back_host(self._h, sino, out))
        return out

    def forward_dev(self, d_img: int, d_sino: int, stream: int = 0) -> None:
        _check("at_forward", lib().at_forward(self._h, C.c_void_p(d_img), C.c_void_p(d_sino), C.c_void_p(stream)))

    def back_dev(self, d_sino: int, d_img: int, stream: int = 0) -> None:
        _check("at_back", lib().at_back(self._h, C.c_void_p(d_sino), C.c_void_p(d_img), C.c_void_p(stream)))


def _plan_array(plans):
    arr = (C.c_void_p * len(plans))(*[p.handle for p in plans])
    return arr


class ProjSet:
    """Several images through their plans in one launch per kernel
    (at_projset_*); images of the same Plan object are projected together, up
    to four per walk of the plan.  Device pointers in, device pointers out."""

    def __init__(self, plans):
        self.plans = list(plans)
        self._h = C.c_void_p()
        _check("at_projset_create", lib().at_projset_create(_plan_array(self.plans), len(self.plans),
                                                            C.byref(self._h)))

    def close(self):
        if self._h:
            lib().at_projset_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ptrs(self, ptrs):
        if len(ptrs) != len(self.plans):
            raise ValueError(f"{len(ptrs)} pointers for {len(self.plans)} plans")
        return (C.c_void_p * len(ptrs))(*[C.c_void_p(p) for p in ptrs])

    def forward_dev(self, d_imgs, d_sinos, stream: int = 0) -> None:
        _check("at_projset_forward", lib().at_projset_forward(self._h, self._ptrs(d_imgs), self._ptrs(d_sinos),
                                                              C.c_void_p(stream)))

    def back_dev(self, d_sinos, d_imgs, stream: int = 0) -> None:
        _check("at_projset_back", lib().at_projset_back(self._h, self._ptrs(d_sinos), self._ptrs(d_imgs),
                                                        C.c_void_p(stream)))

    def _host_call(self, forward: bool, arrays):
        if len(arrays) != len(self.plans):
            raise ValueError(f"{len(arrays)} arrays for {len(self.plans)} plans")
        L = lib()
        ins, outs, res, held = [], [], [], []
        try:
            for p, a in zip(self.plans, arrays):
                shape_in, shape_out = (p.img_shape, p.sino_shape) if forward else (p.sino_shape, p.img_shape)
                a = np.ascontiguousarray(a, np.float32)
                if a.shape != shape_in:
                    raise ValueError(f"array shape {a.shape}, plan expects {shape_in}")
                out = np.zeros(shape_out, np.float32)
                di, do = C.c_void_p(), C.c_void_p()
                _check("at_dev_alloc", L.at_dev_alloc(C.byref(di), a.nbytes))
                held.append(di)
                _check("at_dev_alloc", L.at_dev_alloc(C.byref(do), out.nbytes))
                held.append(do)
                _check("at_memcpy_h2d", L.at_memcpy_h2d(di, a.ctypes.data, a.nbytes, None))
                ins.append(di.value)
                outs.append(do.value)
                res.append(out)
            (self.forward_dev if forward else self.back_dev)(ins, outs)
            for d, out in zip(outs, res):
                _check("at_memcpy_d2h", L.at_memcpy_d2h(out.ctypes.data, C.c_void_p(d), out.nbytes, None))
            _check("at_stream_sync", L.at_stream_sync(None))
        finally:
            for d in held:
                L.at_dev_free(d)
        return res

    def forward(self, imgs):
        """Host arrays in and out (device copies made and freed here)."""
        return self._host_call(True, imgs)

    def back(self, sinos):
        return self._host_call(False, sinos)


class Solver:
    """Batched AT solver over one or more plans (one scan per plan)."""

    def __init__(self, plans, params: Params):
        self.plans = list(plans)
        self.params = params
        self._h = C.c_void_p()
        arr = _plan_array(self.plans)
        prm = params.c()
        _check("at_solver_create", lib().at_solver_create(arr, len(self.plans), C.byref(prm), C.byref(self._h)))

    @staticmethod
    def footprint(plans) -> int:
        arr = _plan_array(list(plans))
        b = C.c_size_t()
        _check("at_solver_footprint", lib().at_solver_footprint(arr, len(plans), C.byref(b)))
        return b.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().at_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_sino(self, scan: int, sino: np.ndarray, stream: int = 0) -> None:
        p = self.plans[scan]
        sino = np.ascontiguousarray(sino, np.float32)
        if sino.shape != p.sino_shape:
            raise ValueError(f"sinogram shape {sino.shape}, scan {scan}'s plan expects {p.sino_shape}")
        self._keep = sino  # host buffer must live until the copy completes
        _check("at_solver_set_sino_host", lib().at_solver_set_sino_host(self._h, scan, sino, C.c_void_p(stream)))
        self.sync(stream)

    def set_sino_dev(self, scan: int, d_sino: int, stream: int = 0) -> None:
        _check("at_solver_set_sino", lib().at_solver_set_sino(self._h, scan, C.c_void_p(d_sino), C.c_void_p(stream)))

    def set_fv(self, scan: int, f: np.ndarray, v: np.ndarray, stream: int = 0) -> None:
        f = np.ascontiguousarray(f, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        _check("at_solver_set_fv_host", lib().at_solver_set_fv_host(self._h, scan, f, v, C.c_void_p(stream)))
        self.sync(stream)

    def reset(self, stream: int = 0) -> None:
        _check("at_solver_reset", lib().at_solver_reset(self._h, C.c_void_p(stream)))

    def run(self, stream: int = 0, sync: bool = True) -> None:
        _check("at_solver_run", lib().at_solver_run(self._h, C.c_void_p(stream)))
        if sync:
            self.sync(stream)

    def step(self, count: int, stream: int = 0, sync: bool = True) -> None:
        _check("at_solver_step", lib().at_solver_step(self._h, count, C.c_void_p(stream)))
        if sync:
            self.sync(stream)

    @staticmethod
    def sync(stream: int = 0) -> None:
        _check("at_stream_sync", lib().at_stream_sync(C.c_void_p(stream)))

    def get(self, scan: int, stream: int = 0):
        p = self.plans[scan]
        f = np.zeros(p.img_shape, np.float32)
        v = np.zeros(p.img_shape, np.float32)
        _check("at_solver_get_host", lib().at_solver_get_host(self._h, scan, f, v, C.c_void_p(stream)))
        return f, v

    def trace(self, scan: int):
        """Scalar trajectory: list of (outer, step, k, exit, s0..s5)."""
        cap = 4096
        buf = np.zeros(cap * 10, np.float64)
        n = C.c_int32()
        _check("at_solver_trace", lib().at_solver_trace(self._h, scan, buf, cap, C.byref(n)))
        recs = buf[: 10 * n.value].reshape(-1, 10)
        return [(int(r[0]), int(r[1]), int(r[2]), int(r[3]), tuple(float(x) for x in r[4:])) for r in recs]

    @property
    def launches_per_outer(self) -> int:
        n = C.c_int32()
        _check("at_solver_launches_per_outer", lib().at_solver_launches_per_outer(self._h, C.byref(n)))
        return n.value


def set_batch_launch_mode(persistent: bool) -> None:
    """Launch form of batched projections made from now on: persistent
    (resident CTAs pulling work units from a queue) or one CTA per unit (the
    default, measured faster); results are bitwise the same."""
    _check("at_set_batch_launch_mode", lib().at_set_batch_launch_mode(1 if persistent else 0))


def reconstruct(plan: Plan, params: Params, sino: np.ndarray):
    """One call through at_reconstruct_host: host sinogram in, (f, v) out."""
    sino = np.ascontiguousarray(sino, np.float32)
    f = np.zeros(plan.img_shape, np.float32)
    v = np.zeros(plan.img_shape, np.float32)
    prm = params.c()
    _check("at_reconstruct_host", lib().at_reconstruct_host(plan.handle, C.byref(prm), sino, f, v))
    return f, v


class Server:
    """Continuous-batching reconstruction server (at_server_*)."""

    def __init__(self, hbm_budget_bytes: int, max_active: int, params: Params | None = None,
                 fp_rays_per_thread: int = 1):
        p = params or Params()
        cfg = _ServerConfig(hbm_budget_bytes, max_active, p.alpha, p.beta, p.epsilon, p.iter_image, p.iter_edge,
                            p.mode, fp_rays_per_thread)
        self._h = C.c_void_p()
        _check("at_server_create", lib().at_server_create(C.byref(cfg), C.byref(self._h)))
        self._plans = {}

    def close(self):
        if self._h:
            lib().at_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, plan: Plan, sino: np.ndarray, iter_alt: int, arrival_s: float = 0.0) -> int:
        sino = np.ascontiguousarray(sino, np.float32)
        rid = C.c_int64()
        _check("at_server_submit", lib().at_server_submit(self._h, plan.handle, sino, iter_alt, arrival_s,
                                                          C.byref(rid)))
        self._plans[rid.value] = plan
        return rid.value

    def submit_psnr(self, plan: Plan, sino: np.ndarray, iter_alt: int, ref: np.ndarray, target_psnr_db: float,
                    arrival_s: float = 0.0, peak: float = 0.0) -> int:
        """A request with a quality stop: it finishes once PSNR(f, ref) (on the
        GPU after every outer iteration) reaches target_psnr_db, or after
        iter_alt outer iterations."""
        sino = np.ascontiguousarray(sino, np.float32)
        ref = np.ascontiguousarray(ref, np.float32)
        if ref.shape != plan.img_shape:
            raise ValueError(f"reference shape {ref.shape}, plan expects {plan.img_shape}")
        rid = C.c_int64()
        _check("at_server_submit_psnr", lib().at_server_submit_psnr(self._h, plan.handle, sino, iter_alt, arrival_s,
                                                                    ref, target_psnr_db, peak, C.byref(rid)))
        self._plans[rid.value] = plan
        return rid.value

    def result_info(self, rid: int) -> dict:
        it, ps, stop = C.c_int32(), C.c_double(), C.c_int32()
        _check("at_server_result_info", lib().at_server_result_info(self._h, rid, C.byref(it), C.byref(ps),
                                                                    C.byref(stop)))
        return {"iterations": it.value, "psnr_db": ps.value, "stopped_by_psnr": bool(stop.value)}

    def run(self, max_seconds: float = 0.0) -> None:
        _check("at_server_run", lib().at_server_run(self._h, max_seconds))

    def result(self, rid: int):
        p = self._plans[rid]
        f = np.zeros(p.img_shape, np.float32)
        v = np.zeros(p.img_shape, np.float32)
        lat, wait = C.c_double(), C.c_double()
        _check("at_server_result", lib().at_server_result(self._h, rid, f, v, C.byref(lat), C.byref(wait)))
        return f, v, lat.value, wait.value

    def stats(self) -> dict:
        st = _ServerStats()
        _check("at_server_get_stats", lib().at_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}


@dataclass
class RowActionParams:
    """msbeam/CPU_OpenMP's constants (proto.h:8-12, main.c:371,391)."""

    alpha: float = 10.0
    beta: float = 0.35
    epsilon: float = 0.001
    lambda0: float = 0.001
    lambda_decay: float = 500.0
    sweeps: int = 10
    phases: int = 4

    def c(self) -> _RowActionParams:
        return _RowActionParams(self.alpha, self.beta, self.epsilon, self.lambda0, self.lambda_decay, self.sweeps,
                                self.phases)


class RowAction:
    """msbeam's row-action AT on the GPU (at_rowaction_*): its parallel beam of
    nproj views x nray rays over an n x n image (defaults: msbeam's 512, 180,
    768)."""

    def __init__(self, n: int = 512, nproj: int = 180, nray: int = 768):
        self.n, self.nproj, self.nray = n, nproj, nray
        self._h = C.c_void_p()
        _check("at_rowaction_create", lib().at_rowaction_create(n, nproj, nray, C.byref(self._h)))
        seg = C.c_int64()
        _check("at_rowaction_segments", lib().at_rowaction_segments(self._h, C.byref(seg)))
        self.segments = seg.value

    def close(self):
        if self._h:
            lib().at_rowaction_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, view: int, ray: int):
        cap = 4 * self.n
        pix = np.zeros(cap, np.int32)
        w = np.zeros(cap, np.float32)
        k = C.c_int32()
        _check("at_rowaction_trace", lib().at_rowaction_trace(self._h, view, ray, pix, w, cap, C.byref(k)))
        return pix[: k.value].copy(), w[: k.value].copy()

    def forward_dev(self, nslices: int, d_f: int, d_g: int, stream: int = 0) -> None:
        _check("at_rowaction_forward", lib().at_rowaction_forward(self._h, nslices, C.c_void_p(d_f), C.c_void_p(d_g),
                                                                  C.c_void_p(stream)))

    def forward(self, f: np.ndarray) -> np.ndarray:
        """msbeam's projection of an n x n image (host arrays)."""
        f = np.ascontiguousarray(f, np.float32)
        L = lib()
        ptr = []
        try:
            for nbytes in (f.nbytes, self.nproj * self.nray * 4):
                p = C.c_void_p()
                _check("at_dev_alloc", L.at_dev_alloc(C.byref(p), nbytes))
                ptr.append(p.value)
            _check("h2d", L.at_memcpy_h2d(C.c_void_p(ptr[0]), f.ctypes.data, f.nbytes, None))
            self.forward_dev(1, ptr[0], ptr[1])
            g = np.zeros((self.nproj, self.nray), np.float32)
            _check("d2h", L.at_memcpy_d2h(g.ctypes.data, C.c_void_p(ptr[1]), g.nbytes, None))
            _check("sync", L.at_stream_sync(None))
        finally:
            for p in ptr:
                L.at_dev_free(C.c_void_p(p))
        return g

    def run_dev(self, nslices: int, d_g: int, d_f: int, d_v: int, params: RowActionParams | None = None,
                stream: int = 0) -> None:
        prm = (params or RowActionParams()).c()
        _check("at_rowaction_run", lib().at_rowaction_run(self._h, nslices, C.c_void_p(d_g), C.c_void_p(d_f),
                                                          C.c_void_p(d_v), C.byref(prm), C.c_void_p(stream)))

    def run(self, g: np.ndarray, params: RowActionParams | None = None):
        """g: [nproj][nray] or [slices][nproj][nray] host sinograms; returns
        (f, v) with matching leading shape."""
        g = np.ascontiguousarray(g, np.float32)
        single = g.ndim == 2
        gs = g.reshape(-1, self.nproj, self.nray)
        B = gs.shape[0]
        L = lib()
        ptr = []
        try:
            for nbytes in (gs.nbytes, B * self.n * self.n * 4, B * self.n * self.n * 4):
                p = C.c_void_p()
                _check("at_dev_alloc", L.at_dev_alloc(C.byref(p), nbytes))
                ptr.append(p.value)
            _check("h2d", L.at_memcpy_h2d(C.c_void_p(ptr[0]), gs.ctypes.data, gs.nbytes, None))
            self.run_dev(B, ptr[0], ptr[1], ptr[2], params)
            f = np.zeros((B, self.n, self.n), np.float32)
            v = np.zeros((B, self.n, self.n), np.float32)
            _check("d2h", L.at_memcpy_d2h(f.ctypes.data, C.c_void_p(ptr[1]), f.nbytes, None))
            _check("d2h", L.at_memcpy_d2h(v.ctypes.data, C.c_void_p(ptr[2]), v.nbytes, None))
            _check("sync", L.at_stream_sync(None))
        finally:
            for p in ptr:
                L.at_dev_free(C.c_void_p(p))
        return (f[0], v[0]) if single else (f, v)


def quality(x: np.ndarray, ref: np.ndarray, peak: float = 0.0, dynamic_range: float | None = None) -> dict:
    """PSNR (peak <= 0: max(ref)) and SSIM computed on the GPU (at_psnr, at_ssim)."""
    x = np.ascontiguousarray(x, np.float32)
    ref = np.ascontiguousarray(ref, np.float32)
    if x.shape != ref.shape or x.ndim != 2:
        raise ValueError(f"quality: shapes {x.shape} and {ref.shape}; two equal 2D images are needed")
    L = lib()
    ptrs = []
    try:
        for a in (x, ref):
            p = C.c_void_p()
            _check("at_dev_alloc", L.at_dev_alloc(C.byref(p), a.nbytes))
            ptrs.append(p)
            _check("at_memcpy_h2d", L.at_memcpy_h2d(p, a.ctypes.data, a.nbytes, None))
        ps, ss = C.c_double(), C.c_double()
        _check("at_psnr", L.at_psnr(ptrs[0], ptrs[1], x.size, peak, C.byref(ps), None))
        dr = float(dynamic_range) if dynamic_range else float(ref.max() - min(ref.min(), 0.0)) or 1.0
        _check("at_ssim", L.at_ssim(ptrs[0], ptrs[1], x.shape[0], x.shape[1], dr, C.byref(ss), None))
        return {"psnr_db": ps.value, "ssim": ss.value}
    finally:
        for p in ptrs:
            L.at_dev_free(p)

// capi.cu -- the C-ABI of include/at_engine.h and the GoldenC drop-in symbols
// of include/goldnc.h.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/goldnc.h"
#include "solver.h"

namespace medimg {

int fp_ctas(const ScanDev &S, int rpt);
cudaError_t launch_fp_single(const Launch &L, const Plan &p, int rpt, void *scratch, cudaStream_t st);
size_t fp_single_scratch_bytes(const Plan &p);
int bp_ctas(const ScanDev &S);
cudaError_t launch_fp(const Launch &L, int kind, int rpt, int nctas, cudaStream_t st);
cudaError_t launch_bp(const Launch &L, int kind, int nctas, cudaStream_t st, const Launch *Lpix, int pix_nctas);
int pix_ctas(const ScanDev &S);
cudaError_t launch_median(const float *in, float *out, int n, cudaStream_t st);

namespace {
thread_local std::string g_err;
thread_local int g_status = AT_OK;
}  // namespace

int set_error(int code, const std::string &msg) {
  g_err = msg;
  g_status = code;
  return code;
}

int cuda_error(cudaError_t e, const char *what) {
  const int code = (e == cudaErrorMemoryAllocation) ? AT_ENOMEM : AT_ECUDA;
  cudaGetLastError();  // clear a non-sticky error
  return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

int projector_rpt(const Plan &p) {
  std::vector<Plan *> v{const_cast<Plan *>(&p)};
  return Solver::choose_rpt(v);
}

int project(const Plan &p, bool forward, const float *in, float *out, cudaStream_t st) {
  Launch L;
  std::memset(&L, 0, sizeof(L));
  fill_scan_plan(L.single, p);
  L.single.buf[0] = const_cast<float *>(in);
  L.single.buf[1] = out;
  L.scans = nullptr;
  L.prefix = nullptr;
  L.nscans = 1;
  L.flow = FLOW_ALWAYS;
  L.stage = ST_NONE;
  L.in_buf = 0;
  L.out_buf = 1;
  L.aux_buf = -1;
  cudaError_t e;
  if (forward) {
    const int rpt = projector_rpt(p);
    if (p.kind == AT_GEOM_FAN || p.kind == AT_GEOM_RAYS) {
      // stream-ordered scratch for the image's row-major and transposed copies
      void *tr = nullptr;
      AT_CUDA_TRY(cudaMallocAsync(&tr, fp_single_scratch_bytes(p), st));
      e = launch_fp_single(L, p, rpt, tr, st);
      cudaFreeAsync(tr, st);
    } else {
      e = launch_fp(L, p.kind, rpt, fp_ctas(L.single, rpt), st);
    }
  } else {
    // stream-ordered scratch: calls on other streams never share it
    const size_t bpb = bp_scratch_bytes(p);
    void *scratch = nullptr;
    if (bpb) {
      AT_CUDA_TRY(cudaMallocAsync(&scratch, bpb, st));
      if ((e = cudaMemsetAsync(scratch, 0, bpb, st)) != cudaSuccess) {
        cudaFreeAsync(scratch, st);
        return cuda_error(e, "back projection scratch");
      }
      carve_bp_scratch(L.single, p, (char *)scratch);
      L.single.bp_split = bp_split_for(p.ntiles, p.nvb);
    }
    L.bp_table = (L.single.pt_use & 1) ? 1 : 0;
    if (p.kind == AT_GEOM_CONE) L.chunks = (p.nviews + p.cone_bp_views - 1) / std::max(1, p.cone_bp_views);
    e = launch_bp(L, p.kind, bp_ctas(L.single), st, &L, pix_ctas(L.single));
    if (scratch) cudaFreeAsync(scratch, st);
  }
  if (e != cudaSuccess) return cuda_error(e, forward ? "forward projection launch" : "back projection launch");
  return AT_OK;
}

__global__ void d2f_kernel(const double *in, float *out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}
__global__ void f2d_kernel(const float *in, double *out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

}  // namespace
}  // namespace medimg

using namespace medimg;

#define AT_API extern "C" __attribute__((visibility("default")))
#define AT_CHECK_ARG(cond, msg) \
  do {                          \
    if (!(cond)) return set_error(AT_EINVAL, msg); \
  } while (0)

AT_API const char *at_last_error(void) { return g_err.c_str(); }

AT_API int at_device_info(char *name, int name_len, int *sm_count, size_t *hbm_bytes) {
  int dev = 0;
  AT_CUDA_TRY(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  AT_CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
  if (name && name_len > 0) {
    std::strncpy(name, prop.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (hbm_bytes) *hbm_bytes = prop.totalGlobalMem;
  return AT_OK;
}

// ---------------------------------------------------------------- plans
AT_API int at_plan_create_fan_ex(const at_fan_geometry *geom, int32_t alpha_precision, at_plan **out) {
  AT_CHECK_ARG(geom && out, "at_plan_create_fan: null argument");
  AT_CHECK_ARG(alpha_precision == AT_ALPHA_FP64 || alpha_precision == AT_ALPHA_FP32,
               "at_plan_create_fan_ex: alpha_precision must be AT_ALPHA_FP64 or AT_ALPHA_FP32");
  *out = nullptr;
  int rc = validate_fan(*geom);
  if (rc) return rc;
  auto P = std::make_unique<at_plan>();
  P->p.kind = AT_GEOM_FAN;
  P->p.geom = *geom;
  P->p.alpha_fp32 = alpha_precision == AT_ALPHA_FP32;
  cudaStream_t st;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  rc = build_fan_plan(P->p, st);
  if (!rc) rc = autotune_fan(P->p, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  *out = P.release();
  return AT_OK;
}

AT_API int at_plan_create_fan(const at_fan_geometry *geom, at_plan **out) {
  return at_plan_create_fan_ex(geom, AT_ALPHA_FP64, out);
}

AT_API int at_plan_create_rays(int32_t n, double pixel_mm, int32_t nviews, int32_t ndets, const double *h_endpoints,
                               at_plan **out) {
  AT_CHECK_ARG(h_endpoints && out, "at_plan_create_rays: null argument");
  *out = nullptr;
  int rc = validate_rays(n, pixel_mm, nviews, ndets, h_endpoints);
  if (rc) return rc;
  auto P = std::make_unique<at_plan>();
  P->p.kind = AT_GEOM_RAYS;
  P->p.geom = at_fan_geometry{};
  P->p.geom.n = n;
  P->p.geom.pixel_mm = pixel_mm;
  P->p.geom.nviews = nviews;
  P->p.geom.ndets = ndets;
  cudaStream_t st;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  rc = build_fan_plan(P->p, st, h_endpoints);
  if (!rc) rc = autotune_fan(P->p, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  *out = P.release();
  return AT_OK;
}

AT_API int at_plan_create_cone(const at_cone_geometry *geom, at_plan **out) {
  AT_CHECK_ARG(geom && out, "at_plan_create_cone: null argument");
  *out = nullptr;
  int rc = validate_cone(*geom);
  if (rc) return rc;
  auto P = std::make_unique<at_plan>();
  P->p.kind = AT_GEOM_CONE;
  P->p.cone = *geom;
  P->p.geom.n = geom->nx;
  P->p.geom.pixel_mm = geom->voxel_mm;
  P->p.geom.nviews = geom->nproj;
  P->p.geom.ndets = geom->ndx * geom->ndy;
  cudaStream_t st;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  rc = build_cone_plan(P->p, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  *out = P.release();
  return AT_OK;
}

AT_API int at_plan_create_goldnc(at_plan **out) {
  AT_CHECK_ARG(out, "at_plan_create_goldnc: null argument");
  *out = nullptr;
  auto P = std::make_unique<at_plan>();
  P->p.kind = AT_GEOM_GOLDNC;
  P->p.geom.n = 512;
  P->p.geom.pixel_mm = 1.0;
  P->p.geom.nviews = 180;
  P->p.geom.ndets = 767;
  cudaStream_t st;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = build_goldnc_plan(P->p, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  *out = P.release();
  return AT_OK;
}

AT_API void at_plan_destroy(at_plan *plan) { delete plan; }

AT_API int at_plan_set_forward_variant(at_plan *plan, int32_t views, int32_t rays, int32_t rows) {
  AT_CHECK_ARG(plan, "at_plan_set_forward_variant: null plan");
  Plan &p = plan->p;
  AT_CHECK_ARG(p.kind == AT_GEOM_FAN || p.kind == AT_GEOM_RAYS,
               "at_plan_set_forward_variant: fan-beam and ray-table plans only");
  // the current tables may be bound into solvers or projection sets made
  // earlier: retire them (freed with the plan) rather than free them
  retire_slab_tables(p);
  if (views == 0 && rays == 0 && rows == 0) return AT_OK;
  cudaStream_t st;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const int rc = build_slab_tables(p, views, rays, rows, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  if (!p.slab.ok) return set_error(AT_EINVAL, "at_plan_set_forward_variant: this slab shape does not fit the plan");
  return AT_OK;
}

AT_API int at_plan_set_back_variant(at_plan *plan, int32_t use) {
  AT_CHECK_ARG(plan, "at_plan_set_back_variant: null plan");
  Plan &p = plan->p;
  AT_CHECK_ARG(p.kind == AT_GEOM_FAN || p.kind == AT_GEOM_RAYS,
               "at_plan_set_back_variant: fan-beam and ray-table plans only");
  AT_CHECK_ARG(use >= 0 && use <= 3, "at_plan_set_back_variant: use is a mask of 1 (single scans) and 2 (groups)");
  if (use && !p.pt_meta_d) {
    cudaStream_t st;
    AT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int rc = build_pixel_table(p, INT64_MAX, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (rc) return rc;
    if (!p.pt_meta_d) return set_error(AT_EINVAL, "at_plan_set_back_variant: the pixel table does not fit this plan");
  }
  p.bp_table = use;
  return AT_OK;
}

AT_API int at_plan_get_stats(const at_plan *plan, at_plan_stats *out) {
  AT_CHECK_ARG(plan && out, "at_plan_get_stats: null argument");
  const Plan &p = plan->p;
  out->kind = p.kind;
  out->n = p.n;
  out->nviews = p.nviews;
  out->ndets = p.ndets;
  out->rays = p.rays;
  out->segments = p.segments;
  out->offgrid = p.offgrid;
  out->device_bytes = p.device_bytes;
  out->max_segments = p.max_segments;
  out->fp_rays_per_thread = p.fp_rpt;
  out->bp_runs = p.nruns;
  out->nz = p.nz;
  out->slab_views = p.slab.ok ? p.slab.views : 0;
  out->slab_rays = p.slab.ok ? p.slab.rays : 0;
  out->slab_rows = p.slab.ok ? p.slab.rows : 0;
  out->slab_wbox = p.slab.ok ? p.slab.wbox : 0;
  out->slab_fallback_ctas = p.slab.ok ? p.slab.fallback : 0;
  out->bp_table_use = p.pt_meta_d ? p.bp_table : 0;
  out->bp_table_bytes = p.pt_bytes;
  out->bp_table_weights = p.pt_entries;
  return AT_OK;
}

AT_API int at_plan_trace_ray(const at_plan *plan, int32_t view, int32_t det, int32_t *h_pix, float *h_w, int32_t cap,
                             int32_t *n_out) {
  AT_CHECK_ARG(plan && n_out, "at_plan_trace_ray: null argument");
  const Plan &p = plan->p;
  if (p.kind == AT_GEOM_GOLDNC) {
    AT_CHECK_ARG(view >= 1 && view <= 45 && det >= 0 && det < 384, "at_plan_trace_ray: (alpha, raynum) out of range");
    const int pair = (view - 1) * 384 + det;
    int32_t off[2];
    AT_CUDA_TRY(cudaMemcpy(off, p.gc_pair_off_d + pair, sizeof(off), cudaMemcpyDeviceToHost));
    const int n = off[1] - off[0];
    *n_out = n;
    std::vector<GcSeg> seg(n);
    if (n) AT_CUDA_TRY(cudaMemcpy(seg.data(), p.gc_seg_d + off[0], sizeof(GcSeg) * n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < n && i < cap; i++) {
      if (h_pix) h_pix[i] = seg[i].pix;
      if (h_w) h_w[i] = seg[i].w;
    }
    return AT_OK;
  }
  AT_CHECK_ARG(view >= 0 && view < p.nviews && det >= 0 && det < p.ndets, "at_plan_trace_ray: ray out of range");
  if (p.kind == AT_GEOM_CONE) return cone_trace_ray(p, (int64_t)view * p.ndets + det, h_pix, h_w, cap, n_out);
  RayHdr h;
  AT_CUDA_TRY(cudaMemcpy(&h, p.rays_d + (size_t)view * p.ndets + det, sizeof(h), cudaMemcpyDeviceToHost));
  const int blk = view * p.nblocks_per_view + det / kRayBlock;
  uint32_t w0;
  AT_CUDA_TRY(cudaMemcpy(&w0, p.blk_word_d + blk, sizeof(w0), cudaMemcpyDeviceToHost));
  const int nw = (h.nseg + 31) / 32;
  std::vector<uint32_t> words(nw);
  for (int w = 0; w < nw; w++)
    AT_CUDA_TRY(cudaMemcpy(&words[w], p.bits_d + w0 + (size_t)w * kRayBlock + det % kRayBlock, sizeof(uint32_t),
                           cudaMemcpyDeviceToHost));
  *n_out = h.nseg;
  // decode exactly as the forward kernel walks
  int idx = h.pix0;
  const int stx = (h.sgn & 1) ? p.n : -p.n, sty = (h.sgn & 2) ? 1 : -1;
  float cx = 0.f, cy = 0.f, prev = 0.f;
  for (int k = 0; k < h.nseg; k++) {
    const bool bx = (words[k >> 5] >> (k & 31)) & 1u;
    const float nx = std::fma(cx, h.lenx, h.ax), ny = std::fma(cy, h.leny, h.ay);
    const float cur = bx ? nx : ny;
    if (k < cap) {
      if (h_pix) h_pix[k] = idx;
      if (h_w) h_w[k] = cur - prev;
    }
    prev = cur;
    idx += bx ? stx : sty;
    cx += bx ? 1.f : 0.f;
    cy += bx ? 0.f : 1.f;
  }
  return AT_OK;
}

// ---------------------------------------------------------------- projectors
AT_API int at_forward(const at_plan *plan, const float *d_img, float *d_sino, void *stream) {
  AT_CHECK_ARG(plan && d_img && d_sino, "at_forward: null argument");
  return project(plan->p, true, d_img, d_sino, (cudaStream_t)stream);
}

AT_API int at_back(const at_plan *plan, const float *d_sino, float *d_img, void *stream) {
  AT_CHECK_ARG(plan && d_img && d_sino, "at_back: null argument");
  return project(plan->p, false, d_sino, d_img, (cudaStream_t)stream);
}

namespace {
int project_host(const Plan &p, bool forward, const float *h_in, float *h_out) {
  const size_t npix = (size_t)p.nz * p.n * p.n, nbins = (size_t)p.nviews * p.ndets;
  const size_t nin = forward ? npix : nbins, nout = forward ? nbins : npix;
  float *din = nullptr, *dout = nullptr;
  cudaStream_t st = nullptr;
  int rc = AT_OK;
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) return cuda_error(e, "stream");
  if ((e = cudaMallocAsync(&din, nin * 4, st)) != cudaSuccess || (e = cudaMallocAsync(&dout, nout * 4, st)) != cudaSuccess) {
    rc = cuda_error(e, "cudaMallocAsync");
  } else if ((e = cudaMemcpyAsync(din, h_in, nin * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
    rc = cuda_error(e, "H2D");
  } else if (!(rc = project(p, forward, din, dout, st))) {
    if ((e = cudaMemcpyAsync(h_out, dout, nout * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) rc = cuda_error(e, "D2H");
  }
  if (din) cudaFreeAsync(din, st);
  if (dout) cudaFreeAsync(dout, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess && !rc) rc = cuda_error(e, "projection");
  if (!rc) rc = check_wait_timeouts();
  cudaStreamDestroy(st);
  return rc;
}
}  // namespace

AT_API int at_forward_host(const at_plan *plan, const float *h_img, float *h_sino) {
  AT_CHECK_ARG(plan && h_img && h_sino, "at_forward_host: null argument");
  return project_host(plan->p, true, h_img, h_sino);
}

AT_API int at_back_host(const at_plan *plan, const float *h_sino, float *h_img) {
  AT_CHECK_ARG(plan && h_img && h_sino, "at_back_host: null argument");
  return project_host(plan->p, false, h_sino, h_img);
}

// ---------------------------------------------------------------- device helpers
AT_API int at_dev_alloc(void **d_ptr, size_t bytes) {
  AT_CHECK_ARG(d_ptr, "at_dev_alloc: null argument");
  AT_CUDA_TRY(cudaMalloc(d_ptr, bytes));
  return AT_OK;
}
AT_API int at_dev_free(void *d_ptr) {
  AT_CUDA_TRY(cudaFree(d_ptr));
  return AT_OK;
}
AT_API int at_memcpy_h2d(void *d_dst, const void *h_src, size_t bytes, void *stream) {
  AT_CUDA_TRY(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return AT_OK;
}
AT_API int at_memcpy_d2h(void *h_dst, const void *d_src, size_t bytes, void *stream) {
  AT_CUDA_TRY(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return AT_OK;
}
AT_API int at_stream_create(void **stream) {
  AT_CHECK_ARG(stream, "at_stream_create: null argument");
  cudaStream_t s;
  AT_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  *stream = s;
  return AT_OK;
}
AT_API int at_stream_destroy(void *stream) {
  AT_CUDA_TRY(cudaStreamDestroy((cudaStream_t)stream));
  return AT_OK;
}
AT_API int at_stream_sync(void *stream) {
  AT_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return check_wait_timeouts();
}

// ---------------------------------------------------------------- solver
AT_API int at_solver_footprint(at_plan *const *plans, int32_t nscans, size_t *bytes) {
  AT_CHECK_ARG(plans && nscans > 0 && bytes, "at_solver_footprint: bad argument");
  std::vector<Plan *> v;
  for (int i = 0; i < nscans; i++) {
    AT_CHECK_ARG(plans[i], "at_solver_footprint: null plan");
    v.push_back(&plans[i]->p);
  }
  *bytes = Solver::footprint(v, Solver::choose_rpt(v));
  return AT_OK;
}

AT_API int at_solver_create(at_plan *const *plans, int32_t nscans, const at_params *params, at_solver **out) {
  AT_CHECK_ARG(plans && nscans > 0 && params && out, "at_solver_create: bad argument");
  *out = nullptr;
  std::vector<Plan *> v;
  for (int i = 0; i < nscans; i++) {
    AT_CHECK_ARG(plans[i], "at_solver_create: null plan");
    v.push_back(&plans[i]->p);
  }
  auto S = std::make_unique<at_solver>();
  int rc = S->s.create(v, *params);
  if (rc) return rc;
  *out = S.release();
  return AT_OK;
}

AT_API void at_solver_destroy(at_solver *s) { delete s; }

AT_API int at_projset_create(at_plan *const *plans, int32_t n, at_projset **out) {
  AT_CHECK_ARG(plans && n > 0 && out, "at_projset_create: bad argument");
  *out = nullptr;
  std::vector<Plan *> v;
  for (int i = 0; i < n; i++) {
    AT_CHECK_ARG(plans[i], "at_projset_create: null plan");
    v.push_back(&plans[i]->p);
  }
  auto P = std::make_unique<at_projset>();
  int rc = P->p.create(v);
  if (rc) return rc;
  *out = P.release();
  return AT_OK;
}

AT_API void at_projset_destroy(at_projset *ps) { delete ps; }

AT_API int at_projset_forward(at_projset *ps, const float *const *d_img, float *const *d_sino, void *stream) {
  AT_CHECK_ARG(ps && d_img && d_sino, "at_projset_forward: null argument");
  return ps->p.project(true, d_img, d_sino, (cudaStream_t)stream);
}

AT_API int at_projset_back(at_projset *ps, const float *const *d_sino, float *const *d_img, void *stream) {
  AT_CHECK_ARG(ps && d_sino && d_img, "at_projset_back: null argument");
  return ps->p.project(false, d_sino, d_img, (cudaStream_t)stream);
}

#define AT_SCAN_ARG(s, scan) \
  AT_CHECK_ARG((s) && (scan) >= 0 && (scan) < (s)->s.nscans, "solver: scan index out of range")

AT_API int at_solver_set_sino(at_solver *s, int32_t scan, const float *d_sino, void *stream) {
  AT_SCAN_ARG(s, scan);
  AT_CHECK_ARG(d_sino, "at_solver_set_sino: null argument");
  const ScanDev &S = s->s.host_scans[scan];
  AT_CUDA_TRY(cudaMemcpyAsync(S.buf[B_G], d_sino, sizeof(float) * S.nbins, cudaMemcpyDeviceToDevice,
                              (cudaStream_t)stream));
  return AT_OK;
}

AT_API int at_solver_set_sino_host(at_solver *s, int32_t scan, const float *h_sino, void *stream) {
  AT_SCAN_ARG(s, scan);
  AT_CHECK_ARG(h_sino, "at_solver_set_sino_host: null argument");
  const ScanDev &S = s->s.host_scans[scan];
  AT_CUDA_TRY(cudaMemcpyAsync(S.buf[B_G], h_sino, sizeof(float) * S.nbins, cudaMemcpyHostToDevice,
                              (cudaStream_t)stream));
  return AT_OK;
}

AT_API int at_solver_reset(at_solver *s, void *stream) {
  AT_CHECK_ARG(s, "at_solver_reset: null argument");
  return s->s.reset((cudaStream_t)stream);
}

AT_API int at_solver_run(at_solver *s, void *stream) {
  AT_CHECK_ARG(s, "at_solver_run: null argument");
  return s->s.run((cudaStream_t)stream);
}

AT_API int at_solver_step(at_solver *s, int32_t count, void *stream) {
  AT_CHECK_ARG(s && count >= 0, "at_solver_step: bad argument");
  return s->s.step(count, (cudaStream_t)stream);
}

AT_API int at_solver_get(at_solver *s, int32_t scan, float *d_f, float *d_v, void *stream) {
  AT_SCAN_ARG(s, scan);
  const ScanDev &S = s->s.host_scans[scan];
  if (d_f)
    AT_CUDA_TRY(cudaMemcpyAsync(d_f, S.buf[B_F], sizeof(float) * S.npix, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  if (d_v)
    AT_CUDA_TRY(cudaMemcpyAsync(d_v, S.buf[B_V], sizeof(float) * S.npix, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return AT_OK;
}

AT_API int at_solver_get_host(at_solver *s, int32_t scan, float *h_f, float *h_v, void *stream) {
  AT_SCAN_ARG(s, scan);
  const ScanDev &S = s->s.host_scans[scan];
  if (h_f)
    AT_CUDA_TRY(cudaMemcpyAsync(h_f, S.buf[B_F], sizeof(float) * S.npix, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  if (h_v)
    AT_CUDA_TRY(cudaMemcpyAsync(h_v, S.buf[B_V], sizeof(float) * S.npix, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  AT_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return check_wait_timeouts();
}

AT_API int at_solver_set_fv_host(at_solver *s, int32_t scan, const float *h_f, const float *h_v, void *stream) {
  AT_SCAN_ARG(s, scan);
  const ScanDev &S = s->s.host_scans[scan];
  if (h_f)
    AT_CUDA_TRY(cudaMemcpyAsync(S.buf[B_F], h_f, sizeof(float) * S.npix, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  if (h_v)
    AT_CUDA_TRY(cudaMemcpyAsync(S.buf[B_V], h_v, sizeof(float) * S.npix, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return AT_OK;
}

AT_API int at_solver_trace(at_solver *s, int32_t scan, double *h_recs, int32_t cap, int32_t *n_out) {
  AT_SCAN_ARG(s, scan);
  AT_CHECK_ARG(n_out, "at_solver_trace: null argument");
  const ScanDev &S = s->s.host_scans[scan];
  Ctl c;
  AT_CUDA_TRY(cudaMemcpy(&c, S.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  const int n = std::min(c.trace_n, kTraceCap);
  *n_out = n;
  if (h_recs && cap > 0 && n > 0)
    AT_CUDA_TRY(cudaMemcpy(h_recs, S.trace, sizeof(double) * 10 * std::min(n, (int)cap), cudaMemcpyDeviceToHost));
  return AT_OK;
}

AT_API int at_solver_launches_per_outer(const at_solver *s, int32_t *n) {
  AT_CHECK_ARG(s && n, "at_solver_launches_per_outer: null argument");
  *n = s->s.launches;
  return AT_OK;
}

AT_API int at_reconstruct_host(const at_plan *plan, const at_params *params, const float *h_sino, float *h_f,
                               float *h_v) {
  AT_CHECK_ARG(plan && params && h_sino, "at_reconstruct_host: null argument");
  at_plan *pl = const_cast<at_plan *>(plan);
  at_solver *s = nullptr;
  int rc = at_solver_create(&pl, 1, params, &s);
  if (rc) return rc;
  cudaStream_t st = s->s.own_stream;
  if (!(rc = at_solver_set_sino_host(s, 0, h_sino, st)) && !(rc = at_solver_run(s, st)))
    rc = at_solver_get_host(s, 0, h_f, h_v, st);
  at_solver_destroy(s);
  return rc;
}

// ---------------------------------------------------------------- GoldenC drop-in
// The caller's globals of origin/GoldenC/src/main.c:8-10, bound if present.
extern "C" {
extern double f[512][512] __attribute__((weak));
extern double v[512][512] __attribute__((weak));
extern double gDelta[180][767] __attribute__((weak));
}

namespace {
constexpr int kGcPix = 512 * 512, kGcBins = 180 * 767;

struct GoldncContext {
  std::mutex mu;
  at_plan *plan = nullptr;
  cudaStream_t st = nullptr;
  double *dd = nullptr;  // staging for FP64 host arrays (kGcPix doubles)
  float *fa = nullptr, *fb = nullptr;
  int iter_alt = 10, iter_image = 10, iter_edge = 10;
  int status = AT_OK;
  // Creates the stream, the staging buffers and then the plan.  `plan` is set
  // last, so a context is either complete or still empty: a failure part way
  // frees what was made and the next call starts over.
  int init() {
    if (plan) return AT_OK;
    cudaStream_t s = nullptr;
    double *d = nullptr;
    float *a = nullptr, *b = nullptr;
    at_plan *p = nullptr;
    int rc = AT_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(double) * kGcPix);
    if (e == cudaSuccess) e = cudaMalloc(&a, sizeof(float) * kGcPix);
    if (e == cudaSuccess) e = cudaMalloc(&b, sizeof(float) * kGcPix);
    if (e != cudaSuccess) rc = cuda_error(e, "GoldenC context set-up");
    if (!rc) rc = at_plan_create_goldnc(&p);
    if (rc) {
      cudaFree(d);
      cudaFree(a);
      cudaFree(b);
      if (s) cudaStreamDestroy(s);
      return rc;
    }
    st = s;
    dd = d;
    fa = a;
    fb = b;
    plan = p;
    return AT_OK;
  }
  int to_dev(const double *h, float *d, int n) {
    AT_CUDA_TRY(cudaMemcpyAsync(dd, h, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    d2f_kernel<<<(n + 255) / 256, 256, 0, st>>>(dd, d, n);
    AT_CUDA_TRY(cudaGetLastError());
    return AT_OK;
  }
  int to_host(const float *d, double *h, int n) {
    f2d_kernel<<<(n + 255) / 256, 256, 0, st>>>(d, dd, n);
    AT_CUDA_TRY(cudaGetLastError());
    AT_CUDA_TRY(cudaMemcpyAsync(h, dd, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    AT_CUDA_TRY(cudaStreamSynchronize(st));
    return AT_OK;
  }
};

GoldncContext &gctx() {
  static GoldncContext *c = new GoldncContext();  // never destroyed: usable from atexit handlers
  return *c;
}

void goldnc_report(const char *fn, int rc) {
  gctx().status = rc;
  if (rc) std::fprintf(stderr, "%s: %s\n", fn, at_last_error());
}

// one GoldenC scan through the batched solver, image or edge step only
int goldnc_step(bool image, double *out, const double *g, const double *fin, const double *vin, double alpha,
                double beta, double eps, int iters) {
  GoldncContext &C = gctx();
  int rc = C.init();
  if (rc) return rc;
  at_params prm{alpha, beta, eps, 1, image ? iters : 2, image ? 1 : iters, 0};
  if (image && iters < 2) return set_error(AT_EINVAL, "minimize_in_IMAGE_variable: IterImage must be >= 2");
  if (!image && iters < 1) return set_error(AT_EINVAL, "minimize_in_EDGE_variable: IterEdge must be >= 1");
  std::vector<Plan *> pl{&C.plan->p};
  Solver S;
  if ((rc = S.create(pl, prm))) return rc;
  const ScanDev &D = S.host_scans[0];
  if ((rc = C.to_dev(fin, D.buf[B_F], kGcPix))) return rc;
  if ((rc = C.to_dev(vin, D.buf[B_V], kGcPix))) return rc;
  if (image) {
    AT_CUDA_TRY(cudaMemcpyAsync(C.dd, g, sizeof(double) * kGcBins, cudaMemcpyHostToDevice, C.st));
    d2f_kernel<<<(kGcBins + 255) / 256, 256, 0, C.st>>>(C.dd, D.buf[B_G], kGcBins);
    AT_CUDA_TRY(cudaGetLastError());
  }
  if ((rc = S.reset_ctl(C.st))) return rc;
  if ((rc = image ? S.enqueue_image(C.st) : S.enqueue_edge(C.st))) return rc;
  return C.to_host(image ? D.buf[B_F] : D.buf[B_V], out, kGcPix);
}
}  // namespace

AT_API int goldnc_status(void) { return gctx().status; }

AT_API void goldnc_set_iterations(int iter_alt, int iter_image, int iter_edge) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  C.iter_alt = iter_alt;
  C.iter_image = iter_image;
  C.iter_edge = iter_edge;
}

AT_API void A(double proj[180][767], double orig[512][512]) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  int rc = C.init();
  if (!rc) rc = C.to_dev(&orig[0][0], C.fa, kGcPix);
  float *sino = nullptr;
  if (!rc) {
    const cudaError_t e = cudaMallocAsync(&sino, sizeof(float) * kGcBins, C.st);
    if (e != cudaSuccess) {
      sino = nullptr;
      rc = cuda_error(e, "cudaMallocAsync");
    }
  }
  if (!rc) rc = project(C.plan->p, true, C.fa, sino, C.st);
  if (!rc) rc = C.to_host(sino, &proj[0][0], kGcBins);
  if (sino) {
    cudaFreeAsync(sino, C.st);
    cudaStreamSynchronize(C.st);
  }
  goldnc_report("A", rc);
}

AT_API void AStar(double back[512][512], double proj[180][767]) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  int rc = C.init();
  float *sino = nullptr;
  if (!rc) {
    const cudaError_t e = cudaMallocAsync(&sino, sizeof(float) * kGcBins, C.st);
    if (e != cudaSuccess) {
      sino = nullptr;
      rc = cuda_error(e, "cudaMallocAsync");
    }
  }
  if (!rc) rc = C.to_dev(&proj[0][0], sino, kGcBins);
  if (!rc) rc = project(C.plan->p, false, sino, C.fa, C.st);
  if (!rc) rc = C.to_host(C.fa, &back[0][0], kGcPix);
  if (sino) {
    cudaFreeAsync(sino, C.st);
    cudaStreamSynchronize(C.st);
  }
  goldnc_report("AStar", rc);
}

AT_API void medfilt2(double fimg[512][512]) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  int rc = C.init();
  if (!rc) rc = C.to_dev(&fimg[0][0], C.fa, kGcPix);
  if (!rc) {
    cudaError_t e = launch_median(C.fa, C.fb, 512, C.st);
    if (e != cudaSuccess) rc = cuda_error(e, "median launch");
  }
  if (!rc) rc = C.to_host(C.fb, &fimg[0][0], kGcPix);
  goldnc_report("medfilt2", rc);
}

AT_API void minimize_in_IMAGE_variable(double out[512][512], double g[180][767], double fimg[512][512],
                                       double vimg[512][512], double alpha, double epsilon, int IterImage) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  const int rc = goldnc_step(true, &out[0][0], &g[0][0], &fimg[0][0], &vimg[0][0], alpha, 0.0, epsilon, IterImage);
  goldnc_report("minimize_in_IMAGE_variable", rc);
}

AT_API void minimize_in_EDGE_variable(double out[512][512], double fimg[512][512], double vimg[512][512], double alpha,
                                      double beta, double epsilon, int IterEdge) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  const int rc = goldnc_step(false, &out[0][0], nullptr, &fimg[0][0], &vimg[0][0], alpha, beta, epsilon, IterEdge);
  goldnc_report("minimize_in_EDGE_variable", rc);
}

AT_API void MumfordShah(double alpha, double beta, double epsilon) {
  GoldncContext &C = gctx();
  std::lock_guard<std::mutex> lk(C.mu);
  int rc = AT_OK;
  if (&f == nullptr || &v == nullptr || &gDelta == nullptr) {
    rc = set_error(AT_ESTATE, "MumfordShah: the program defines no globals f, v, gDelta");
  } else if (!(rc = C.init())) {
    at_params prm{alpha, beta, epsilon, C.iter_alt, C.iter_image, C.iter_edge, 0};
    std::vector<Plan *> pl{&C.plan->p};
    Solver S;
    if (!(rc = S.create(pl, prm))) {
      // f and v are written together, after both have reached the host: a
      // failure leaves the program's globals as they were
      const ScanDev &D = S.host_scans[0];
      std::vector<double> hf(kGcPix), hv(kGcPix);
      if (!(rc = C.to_dev(&gDelta[0][0], D.buf[B_G], kGcBins)) && !(rc = S.run(C.st)) &&
          !(rc = C.to_host(D.buf[B_F], hf.data(), kGcPix)) && !(rc = C.to_host(D.buf[B_V], hv.data(), kGcPix))) {
        std::memcpy(&f[0][0], hf.data(), sizeof(double) * kGcPix);
        std::memcpy(&v[0][0], hv.data(), sizeof(double) * kGcPix);
      }
    }
  }
  goldnc_report("MumfordShah", rc);
}

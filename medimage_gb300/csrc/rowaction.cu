// rowaction.cu -- the row-action AT of msbeam/CPU_OpenMP on the GPU.
//
// msbeam (main.c:213-394) sweeps the rays of a parallel beam one at a time:
// for each ray it traces the pixels (wray, proj.c:67-211), takes one gradient
// step of the image on them (minIMAGE, main.c:213-261) and one of the edge
// field (minEDGE, main.c:263-301), with a step length lambda that shrinks
// after every sweep (main.c:371,391).  Its OpenMP loop runs views in parallel
// and lets the updates race.  Here the order is fixed instead: within a view,
// rays that are `phases` apart never touch each other's pixels or their
// four neighbours (checked on every ray of msbeam's geometry for 3 and more),
// so the rays nr = phase, phase + phases, ... of one view run concurrently,
// one CTA per ray, and views and phases follow one another.  The result is
// deterministic, and equal (up to the order of the ray sum) to one thread
// running the rays in that order.
//
// The traces are msbeam's own, computed once on the GPU with its float/double
// mix written as explicitly rounded intrinsics (bit-identical to the
// reference's wray) and stored per ray.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "at_internal.h"

namespace medimg {
namespace {

struct RaGeom {
  int n, nproj, nray, mid;
};

constexpr double kFtol = 1e-8;     // F_TOL, proto.h:14
constexpr double kGridTol = 1e-2;  // GRID_TOL, proto.h:15

// proj.c:67-211 for ray (np, nr); kMode 0 counts, 1 writes
template <int kMode>
__device__ int ms_wray(const RaGeom G, const float2 *trig, int np, int nr, int *line, float *weight) {
  // posit, proj.c:53-65
  const float sinth = trig[np].x, costh = trig[np].y;
  const float tmp_length = (float)(nr - G.mid);
  float sorx = __fmul_rn(-sinth, tmp_length), sory = __fmul_rn(costh, tmp_length);
  float cf = costh, sf = sinth;
  if ((double)sf < -kFtol) {
    sf = -sf;
    cf = -cf;
  }
  int flip = 0;
  if ((double)__fmul_rn(sf, cf) < -kFtol * kFtol) {
    flip = 1;
    cf = -cf;
  }
  if (flip > 0) sorx = -sorx;
  if (fabs((double)sf) <= kFtol) sf = (float)((sf < 0) ? -kFtol * kFtol : kFtol * kFtol);
  if (fabs((double)cf) <= kFtol) cf = (float)((cf < 0) ? -kFtol * kFtol : kFtol * kFtol);
  float tanphi, rtnphi;
  if (fabs((double)cf) > kFtol) tanphi = __fdiv_rn(sf, cf);
  else tanphi = (float)(1 / (kFtol * kFtol));
  if (fabs((double)sf) > kFtol) rtnphi = __fdiv_rn(cf, sf);
  else rtnphi = (float)(1 / (kFtol * kFtol));
  int flipxy = 0;
  if ((double)tanphi > 1 + kFtol) {
    flipxy = 1;
    tanphi = __fdiv_rn(1.f, tanphi);
    rtnphi = __fdiv_rn(1.f, rtnphi);
    sf = sory;
    sory = sorx;
    sorx = sf;
  }
  const float rcosphi = __double2float_rn(__dsqrt_rn((double)__fadd_rn(1.f, __fmul_rn(tanphi, tanphi))));
  sory = __double2float_rn(__dadd_rn((double)sory, G.n / 2.0));
  sorx = __double2float_rn(__dadd_rn((double)sorx, G.n / 2.0));
  float c = __fsub_rn(sory, __fmul_rn(sorx, tanphi));
  int ix, iy;
  float yc;
  if ((double)__fsub_rn(c, (float)G.n) >= kGridTol) return 0;
  if ((double)c < -kGridTol) {
    c = __fmul_rn(-c, rtnphi);
    if ((double)__fsub_rn(c, (float)G.n) >= kGridTol) return 0;
    ix = (int)c;
    iy = 0;
    const float fp = __fsub_rn((float)(ix + 1), c);
    yc = __fmul_rn(fp, tanphi);
    yc = __double2float_rn(__dadd_rn((double)yc, -1.0));
  } else {
    ix = 0;
    iy = (int)c;
    const float fp = __fsub_rn((float)(iy + 1), c);
    yc = -fp;
    yc = __fadd_rn(yc, tanphi);
  }
  int next = (yc >= 0) ? 1 : 2;
  int index, incx, incy;
  if (flipxy > 0) {
    index = iy + ix * G.n;
    incx = G.n;
    incy = 1;
    if (flip > 0) {
      index = G.n - 1 - iy + ix * G.n;
      incy = -1;
    }
  } else {
    index = iy * G.n + ix;
    incx = 1;
    incy = G.n;
    if (flip > 0) {
      index = G.n - 1 - ix + iy * G.n;
      incx = -1;
    }
  }
  int numb = 0;
  const int cap = 4 * G.n;  // a walk visits at most 2n pixels; this only guards the loop
  for (int guard = 0; guard < cap; guard++) {
    if (next == 1) {
      if (iy + 1 >= G.n || ix < 0) return numb;
      if (kMode == 1) {
        weight[numb] = __fmul_rn(rcosphi, __fsub_rn(1.f, __fmul_rn(yc, rtnphi)));
        line[numb] = index;
      }
      ++numb;
      iy++;
      index += incy;
      if (ix + 1 >= G.n) return numb;
      if (kMode == 1) {
        weight[numb] = __fmul_rn(rcosphi, __fmul_rn(yc, rtnphi));
        line[numb] = index;
      }
      ++numb;
      ix++;
      index += incx;
      yc = __double2float_rn(__dadd_rn((double)yc, __dsub_rn((double)tanphi, 1.0)));
      next = (yc >= 0) ? 1 : 2;
    } else {
      if (iy >= G.n || ix + 1 >= G.n || ix < 0) return numb;
      if (kMode == 1) {
        weight[numb] = rcosphi;
        line[numb] = index;
      }
      ++numb;
      ix++;
      index += incx;
      yc = __fadd_rn(yc, tanphi);
      next = (yc >= 0) ? 1 : 2;
    }
  }
  return numb;
}

__global__ void ra_count_kernel(const RaGeom G, const float2 *trig, int *count) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= G.nproj * G.nray) return;
  count[ray] = ms_wray<0>(G, trig, ray / G.nray, ray % G.nray, nullptr, nullptr);
}

__global__ void ra_fill_kernel(const RaGeom G, const float2 *trig, const int64_t *off, int *line, float *weight) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= G.nproj * G.nray) return;
  ms_wray<1>(G, trig, ray / G.nray, ray % G.nray, line + off[ray], weight + off[ray]);
}

struct RaArgs {
  RaGeom G;
  const int64_t *off;
  const int *line;
  const float *weight;
  const float *g;  // [slice][nproj][nray]
  float *f, *v;    // [slice][n][n]
  int view, phase, phases, rays_in_phase;
  float lambda, alpha, eps2;     // eps2 = sqr((float)epsilon)
  double beta4e, betaeps;        // beta / (4 epsilon), beta * epsilon
};

constexpr int kRaWarps = 4;       // rays per CTA of the forward projection
constexpr int kRaThreads = 256;   // threads per ray of a sweep step
constexpr int kRaMaxSeg = 2048;   // per ray: at most 2n pixels, n <= 1024

// one CTA per ray of (view, phase), its pixels spread over the threads;
// blockIdx.y = slice
__global__ void __launch_bounds__(kRaThreads) ra_step_kernel(const RaArgs A) {
  __shared__ float d[kRaMaxSeg];
  __shared__ float part[kRaThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k = blockIdx.x;
  const int nr = A.phase + k * A.phases;
  const int n = A.G.n, ray = A.view * A.G.nray + nr;
  const int64_t o0 = A.off[ray], o1 = A.off[ray + 1];
  const int numb = (int)(o1 - o0);
  const int *line = A.line + o0;
  const float *wgt = A.weight + o0;
  float *f = A.f + (size_t)blockIdx.y * n * n;
  float *v = A.v + (size_t)blockIdx.y * n * n;
  // minIMAGE, main.c:213-261: the ray's projection, summed in a fixed tree
  float af = 0.f;
  for (int i = tid; i < numb; i += kRaThreads) af = __fadd_rn(af, __fmul_rn(f[line[i]], wgt[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) af = __fadd_rn(af, __shfl_xor_sync(0xffffffffu, af, o));
  if (lane == 0) part[warp] = af;
  __syncthreads();
  af = 0.f;
#pragma unroll
  for (int w = 0; w < kRaThreads / 32; w++) af = __fadd_rn(af, part[w]);
  af = __fsub_rn(af, A.g[(size_t)blockIdx.y * A.G.nproj * A.G.nray + ray]);
  for (int i = tid; i < numb; i += kRaThreads) {
    const int ind = line[i], x = ind / n, y = ind % n;
    const float fc = f[ind], vc = v[ind], vc2 = __fmul_rn(vc, vc);
    float tmp = 0.f, lap = 0.f;
    float fd = 0.f, fr = 0.f;  // neighbours past the edge are zero (never read)
    if (x + 1 < n) fd = f[ind + n];
    if (y + 1 < n) fr = f[ind + 1];
    tmp = __fadd_rn(tmp, __fmul_rn(vc2, __fsub_rn(fd, fc)));
    tmp = __fadd_rn(tmp, __fmul_rn(vc2, __fsub_rn(fr, fc)));
    if (x - 1 >= 0) tmp = __fsub_rn(tmp, __fmul_rn(__fmul_rn(v[ind - n], v[ind - n]), __fsub_rn(fc, f[ind - n])));
    else tmp = __fsub_rn(tmp, __fsub_rn(fc, 0.f));
    if (y - 1 >= 0) tmp = __fsub_rn(tmp, __fmul_rn(__fmul_rn(v[ind - 1], v[ind - 1]), __fsub_rn(fc, f[ind - 1])));
    else tmp = __fsub_rn(tmp, __fsub_rn(fc, 0.f));
    if (x + 1 < n) lap = __fadd_rn(lap, f[ind + n]);
    if (y + 1 < n) lap = __fadd_rn(lap, f[ind + 1]);
    if (x - 1 >= 0) lap = __fadd_rn(lap, f[ind - n]);
    if (y - 1 >= 0) lap = __fadd_rn(lap, f[ind - 1]);
    lap = __fsub_rn(lap, __fmul_rn(4.f, fc));
    d[i] = __fadd_rn(__fmul_rn(-af, wgt[i]), __fmul_rn(A.alpha, __fadd_rn(tmp, __fmul_rn(A.eps2, lap))));
  }
  __syncthreads();  // every read of f before any write (main.c:255-260 updates after the loop)
  for (int i = tid; i < numb; i += kRaThreads) {
    const int ind = line[i];
    float fn = __fadd_rn(f[ind], __fmul_rn(A.lambda, d[i]));
    f[ind] = fn < 0 ? 0.f : fn;
  }
  __syncthreads();
  // minEDGE, main.c:263-301
  for (int i = tid; i < numb; i += kRaThreads) {
    const int ind = line[i], x = ind / n, y = ind % n;
    const float fc = f[ind], vc = v[ind];
    float a = 0.f, c = 0.f;
    float fu = 0.f, fl = 0.f;
    if (x - 1 >= 0) fu = f[ind - n];
    if (y - 1 >= 0) fl = f[ind - 1];
    const float gx = __fsub_rn(fc, fu);
    const float gy = __fsub_rn(fc, fl);
    a = __fadd_rn(a, __fmul_rn(gx, gx));
    a = __fadd_rn(a, __fmul_rn(gy, gy));
    a = __fmul_rn(a, vc);
    const float b = __fsub_rn(vc, 1.f);
    if (x + 1 < n) c = __fadd_rn(c, v[ind + n]);
    if (y + 1 < n) c = __fadd_rn(c, v[ind + 1]);
    if (x - 1 >= 0) c = __fadd_rn(c, v[ind - n]);
    if (y - 1 >= 0) c = __fadd_rn(c, v[ind - 1]);
    c = __fsub_rn(c, __fmul_rn(4.f, vc));
    // -ALPHA*a in float, the beta terms in double, as main.c:298 evaluates them
    const double dd = __dadd_rn(__dsub_rn((double)__fmul_rn(-A.alpha, a), __dmul_rn(A.beta4e, (double)b)),
                                __dmul_rn(A.betaeps, (double)c));
    d[i] = __double2float_rn(dd);
  }
  __syncthreads();
  for (int i = tid; i < numb; i += kRaThreads) {
    const int ind = line[i];
    float vn = __fadd_rn(v[ind], __fmul_rn(A.lambda, d[i]));
    vn = vn < 0 ? 0.f : vn;
    v[ind] = vn > 1 ? 1.f : vn;
  }
}

// msbeam's A (proj.c:14-32) on its traces: g[ray] = sum f[pixel] * weight,
// a warp per ray (the sum in tree order); blockIdx.y = slice
__global__ void __launch_bounds__(32 * kRaWarps) ra_forward_kernel(const RaGeom G, const int64_t *off, const int *line,
                                                                 const float *weight, const float *f, float *g) {
  const int ray = blockIdx.x * kRaWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int rays = G.nproj * G.nray;
  if (ray >= rays) return;
  const float *fs = f + (size_t)blockIdx.y * G.n * G.n;
  float acc = 0.f;
  for (int64_t i = off[ray] + lane; i < off[ray + 1]; i += 32) acc = __fadd_rn(acc, __fmul_rn(fs[line[i]], weight[i]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
  if (lane == 0) g[(size_t)blockIdx.y * rays + ray] = acc;
}

__global__ void ra_init_kernel(float *f, float *v, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) {
    f[i] = 0.f;
    v[i] = 1.f;
  }
}

}  // namespace
}  // namespace medimg

// A run is one launch per (sweep, view, phase), a few microseconds of work
// each, so it is captured as a CUDA graph and replayed; the graph is kept for
// the next call with the same slice count, buffers and parameters.
struct RaGraphKey {
  int nslices = 0;
  const float *g = nullptr;
  float *f = nullptr, *v = nullptr;
  float alpha = 0.f, lambda0 = 0.f, lambda_decay = 0.f;
  double beta = 0.0, epsilon = 0.0;
  int sweeps = -1, phases = 0;
  bool operator==(const RaGraphKey &o) const {
    return nslices == o.nslices && g == o.g && f == o.f && v == o.v && alpha == o.alpha && lambda0 == o.lambda0 &&
           lambda_decay == o.lambda_decay && beta == o.beta && epsilon == o.epsilon && sweeps == o.sweeps &&
           phases == o.phases;
  }
};

struct at_rowaction {
  medimg::RaGeom G{};
  float2 *trig = nullptr;
  int64_t *off = nullptr;
  int *line = nullptr;
  float *weight = nullptr;
  int64_t segments = 0;
  // the captured run (see RaGraphKey); calls on one handle are serialised by
  // the graph's launches
  mutable cudaGraphExec_t exec = nullptr;
  mutable RaGraphKey key{};
  mutable cudaStream_t cap = nullptr;
  mutable cudaEvent_t done = nullptr;  // after the last launch of `exec`
  ~at_rowaction() {
    if (done) cudaEventSynchronize(done);
    if (exec) cudaGraphExecDestroy(exec);
    if (done) cudaEventDestroy(done);
    if (cap) cudaStreamDestroy(cap);
    cudaFree(trig);
    cudaFree(off);
    cudaFree(line);
    cudaFree(weight);
  }
};

using namespace medimg;

namespace {
// msbeam's run (main.c:365-394): f = 0, v = 1, then `sweeps` sweeps of every
// view's rays, phase by phase, the step length shrinking after each sweep
void enqueue_run(const at_rowaction &ra, int nslices, const float *d_g, float *d_f, float *d_v,
                 const at_rowaction_params &prm, cudaStream_t st) {
  const size_t npix = (size_t)ra.G.n * ra.G.n * nslices;
  ra_init_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, st>>>(d_f, d_v, npix);  // main.c:365-369
  RaArgs A;
  std::memset(&A, 0, sizeof(A));
  A.G = ra.G;
  A.off = ra.off;
  A.line = ra.line;
  A.weight = ra.weight;
  A.g = d_g;
  A.f = d_f;
  A.v = d_v;
  A.phases = prm.phases;
  A.alpha = prm.alpha;
  const float epsf = prm.epsilon;
  A.eps2 = epsf * epsf;
  A.beta4e = prm.beta / (4 * prm.epsilon);
  A.betaeps = prm.beta * prm.epsilon;
  float lambda = prm.lambda0;
  for (int it = 0; it < prm.sweeps; it++) {
    A.lambda = lambda;
    for (int view = 0; view < ra.G.nproj; view++)
      for (int ph = 0; ph < prm.phases; ph++) {
        A.view = view;
        A.phase = ph;
        A.rays_in_phase = (ra.G.nray - ph + prm.phases - 1) / prm.phases;
        dim3 grid(A.rays_in_phase, nslices);
        ra_step_kernel<<<grid, kRaThreads, 0, st>>>(A);
      }
    lambda = lambda / (1 + prm.lambda_decay * lambda);  // main.c:391
  }
}
}  // namespace

#define AT_API extern "C" __attribute__((visibility("default")))

AT_API int at_rowaction_create(int32_t n, int32_t nproj, int32_t nray, at_rowaction **out) {
  if (!out) return set_error(AT_EINVAL, "at_rowaction_create: null argument");
  *out = nullptr;
  if (n < 8 || n > 1024 || nproj < 1 || nproj > 65536 || nray < 2 || nray > 65536 ||
      (int64_t)nproj * nray > (1ll << 30))
    return set_error(AT_EINVAL, "at_rowaction_create: need n in [8, 1024], nproj and nray in range");
  auto R = std::make_unique<at_rowaction>();
  R->G = RaGeom{n, nproj, nray, nray / 2};
  // posit, proj.c:56-57: sin and cos of PI/NPROJ*np in double, kept as float
  constexpr double kMsPi = 3.14159265359;  // proto.h:17
  std::vector<float2> trig(nproj);
  for (int p = 0; p < nproj; p++) trig[p] = make_float2((float)std::sin(kMsPi / nproj * p), (float)std::cos(kMsPi / nproj * p));
  const int rays = nproj * nray;
  AT_CUDA_TRY(cudaMalloc(&R->trig, sizeof(float2) * nproj));
  AT_CUDA_TRY(cudaMemcpy(R->trig, trig.data(), sizeof(float2) * nproj, cudaMemcpyHostToDevice));
  int *cnt = nullptr;
  const auto free_cnt = scope_exit([&] { cudaFree(cnt); });
  AT_CUDA_TRY(cudaMalloc(&cnt, sizeof(int) * rays));
  ra_count_kernel<<<(rays + 127) / 128, 128>>>(R->G, R->trig, cnt);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<int> h(rays);
  AT_CUDA_TRY(cudaMemcpy(h.data(), cnt, sizeof(int) * rays, cudaMemcpyDeviceToHost));
  std::vector<int64_t> off(rays + 1, 0);
  for (int r = 0; r < rays; r++) {
    if (h[r] > kRaMaxSeg) return set_error(AT_EINVAL, "at_rowaction_create: a ray crosses more than 2048 pixels");
    off[r + 1] = off[r] + h[r];
  }
  R->segments = off[rays];
  AT_CUDA_TRY(cudaMalloc(&R->off, sizeof(int64_t) * (rays + 1)));
  AT_CUDA_TRY(cudaMalloc(&R->line, sizeof(int) * std::max<int64_t>(R->segments, 1)));
  AT_CUDA_TRY(cudaMalloc(&R->weight, sizeof(float) * std::max<int64_t>(R->segments, 1)));
  AT_CUDA_TRY(cudaMemcpy(R->off, off.data(), sizeof(int64_t) * (rays + 1), cudaMemcpyHostToDevice));
  ra_fill_kernel<<<(rays + 127) / 128, 128>>>(R->G, R->trig, R->off, R->line, R->weight);
  AT_CUDA_TRY(cudaGetLastError());
  AT_CUDA_TRY(cudaDeviceSynchronize());
  *out = R.release();
  return AT_OK;
}

AT_API void at_rowaction_destroy(at_rowaction *ra) { delete ra; }

AT_API int at_rowaction_segments(const at_rowaction *ra, int64_t *segments) {
  if (!ra || !segments) return set_error(AT_EINVAL, "at_rowaction_segments: null argument");
  *segments = ra->segments;
  return AT_OK;
}

AT_API int at_rowaction_trace(const at_rowaction *ra, int32_t view, int32_t ray, int32_t *h_pix, float *h_w,
                              int32_t cap, int32_t *n_out) {
  if (!ra || !n_out) return set_error(AT_EINVAL, "at_rowaction_trace: null argument");
  if (view < 0 || view >= ra->G.nproj || ray < 0 || ray >= ra->G.nray)
    return set_error(AT_EINVAL, "at_rowaction_trace: ray out of range");
  const int r = view * ra->G.nray + ray;
  int64_t o[2];
  AT_CUDA_TRY(cudaMemcpy(o, ra->off + r, sizeof(o), cudaMemcpyDeviceToHost));
  const int n = (int)(o[1] - o[0]), m = std::min(n, (int)cap);
  if (m > 0 && h_pix) AT_CUDA_TRY(cudaMemcpy(h_pix, ra->line + o[0], sizeof(int) * m, cudaMemcpyDeviceToHost));
  if (m > 0 && h_w) AT_CUDA_TRY(cudaMemcpy(h_w, ra->weight + o[0], sizeof(float) * m, cudaMemcpyDeviceToHost));
  *n_out = n;
  return AT_OK;
}

AT_API int at_rowaction_forward(const at_rowaction *ra, int32_t nslices, const float *d_f, float *d_g, void *stream) {
  if (!ra || !d_f || !d_g) return set_error(AT_EINVAL, "at_rowaction_forward: null argument");
  if (nslices < 1 || nslices > 65535) return set_error(AT_EINVAL, "at_rowaction_forward: nslices must be in [1, 65535]");
  const int rays = ra->G.nproj * ra->G.nray;
  dim3 grid((rays + kRaWarps - 1) / kRaWarps, nslices);
  ra_forward_kernel<<<grid, 32 * kRaWarps, 0, (cudaStream_t)stream>>>(ra->G, ra->off, ra->line, ra->weight, d_f, d_g);
  AT_CUDA_TRY(cudaGetLastError());
  return AT_OK;
}

AT_API int at_rowaction_run(const at_rowaction *ra, int32_t nslices, const float *d_g, float *d_f, float *d_v,
                            const at_rowaction_params *prm, void *stream) {
  if (!ra || !d_g || !d_f || !d_v || !prm) return set_error(AT_EINVAL, "at_rowaction_run: null argument");
  if (nslices < 1 || nslices > 65535) return set_error(AT_EINVAL, "at_rowaction_run: nslices must be in [1, 65535]");
  if (prm->sweeps < 0 || prm->phases < 3 || prm->phases > ra->G.nray)
    return set_error(AT_EINVAL, "at_rowaction_run: need sweeps >= 0 and phases >= 3 (rays closer than 3 apart share pixels)");
  cudaStream_t st = (cudaStream_t)stream;
  RaGraphKey key;
  key.nslices = nslices;
  key.g = d_g;
  key.f = d_f;
  key.v = d_v;
  key.alpha = prm->alpha;
  key.lambda0 = prm->lambda0;
  key.lambda_decay = prm->lambda_decay;
  key.beta = prm->beta;
  key.epsilon = prm->epsilon;
  key.sweeps = prm->sweeps;
  key.phases = prm->phases;
  if (!ra->exec || !(ra->key == key)) {
    if (ra->exec) {
      AT_CUDA_TRY(cudaEventSynchronize(ra->done));  // its last launch has ended
      cudaGraphExecDestroy(ra->exec);
    }
    ra->exec = nullptr;
    if (!ra->cap) AT_CUDA_TRY(cudaStreamCreateWithFlags(&ra->cap, cudaStreamNonBlocking));
    if (!ra->done) AT_CUDA_TRY(cudaEventCreateWithFlags(&ra->done, cudaEventDisableTiming));
    AT_CUDA_TRY(cudaStreamBeginCapture(ra->cap, cudaStreamCaptureModeThreadLocal));
    enqueue_run(*ra, nslices, d_g, d_f, d_v, *prm, ra->cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ra->cap, &graph);
    if (e != cudaSuccess) return cuda_error(e, "at_rowaction_run: capture");
    const cudaError_t ei = cudaGraphInstantiate(&ra->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      ra->exec = nullptr;
      return cuda_error(ei, "at_rowaction_run: graph instantiation");
    }
    ra->key = key;
  }
  AT_CUDA_TRY(cudaGraphLaunch(ra->exec, st));
  AT_CUDA_TRY(cudaEventRecord(ra->done, st));
  return AT_OK;
}

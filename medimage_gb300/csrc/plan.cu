// plan.cu -- one-time projector plans, built on the GPU in FP64.
//
// Compiled with --fmad=false: every FP64 expression below is evaluated as
// separately rounded IEEE operations in the reference's order, so the traced
// pixel sequences are bit-identical to the reference's CPU traversal.  Trig
// tables come from the host's libm (see geometry.cpp), as in the reference.
//
// Fan beam  : helical/rebin/src/tracing.cpp:22-147 on the end points of
//             helical/rebin/src/ms2d.cpp:172-183.
// GoldenC   : origin/GoldenC/src/proj.c:38-200 (tile walks).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "at_internal.h"

namespace medimg {

// ---------------------------------------------------------------------------
// fan beam
// ---------------------------------------------------------------------------
struct FanDevTables {
  const double *scos, *ssin, *dcos, *dsin;
};

// Where a ray's end points come from: the fan geometry's tables
// (helical/rebin/src/ms2d.cpp:172-183) or a caller's table of
// (sx, sy, dx, dy) per ray, the arguments of the reference tracer's
// forward_proj (helical/rebin/src/tracing.cpp:22).
struct RaySource {
  at_fan_geometry g;
  FanDevTables T;
  const double *ends;  // [rays][4] for AT_GEOM_RAYS, else null
};

// Real = double: the reference's FP64 arithmetic (bit-identical traversal).
// Real = float: the same steps in FP32 throughout (tables, end points, lambda
// entry/exit, start pixel, crossing merge): the plain form, used to measure
// what the FP64 traversal buys.
template <typename Real>
__device__ __forceinline__ void ray_endpoints(const RaySource &R, int view, int det, Real &sx, Real &sy, Real &dx,
                                              Real &dy) {
  if (R.ends) {
    const double *e = R.ends + ((size_t)view * R.g.ndets + det) * 4;
    sx = (Real)e[0];
    sy = (Real)e[1];
    dx = (Real)e[2];
    dy = (Real)e[3];
    return;
  }
  const at_fan_geometry &g = R.g;
  const Real vx = (Real)g.pixel_mm, vy = (Real)g.pixel_mm;
  const Real sod = (Real)g.sod_mm, sdd = (Real)g.sdd_mm, two = (Real)2.0;
  // ms2d.cpp:172-183
  const Real scos = (Real)R.T.scos[view], ssin = (Real)R.T.ssin[view];
  const Real dcos = (Real)R.T.dcos[det], dsin = (Real)R.T.dsin[det];
  sx = sod * scos + (Real)g.n * vx / two;
  sy = sod * ssin + (Real)g.n * vy / two;
  dx = sdd * (dcos * scos - dsin * ssin) + sx;
  dy = sdd * (dsin * scos + dcos * ssin) + sy;
}

// Traces ray (view, det).  Mode 0: fill the header and count segments.
// Mode 1: also write the decision words into the block-interleaved array.
template <int kMode, typename Real>
__device__ void fan_trace_ray(const RaySource &R, int view, int det, RayHdr *hdr, int *offgrid, uint32_t *bits,
                              uint32_t word_stride) {
  const int NX = R.g.n, NY = R.g.n;
  const Real vx = (Real)R.g.pixel_mm, vy = (Real)R.g.pixel_mm;
  const Real zero = (Real)0.0, tiny = (Real)1.e-4, huge = (Real)1.e6;
  Real sx, sy, dx, dy;
  ray_endpoints<Real>(R, view, det, sx, sy, dx, dy);
  // tracing.cpp:39-87
  int index = 0;
  const Real ray_x = dx - sx, ray_y = dy - sy;
  const Real L = sqrt(ray_x * ray_x + ray_y * ray_y);
  Real lambda_min = zero, lambda_max = L;
  const int signx = (ray_x > zero) ? 1 : -1;
  const int signy = (ray_y > zero) ? 1 : -1;
  const Real absx = fabs(ray_x), absy = fabs(ray_y);
  const Real len_x = (absx > tiny) ? (L / absx) * vx : huge;
  const Real len_y = (absy > tiny) ? (L / absy) * vy : huge;
  Real tempx = (Real)NX * vx, tempy = (Real)NY * vy;
  Real l0, lN, temp;
  l0 = (L * (zero - sx)) / (dx - sx);
  lN = (L * (tempx - sx)) / (dx - sx);
  temp = (l0 < lN) ? l0 : lN;
  lambda_min = (lambda_min > temp) ? lambda_min : temp;
  if (lambda_min == temp) index = 1;
  temp = (l0 > lN) ? l0 : lN;
  lambda_max = (lambda_max < temp) ? lambda_max : temp;
  l0 = (L * (zero - sy)) / (dy - sy);
  lN = (L * (tempy - sy)) / (dy - sy);
  temp = (l0 < lN) ? l0 : lN;
  lambda_min = (lambda_min > temp) ? lambda_min : temp;
  if (lambda_min == temp) index = 2;
  temp = (l0 > lN) ? l0 : lN;
  lambda_max = (lambda_max < temp) ? lambda_max : temp;

  RayHdr h;
  h.pix0 = 0;
  h.nseg = 0;
  h.xy0 = 0;
  h.sgn = (signx > 0 ? 1 : 0) | (signy > 0 ? 2 : 0);
  h.ax = h.ay = 0.f;
  h.lenx = (float)len_x;
  h.leny = (float)len_y;
  if (lambda_min >= lambda_max) {
    if (kMode == 0) {
      *hdr = h;
      *offgrid = 0;
    }
    return;
  }
  Real lambda0 = lambda_min, lambda_x, lambda_y;
  int v_x, v_y;
  if (index == 1) {  // tracing.cpp:91-102
    v_x = (signx == 1) ? 0 : NX - 1;
    lambda_x = lambda0 + len_x;
    v_y = (int)((sy + lambda0 * ray_y / L) / vy);
    tempy = (Real)v_y * vy;
    lambda_y = (absy < tiny) ? huge : (L * ((tempy + (Real)(signy > 0) * vy) - sy)) / (dy - sy);
  } else {  // tracing.cpp:104-115
    v_y = (signy == 1) ? 0 : NY - 1;
    lambda_y = lambda0 + len_y;
    v_x = (int)((sx + lambda0 * ray_x / L) / vx);
    tempx = (Real)v_x * vx;
    lambda_x = (absx < tiny) ? huge : (L * ((tempx + (Real)(signx > 0) * vx) - sx)) / (dx - sx);
  }
  h.pix0 = v_x * NY + v_y;
  h.xy0 = (v_x & 0xffff) | (v_y << 16);
  h.ax = (float)(lambda_x - lambda_min);
  h.ay = (float)(lambda_y - lambda_min);
  int numb = 0, bad = 0;
  uint32_t word = 0;
  const Real stop = lambda_max - (Real)5.e-2;
  while (lambda0 < stop) {  // tracing.cpp:118-146
    if ((unsigned)v_x >= (unsigned)NX || (unsigned)v_y >= (unsigned)NY) bad++;
    const bool xstep = lambda_x <= lambda_y;
    if (kMode == 1) {
      if (xstep) word |= 1u << (numb & 31);
      if ((numb & 31) == 31) {
        bits[(size_t)(numb >> 5) * word_stride] = word;
        word = 0;
      }
    }
    ++numb;
    if (xstep) {
      lambda0 = lambda_x;
      lambda_x += len_x;
      v_x += signx;
    } else {
      lambda0 = lambda_y;
      lambda_y += len_y;
      v_y += signy;
    }
  }
  if (kMode == 1 && (numb & 31) != 0) bits[(size_t)(numb >> 5) * word_stride] = word;
  if (kMode == 0) {
    h.nseg = numb;
    *hdr = h;
    *offgrid = bad;
  }
}

template <typename Real>
__global__ void fan_count_kernel(const RaySource R, RayHdr *hdr, int *offgrid) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= R.g.nviews * R.g.ndets) return;
  const int view = ray / R.g.ndets, det = ray % R.g.ndets;
  fan_trace_ray<0, Real>(R, view, det, hdr + ray, offgrid + ray, nullptr, 0);
}

template <typename Real>
__global__ void fan_fill_kernel(const RaySource R, int nblocks_per_view, const uint32_t *blk_word, uint32_t *bits) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= R.g.nviews * R.g.ndets) return;
  const int view = ray / R.g.ndets, det = ray % R.g.ndets;
  const int blk = view * nblocks_per_view + det / kRayBlock;
  uint32_t *dst = bits + blk_word[blk] + (det % kRayBlock);
  fan_trace_ray<1, Real>(R, view, det, nullptr, nullptr, dst, kRayBlock);
}

// Segments each pixel receives from each block of kBpViewBlock views, for the
// back projector's fixed-point range when no geometric bound is known.
__global__ void pixel_hits_kernel(int n, int view0, int view1, int ndets, int nbpv, const RayHdr *hdr,
                                  const uint32_t *bits, const uint32_t *blk_word, unsigned *hits) {
  const int ray = view0 * ndets + blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= view1 * ndets) return;
  const RayHdr h = hdr[ray];
  const int view = ray / ndets, det = ray % ndets;
  const uint32_t *wp = bits + blk_word[view * nbpv + det / kRayBlock] + (det % kRayBlock);
  int x = h.xy0 & 0xffff, y = h.xy0 >> 16;
  const int sx = (h.sgn & 1) ? 1 : -1, sy = (h.sgn & 2) ? 1 : -1;
  uint32_t word = 0;
  for (int k = 0; k < h.nseg; k++) {
    if ((k & 31) == 0) word = wp[(size_t)(k >> 5) * kRayBlock];
    if ((unsigned)x < (unsigned)n && (unsigned)y < (unsigned)n) atomicAdd(hits + (size_t)x * n + y, 1u);
    if ((word >> (k & 31)) & 1u) x += sx;
    else y += sy;
  }
}

__global__ void max_kernel(const unsigned *v, size_t n, unsigned *out) {
  unsigned m = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = max(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

namespace {
template <typename T>
int dev_alloc(T **p, size_t count, int64_t &acct) {
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
  if (e != cudaSuccess) return set_error(AT_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  acct += (int64_t)(sizeof(T) * count);
  return AT_OK;
}
}  // namespace

// ---------------------------------------------------------------------------
// back-projection runs: the traversal of every ray cut into its runs through
// 16x16 pixel tiles, so the back projector can own a tile and walk exactly the
// forward projector's segments inside it.
// ---------------------------------------------------------------------------
template <int kMode>
__global__ void fan_runs_kernel(int n, int nviews, int ndets, int nbpv, const RayHdr *hdr, const uint32_t *bits,
                                const uint32_t *blk_word, int tiles_y, int nvb, int *tile_count,
                                unsigned long long *cursor, uint4 *ent, unsigned long long *keys) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= nviews * ndets) return;
  const RayHdr h = hdr[ray];
  if (h.nseg == 0) return;
  const int view = ray / ndets, det = ray % ndets;
  const uint32_t wbase = blk_word[view * nbpv + det / kRayBlock] + (det % kRayBlock);
  const uint32_t *wp = bits + wbase;
  int x = h.xy0 & 0xffff, y = h.xy0 >> 16;
  const int sx = (h.sgn & 1) ? 1 : -1, sy = (h.sgn & 2) ? 1 : -1;
  int cx = 0, cur_tile = -1, run_k = 0, run_cx = 0, run_x = 0, run_y = 0, prevx = 0, run_prevx = 0;
  uint32_t word = 0, run_bits = 0;  // run_bits: the run's decisions, bit j = segment run_k + j
  auto close_run = [&](int k_end) {
    if (cur_tile < 0) return;
    const int nk = k_end - run_k;
    const int vb = view / kBpViewBlock;
    if (kMode == 0) {
      atomicAdd(&tile_count[(size_t)cur_tile * nvb + vb], 1);
    } else {
      const unsigned long long pos = atomicAdd(cursor, 1ull);
      ent[pos] = make_uint4((unsigned)ray, (unsigned)run_k | ((unsigned)nk << 14) | ((unsigned)run_cx << 19), run_bits,
                            (unsigned)(run_x & 15) | ((unsigned)(run_y & 15) << 4) | ((h.sgn & 1u) << 8) |
                                (((h.sgn >> 1) & 1u) << 9) | ((unsigned)run_prevx << 10));
      // by tile, then view block, then longest runs first, then ray order
      static_assert(kBpViewBlock <= 64, "view-in-block field is 6 bits");
      keys[pos] = ((unsigned long long)cur_tile << 38) | ((unsigned long long)vb << 28) |
                  ((unsigned long long)(63 - nk) << 22) | ((unsigned long long)(view % kBpViewBlock) << 16) |
                  (unsigned)det;
    }
  };
  for (int k = 0; k < h.nseg; k++) {
    if ((k & 31) == 0) word = wp[(size_t)(k >> 5) * kRayBlock];
    const bool inside = (unsigned)x < (unsigned)n && (unsigned)y < (unsigned)n;
    const int t = inside ? (x >> 4) * tiles_y + (y >> 4) : -1;
    if (t != cur_tile) {
      close_run(k);
      cur_tile = t;
      run_k = k;
      run_cx = cx;
      run_x = x;
      run_y = y;
      run_prevx = prevx;
      run_bits = 0;
    }
    const int bit = (word >> (k & 31)) & 1;
    // a tile run has at most 31 segments (16 + 16 - 1); off-grid stretches are not runs
    if (cur_tile >= 0) run_bits |= (uint32_t)bit << (k - run_k);
    if (bit) {
      x += sx;
      cx++;
    } else {
      y += sy;
    }
    prevx = bit;
  }
  close_run(h.nseg);
}

__global__ void gather_runs_kernel(const uint4 *src, const unsigned *idx, uint4 *dst, int64_t count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) dst[i] = src[idx[i]];
}

__global__ void iota_kernel(unsigned *v, int64_t count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) v[i] = (unsigned)i;
}

int build_fan_runs(Plan &p, cudaStream_t st) {
  const int nrays = p.nviews * p.ndets, tpb = 128;
  p.ntiles_y = (p.n + kBpTile - 1) / kBpTile;
  p.ntiles = p.ntiles_y * p.ntiles_y;
  p.nvb = (p.nviews + kBpViewBlock - 1) / kBpViewBlock;
  const size_t ncell = (size_t)p.ntiles * p.nvb;
  int *cnt_d = nullptr;
  unsigned long long *cur_d = nullptr;
  uint4 *tmp_ent = nullptr;
  unsigned long long *keys = nullptr, *keys_out = nullptr;
  unsigned *idx = nullptr, *idx_out = nullptr, *hits = nullptr;
  void *temp = nullptr;
  const auto free_temps = scope_exit([&] {
    cudaFree(hits);
    cudaFree(temp);
    cudaFree(tmp_ent);
    cudaFree(keys);
    cudaFree(keys_out);
    cudaFree(idx);
    cudaFree(idx_out);
    cudaFree(cnt_d);
    cudaFree(cur_d);
  });
  AT_CUDA_TRY(cudaMalloc(&cnt_d, sizeof(int) * ncell));
  AT_CUDA_TRY(cudaMalloc(&cur_d, sizeof(unsigned long long)));
  AT_CUDA_TRY(cudaMemsetAsync(cnt_d, 0, sizeof(int) * ncell, st));
  AT_CUDA_TRY(cudaMemsetAsync(cur_d, 0, sizeof(unsigned long long), st));
  fan_runs_kernel<0><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(p.n, p.nviews, p.ndets, p.nblocks_per_view, p.rays_d,
                                                              p.bits_d, p.blk_word_d, p.ntiles_y, p.nvb, cnt_d,
                                                              nullptr, nullptr, nullptr);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<int> cnt(ncell);
  AT_CUDA_TRY(cudaMemcpyAsync(cnt.data(), cnt_d, sizeof(int) * ncell, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int32_t> off(ncell + 1);
  int64_t tot = 0;
  for (size_t t = 0; t < ncell; t++) {
    off[t] = (int32_t)tot;
    tot += cnt[t];
  }
  if (tot >= (1ll << 31)) return set_error(AT_EINVAL, "plan: too many back-projection runs");
  off[ncell] = (int32_t)tot;
  p.nruns = tot;
  AT_CUDA_TRY(cudaMalloc(&tmp_ent, sizeof(uint4) * std::max<int64_t>(tot, 1)));
  AT_CUDA_TRY(cudaMalloc(&keys, sizeof(unsigned long long) * std::max<int64_t>(tot, 1)));
  AT_CUDA_TRY(cudaMalloc(&keys_out, sizeof(unsigned long long) * std::max<int64_t>(tot, 1)));
  AT_CUDA_TRY(cudaMalloc(&idx, sizeof(unsigned) * std::max<int64_t>(tot, 1)));
  AT_CUDA_TRY(cudaMalloc(&idx_out, sizeof(unsigned) * std::max<int64_t>(tot, 1)));
  fan_runs_kernel<1><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(p.n, p.nviews, p.ndets, p.nblocks_per_view, p.rays_d,
                                                              p.bits_d, p.blk_word_d, p.ntiles_y, p.nvb, nullptr,
                                                              cur_d, tmp_ent, keys);
  AT_CUDA_TRY(cudaGetLastError());
  iota_kernel<<<(int)((tot + 255) / 256) + 1, 256, 0, st>>>(idx, tot);
  AT_CUDA_TRY(cudaGetLastError());
  // keys are unique (tile, view block, 63-nk, view, det): the sorted order is deterministic
  size_t temp_bytes = 0;
  AT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys, keys_out, idx, idx_out, (int64_t)tot, 0, 64, st));
  AT_CUDA_TRY(cudaMalloc(&temp, std::max<size_t>(temp_bytes, 1)));
  AT_CUDA_TRY(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys_out, idx, idx_out, (int64_t)tot, 0, 64, st));
  int rc;
  if ((rc = dev_alloc(&p.run_d, tot, p.device_bytes))) return rc;
  if ((rc = dev_alloc(&p.tile_off_d, ncell + 1, p.device_bytes))) return rc;
  gather_runs_kernel<<<(int)((tot + 255) / 256) + 1, 256, 0, st>>>(tmp_ent, idx_out, p.run_d, tot);
  AT_CUDA_TRY(cudaGetLastError());
  AT_CUDA_TRY(cudaMemcpyAsync(p.tile_off_d, off.data(), sizeof(int32_t) * (ncell + 1), cudaMemcpyHostToDevice, st));
  // Terms one pixel can receive within one view block bound the fixed-point
  // scale.  Fan beam: rays through a pixel are at least d_min * pitch apart
  // (d_min = closest approach of the image to the source), so at most
  // ceil(pixel diagonal / that) + 1 of them cross it per view.  Ray tables: the
  // exact count, taken from the traversal.
  double per_block;
  if (p.kind == AT_GEOM_FAN) {
    const at_fan_geometry &g = p.geom;
    const double dmin = g.sod_mm - g.n * g.pixel_mm * std::sqrt(2.0) / 2.0;
    const double spacing = dmin * g.det_pitch_deg * M_PI / 180.0;
    const int per_view = (int)std::ceil(std::sqrt(2.0) * g.pixel_mm / spacing) + 1;
    per_block = (double)per_view * kBpViewBlock;
  } else {
    const size_t cells = (size_t)p.n * p.n;
    unsigned *mx = nullptr;
    AT_CUDA_TRY(cudaMalloc(&hits, sizeof(unsigned) * (cells + 1)));
    mx = hits + cells;
    AT_CUDA_TRY(cudaMemsetAsync(mx, 0, sizeof(unsigned), st));
    for (int vb = 0; vb < p.nvb; vb++) {
      const int v0 = vb * kBpViewBlock, v1 = std::min(p.nviews, v0 + kBpViewBlock);
      AT_CUDA_TRY(cudaMemsetAsync(hits, 0, sizeof(unsigned) * cells, st));
      pixel_hits_kernel<<<((v1 - v0) * p.ndets + 127) / 128, 128, 0, st>>>(p.n, v0, v1, p.ndets, p.nblocks_per_view,
                                                                          p.rays_d, p.bits_d, p.blk_word_d, hits);
      AT_CUDA_TRY(cudaGetLastError());
      max_kernel<<<256, 256, 0, st>>>(hits, cells, mx);
      AT_CUDA_TRY(cudaGetLastError());
    }
    unsigned m = 0;
    AT_CUDA_TRY(cudaMemcpyAsync(&m, mx, sizeof(m), cudaMemcpyDeviceToHost, st));
    AT_CUDA_TRY(cudaStreamSynchronize(st));
    per_block = std::max(1u, m);
  }
  // terms stay below 2^22 so the kernel can round them with one FFMA
  p.bp_term_bits = std::min(22, 31 - (int)std::ceil(std::log2(per_block + 1.0)));
  if (p.bp_term_bits < 16) return set_error(AT_EINVAL, "plan: detector far finer than the pixel grid (back projector precision)");
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  return AT_OK;
}

int build_fan_plan(Plan &p, cudaStream_t st, const double *h_ends) {
  const at_fan_geometry &g = p.geom;
  const int nv = g.nviews, nd = g.ndets, nrays = nv * nd;
  p.n = g.n;
  p.nviews = nv;
  p.ndets = nd;
  p.rays = nrays;
  double *tab_d = nullptr;
  int rc;
  RaySource R{};
  R.g = g;
  if (h_ends) {
    AT_CUDA_TRY(cudaMalloc(&tab_d, sizeof(double) * 4 * (size_t)nrays));
    AT_CUDA_TRY(cudaMemcpyAsync(tab_d, h_ends, sizeof(double) * 4 * (size_t)nrays, cudaMemcpyHostToDevice, st));
    R.ends = tab_d;
  } else {
    std::vector<double> scos(nv), ssin(nv), dcos(nd), dsin(nd);
    fan_tables(g, scos.data(), ssin.data(), dcos.data(), dsin.data());
    AT_CUDA_TRY(cudaMalloc(&tab_d, sizeof(double) * 2 * (nv + nd)));
    AT_CUDA_TRY(cudaMemcpyAsync(tab_d, scos.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaMemcpyAsync(tab_d + nv, ssin.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaMemcpyAsync(tab_d + 2 * nv, dcos.data(), sizeof(double) * nd, cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaMemcpyAsync(tab_d + 2 * nv + nd, dsin.data(), sizeof(double) * nd, cudaMemcpyHostToDevice, st));
    AT_CUDA_TRY(cudaStreamSynchronize(st));  // the host tables go out of scope
    R.T = FanDevTables{tab_d, tab_d + nv, tab_d + 2 * nv, tab_d + 2 * nv + nd};
  }

  if ((rc = dev_alloc(&p.rays_d, nrays, p.device_bytes))) return rc;
  int *off_d = nullptr;
  AT_CUDA_TRY(cudaMalloc(&off_d, sizeof(int) * nrays));
  const int tpb = 128;
  if (p.alpha_fp32)
    fan_count_kernel<float><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(R, p.rays_d, off_d);
  else
    fan_count_kernel<double><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(R, p.rays_d, off_d);
  AT_CUDA_TRY(cudaGetLastError());

  std::vector<RayHdr> hdr(nrays);
  std::vector<int> off(nrays);
  AT_CUDA_TRY(cudaMemcpyAsync(hdr.data(), p.rays_d, sizeof(RayHdr) * nrays, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(off.data(), off_d, sizeof(int) * nrays, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(off_d);

  p.nblocks_per_view = (nd + kRayBlock - 1) / kRayBlock;
  p.nblocks = nv * p.nblocks_per_view;
  std::vector<uint32_t> blk_word(p.nblocks + 1);
  std::vector<uint8_t> blk_off(p.nblocks);
  uint64_t words = 0;
  int64_t segs = 0, bad = 0;
  int maxseg = 0;
  for (int v = 0; v < nv; v++)
    for (int b = 0; b < p.nblocks_per_view; b++) {
      int mx = 0, boff = 0;
      for (int d = b * kRayBlock; d < std::min(nd, (b + 1) * kRayBlock); d++) {
        const RayHdr &h = hdr[(size_t)v * nd + d];
        mx = std::max(mx, h.nseg);
        segs += h.nseg;
        bad += off[(size_t)v * nd + d];
        boff |= off[(size_t)v * nd + d] != 0;
      }
      maxseg = std::max(maxseg, mx);
      const int blk = v * p.nblocks_per_view + b;
      const int nw = (mx + 31) / 32;
      if (nw > 255) return set_error(AT_EINVAL, "ray longer than 8160 segments");
      blk_word[blk] = (uint32_t)words;
      blk_off[blk] = (uint8_t)boff;
      words += (uint64_t)nw * kRayBlock;
    }
  if (words >= (1ull << 32)) return set_error(AT_EINVAL, "plan exceeds 2^32 decision words");
  blk_word[p.nblocks] = (uint32_t)words;
  p.segments = segs;
  p.offgrid = bad;
  p.max_segments = maxseg;

  // one spare block of zero words at the end: readers may fetch the word after
  // a ray's last one without a bounds check
  if ((rc = dev_alloc(&p.bits_d, words + kRayBlock, p.device_bytes))) return rc;
  if ((rc = dev_alloc(&p.blk_word_d, p.nblocks + 1, p.device_bytes))) return rc;
  if ((rc = dev_alloc(&p.blk_off_d, p.nblocks, p.device_bytes))) return rc;
  AT_CUDA_TRY(cudaMemsetAsync(p.bits_d, 0, sizeof(uint32_t) * (words + kRayBlock), st));
  AT_CUDA_TRY(cudaMemcpyAsync(p.blk_word_d, blk_word.data(), sizeof(uint32_t) * (p.nblocks + 1),
                              cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaMemcpyAsync(p.blk_off_d, blk_off.data(), p.nblocks, cudaMemcpyHostToDevice, st));
  if (p.alpha_fp32)
    fan_fill_kernel<float><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(R, p.nblocks_per_view, p.blk_word_d, p.bits_d);
  else
    fan_fill_kernel<double><<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(R, p.nblocks_per_view, p.blk_word_d, p.bits_d);
  AT_CUDA_TRY(cudaGetLastError());

  if ((rc = build_fan_runs(p, st))) return rc;
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(tab_d);
  return AT_OK;
}

// ---------------------------------------------------------------------------
// GoldenC parallel beam
// ---------------------------------------------------------------------------
constexpr int kGcN = 512, kGcDets = 767, kGcTile = 128, kGcRays = 384, kGcAlphas = 45;
constexpr int kGcPairs = kGcAlphas * kGcRays;  // (alpha, raynum) pairs
constexpr int kGcWalks = kGcPairs * 16;        // (alpha, raynum, tile)

struct GcTrig {
  double sf, cf, hx, hy, tanphi, rtnphi;
};

// proj.c:55-200.  walk = pair*16 + tile.  Mode 0 counts, mode 1 writes.
template <int kMode>
__device__ int gc_walk_dev(const GcTrig *trig, int walk, GcSeg *out) {
  const int pair = walk >> 4, tile = walk & 15;
  const int alpha = 1 + pair / kGcRays, raynum = pair % kGcRays;
  const GcTrig t = trig[alpha - 1];
  const int ind = raynum - (kGcDets / 2);
  const int col = tile % 4;
  const int dxo = kGcTile * (3 - col), dyo = kGcTile * (tile / 4);
  double c = t.cf * ind + t.sf * ind * t.tanphi;
  c = (kGcN / 2 - dyo) - t.tanphi * (kGcN / 2 - kGcTile * col) - c;
  int ix, iy, next;
  double fp, w, xc, yc;
  if (c < 0) {
    c = -c * t.rtnphi;
    ix = (int)c;
    iy = 0;
    fp = ((double)(ix + 1)) - c;
    ix = kGcTile - ix - 1;
    w = t.hy * fp;
    yc = fp * t.tanphi;
    xc = -fp;
    next = 2;
  } else {
    ix = kGcTile - 1;
    iy = (int)c;
    fp = ((double)(iy + 1)) - c;
    yc = -fp;
    w = t.hx * fp;
    xc = fp * t.rtnphi;
    next = 1;
  }
  int n = 0;
  while (ix >= 0 && ix < kGcTile && iy >= 0 && iy < kGcTile) {
    double emit;
    const int ex = ix, ey = iy;
    if (next == 1) {
      xc -= 1.0;
      yc += t.tanphi;
      if (xc > 0) {
        emit = t.hy;
        w -= t.hy;
        ix -= 1;
      } else {
        emit = w;
        w = t.hy - w;
        iy++;
        next = 2;
      }
    } else {
      yc -= 1.0;
      xc += t.rtnphi;
      if (yc > 0) {
        w -= t.hx;
        emit = t.hx;
        iy++;
      } else {
        emit = w;
        w = t.hx - w;
        ix -= 1;
        next = 1;
      }
    }
    if (kMode == 1) {
      out[n].pix = (ey + dyo) * kGcN + (ex + dxo);
      out[n].w = (float)emit;
    }
    n++;
  }
  return n;
}

__global__ void gc_count_kernel(const GcTrig *trig, int *count) {
  const int walk = blockIdx.x * blockDim.x + threadIdx.x;
  if (walk >= kGcWalks) return;
  count[walk] = gc_walk_dev<0>(trig, walk, nullptr);
}

__global__ void gc_fill_kernel(const GcTrig *trig, const int64_t *walk_off, GcSeg *seg) {
  const int walk = blockIdx.x * blockDim.x + threadIdx.x;
  if (walk >= kGcWalks) return;
  gc_walk_dev<1>(trig, walk, seg + walk_off[walk]);
}

__global__ void gc_pix_count_kernel(const GcSeg *seg, int64_t nseg, int *cnt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nseg) return;
  atomicAdd(&cnt[seg[i].pix], 1);
}

__global__ void gc_pix_fill_kernel(const GcSeg *seg, const int32_t *pair_off, int64_t nseg, int *cursor,
                                   GcEntry *ent) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nseg) return;
  // pair of segment i: binary search in pair_off
  int lo = 0, hi = kGcPairs;  // pair_off[lo] <= i < pair_off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (pair_off[mid] <= i) lo = mid;
    else hi = mid;
  }
  const int pos = atomicAdd(&cursor[seg[i].pix], 1);
  ent[pos].pair = lo;
  ent[pos].w = seg[i].w;
}

// orders each pixel's entries by pair so the gather sums in a fixed order
__global__ void gc_pix_sort_kernel(const int32_t *pix_off, GcEntry *ent) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= kGcN * kGcN) return;
  const int b = pix_off[pix], e = pix_off[pix + 1];
  for (int i = b + 1; i < e; i++) {
    const GcEntry x = ent[i];
    int j = i - 1;
    while (j >= b && ent[j].pair > x.pair) {
      ent[j + 1] = ent[j];
      j--;
    }
    ent[j + 1] = x;
  }
}

int build_goldnc_plan(Plan &p, cudaStream_t st) {
  p.kind = AT_GEOM_GOLDNC;
  p.n = kGcN;
  p.nviews = 180;
  p.ndets = kGcDets;
  p.rays = 180 * kGcDets;
  std::vector<GcTrig> trig(kGcAlphas);
  for (int a = 1; a <= kGcAlphas; a++) {  // proj.c:43-48, host libm
    GcTrig &t = trig[a - 1];
    const double ang = 3.141593 / 180 * a;
    t.sf = std::sin(ang);
    t.cf = std::cos(ang);
    t.hx = ((double)1.0) / t.sf;
    t.hy = ((double)1.0) / t.cf;
    t.tanphi = t.sf / t.cf;
    t.rtnphi = t.cf / t.sf;
  }
  GcTrig *trig_d = nullptr;
  int *cnt_d = nullptr;
  AT_CUDA_TRY(cudaMalloc(&trig_d, sizeof(GcTrig) * kGcAlphas));
  AT_CUDA_TRY(cudaMemcpyAsync(trig_d, trig.data(), sizeof(GcTrig) * kGcAlphas, cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaMalloc(&cnt_d, sizeof(int) * kGcWalks));
  gc_count_kernel<<<(kGcWalks + 127) / 128, 128, 0, st>>>(trig_d, cnt_d);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<int> cnt(kGcWalks);
  AT_CUDA_TRY(cudaMemcpyAsync(cnt.data(), cnt_d, sizeof(int) * kGcWalks, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int64_t> walk_off(kGcWalks + 1);
  std::vector<int32_t> pair_off(kGcPairs + 1);
  int64_t tot = 0;
  int maxseg = 0;
  for (int w = 0; w < kGcWalks; w++) {
    if ((w & 15) == 0) pair_off[w >> 4] = (int32_t)tot;
    walk_off[w] = tot;
    tot += cnt[w];
  }
  walk_off[kGcWalks] = tot;
  pair_off[kGcPairs] = (int32_t)tot;
  for (int q = 0; q < kGcPairs; q++) maxseg = std::max(maxseg, pair_off[q + 1] - pair_off[q]);
  p.max_segments = maxseg;
  p.segments = tot;  // traced segments (each feeds up to 8 bins)
  int rc;
  int64_t *walk_off_d = nullptr;
  AT_CUDA_TRY(cudaMalloc(&walk_off_d, sizeof(int64_t) * (kGcWalks + 1)));
  AT_CUDA_TRY(cudaMemcpyAsync(walk_off_d, walk_off.data(), sizeof(int64_t) * (kGcWalks + 1),
                              cudaMemcpyHostToDevice, st));
  if ((rc = dev_alloc(&p.gc_seg_d, tot, p.device_bytes))) return rc;
  if ((rc = dev_alloc(&p.gc_pair_off_d, kGcPairs + 1, p.device_bytes))) return rc;
  AT_CUDA_TRY(cudaMemcpyAsync(p.gc_pair_off_d, pair_off.data(), sizeof(int32_t) * (kGcPairs + 1),
                              cudaMemcpyHostToDevice, st));
  gc_fill_kernel<<<(kGcWalks + 127) / 128, 128, 0, st>>>(trig_d, walk_off_d, p.gc_seg_d);
  AT_CUDA_TRY(cudaGetLastError());

  // transpose to per-pixel lists
  int *pcnt_d = nullptr;
  AT_CUDA_TRY(cudaMalloc(&pcnt_d, sizeof(int) * kGcN * kGcN));
  AT_CUDA_TRY(cudaMemsetAsync(pcnt_d, 0, sizeof(int) * kGcN * kGcN, st));
  const int nb = (int)((tot + 255) / 256);
  gc_pix_count_kernel<<<nb, 256, 0, st>>>(p.gc_seg_d, tot, pcnt_d);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<int> pcnt(kGcN * kGcN);
  AT_CUDA_TRY(cudaMemcpyAsync(pcnt.data(), pcnt_d, sizeof(int) * kGcN * kGcN, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int32_t> pix_off(kGcN * kGcN + 1);
  int64_t acc = 0;
  for (int i = 0; i < kGcN * kGcN; i++) {
    pix_off[i] = (int32_t)acc;
    acc += pcnt[i];
  }
  pix_off[kGcN * kGcN] = (int32_t)acc;
  if ((rc = dev_alloc(&p.gc_pix_off_d, kGcN * kGcN + 1, p.device_bytes))) return rc;
  if ((rc = dev_alloc(&p.gc_ent_d, tot, p.device_bytes))) return rc;
  AT_CUDA_TRY(cudaMemcpyAsync(p.gc_pix_off_d, pix_off.data(), sizeof(int32_t) * (kGcN * kGcN + 1),
                              cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaMemcpyAsync(pcnt_d, pix_off.data(), sizeof(int32_t) * kGcN * kGcN, cudaMemcpyHostToDevice, st));
  gc_pix_fill_kernel<<<nb, 256, 0, st>>>(p.gc_seg_d, p.gc_pair_off_d, tot, pcnt_d, p.gc_ent_d);
  AT_CUDA_TRY(cudaGetLastError());
  gc_pix_sort_kernel<<<(kGcN * kGcN + 255) / 256, 256, 0, st>>>(p.gc_pix_off_d, p.gc_ent_d);
  AT_CUDA_TRY(cudaGetLastError());
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(pcnt_d);
  cudaFree(walk_off_d);
  cudaFree(cnt_d);
  cudaFree(trig_d);
  return AT_OK;
}

Plan::~Plan() {
  cudaFree(rays_d);
  cudaFree(bits_d);
  cudaFree(blk_word_d);
  cudaFree(blk_off_d);
  cudaFree(run_d);
  cudaFree(tile_off_d);
  cudaFree(gc_seg_d);
  cudaFree(gc_pair_off_d);
  cudaFree(gc_ent_d);
  cudaFree(gc_pix_off_d);
  cudaFree(cone_trig_d);
  free_slab_tables(slab);
  for (auto &r : retired_slabs) free_slab_tables(r);
  free_pixel_table(*this);
}

}  // namespace medimg

// cone.cu -- 3D cone-beam projectors, traced on the fly.
//
// Each thread walks one ray with the reference's single-precision Siddon
// (industry3d/src/tracing.cpp:123-307) from the end points of its cone()
// (tracing.cpp:51-81).  Every operation is an explicitly rounded intrinsic
// (__fadd_rn, __fmul_rn, ...) in the reference's order, so the visited voxels
// and the FP32 weights are bit-identical to the reference's whatever the
// compiler's contraction settings.  Nothing per ray is stored: at 512^3 with
// 720 x 768 x 1024 rays a stored traversal would take hundreds of GB.
//
// Forward: thread per ray (detector columns fastest, so a warp's rays are
// neighbours and share voxels in L1/L2), FP32 products summed per 32 segments
// and the partial sums Kahan-folded, then the fused epilogue of the 2D
// projectors.  Back: thread per ray, in chunks of views, each term w*r scaled
// to an integer (one FFMA, magic-number rounding) and added with a 32-bit
// reduction into the chunk's accumulator, whose sums a fold pass moves into
// exact 64-bit ones between chunks; integer sums do not depend on order, so
// the result is deterministic without float atomics.  A per-voxel pass adds
// the last chunk, converts, runs the epilogue and leaves both accumulators
// zero.
#include <algorithm>
#include <cmath>
#include <vector>

#include "epilogue.cuh"
#include "solver.h"

namespace medimg {

// State of one ray's walk (tracing.cpp:131-265).
struct ConeWalk {
  float lam0, lx, ly, lz, len_x, len_y, len_z;
  float stop;  // the smallest float >= lambda_max - 0.05 (see cone_start)
  int vx, vy, vz, sx, sy, sz;
  bool empty;
};

// tracing.cpp:51-81 (cone) with utility.cpp:82-98 (rotate_2d: d = R x summed
// from zero, k-major); cos and sin per view come from the host's libm
__device__ __forceinline__ void cone_endpoints(const ScanDev &S, int view, int row, int col, float &sx, float &sy,
                                               float &sz, float &dx, float &dy, float &dz) {
  const float2 cs = S.cone_trig[view];
  const float c = cs.x, s = cs.y, ns = -cs.y;
  const float X0 = 0.0f, X1 = -S.sod;  // source (0, -SOD, 0)
  float srcX = __fadd_rn(__fadd_rn(0.0f, __fmul_rn(c, X0)), __fmul_rn(ns, X1));
  float srcY = __fadd_rn(__fadd_rn(0.0f, __fmul_rn(s, X0)), __fmul_rn(c, X1));
  float srcZ = 0.0f;
  float dX = __double2float_rn(__dadd_rn((double)(col - S.half_cols), 0.5));
  dX = __fmul_rn(dX, S.pitch);
  const float dY = __fsub_rn(S.sdd, S.sod);
  float dZ = __double2float_rn(__dsub_rn((double)(S.half_rows - row), 0.5));
  dZ = __fmul_rn(dZ, S.pitch);
  const float dstX = __fadd_rn(__fadd_rn(0.0f, __fmul_rn(c, dX)), __fmul_rn(ns, dY));
  const float dstY = __fadd_rn(__fadd_rn(0.0f, __fmul_rn(s, dX)), __fmul_rn(c, dY));
  srcX = __fdiv_rn(srcX, S.voxel);
  srcZ = __fdiv_rn(srcZ, S.voxel);
  srcY = __fdiv_rn(srcY, S.voxel);
  const float dxv = __fdiv_rn(dstX, S.voxel), dyv = __fdiv_rn(dstY, S.voxel), dzv = __fdiv_rn(dZ, S.voxel);
  const double hx = S.n / 2.0, hz = S.nz / 2.0;  // NX/2.0 = NY/2.0, NZ/2.0
  sx = __double2float_rn(__dadd_rn((double)srcX, hx));
  sy = __double2float_rn(__dadd_rn((double)srcY, hx));
  sz = __double2float_rn(__dadd_rn((double)srcZ, hz));
  dx = __double2float_rn(__dadd_rn((double)dxv, hx));
  dy = __double2float_rn(__dadd_rn((double)dyv, hx));
  dz = __double2float_rn(__dadd_rn((double)dzv, hz));
}

// LAMBDA_X/Y/Z of tracing.cpp:101-103: L*((float)i - s)/(d - s)
__device__ __forceinline__ float lam_at(float i, float s, float d, float L) {
  return __fdiv_rn(__fmul_rn(L, __fsub_rn(i, s)), __fsub_rn(d, s));
}

// tracing.cpp:131-265: entry plane, first voxel and first crossings
__device__ __forceinline__ ConeWalk cone_start(int nx, int ny, int nz, float sx, float sy, float sz, float dx,
                                               float dy, float dz) {
  ConeWalk w;
  int index = 0;
  const float ray_x = __fsub_rn(dx, sx), ray_y = __fsub_rn(dy, sy), ray_z = __fsub_rn(dz, sz);
  const float L =
      __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ray_x, ray_x), __fmul_rn(ray_y, ray_y)), __fmul_rn(ray_z, ray_z)));
  float lambda_min = 0.0f, lambda_max = L;
  w.sx = (ray_x > 0) ? 1 : -1;
  w.sy = (ray_y > 0) ? 1 : -1;
  w.sz = (ray_z > 0) ? 1 : -1;
  const float ax = fabsf(ray_x), ay = fabsf(ray_y), az = fabsf(ray_z);
  w.len_x = ((double)ax > 1.e-4) ? __fdiv_rn(L, ax) : 1.e6f;
  w.len_y = ((double)ay > 1.e-4) ? __fdiv_rn(L, ay) : 1.e6f;
  w.len_z = ((double)az > 1.e-4) ? __fdiv_rn(L, az) : 1.e6f;
  float l0, lN, t;
  l0 = lam_at(0.f, sx, dx, L);
  lN = lam_at((float)nx, sx, dx, L);
  t = (l0 < lN) ? l0 : lN;
  lambda_min = (lambda_min > t) ? lambda_min : t;
  if (lambda_min == t) index = 1;
  t = (l0 > lN) ? l0 : lN;
  lambda_max = (lambda_max < t) ? lambda_max : t;
  l0 = lam_at(0.f, sy, dy, L);
  lN = lam_at((float)ny, sy, dy, L);
  t = (l0 < lN) ? l0 : lN;
  lambda_min = (lambda_min > t) ? lambda_min : t;
  if (lambda_min == t) index = 2;
  t = (l0 > lN) ? l0 : lN;
  lambda_max = (lambda_max < t) ? lambda_max : t;
  l0 = lam_at(0.f, sz, dz, L);
  lN = lam_at((float)nz, sz, dz, L);
  t = (l0 < lN) ? l0 : lN;
  lambda_min = (lambda_min > t) ? lambda_min : t;
  if (lambda_min == t) index = 3;
  t = (l0 > lN) ? l0 : lN;
  lambda_max = (lambda_max < t) ? lambda_max : t;
  w.empty = !(lambda_min < lambda_max);  // tracing.cpp:214 (also false for NaN, as there)
  if (w.empty) return w;
  const float lam = lambda_min;
  auto first = [&](float s, float r) { return (int)__fadd_rn(s, __fdiv_rn(__fmul_rn(lam, r), L)); };
  auto cross = [&](int v, int sg, float s, float d, float a) {
    return ((double)a < 1.e-4) ? 1.e6f : lam_at(__fadd_rn((float)v, (float)(sg > 0)), s, d, L);
  };
  if (index == 1) {
    w.vx = (w.sx == 1) ? 0 : nx - 1;
    w.lx = __fadd_rn(lam, w.len_x);
    w.vy = first(sy, ray_y);
    w.ly = cross(w.vy, w.sy, sy, dy, ay);
    w.vz = first(sz, ray_z);
    w.lz = cross(w.vz, w.sz, sz, dz, az);
  } else if (index == 2) {
    w.vy = (w.sy == 1) ? 0 : ny - 1;
    w.ly = __fadd_rn(lam, w.len_y);
    w.vx = first(sx, ray_x);
    w.lx = cross(w.vx, w.sx, sx, dx, ax);
    w.vz = first(sz, ray_z);
    w.lz = cross(w.vz, w.sz, sz, dz, az);
  } else {
    w.vz = (w.sz == 1) ? 0 : nz - 1;
    w.lz = __fadd_rn(lam, w.len_z);
    w.vx = first(sx, ray_x);
    w.lx = cross(w.vx, w.sx, sx, dx, ax);
    w.vy = first(sy, ray_y);
    w.ly = cross(w.vy, w.sy, sy, dy, ay);
  }
  w.lam0 = lam;
  // the loop test of tracing.cpp:267, (double)lambda0 < (double)lambda_max -
  // 0.05, as one float compare: a float x is below a double D exactly when it
  // is below D rounded up to a float
  w.stop = __double2float_ru(__dsub_rn((double)lambda_max, 5.e-2));
  return w;
}

// tracing.cpp:267-306: calls f(on_grid, voxel, weight) per segment and
// end_block() after every 32 segments and once after the last (possibly empty)
// block.  Each step crosses one plane of the (nx+1) + (ny+1) + (nz+1) inside
// the clipped segment, so the walk ends within nx + ny + nz + 3 steps; the
// block bound is only a guard.  Idx is the voxel index type: 32-bit when
// every index the walk can form fits (cone_index32).
// xst / yst: the index strides of x and y (ny and 1 in the volume's layout;
// 1 and nx for an x-contiguous copy), z slices of nx*ny either way.
template <typename Idx, typename F, typename B>
__device__ __forceinline__ void cone_walk_strided(ConeWalk &w, int nx, int ny, int nz, Idx xst, Idx yst, F &&f,
                                                  B &&end_block) {
  const Idx nxy = (Idx)nx * ny;
  const Idx sxs = (Idx)w.sx * xst, sys = (Idx)w.sy * yst, szs = (Idx)w.sz * nxy;
  Idx addr = (Idx)w.vz * nxy + (Idx)w.vx * xst + (Idx)w.vy * yst;
  const int guard = (nx + ny + nz + 16) / 32 + 2;
  for (int blk = 0; blk < guard; blk++) {
    int j = 0;
#pragma unroll 4
    for (; j < 32; j++) {
      if (!(w.lam0 < w.stop)) break;
      const bool on =
          (unsigned)w.vx < (unsigned)nx && (unsigned)w.vy < (unsigned)ny && (unsigned)w.vz < (unsigned)nz;
      // the reference's three-way test (x if lx is the smallest or tied, else
      // y if ly <= lz, else z) as selects: neighbouring rays step
      // differently, so branches would run every path for the whole warp
      const bool bx = (w.lx <= w.ly) & (w.lx <= w.lz);
      const bool by = !bx & (w.ly <= w.lz);
      const bool bz = !bx & !by;
      const float cur = bx ? w.lx : (by ? w.ly : w.lz);
      f(on, addr, __fsub_rn(cur, w.lam0));
      w.lam0 = cur;
      const float nlx = __fadd_rn(w.lx, w.len_x), nly = __fadd_rn(w.ly, w.len_y), nlz = __fadd_rn(w.lz, w.len_z);
      w.lx = bx ? nlx : w.lx;
      w.ly = by ? nly : w.ly;
      w.lz = bz ? nlz : w.lz;
      w.vx += bx ? w.sx : 0;
      w.vy += by ? w.sy : 0;
      w.vz += bz ? w.sz : 0;
      addr += bx ? sxs : (by ? sys : szs);
    }
    end_block();
    if (j < 32) break;
  }
}

template <typename Idx, typename F, typename B>
__device__ __forceinline__ void cone_walk(ConeWalk &w, int nx, int ny, int nz, F &&f, B &&end_block) {
  cone_walk_strided<Idx>(w, nx, ny, nz, (Idx)ny, (Idx)1, f, end_block);
}

// 32-bit voxel indices hold every index a walk can form (each coordinate one
// step outside the grid at most)
__host__ __device__ __forceinline__ bool cone_index32(int n, int nz) {
  return (int64_t)(nz + 2) * n * n < (int64_t)1 << 31;
}

__device__ __forceinline__ ConeWalk cone_ray(const ScanDev &S, int64_t ray) {
  const int per_view = S.ndx * S.ndy;
  const int view = (int)(ray / per_view), rem = (int)(ray % per_view);
  float sx, sy, sz, dx, dy, dz;
  cone_endpoints(S, view, rem / S.ndy, rem % S.ndy, sx, sy, sz, dx, dy, dz);
  return cone_start(S.n, S.n, S.nz, sx, sy, sz, dx, dy, dz);
}

constexpr int kConeThreads = 128;

// Order in which the projectors take rays: bands of kConeBandRows detector
// rows, every view of a band before the next band, then rows, then columns
// (a warp's rays are neighbours in a row).  The rays of one band only cross a
// slab of the volume a few dozen slices thick (the cone angle is small), so
// the views in flight share that slab in L2 instead of each view sweeping the
// whole volume through it.  0 = view-major order (bins in sinogram order).
constexpr int kConeBandRows = 16;

// the sinogram bin ([view][row][col]) of work item i
__device__ __forceinline__ int64_t cone_bin_of(const ScanDev &S, int64_t i) {
  if (kConeBandRows == 0) return i;
  const int64_t full = (int64_t)kConeBandRows * S.ndy * S.nviews;  // items of one full band
  const int64_t b = i / full, off = i - b * full;
  const int rows_b = min(kConeBandRows, S.ndx - (int)b * kConeBandRows);
  const int64_t per_view = (int64_t)rows_b * S.ndy;
  const int view = (int)(off / per_view), r2 = (int)(off - view * per_view);
  const int row = (int)b * kConeBandRows + r2 / S.ndy, col = r2 % S.ndy;
  return ((int64_t)view * S.ndx + row) * S.ndy + col;
}

// the bin of work item i of the back projection's chunk of views [v0, v0+nv):
// the same band order over those views only
__device__ __forceinline__ int64_t cone_bin_of_chunk(const ScanDev &S, int64_t i, int v0, int nv) {
  const int64_t full = (int64_t)kConeBandRows * S.ndy * nv;
  const int64_t b = i / full, off = i - b * full;
  const int rows_b = min(kConeBandRows, S.ndx - (int)b * kConeBandRows);
  const int64_t per_view = (int64_t)rows_b * S.ndy;
  const int view = v0 + (int)(off / per_view), r2 = (int)(off - (view - v0) * per_view);
  const int row = (int)b * kConeBandRows + r2 / S.ndy, col = r2 % S.ndy;
  return ((int64_t)view * S.ndx + row) * S.ndy + col;
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// at least ten CTAs per SM (C4 forward: 153 ms against 156 ms with the
// compiler's own register choice, 155 ms with twelve, 168 ms with sixteen)
__global__ void __launch_bounds__(kConeThreads, 10) cone_fp_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = blockIdx.x - cta0;
  const int64_t item = (int64_t)local_cta * kConeThreads + threadIdx.x;
  FF s0 = ff_zero();
  if (item < S.nbins) {
    const int64_t ray = cone_bin_of(S, item);
    const float *__restrict__ vol = S.buf[L.in_buf];
    ConeWalk w = cone_ray(S, ray);
    float acc = 0.f, comp = 0.f, part = 0.f;
    // FP32 products summed per 32 segments, the partial sums Kahan-folded
    auto seg = [&](bool on, auto addr, float wt) {
      float val = 0.f;
      if (on) val = __ldg(vol + addr);  // off-grid voxels are never read
      part = fmaf(wt, val, part);
    };
    auto fold = [&]() {
      kahan_add(acc, comp, part);
      part = 0.f;
    };
    if (w.empty)
      fold();
    else if (cone_index32(S.n, S.nz))
      cone_walk<int>(w, S.n, S.n, S.nz, seg, fold);
    else
      cone_walk<int64_t>(w, S.n, S.n, S.nz, seg, fold);
    fp_epilogue(S, L, (int)ray, acc - comp, s0);
  }
  if (stage_reduces(L.stage)) {
    FF v[1] = {s0};
    reduce_and_finalize<1>(S, L, v, local_cta, ncta);
  }
}

// ---------------------------------------------------------------------------
// back
// ---------------------------------------------------------------------------
constexpr int kConeTermBits = 22;  // |term| < 2^22, so one FFMA rounds it

// fixed-point exponent from the scan's largest |r| (the 64 partial maxima of
// sino_absmax_kernel); every CTA of both passes computes the same value.  Must
// be reached by the whole CTA.
__device__ __forceinline__ int cone_bp_sexp(const ScanDev &S) {
  static_assert(kBpMaxParts == 64, "two partial maxima per lane");
  __shared__ int s_sexp;
  if (threadIdx.x < 32) {
    float m = fmaxf(S.bpmax[threadIdx.x], S.bpmax[threadIdx.x + 32]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    // a segment is at most sqrt(3) voxels long: |w r| < 2 m
    int ex = 0;
    frexpf(fmaxf(2.f * m, 1e-30f), &ex);
    if (threadIdx.x == 0) s_sexp = min(kConeTermBits - ex, 120);
  }
  __syncthreads();
  return s_sexp;
}

// v added to *p as a reduction (PTX red: no value comes back, so the walk
// never waits on it)
__device__ __forceinline__ void red_add(int *p, int v) {
  asm volatile("red.relaxed.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One chunk of views (L.chunk; S.bp_vchunk views each), rays in band order,
// a grid-stride loop over the chunk's rays.  Each term w*r is rounded to an
// integer below 2^22 (one FFMA, magic-number rounding) and added with a 32-bit
// reduction (red_add) into the chunk's accumulator; the chunk is short enough that no
// voxel's sum can leave 32 bits (cone_bp_views_per_chunk), and the fold pass
// moves it into the exact 64-bit sum before the next chunk.  Integer sums do
// not depend on order, so the result is deterministic, and bitwise the same
// as adding every term into 64 bits.
__global__ void __launch_bounds__(kConeThreads) cone_bp_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int v0 = L.chunk * S.bp_vchunk;
  if (v0 >= S.nviews) return;  // a scan with fewer chunks than the launch's largest
  const int nv = min(S.bp_vchunk, S.nviews - v0);
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = blockIdx.x - cta0;
  const int sexp = cone_bp_sexp(S);
  const float scale = ldexpf(1.f, sexp);
  const int64_t nitems = (int64_t)nv * S.ndets;
  constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
  constexpr int kMagicBits = 0x4B400000;
  auto none = [] {};
  for (int64_t item = (int64_t)local_cta * kConeThreads + threadIdx.x; item < nitems;
       item += (int64_t)ncta * kConeThreads) {
    const int64_t ray = cone_bin_of_chunk(S, item, v0, nv);
    const float r = S.buf[L.in_buf][ray];
    if (r == 0.f) continue;
    const float rs = r * scale;
    ConeWalk w = cone_ray(S, ray);
    if (w.empty) continue;
    // a warp's rays are neighbouring detector columns of one view; they lie
    // side by side along the view's column direction (cos, sin) in (x, y).
    // Where that is closer to x, they add into the x-contiguous accumulator,
    // so the lanes of one reduction instruction share sectors
    const float2 cs = __ldg(S.cone_trig + (int)(ray / S.ndets));
    const bool xfast = fabsf(cs.x) > fabsf(cs.y);
    int *acc = xfast ? S.bp_acc32x : S.bp_acc32;
    auto seg = [&](bool on, auto addr, float wt) {
      if (on) red_add(acc + addr, __float_as_int(fmaf(wt, rs, kMagic)) - kMagicBits);
    };
    if (cone_index32(S.n, S.nz)) {
      if (xfast) cone_walk_strided<int>(w, S.n, S.n, S.nz, 1, S.n, seg, none);
      else cone_walk<int>(w, S.n, S.n, S.nz, seg, none);
    } else {
      if (xfast) cone_walk_strided<int64_t>(w, S.n, S.n, S.nz, (int64_t)1, (int64_t)S.n, seg, none);
      else cone_walk<int64_t>(w, S.n, S.n, S.nz, seg, none);
    }
  }
}

// The chunk sums of one kPixRows x 32 tile of slice z: the volume-layout
// accumulator's at (x, y) plus the x-contiguous one's, read through a
// shared-memory transpose so both reads are coalesced; both left zero.
__device__ __forceinline__ void cone_chunk_sums(const ScanDev &S, int z, int bx, int by, int (&out)[kPixRows / 8]) {
  __shared__ int tx[32][kPixRows + 1];
  const int n = S.n, lane = threadIdx.x & 31, wrow = threadIdx.x >> 5;
  // x-contiguous copy: row y of slice z holds x = 0..n-1; lanes along x
#pragma unroll
  for (int j = 0; j < 32 / 8; j++) {
    const int yy = by + j * 8 + wrow;
    for (int xo = lane; xo < kPixRows; xo += 32) {
      const int xx = bx + xo;
      int v = 0;
      if (xx < n && yy < n && z < S.nz) {
        const int64_t i = ((int64_t)z * n + yy) * n + xx;
        v = S.bp_acc32x[i];
        if (v != 0) S.bp_acc32x[i] = 0;
      }
      tx[yy - by][xo] = v;
    }
  }
  __syncthreads();
  const int y = by + lane;
#pragma unroll
  for (int j = 0; j < kPixRows / 8; j++) {
    const int x = bx + j * 8 + wrow;
    int v = tx[lane][j * 8 + wrow];
    if (x < n && y < n && z < S.nz) {
      const int64_t i = ((int64_t)z * n + x) * n + y;
      const int a = S.bp_acc32[i];
      if (a != 0) S.bp_acc32[i] = 0;
      v += a;  // |v| < 2^31: each accumulator's chunk sum is below 2^30
    }
    out[j] = v;
  }
}

// per voxel, over the pixel-pass CTAs: the chunk's 32-bit sums into the
// 64-bit ones, leaving the 32-bit sums zero for the next chunk
__global__ void __launch_bounds__(256) cone_bp_fold_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int local_cta = blockIdx.x - cta0;
  const int n = S.n, tiles_y = (n + 31) >> 5, tiles = ((n + kPixRows - 1) / kPixRows) * tiles_y;
  const int z = local_cta / tiles, t = local_cta % tiles;
  const int y = (t % tiles_y) * 32 + (threadIdx.x & 31);
  int part[kPixRows / 8];
  cone_chunk_sums(S, z, (t / tiles_y) * kPixRows, (t % tiles_y) * 32, part);
#pragma unroll
  for (int j = 0; j < kPixRows / 8; j++) {
    const int x = (t / tiles_y) * kPixRows + j * 8 + (threadIdx.x >> 5);
    if (x < n && y < n && z < S.nz && part[j] != 0) {
      const int64_t i = ((int64_t)z * n + x) * n + y;
      S.bp_acc[i] += (unsigned long long)(long long)part[j];
    }
  }
}

// per voxel, over the pixel-pass CTAs (kPixRows x 32 tiles of each slice,
// each thread kPixRows / 8 rows 8 apart): the last chunk's sums added to the
// 64-bit ones, converted, the epilogue run, and both accumulators left zero
__global__ void __launch_bounds__(256) cone_bp_finish_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = blockIdx.x - cta0;
  const int n = S.n, tiles_y = (n + 31) >> 5, tiles = ((n + kPixRows - 1) / kPixRows) * tiles_y;
  const int z = local_cta / tiles, t = local_cta % tiles;
  const int y = (t % tiles_y) * 32 + (threadIdx.x & 31);
  const int sexp = cone_bp_sexp(S);
  int part[kPixRows / 8];
  cone_chunk_sums(S, z, (t / tiles_y) * kPixRows, (t % tiles_y) * 32, part);
  FF s0 = ff_zero();
#pragma unroll
  for (int j = 0; j < kPixRows / 8; j++) {
    const int x = (t / tiles_y) * kPixRows + j * 8 + (threadIdx.x >> 5);
    if (x < n && y < n && z < S.nz) {
      const int64_t i = ((int64_t)z * n + x) * n + y;
      const long long total = (long long)S.bp_acc[i] + part[j];
      S.bp_acc[i] = 0ull;
      const float val = (float)((double)total * ldexp(1.0, -sexp));
      bp_epilogue(S, L, z, x, y, val, s0);
    }
  }
  if (stage_reduces(L.stage)) {
    FF v[1] = {s0};
    reduce_and_finalize<1>(S, L, v, local_cta, ncta);
  }
}

// ---------------------------------------------------------------------------
// plan support: segment count, one traced ray
// ---------------------------------------------------------------------------
__global__ void cone_count_kernel(const ScanDev S, unsigned long long *segs, unsigned long long *offgrid,
                                  int *maxseg) {
  const int64_t ray = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned long long cnt = 0, off = 0;
  if (ray < S.nbins) {
    ConeWalk w = cone_ray(S, ray);
    if (!w.empty)
      cone_walk<int64_t>(
          w, S.n, S.n, S.nz,
          [&](bool on, int64_t, float) {
            cnt++;
            off += on ? 0 : 1;
          },
          [] {});
  }
  const unsigned mine = (unsigned)cnt;
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    off += __shfl_xor_sync(0xffffffffu, off, o);
  }
  const unsigned mx = __reduce_max_sync(0xffffffffu, mine);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(segs, cnt);
    atomicAdd(offgrid, off);
    atomicMax(maxseg, (int)mx);
  }
}

__global__ void cone_trace_one_kernel(const ScanDev S, int64_t ray, int cap, int *pix, float *wgt, int *count) {
  ConeWalk w = cone_ray(S, ray);
  int k = 0;
  if (!w.empty)
    cone_walk<int64_t>(
        w, S.n, S.n, S.nz,
        [&](bool, int64_t addr, float wt) {
          if (k < cap) {
            pix[k] = (int)addr;
            wgt[k] = wt;
          }
          k++;
        },
        [] {});
  *count = k;
}

int cone_ctas(const ScanDev &S) { return (int)(((int64_t)S.nbins + kConeThreads - 1) / kConeThreads); }

// CTAs of one back-projection chunk (the rays of bp_vchunk views, one per thread)
int cone_bp_ctas(const ScanDev &S) {
  const int64_t items = (int64_t)std::min(S.nviews, std::max(1, S.bp_vchunk)) * S.ndets;
  return (int)((items + kConeThreads - 1) / kConeThreads);
}

// Views per back-projection chunk.  All rays of a view leave the source point;
// the detector cell centres lie on a grid of pitch p.  A voxel of edge a whose
// nearest point is at depth d >= dmin from the source (dmin = SOD minus the
// volume's radius about the rotation axis) casts a shadow of diameter at most
// sqrt(3) a (SDD / dmin) (1 + tan_max) on the detector, tan_max bounding the
// ratio of a point's distance from the central axis to its depth; at most
// (floor(diameter / p) + 1)^2 cell centres fall in it, so that many rays per
// view cross the voxel, each once.  Terms are below 2^22, so a 32-bit sum
// stays exact for 2^9 terms; chunks are sized for half that.
int cone_bp_views_per_chunk(const at_cone_geometry &g) {
  const double a = g.voxel_mm;
  const double R = 0.5 * a * std::sqrt((double)g.nx * g.nx + (double)g.ny * g.ny);
  const double Z = 0.5 * a * g.nz;
  const double dmin = (double)g.sod_mm - R;
  if (!(dmin > 0.0)) return 1;
  const double tan_max = std::sqrt(R * R + Z * Z) / dmin;
  const double diam = std::sqrt(3.0) * a * ((double)g.sdd_mm / dmin) * (1.0 + tan_max);
  const double per_axis = std::floor(diam / (double)g.pitch_mm) + 1.0;
  const double per_view = per_axis * per_axis;
  const double v = std::floor(256.0 / per_view);
  return (int)std::max(1.0, std::min(v, (double)g.nproj));
}

cudaError_t launch_cone_fp(const Launch &L, int nctas, cudaStream_t st) {
  cone_fp_kernel<<<nctas, kConeThreads, 0, st>>>(L);
  return cudaGetLastError();
}

// the max |r| pass has run; tracing pass over `L` (ray CTAs), then the
// finishing pass over `Lpix` (pixel-pass CTAs)
// (and L.chunks chunks of views, each folded into the 64-bit sums before the
// next; the last one is added by the finishing pass)
cudaError_t launch_cone_bp(const Launch &L, int nctas, const Launch &Lpix, int pix_nctas, cudaStream_t st) {
  const int chunks = std::max(1, L.chunks);
  for (int c = 0; c < chunks; c++) {
    Launch Lc = L;
    Lc.chunk = c;
    cone_bp_kernel<<<nctas, kConeThreads, 0, st>>>(Lc);
    if (c + 1 < chunks) cone_bp_fold_kernel<<<pix_nctas, 256, 0, st>>>(Lpix);
  }
  cone_bp_finish_kernel<<<pix_nctas, 256, 0, st>>>(Lpix);
  return cudaGetLastError();
}

// launches of one cone back projection (max |r| pass, chunks, folds, finish)
int cone_bp_launches(int chunks) { return 2 * std::max(1, chunks) + 1; }

int build_cone_plan(Plan &p, cudaStream_t st) {
  const at_cone_geometry &g = p.cone;
  p.n = g.nx;
  p.nz = g.nz;
  p.nviews = g.nproj;
  p.ndets = g.ndx * g.ndy;
  p.rays = (int64_t)p.nviews * p.ndets;
  p.cone_bp_views = cone_bp_views_per_chunk(g);
  std::vector<float2> trig(g.nproj);
  cone_trig(g, trig.data());
  AT_CUDA_TRY(cudaMalloc(&p.cone_trig_d, sizeof(float2) * g.nproj));
  p.device_bytes += sizeof(float2) * g.nproj;
  AT_CUDA_TRY(cudaMemcpyAsync(p.cone_trig_d, trig.data(), sizeof(float2) * g.nproj, cudaMemcpyHostToDevice, st));
  ScanDev S;
  fill_scan_plan(S, p);
  unsigned long long *cnt = nullptr;
  const auto free_cnt = scope_exit([&] { cudaFree(cnt); });
  AT_CUDA_TRY(cudaMalloc(&cnt, 3 * sizeof(unsigned long long)));
  AT_CUDA_TRY(cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned long long), st));
  cone_count_kernel<<<(unsigned)((p.rays + 255) / 256), 256, 0, st>>>(S, cnt, cnt + 1, (int *)(cnt + 2));
  AT_CUDA_TRY(cudaGetLastError());
  unsigned long long h[3];
  AT_CUDA_TRY(cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  p.segments = (int64_t)h[0];
  p.offgrid = (int64_t)h[1];
  p.max_segments = (int)(unsigned)(h[2] & 0xffffffffu);
  return AT_OK;
}

int cone_trace_ray(const Plan &p, int64_t ray, int32_t *h_pix, float *h_w, int32_t cap, int32_t *n_out) {
  ScanDev S;
  fill_scan_plan(S, p);
  const int dcap = std::max(cap, 1);
  int *pix = nullptr, *cnt = nullptr;
  float *wgt = nullptr;
  const auto free_temps = scope_exit([&] {
    cudaFree(pix);
    cudaFree(wgt);
    cudaFree(cnt);
  });
  AT_CUDA_TRY(cudaMalloc(&pix, sizeof(int) * dcap));
  AT_CUDA_TRY(cudaMalloc(&wgt, sizeof(float) * dcap));
  AT_CUDA_TRY(cudaMalloc(&cnt, sizeof(int)));
  cone_trace_one_kernel<<<1, 1>>>(S, ray, dcap, pix, wgt, cnt);
  AT_CUDA_TRY(cudaGetLastError());
  int n = 0;
  AT_CUDA_TRY(cudaMemcpy(&n, cnt, sizeof(int), cudaMemcpyDeviceToHost));
  const int m = std::min(n, cap);
  if (m > 0 && h_pix) AT_CUDA_TRY(cudaMemcpy(h_pix, pix, sizeof(int) * m, cudaMemcpyDeviceToHost));
  if (m > 0 && h_w) AT_CUDA_TRY(cudaMemcpy(h_w, wgt, sizeof(float) * m, cudaMemcpyDeviceToHost));
  *n_out = n;
  return AT_OK;
}

}  // namespace medimg

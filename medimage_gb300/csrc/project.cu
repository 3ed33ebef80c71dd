// project.cu -- forward (A f) and back (A^T r) projection kernels with the
// solver's fused epilogues.
//
// Fan beam, forward: each thread walks RPT adjacent rays of one view through
// the plan's decision bits (1 bit per segment, block-interleaved so a warp's
// word loads are coalesced), reads the traversed pixels through the read-only
// cache, accumulates FP32 products per 32-segment word and folds the word sums
// into a Kahan-compensated total.  The traversal (pixel sequence) is the
// reference's FP64 one (helical/rebin/src/tracing.cpp:118-146); weights are
// differences of FP32 boundary crossings.
// Fan beam, back: one CTA per 16x16 pixel tile walks the plan's (ray, tile)
// runs with the forward walk's bits and crossing formula (so A^T is the exact
// transpose of the FP32 A), accumulating in 64-bit fixed point in shared
// memory: integer sums do not depend on arrival order (deterministic).
// GoldenC: forward = one warp per traced (alpha, raynum) pair summing its 16
// tile walks into the 8 symmetric bins of proj.c:114-127; back = one thread
// per pixel over the transposed walk lists, with the 90-degree column of
// proj.c:225.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "epilogue.cuh"
#include "solver.h"

namespace medimg {


// ---------------------------------------------------------------------------
// fan-beam forward projection
// ---------------------------------------------------------------------------
// A thread walks its ray by the plan's decision bits and gathers one pixel
// per segment.  The 32 rays of a warp are neighbours in one view, so at a
// given step they lie side by side across the ray direction: a warp whose
// rays run closer to the y axis reads a transposed copy of the image (made
// just before the walk), where its pixels share sectors.
//
// A batch's scans that share one plan form a group (up to kGroupMax, listed in
// the lead scan's ScanDev).  Their input images are first interleaved into the
// lead's pack buffer (fp_pack_kernel, one float4 per pixel, row-major and
// transposed); the lead's CTAs then walk each ray once and one 16-byte gather
// per segment feeds every member, so the walk (decision bits, crossing
// arithmetic) and the gathers are shared.  Each member's sum is formed exactly
// as it would be alone, so results do not depend on the grouping or on the
// copy a warp reads.

// The members' values of element p as one T (float, float2 or float4; zeros
// for absent or finished members)
template <typename T>
__device__ __forceinline__ T pack_elem(const float *const (&src)[kGroupMax], int p) {
  float v[kGroupMax];
#pragma unroll
  for (int m = 0; m < kGroupMax; m++) v[m] = src[m] ? __ldg(src[m] + p) : 0.f;
  if constexpr (sizeof(T) == 4) return v[0];
  else if constexpr (sizeof(T) == 8) return make_float2(v[0], v[1]);
  else return make_float4(v[0], v[1], v[2], v[3]);
}

// Images of a scan (or a group) into its pack buffer, row-major and transposed,
// 32 x 32 pixels at a time through shared memory so that both copies are
// written in whole rows: tiles (local, local + ncta, ...) of the scan's CTAs.
template <typename T>
__device__ __forceinline__ void pack_image_tiles(const float *const (&src)[kGroupMax], int n, T *pk, int local,
                                                 int ncta, float4 (*raw)[33]) {
  T(*tile)[33] = reinterpret_cast<T(*)[33]>(raw);  // 32 x 33 elements of T
  const int lane = threadIdx.x & 31, row = threadIdx.x >> 5;  // 8 rows of 32 threads
  const int tiles_y = (n + 31) / 32;
  const size_t npix = (size_t)n * n;
  for (int t = local; t < tiles_y * tiles_y; t += ncta) {
    const int x0 = (t / tiles_y) * 32, y0 = (t % tiles_y) * 32;
    for (int r = row; r < 32; r += 8) {
      const int x = x0 + r, y = y0 + lane;
      if (x < n && y < n) {
        const T v = pack_elem<T>(src, x * n + y);
        pk[(size_t)x * n + y] = v;
        tile[r][lane] = v;
      }
    }
    __syncthreads();
    for (int r = row; r < 32; r += 8) {
      const int y = y0 + r, x = x0 + lane;
      if (x < n && y < n) pk[npix + (size_t)y * n + x] = tile[lane][r];
    }
    __syncthreads();
  }
}

// Interleaves each group's projector inputs into the lead's pack buffer, one
// float2 per element for a pair, one float4 for three or four members, zeros
// for absent or finished members; images twice, row-major and transposed
// (the forward projector reads whichever puts a warp's neighbouring rays in
// fewer sectors), and for a scan alone only its image as floats, row-major and
// transposed: images (bins = 0, over the pixel-pass CTAs) before a grouped
// forward projection, sinograms (bins = 1, over the sinogram-pass CTAs) before
// a grouped back projection.
__global__ void __launch_bounds__(256) fp_pack_kernel(const Launch L, int bins) {
  const int scan = find_scan(L.prefix, L.nscans, blockIdx.x);
  const ScanDev &S = L.scans[scan];
  if (S.nmem == 0 || (S.nmem == 1 && bins)) return;  // a scan alone: its sinogram is read in place
  const float *src[kGroupMax];
  bool any = false;
#pragma unroll
  for (int m = 0; m < kGroupMax; m++) {
    const ScanDev &Mm = L.scans[S.mem[m < S.nmem ? m : 0]];
    src[m] = (m < S.nmem && flow_active(Mm, L.flow)) ? Mm.buf[L.in_buf] : nullptr;
    any |= src[m] != nullptr;
  }
  if (!any) return;
  const int cta0 = __ldg(L.prefix + scan), ncta = __ldg(L.prefix + scan + 1) - cta0;
  const int local = blockIdx.x - cta0;
  if (!bins) {
    __shared__ float4 raw[32][33];
    if (S.nmem == 1) pack_image_tiles<float>(src, S.n, reinterpret_cast<float *>(S.pack), local, ncta, raw);
    else if (S.nmem == 2) pack_image_tiles<float2>(src, S.n, reinterpret_cast<float2 *>(S.pack), local, ncta, raw);
    else pack_image_tiles<float4>(src, S.n, S.pack, local, ncta, raw);
    return;
  }
  for (int p = local * blockDim.x + threadIdx.x; p < S.nbins; p += ncta * blockDim.x) {
    if (S.nmem == 2) reinterpret_cast<float2 *>(S.pack)[p] = pack_elem<float2>(src, p);
    else S.pack[p] = pack_elem<float4>(src, p);
  }
}

// RPT rays per thread; G scans per walk: 1, or a group's 2 or 4 members
// gathered as one float2 / float4 (three members take the float4 form).
// `unit` is the CTA's index in the ordinary launch (blockIdx.x), or the work
// unit a persistent CTA pulled from the queue.
template <int RPT, int G>
__device__ __forceinline__ void fan_fp_body(const Launch &L, const int unit) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, unit) : 0;
  const ScanDev &S = scan_of(L, scan);
  const int nm = L.scans ? S.nmem : 1;
  const ScanDev *M[G];
  bool act[G];
  bool any = false;
#pragma unroll
  for (int m = 0; m < G; m++) {
    M[m] = L.scans ? &L.scans[S.mem[m < nm ? m : 0]] : &L.single;
    act[m] = m < nm && flow_active(*M[m], L.flow);
    any |= act[m];
  }
  if (!any) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = unit - cta0;
  const int lane = threadIdx.x & 31;
  const int lw = local_cta * (int)(blockDim.x >> 5) + (threadIdx.x >> 5);
  const int nblk = S.nviews * S.nbpv;
  int view, in_blk, blk;
  bool warp_live;
  if constexpr (RPT == 1) {
    // A warp walks 16 adjacent rays of each of two neighbouring views: rays
    // of the same detector in the two views nearly coincide, so at any step
    // the warp's pixels span half the width across the rays that 32 rays of
    // one view would (measured on the C2 traversal: 28 % fewer cache lines
    // per gather for floats, 20 % for float4).  A CTA's four warps cover 64
    // rays of each view.
    const int per_pair = S.nbpv * 8;  // warps per view pair
    const int vp = lw / per_pair, rem = lw - vp * per_pair;
    view = 2 * vp + (lane >> 4);
    in_blk = (rem & 7) * 16 + (lane & 15);
    blk = min(view * S.nbpv + (rem >> 3), nblk - 1);  // (clamped for a missing second view)
    warp_live = 2 * vp < S.nviews;
  } else {
    constexpr int kWarpsPerBlock = 4 / RPT;  // warps per 128-ray bit block
    blk = lw / kWarpsPerBlock;
    view = blk / max(1, S.nbpv);
    in_blk = (lw % kWarpsPerBlock) * 32 * RPT + lane * RPT;  // first ray of this thread within the block
    warp_live = blk < nblk;
  }
  FF s0[G];
#pragma unroll
  for (int m = 0; m < G; m++) s0[m] = ff_zero();
  if (warp_live) {
    const bool view_ok = view < S.nviews;
    const int det0 = (blk % S.nbpv) * kRayBlock + in_blk;
    static_assert(G == 1 || G == 2 || G == 4, "members are gathered as one float, float2 or float4");
    const float *__restrict__ img = M[0]->buf[L.in_buf];  // (or its transposed copy, below)
    const float4 *__restrict__ pack = S.pack;
    const float2 *__restrict__ pack2 = reinterpret_cast<const float2 *>(S.pack);
    const unsigned npix = (unsigned)S.npix;
    int idx[RPT], stx[RPT], sty[RPT], nseg[RPT];
    float ax[RPT], ay[RPT], lx[RPT], ly[RPT], cx[RPT], cy[RPT], prev[RPT], acc[RPT][G], comp[RPT][G];
    int my_max = 0;
#pragma unroll
    for (int r = 0; r < RPT; r++) {
      const int det = det0 + r;
      nseg[r] = 0;
      idx[r] = 0;
      stx[r] = sty[r] = 0;
      ax[r] = ay[r] = lx[r] = ly[r] = 0.f;
      if (view_ok && det < S.ndets) {
        const uint4 *hp = reinterpret_cast<const uint4 *>(S.rays + (size_t)view * S.ndets + det);
        const uint4 h0 = __ldg(hp), h1 = __ldg(hp + 1);
        idx[r] = (int)h0.x;
        nseg[r] = (int)h0.y;
        stx[r] = (h0.w & 1u) ? S.n : -S.n;
        sty[r] = (h0.w & 2u) ? 1 : -1;
        ax[r] = __uint_as_float(h1.x);
        ay[r] = __uint_as_float(h1.y);
        lx[r] = __uint_as_float(h1.z);
        ly[r] = __uint_as_float(h1.w);
      }
      cx[r] = cy[r] = prev[r] = 0.f;
#pragma unroll
      for (int m = 0; m < G; m++) acc[r][m] = comp[r][m] = 0.f;
      my_max = max(my_max, nseg[r]);
    }
    // With a transposed copy of the inputs (L.tr: the scan's pack buffer), a
    // warp whose rays run closer to the y axis gathers from it: its rays then
    // lie side by side along x, and in the transposed copy neighbouring x share
    // a sector (the row-major copy serves rays closer to the x axis).  Blocks
    // with rays off the grid keep the row-major copy, whose index checks they
    // rely on.
    const float4 *__restrict__ pk4 = pack;
    const float2 *__restrict__ pk2 = pack2;
    // (blocks of both views for the paired layout)
    const bool off_any = __any_sync(0xffffffffu, __ldg(S.blk_off + blk) != 0);
    if (L.tr) {
      const float lx0 = __shfl_sync(0xffffffffu, lx[0], 0), ly0 = __shfl_sync(0xffffffffu, ly[0], 0);
      if (!off_any && lx0 > ly0) {
        pk4 += npix;
        pk2 += npix;
        if constexpr (G == 1) img = reinterpret_cast<const float *>(S.pack) + npix;
#pragma unroll
        for (int r = 0; r < RPT; r++) {
          if (nseg[r] == 0) continue;
          const int xy = __ldg(&S.rays[(size_t)view * S.ndets + det0 + r].xy0);
          const int x0 = xy & 0xffff, y0 = xy >> 16;
          idx[r] = y0 * S.n + x0;
          const int sx = stx[r] > 0 ? 1 : -1, sy = sty[r] > 0 ? S.n : -S.n;
          stx[r] = sx;
          sty[r] = sy;
        }
      }
    }
    // warp-uniform trip count, and the words that are full for every ray
    int my_min = nseg[0];
#pragma unroll
    for (int r = 1; r < RPT; r++) my_min = min(my_min, nseg[r]);
    const int nwords = ((int)__reduce_max_sync(0xffffffffu, (unsigned)my_max) + 31) >> 5;
    // blocks holding a ray that leaves the grid take the checked path throughout
    const int wfull = off_any ? 0 : (int)(__reduce_min_sync(0xffffffffu, (unsigned)my_min) >> 5);
    const uint32_t *wp = S.bits + __ldg(S.blk_word + blk) + in_blk;
    // a lane reads only its own ray's words: with two views a warp spans two
    // blocks, whose word counts differ
    const int my_words = (my_max + 31) >> 5;
    auto load_bits = [&](int w, uint32_t(&bw)[RPT]) {
      if constexpr (RPT == 4) {
        const uint4 t = __ldg(reinterpret_cast<const uint4 *>(wp + (size_t)w * kRayBlock));
        bw[0] = t.x;
        bw[1] = t.y;
        bw[2] = t.z;
        bw[3] = t.w;
      } else if constexpr (RPT == 2) {
        const uint2 t = __ldg(reinterpret_cast<const uint2 *>(wp + (size_t)w * kRayBlock));
        bw[0] = t.x;
        bw[1] = t.y;
      } else {
        bw[0] = w < my_words ? __ldg(wp + (size_t)w * kRayBlock) : 0u;
      }
    };
    for (int w = 0; w < nwords; w++) {
      uint32_t bw[RPT];
      load_bits(w, bw);
      float part[RPT][G];
#pragma unroll
      for (int r = 0; r < RPT; r++)
#pragma unroll
        for (int m = 0; m < G; m++) part[r][m] = 0.f;
      const int base = w << 5;
      if (w < wfull) {
        // every ray of the warp has 32 segments in this word and none of them
        // leaves the grid: no per-segment checks
#pragma unroll
        for (int b = 0; b < 32; b++) {
#pragma unroll
          for (int r = 0; r < RPT; r++) {
            const bool bx = (bw[r] >> b) & 1u;
            const float nx = fmaf(cx[r], lx[r], ax[r]);
            const float ny = fmaf(cy[r], ly[r], ay[r]);
            const float cur = bx ? nx : ny;
            const float wt = cur - prev[r];
            prev[r] = cur;
            if constexpr (G == 1) {
              part[r][0] = fmaf(wt, __ldg(img + idx[r]), part[r][0]);
            } else if constexpr (G == 2) {
              const float2 v = __ldg(pk2 + idx[r]);
              part[r][0] = fmaf(wt, v.x, part[r][0]);
              part[r][1] = fmaf(wt, v.y, part[r][1]);
            } else {
              const float4 v = __ldg(pk4 + idx[r]);
              part[r][0] = fmaf(wt, v.x, part[r][0]);
              part[r][1] = fmaf(wt, v.y, part[r][1]);
              part[r][2] = fmaf(wt, v.z, part[r][2]);
              part[r][3] = fmaf(wt, v.w, part[r][3]);
            }
            idx[r] += bx ? stx[r] : sty[r];
            cx[r] += bx ? 1.f : 0.f;
            cy[r] += bx ? 0.f : 1.f;
          }
        }
      } else {
#pragma unroll 8
        for (int b = 0; b < 32; b++) {
#pragma unroll
          for (int r = 0; r < RPT; r++) {
            const bool bx = (bw[r] >> b) & 1u;
            const float nx = fmaf(cx[r], lx[r], ax[r]);
            const float ny = fmaf(cy[r], ly[r], ay[r]);
            const float cur = bx ? nx : ny;
            const float wt = cur - prev[r];
            prev[r] = cur;
            const bool on = (base + b) < nseg[r] && (unsigned)idx[r] < npix;
            if constexpr (G == 1) {
              float val = 0.f;
              if (on) val = __ldg(img + idx[r]);
              part[r][0] = fmaf(wt, val, part[r][0]);
            } else if constexpr (G == 2) {
              float2 v = make_float2(0.f, 0.f);
              if (on) v = __ldg(pk2 + idx[r]);
              part[r][0] = fmaf(wt, v.x, part[r][0]);
              part[r][1] = fmaf(wt, v.y, part[r][1]);
            } else {
              float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
              if (on) v = __ldg(pk4 + idx[r]);
              part[r][0] = fmaf(wt, v.x, part[r][0]);
              part[r][1] = fmaf(wt, v.y, part[r][1]);
              part[r][2] = fmaf(wt, v.z, part[r][2]);
              part[r][3] = fmaf(wt, v.w, part[r][3]);
            }
            idx[r] += bx ? stx[r] : sty[r];
            cx[r] += bx ? 1.f : 0.f;
            cy[r] += bx ? 0.f : 1.f;
          }
        }
      }
      // fold only words that hold segments of this ray, so the result does not
      // depend on how many rays share the warp's trip count
#pragma unroll
      for (int r = 0; r < RPT; r++)
        if (base < nseg[r])
#pragma unroll
          for (int m = 0; m < G; m++) kahan_add(acc[r][m], comp[r][m], part[r][m]);
    }
    const int row0 = view * S.ndets;
#pragma unroll
    for (int r = 0; r < RPT; r++) {
      const int det = det0 + r;
      if (view_ok && det < S.ndets)
#pragma unroll
        for (int m = 0; m < G; m++)
          if (act[m]) fp_epilogue(*M[m], L, row0 + det, acc[r][m] - comp[r][m], s0[m]);
    }
  }
  if (stage_reduces(L.stage)) {
    if constexpr (G == 1) {
      reduce_and_finalize<1>(*M[0], L, s0, local_cta, ncta);
    } else {
      unsigned mask = 0;
#pragma unroll
      for (int m = 0; m < G; m++) mask |= act[m] ? 1u << m : 0u;
      reduce_and_finalize_group<G>(M, mask, L, s0, local_cta, ncta);
    }
  }
}

template <int RPT, int G>
__global__ void __launch_bounds__(128) fan_fp_kernel(const Launch L) {
  fan_fp_body<RPT, G>(L, blockIdx.x);
}
// The grouped walk of four members with at least seven CTAs per SM (up to 73
// registers): C2, 16 slices per step, 4.09 slices/s against 4.02 with the
// compiler's own choice (64 registers and a spill) or eight CTAs, 4.05 with
// six, 4.01 with five.
template <>
__global__ void __launch_bounds__(128, 7) fan_fp_kernel<1, 4>(const Launch L) {
  fan_fp_body<1, 4>(L, blockIdx.x);
}

// the same work from a queue, over a grid of resident CTAs
template <int RPT, int G>
__global__ void __launch_bounds__(128) fan_fp_queue_kernel(const Launch L) {
  persistent_loop(L, [&](int unit) { fan_fp_body<RPT, G>(L, unit); });
}


// ---------------------------------------------------------------------------
// fan-beam back projection (gather over tile runs)
// ---------------------------------------------------------------------------
// CTA = one 16x16 pixel tile, 256 threads.  The plan lists every (ray, tile)
// run of the traversal that crosses the tile, longest first; warps take 32
// runs at a time and walk them with the forward walk's decision bits and
// crossing formula, so each segment gets the forward projector's weight
// bit-for-bit.  Runs are grouped in blocks of 64 views.  Each contribution w*r
// is scaled to an integer (a power of two per scan, from the largest |r| of
// its sinogram, sized so that one view block's contributions to a pixel cannot
// overflow 32 bits) and added to a shared-memory 32-bit accumulator; after
// each view block every thread folds its pixel into an exact 64-bit register
// sum.  A tile's view blocks may be split over several CTAs (load balance when
// a launch has few tiles); their 64-bit sums add exactly in global memory.
// Integer addition is associative, so the result does not depend on the order
// in which lanes, warps or views arrive (deterministic, no float atomics).
// Scans of a batch that share the plan are back-projected together (up to
// kGroupMax, listed in the lead scan; their residuals interleaved by
// fp_pack_kernel): each run is loaded and walked once and its weights go to
// every member's accumulator, each with the member's own residual and scale,
// so each member's integer sum is exactly the one it gets alone.
// Lanes of a warp that add to the same pixel in one instruction serialise, and
// a warp's runs (similar lengths through one tile, from nearby views) often
// meet: each member therefore keeps C accumulator copies, lane l adding to copy
// l % C, with copies 32/C banks apart.
constexpr int kBpPitch = kBpTile + 1;  // padded row pitch of the accumulator
constexpr int kBpAccWords = kBpTile * kBpPitch;
constexpr int kBpCopies1 = 4;  // copies, single-scan launches (C2: 1 copy 0.33 ms, 4 copies 0.275 ms)
constexpr int kBpCopiesG = 8;  // copies per member, grouped launches (four slices: 2 copies 0.90 ms, 4 0.785, 8 0.764;
                                // sixteen slices: 8 copies 2.52 ms, 4 copies at five or six CTAs per SM 2.70-2.72)
template <int C>
constexpr int bp_copy_stride() {
  return kBpAccWords + ((32 / C - kBpAccWords % 32) % 32 + 32) % 32;
}

// max |r| of each scan's input sinogram, in kBpMaxParts partial maxima
__global__ void __launch_bounds__(256) sino_absmax_kernel(const Launch L) {
  const int scan = blockIdx.x / kBpMaxParts, part = blockIdx.x % kBpMaxParts;
  const ScanDev &S = scan_of(L, L.scans ? scan : 0);
  if (!flow_active(S, L.flow)) return;
  const float *__restrict__ sino = S.buf[L.in_buf];
  float m = 0.f;
  for (int i = part * blockDim.x + threadIdx.x; i < S.nbins; i += kBpMaxParts * blockDim.x)
    m = fmaxf(m, fabsf(__ldg(sino + i)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ float wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, wm[w]);
    S.bpmax[part] = m;
  }
}

// v added to the shared-memory word *p as a reduction (PTX red: no value
// comes back, so the walk never waits on it)
__device__ __forceinline__ void red_shared_add(int *p, int v) {
  asm volatile("red.shared.add.s32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}

// The residuals of bin for the G members: one float, or the group's
// interleaved float2 / float4.
template <int G>
__device__ __forceinline__ void bp_load_r(const float *__restrict__ sino, const float4 *__restrict__ spack,
                                          unsigned bin, float (&r)[G]) {
  if constexpr (G == 1) {
    r[0] = __ldg(sino + bin);
  } else if constexpr (G == 2) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(spack) + bin);
    r[0] = v.x;
    r[1] = v.y;
  } else {
    static_assert(G == 4, "members are read as one float, float2 or float4");
    const float4 v = __ldg(spack + bin);
    r[0] = v.x;
    r[1] = v.y;
    r[2] = v.z;
    r[3] = v.w;
  }
}

// w*r*scale + 1.5*2^23 rounds w*r*scale to an integer in the float's low
// mantissa bits (|w*r*scale| < 2^22), so one FFMA does the scaling and the
// round-to-nearest conversion
constexpr float kBpMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kBpMagicBits = 0x4B400000;

// bytes at p (16-byte aligned, a multiple of 16) fetched into L2 ahead of use
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Back projection from the plan's pixel table: thread (warp, lane) owns pixel
// ((warp/2)*4 + lane/8, (warp%2)*8 + lane%8) of the tile and gathers, view by
// view, the terms of the rays that cross it, in the same fixed point as the
// tile-run walk (32-bit sums per view block, folded into 64 bits).  Each warp
// reads its own stream (the table's words and weights of its 32 pixels, view
// after view); one lane asks L2 for the stream's chunks of kPtChunk views two
// chunks ahead, so the loads of a view wait on L2, not on HBM.  Returns the
// sums in the tile-run mapping (thread x*16 + y), through shared memory.
template <int G>
__device__ __forceinline__ void bp_table_sums(const ScanDev &S, const float *__restrict__ sino,
                                              const float4 *__restrict__ spack, int tile, int vb0, int vb1,
                                              const float (&scale)[G], const bool (&use)[G], long long (&total)[G],
                                              long long *xch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t stream = (size_t)tile * 8 + warp;
  const int nch = (S.nviews + kPtChunk - 1) / kPtChunk;
  const uint32_t *__restrict__ meta0 = S.pt_meta + stream * (size_t)S.nviews * 32;
  const uint32_t *__restrict__ meta = meta0 + lane;
  const int64_t *__restrict__ woff = S.pt_woff + stream * (size_t)(nch + 1);
  const int ch_end = (min(S.nviews, vb1 * kBpViewBlock) + kPtChunk - 1) / kPtChunk;
  auto prefetch_chunk = [&](int c) {
    if (lane == 0 && c < ch_end) {
      const int cv0 = c * kPtChunk, cv1 = min(S.nviews, cv0 + kPtChunk);
      prefetch_l2(meta0 + (size_t)cv0 * 32, (unsigned)(cv1 - cv0) * 128u);
      const int64_t a = __ldg(woff + c) & ~3ll, b = (__ldg(woff + c + 1) + 3) & ~3ll;
      if (b > a) prefetch_l2(S.pt_w + a, (unsigned)(b - a) * 4u);
    }
  };
  static_assert(kBpViewBlock % kPtChunk == 0, "view blocks are whole chunks");
  prefetch_chunk(vb0 * (kBpViewBlock / kPtChunk));
  prefetch_chunk(vb0 * (kBpViewBlock / kPtChunk) + 1);
  // Views go V at a time: a lane's rays of those views are numbered as slots
  // 0..E-1 (view j's rays from p[j]), and the loads of U slots issue together,
  // so one round trip to memory serves several views.
  constexpr int V = G == 4 ? 2 : 4;
  constexpr int U = G == 4 ? 4 : 8;
  static_assert(kPtChunk % V == 0 && kBpViewBlock % V == 0, "view groups stay inside a chunk");
  for (int vb = vb0; vb < vb1; vb++) {
    const int v0 = vb * kBpViewBlock, v1 = min(S.nviews, v0 + kBpViewBlock);
    const float *__restrict__ wblk = S.pt_w + __ldg(woff + vb * (kBpViewBlock / kPtChunk));
    int wrun = 0;  // the view's first weight, from wblk
    int acc[G];
#pragma unroll
    for (int m = 0; m < G; m++) acc[m] = 0;
    uint32_t mn[V];
#pragma unroll
    for (int j = 0; j < V; j++) mn[j] = (v0 + j < v1) ? __ldg(meta + (size_t)(v0 + j) * 32) : 0u;
    for (int v = v0; v < v1; v += V) {
      if (v % kPtChunk == 0) prefetch_chunk(v / kPtChunk + 2);
      uint32_t mc[V];
#pragma unroll
      for (int j = 0; j < V; j++) {
        mc[j] = mn[j];
        mn[j] = (v + V + j < v1) ? __ldg(meta + (size_t)(v + V + j) * 32) : 0u;
      }
      // slot s of view j: weight wblk[wo[j] + s], bin bo[j] + s
      int p[V + 1], wo[V], bo[V];
      p[0] = 0;
#pragma unroll
      for (int j = 0; j < V; j++) {
        const int d0 = (int)(mc[j] & 0x7fffu), n = (int)((mc[j] >> 15) & 63u), pre = (int)(mc[j] >> 21);
        wo[j] = wrun + pre - p[j];
        bo[j] = (v + j) * S.ndets + d0 - p[j];
        p[j + 1] = p[j] + n;
        wrun += __shfl_sync(0xffffffffu, pre + n, 31);
      }
      const int E = p[V];
      const int emax = (int)__reduce_max_sync(0xffffffffu, (unsigned)E);
      for (int s0 = 0; s0 < emax; s0 += U) {
        float wt[U], r[U][G];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int sl = s0 + u;
          int a = wo[0], b = bo[0];
#pragma unroll
          for (int j = 1; j < V; j++)
            if (sl >= p[j]) {
              a = wo[j];
              b = bo[j];
            }
          wt[u] = 0.f;
#pragma unroll
          for (int m = 0; m < G; m++) r[u][m] = 0.f;
          if (sl < E) {
            wt[u] = __ldg(wblk + a + sl);
            bp_load_r<G>(sino, spack, (unsigned)(b + sl), r[u]);
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++)
          if (s0 + u < E)
#pragma unroll
            for (int m = 0; m < G; m++)
              if (use[m]) acc[m] += __float_as_int(fmaf(wt[u], r[u][m] * scale[m], kBpMagic)) - kBpMagicBits;
      }
    }
#pragma unroll
    for (int m = 0; m < G; m++) total[m] += acc[m];
  }
  const int own = (((warp >> 1) << 2) + (lane >> 3)) * kBpTile + ((warp & 1) << 3) + (lane & 7);
#pragma unroll
  for (int m = 0; m < G; m++) xch[m * 256 + own] = total[m];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < G; m++) total[m] = xch[m * 256 + threadIdx.x];
}

template <int G, int C, int kMode>
__device__ __forceinline__ void fan_bp_body(const Launch &L, const int unit) {
  constexpr int kStride = bp_copy_stride<C>();  // one copy
  constexpr int kMemStride = C * kStride;       // one member
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, unit) : 0;
  const ScanDev &S = scan_of(L, scan);
  const int nm = L.scans ? S.nmem : 1;
  const ScanDev *M[G];
  bool act[G];
  bool any = false;
#pragma unroll
  for (int m = 0; m < G; m++) {
    M[m] = L.scans ? &L.scans[S.mem[m < nm ? m : 0]] : &L.single;
    act[m] = m < nm && flow_active(*M[m], L.flow);
    any |= act[m];
  }
  if (!any) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = unit - cta0;
  const int ntiles = S.ntiles_y * S.ntiles_y;
  // CTA = (split, tile): split s walks view blocks [s*nvb/split, (s+1)*nvb/split)
  const int tile = local_cta % ntiles, split = local_cta / ntiles;
  const int vb0 = split * S.nvb / S.bp_split, vb1 = (split + 1) * S.nvb / S.bp_split;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool real = split < S.bp_split;
  // gather from the pixel table instead of walking tile runs (kMode: the
  // launch's Launch::bp_table)
  const bool table = kMode == 1 || (kMode == 2 && (S.pt_use & (nm > 1 ? 2 : 1)) != 0);
  static_assert(kMemStride >= 512, "the accumulators double as the table path's 64-bit exchange");
  __shared__ __align__(16) int acc[kMode == 1 ? G * 512 : G * kMemStride];
  __shared__ float wmax[G][8];
  __shared__ int last_split;
  if (!table)
    for (int i = threadIdx.x; i < G * kMemStride; i += blockDim.x) acc[i] = 0;
  int *const my_acc = acc + (lane % C) * kStride;
  // one scan: its sinogram; a group: the members' sinograms interleaved, one
  // float4 per bin (the lead's pack buffer)
  const float *__restrict__ sino = M[0]->buf[L.in_buf];
  const float4 *__restrict__ spack = S.pack;
  const int32_t *toff = S.tile_off + (size_t)(real ? tile : 0) * S.nvb;
  // fixed-point scale from the largest |r| of each member's sinogram (the same
  // in every split of a tile, so split sums add exactly)
#pragma unroll
  for (int m = 0; m < G; m++) {
    float mx = (act[m] && threadIdx.x < kBpMaxParts) ? M[m]->bpmax[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) wmax[m][warp] = mx;
  }
  __syncthreads();
  int sexp[G];
  float scale[G];
  bool use[G];
  bool any_use = false;
#pragma unroll
  for (int m = 0; m < G; m++) {
    float mx = wmax[m][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = fmaxf(mx, wmax[m][w]);
    // every |w r| <= 1.5 * pixel * max|r| < 2^ex; terms are scaled below
    // 2^bp_term_bits, so one view block's terms fit a 32-bit accumulator
    int ex = 0;
    frexpf(fmaxf(1.5f * S.pixel_mm * mx, 1e-30f), &ex);
    sexp[m] = min(S.bp_term_bits - ex, 120);
    scale[m] = ldexpf(1.f, sexp[m]);
    use[m] = real && act[m] && mx > 0.f;
    any_use |= use[m];
  }
  const int own = (threadIdx.x >> 4) * kBpPitch + (threadIdx.x & 15);  // this thread's pixel
  long long total[G];  // exact sums over view blocks
#pragma unroll
  for (int m = 0; m < G; m++) total[m] = 0;
  constexpr float kMagic = kBpMagic;
  constexpr int kMagicBits = kBpMagicBits;
  if (table) {
    if (any_use)
      bp_table_sums<G>(S, sino, spack, tile, vb0, vb1, scale, use, total, reinterpret_cast<long long *>(acc));
  } else if (any_use) {
    for (int vb = vb0; vb < vb1; vb++) {
      const int b0 = __ldg(toff + vb), b1 = __ldg(toff + vb + 1);
      // two-stage pipeline: the next chunk's dependent loads fly during this walk
      const uint4 kZ = make_uint4(0u, 0u, 0u, 0u);
      int c = b0 + warp * 32;
      uint4 e = (c + lane < b1) ? __ldg(S.run + c + lane) : kZ;
      uint4 h1 = __ldg(reinterpret_cast<const uint4 *>(S.rays + e.x) + 1);
      auto load_r = [&](unsigned bin, float(&r)[G]) { bp_load_r<G>(sino, spack, bin, r); };
      float r0[G];
      load_r(e.x, r0);
      for (; c < b1; c += blockDim.x) {
        const int cn = c + blockDim.x;
        const uint4 en = (cn + lane < b1) ? __ldg(S.run + cn + lane) : kZ;
        const uint4 h1n = __ldg(reinterpret_cast<const uint4 *>(S.rays + en.x) + 1);
        float rn[G], rs[G];
        load_r(en.x, rn);
#pragma unroll
        for (int m = 0; m < G; m++) rs[m] = r0[m] * scale[m];
        const bool valid = c + lane < b1;
        const int k_in = (int)(e.y & 0x3fffu), nk = valid ? (int)((e.y >> 14) & 31u) : 0;
        const int cx_in = (int)(e.y >> 19);
        const float ax = __uint_as_float(h1.x), ay = __uint_as_float(h1.y);
        const float lx = __uint_as_float(h1.z), ly = __uint_as_float(h1.w);
        uint32_t wnd = e.z;  // the run's decision bits
        float cxf = (float)cx_in, cyf = (float)(k_in - cx_in);
        float prev = 0.f;
        if (k_in > 0) prev = (e.w & 1024u) ? fmaf(cxf - 1.f, lx, ax) : fmaf(cyf - 1.f, ly, ay);
        int sidx = (int)(e.w & 15u) * kBpPitch + (int)((e.w >> 4) & 15u);
        const int dsx = (e.w & 256u) ? kBpPitch : -kBpPitch, dsy = (e.w & 512u) ? 1 : -1;
        const int steps = (int)__reduce_max_sync(0xffffffffu, (unsigned)nk);
        const int common = (int)__reduce_min_sync(0xffffffffu, (unsigned)nk);
        int t = 0;
        // steps every run of the warp has (runs are sorted longest first, so
        // most steps): no per-lane test
#pragma unroll 4
        for (; t < common; t++) {
          const bool bx = wnd & 1u;
          wnd >>= 1;
          const float nx = fmaf(cxf, lx, ax), ny = fmaf(cyf, ly, ay);
          const float cur = bx ? nx : ny;
          const float wt = cur - prev;
          prev = cur;
#pragma unroll
          for (int m = 0; m < G; m++)
            if (use[m]) red_shared_add(&my_acc[m * kMemStride + sidx], __float_as_int(fmaf(wt, rs[m], kMagic)) - kMagicBits);
          sidx += bx ? dsx : dsy;
          cxf += bx ? 1.f : 0.f;
          cyf += bx ? 0.f : 1.f;
        }
#pragma unroll 2
        for (; t < steps; t++) {
          const bool bx = wnd & 1u;
          wnd >>= 1;
          const float nx = fmaf(cxf, lx, ax), ny = fmaf(cyf, ly, ay);
          const float cur = bx ? nx : ny;
          const float wt = cur - prev;
          prev = cur;
          if (t < nk)
#pragma unroll
            for (int m = 0; m < G; m++)
              if (use[m]) red_shared_add(&my_acc[m * kMemStride + sidx], __float_as_int(fmaf(wt, rs[m], kMagic)) - kMagicBits);
          sidx += bx ? dsx : dsy;
          cxf += bx ? 1.f : 0.f;
          cyf += bx ? 0.f : 1.f;
        }
        e = en;
        h1 = h1n;
#pragma unroll
        for (int m = 0; m < G; m++) r0[m] = rn[m];
      }
      __syncthreads();
#pragma unroll
      for (int m = 0; m < G; m++)
#pragma unroll
        for (int c = 0; c < C; c++) {
          total[m] += acc[m * kMemStride + c * kStride + own];
          acc[m * kMemStride + c * kStride + own] = 0;
        }
      __syncthreads();
    }
  }
  const int x = (tile / S.ntiles_y) * kBpTile + (threadIdx.x >> 4);
  const int y = (tile % S.ntiles_y) * kBpTile + (threadIdx.x & 15);
  const bool mine = real && x < S.n && y < S.n;
  bool finish = real;
  if (S.bp_split > 1) {
    // exact integer sums meet in each member's 64-bit accumulator; the tile's
    // last split to arrive (one ticket for the group) takes the totals, leaves
    // zeros and finishes
#pragma unroll
    for (int m = 0; m < G; m++)
      if (act[m] && mine && total[m] != 0)
        atomicAdd(M[m]->bp_acc + (size_t)x * S.n + y, (unsigned long long)total[m]);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last_split = real && atomicAdd(&S.bp_cnt[tile], 1) == S.bp_split - 1;
    __syncthreads();
    finish = last_split;
    if (finish) {
      __threadfence();
#pragma unroll
      for (int m = 0; m < G; m++)
        total[m] = (act[m] && mine) ? (long long)atomicExch(M[m]->bp_acc + (size_t)x * S.n + y, 0ull) : 0;
      if (threadIdx.x == 0) S.bp_cnt[tile] = 0;
    }
  }
  FF s0[G];
#pragma unroll
  for (int m = 0; m < G; m++) {
    s0[m] = ff_zero();
    if (act[m] && finish && mine) {
      const float val = (float)((double)total[m] * ldexp(1.0, -sexp[m]));
      bp_epilogue(*M[m], L, 0, x, y, val, s0[m]);
    }
  }
  if (stage_reduces(L.stage)) {
    if constexpr (G == 1) {
      reduce_and_finalize<1>(*M[0], L, s0, local_cta, ncta);
    } else {
      unsigned mask = 0;
#pragma unroll
      for (int m = 0; m < G; m++) mask |= act[m] ? 1u << m : 0u;
      reduce_and_finalize_group<G>(M, mask, L, s0, local_cta, ncta);
    }
  }
}

template <int M>
__global__ void __launch_bounds__(256) fan_bp_kernel(const Launch L) { fan_bp_body<1, kBpCopies1, M>(L, blockIdx.x); }
// queued (persistent) launches choose per CTA
__global__ void __launch_bounds__(256) fan_bp_queue_kernel(const Launch L) {
  persistent_loop(L, [&](int unit) { fan_bp_body<1, kBpCopies1, 2>(L, unit); });
}
// four CTAs per SM (at most 64 registers; some setup state spills, and the
// walk's latency is hidden better than at three CTAs with 80: two outer
// iterations of four C2 slices 52.8 -> 51.3 ms)
// table forms: three CTAs (85 registers for the loads of several views in flight)
template <int M>
__global__ void __launch_bounds__(256, M != 0 ? 3 : 4) fan_bp_group_kernel(const Launch L) {
  fan_bp_body<kGroupMax, kBpCopiesG, M>(L, blockIdx.x);
}
__global__ void __launch_bounds__(256, 4) fan_bp_group_queue_kernel(const Launch L) {
  persistent_loop(L, [&](int unit) { fan_bp_body<kGroupMax, kBpCopiesG, 2>(L, unit); });
}
// in a batch with groups, the scans alone and the pairs
template <int M>
__device__ __forceinline__ void fan_bp_small_body(const Launch &L, int unit) {
  const ScanDev &S = L.scans[find_scan(L.prefix, L.nscans, unit)];
  if (S.nmem <= 1)
    fan_bp_body<1, kBpCopiesG, M>(L, unit);
  else
    fan_bp_body<2, kBpCopiesG, M>(L, unit);
}
// tile runs: four CTAs per SM (C3 batched: 11.84 slices/s against 11.62 with
// three, 11.70 with five); the table forms: three
template <int M>
__global__ void __launch_bounds__(256, M == 0 ? 4 : 3) fan_bp_small_kernel(const Launch L) {
  fan_bp_small_body<M>(L, blockIdx.x);
}
__global__ void __launch_bounds__(256, 3) fan_bp_small_queue_kernel(const Launch L) {
  persistent_loop(L, [&](int unit) { fan_bp_small_body<2>(L, unit); });
}

// ---------------------------------------------------------------------------
// GoldenC parallel beam
// ---------------------------------------------------------------------------
constexpr int kGcN = 512, kGcDets = 767, kGcRays = 384, kGcPairs = 45 * 384;
constexpr int kGcLast = kGcN - 1;
constexpr int kGcSpecial = 2 * kGcDets;  // bins of views 0 and 90
constexpr int kGcFpWarps = kGcPairs + kGcSpecial;

__device__ __forceinline__ int gc_sym_pix(int s, int X, int Y) {
  switch (s) {  // proj.c:114-127 image samples
    case 0: return Y * kGcN + X;
    case 1: return (kGcLast - X) * kGcN + Y;
    case 2: return (kGcLast - Y) * kGcN + (kGcLast - X);
    case 3: return X * kGcN + (kGcLast - Y);
    case 4: return X * kGcN + Y;
    case 5: return (kGcLast - Y) * kGcN + X;
    case 6: return (kGcLast - X) * kGcN + (kGcLast - Y);
    default: return Y * kGcN + (kGcLast - X);
  }
}

__device__ __forceinline__ bool gc_sym_present(int s, int a, int r) {
  return !(((s & 2) && r == 383) || (s >= 4 && a == 45));
}

__device__ __forceinline__ int gc_sym_bin(int s, int a, int r) {
  const int view = (s < 4) ? ((s & 1) ? 90 + a : a) : ((s & 1) ? 180 - a : 90 - a);
  const int det = (s & 2) ? (kGcDets - 1 - r) : r;
  return view * kGcDets + det;
}

__global__ void __launch_bounds__(128) gc_fp_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = blockIdx.x - cta0;
  const int lane = threadIdx.x & 31;
  const int gw = local_cta * 4 + (threadIdx.x >> 5);
  const float *__restrict__ img = S.buf[L.in_buf];
  FF s0 = ff_zero();
  if (gw < kGcPairs) {
    const int a = 1 + gw / kGcRays, r = gw % kGcRays;
    float acc[8];
#pragma unroll
    for (int s = 0; s < 8; s++) acc[s] = 0.f;
    const int b = __ldg(S.gc_pair_off + gw), e = __ldg(S.gc_pair_off + gw + 1);
    for (int i = b + lane; i < e; i += 32) {
      const int2 sg = __ldg(reinterpret_cast<const int2 *>(S.gc_seg) + i);
      const int X = sg.x % kGcN, Y = sg.x / kGcN;
      const float w = __int_as_float(sg.y);
#pragma unroll
      for (int s = 0; s < 8; s++) acc[s] = fmaf(__ldg(img + gc_sym_pix(s, X, Y)), w, acc[s]);
    }
#pragma unroll
    for (int s = 0; s < 8; s++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[s] += __shfl_xor_sync(0xffffffffu, acc[s], o);
#pragma unroll
    for (int s = 0; s < 8; s++)
      if (lane == s && gc_sym_present(s, a, r)) fp_epilogue(S, L, gc_sym_bin(s, a, r), acc[s], s0);
  } else if (gw < kGcFpWarps) {
    // views 0 (row sums, proj.c:17-26) and 90 (column sums at 256+ind, proj.c:27-36)
    const int q = gw - kGcPairs;
    const int view = q < kGcDets ? 0 : 90;
    const int r = q % kGcDets;
    const int ind = r - kGcDets / 2;
    float acc = 0.f;
    if (ind <= kGcN / 2 - 1 && ind >= 1 - kGcN / 2) {
      if (view == 0) {
        const float *row = img + (kGcN / 2 - 1 + ind) * kGcN;
        for (int t = lane; t < kGcN; t += 32) acc += __ldg(row + t);
      } else {
        const int col = kGcN / 2 + ind;
        for (int t = lane; t < kGcN; t += 32) acc += __ldg(img + t * kGcN + col);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) fp_epilogue(S, L, view * kGcDets + r, acc, s0);
  }
  if (stage_reduces(L.stage)) {
    FF v[1] = {s0};
    reduce_and_finalize<1>(S, L, v, local_cta, ncta);
  }
}

__global__ void __launch_bounds__(256) gc_bp_kernel(const Launch L) {
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  if (!flow_active(S, L.flow)) return;
  const int cta0 = L.scans ? __ldg(L.prefix + scan) : 0;
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - cta0 : gridDim.x;
  const int local_cta = blockIdx.x - cta0;
  const int x = (local_cta >> 4) * 8 + (threadIdx.x >> 5);  // row
  const int y = (local_cta & 15) * 32 + (threadIdx.x & 31); // column
  const float *__restrict__ sino = S.buf[L.in_buf];
  float acc = 0.f, comp = 0.f;
  // views 0 and 90 (proj.c:210-230; column 255+ind at 90 degrees)
  if (x <= kGcN - 2) acc += __ldg(sino + 0 * kGcDets + x + 128);
  if (y <= kGcN - 2) acc += __ldg(sino + 90 * kGcDets + y + 128);
#pragma unroll 1
  for (int s = 0; s < 8; s++) {
    int X, Y;  // symmetry-0 pixel whose image under s is (x, y)
    switch (s) {
      case 0: Y = x; X = y; break;
      case 1: X = kGcLast - x; Y = y; break;
      case 2: Y = kGcLast - x; X = kGcLast - y; break;
      case 3: X = x; Y = kGcLast - y; break;
      case 4: X = x; Y = y; break;
      case 5: Y = kGcLast - x; X = y; break;
      case 6: X = kGcLast - x; Y = kGcLast - y; break;
      default: Y = x; X = kGcLast - y; break;
    }
    const int p = Y * kGcN + X;
    const int b = __ldg(S.gc_pix_off + p), e = __ldg(S.gc_pix_off + p + 1);
    float part = 0.f;
    for (int i = b; i < e; i++) {
      const int2 en = __ldg(reinterpret_cast<const int2 *>(S.gc_ent) + i);
      const int a = 1 + en.x / kGcRays, r = en.x % kGcRays;
      if (!gc_sym_present(s, a, r)) continue;
      part = fmaf(__ldg(sino + gc_sym_bin(s, a, r)), __int_as_float(en.y), part);
    }
    kahan_add(acc, comp, part);
  }
  FF s0 = ff_zero();
  bp_epilogue(S, L, 0, x, y, acc - comp, s0);
  if (stage_reduces(L.stage)) {
    FF v[1] = {s0};
    reduce_and_finalize<1>(S, L, v, local_cta, ncta);
  }
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
int cone_ctas(const ScanDev &S);
cudaError_t launch_cone_fp(const Launch &L, int nctas, cudaStream_t st);
cudaError_t launch_fp_slab(const Launch &L, int G, int nctas, int threads, size_t smem, cudaStream_t st);
size_t slab_smem_bytes(int G, int rows, int wbox);
int encode_pack_tmap(CUtensorMap *out, const void *pack, int n, int G, int wbox, int rows);
cudaError_t launch_cone_bp(const Launch &L, int nctas, const Launch &Lpix, int pix_nctas, cudaStream_t st);

// CTAs of `kernel` (with `threads` threads) resident on the whole device at
// once: the grid of its persistent (queue) form
template <typename K>
int resident_ctas(K kernel, int threads) {
  int nb = 0, dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess)
    return 152;
  return std::max(1, nb * sms);
}

// launches `kernel`, or its queue form `qkernel` over the resident CTAs when
// the launch carries a work queue
template <typename K>
void launch_maybe_queued(K kernel, K qkernel, int &resident, const Launch &L, int nctas, int threads,
                         cudaStream_t st) {
  if (nctas <= 0) return;
  if (L.queue) {
    if (resident <= 0) resident = resident_ctas(qkernel, threads);
    qkernel<<<std::min(nctas, resident), threads, 0, st>>>(L);
  } else {
    kernel<<<nctas, threads, 0, st>>>(L);
  }
}

int fp_ctas(const ScanDev &S, int rpt) {
  if (S.kind == AT_GEOM_GOLDNC) return (kGcFpWarps + 3) / 4;
  if (S.kind == AT_GEOM_CONE) return cone_ctas(S);
  // one ray per thread: warps of two views (an odd view count adds a half-empty pair)
  const int views = rpt == 1 ? (S.nviews + 1) / 2 * 2 : S.nviews;
  const int warps = views * S.nbpv * (4 / rpt);
  return (warps + 3) / 4;
}

// CTAs of a grouped forward projection (one ray per thread)
int fp_group_ctas(const ScanDev &S) {
  if (S.kind != AT_GEOM_FAN && S.kind != AT_GEOM_RAYS) return 0;
  constexpr int w = kFpGroupThreads / 32;
  static_assert(kFpGroupThreads == 128, "a grouped CTA holds four warps (two views x 64 rays)");
  return ((S.nviews + 1) / 2 * 2 * S.nbpv * 4 + w - 1) / w;
}

int cone_bp_ctas(const ScanDev &S);

int bp_ctas(const ScanDev &S) {
  if (S.kind == AT_GEOM_GOLDNC) return (kGcN / 8) * (kGcN / 32);
  if (S.kind == AT_GEOM_CONE) return cone_bp_ctas(S);
  return S.ntiles_y * S.ntiles_y * std::max(1, S.bp_split);
}

// CTAs per back-projection tile for a launch over `tiles` tiles: enough for
// about four waves of six 256-thread CTAs per SM (152 SMs), at most one per
// view block.  Results do not depend on it (split sums are exact integers).
int bp_split_for(int tiles, int nvb) {
  constexpr int kTarget = 4 * 6 * 152;
  int s = (kTarget + tiles - 1) / std::max(1, tiles);
  return std::max(1, std::min({s, nvb, kBpMaxSplit}));
}

int pix_ctas(const ScanDev &S) { return ((S.n + kPixRows - 1) / kPixRows) * ((S.n + 31) / 32) * S.nz; }

cudaError_t launch_fp(const Launch &L, int kind, int rpt, int nctas, cudaStream_t st) {
  if (kind == AT_GEOM_GOLDNC) {
    gc_fp_kernel<<<nctas, 128, 0, st>>>(L);
  } else if (kind == AT_GEOM_CONE) {
    return launch_cone_fp(L, nctas, st);
  } else if (rpt == 4) {
    static int res = 0;
    launch_maybe_queued(fan_fp_kernel<4, 1>, fan_fp_queue_kernel<4, 1>, res, L, nctas, 128, st);
  } else if (rpt == 2) {
    static int res = 0;
    launch_maybe_queued(fan_fp_kernel<2, 1>, fan_fp_queue_kernel<2, 1>, res, L, nctas, 128, st);
  } else {
    static int res = 0;
    launch_maybe_queued(fan_fp_kernel<1, 1>, fan_fp_queue_kernel<1, 1>, res, L, nctas, 128, st);
  }
  return cudaGetLastError();
}

// Forward projection of a batch whose scans sharing a plan are grouped: the
// members' inputs are interleaved (over the pixel-pass CTAs of Lpix), then
// each group's rays are walked once, one ray per thread, in one launch per
// form: groups of three or four over L's CTAs, scans alone over L1's, pairs
// over L2's.  Returns the number of launches.
int launch_fp_group(const Launch &L, const Launch &Lpix, const Launch &L1, const Launch &L2, int nctas, int pix_nctas,
                    int nctas1, int nctas2, const SlabLaunch *slab, cudaStream_t st) {
  int n = 1;
  fp_pack_kernel<<<pix_nctas, 256, 0, st>>>(Lpix, 0);
  if (slab) {  // every plan of the batch has slab tables of one CTA shape
    const int G[3] = {kGroupMax, 1, 2};
    const Launch *Ls[3] = {&L, &L1, &L2};
    const int nc[3] = {nctas, nctas1, nctas2};
    for (int i = 0; i < 3; i++) {
      if (nc[i] <= 0) continue;
      const cudaError_t e = launch_fp_slab(*Ls[i], G[i], nc[i], slab->threads, slab->smem[i], st);
      if (e != cudaSuccess) return -1;
      n++;
    }
    return n;
  }
  Launch Lg = L, Lg1 = L1, Lg2 = L2;
  Lg.tr = Lg1.tr = Lg2.tr = 1;
  static int res4 = 0, res1 = 0, res2 = 0;
  launch_maybe_queued(fan_fp_kernel<1, kGroupMax>, fan_fp_queue_kernel<1, kGroupMax>, res4, Lg, nctas,
                      kFpGroupThreads, st);
  launch_maybe_queued(fan_fp_kernel<1, 1>, fan_fp_queue_kernel<1, 1>, res1, Lg1, nctas1, kFpGroupThreads, st);
  launch_maybe_queued(fan_fp_kernel<1, 2>, fan_fp_queue_kernel<1, 2>, res2, Lg2, nctas2, kFpGroupThreads, st);
  return n + (nctas > 0) + (nctas1 > 0) + (nctas2 > 0);
}

// out[p] = in[p] and out[n*n + y*n + x] = in[x*n + y] for an n x n image
// (the row-major and transposed copies the forward projectors read), through
// 32 x 32 shared-memory tiles (coalesced reads and writes)
__global__ void __launch_bounds__(256) pack_single_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                           int n) {
  __shared__ float t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  const size_t npix = (size_t)n * n;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int x = by + r, y = bx + threadIdx.x;
    if (x < n && y < n) {
      const float v = in[(size_t)x * n + y];
      t[r][threadIdx.x] = v;
      out[(size_t)x * n + y] = v;
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int y = bx + r, x = by + threadIdx.x;
    if (x < n && y < n) out[npix + (size_t)y * n + x] = t[threadIdx.x][r];
  }
}

// Device scratch of one fan-beam / ray-table forward projection outside a
// batch: the image's two copies (2 n^2 floats) and, for the slab projector,
// its TMA descriptor.
size_t fp_single_scratch_bytes(const Plan &p) {
  return ((sizeof(float) * 2 * (size_t)p.n * p.n + 255) & ~(size_t)255) + sizeof(CUtensorMap);
}

// One fan-beam / ray-table forward projection outside a batch: the image's
// row-major and transposed copies into `scratch` (fp_single_scratch_bytes),
// then the slab projector when the plan has slab tables, else the L1 walk
// reading the transposed copy where rays run closer to the y axis.  The TMA
// descriptor is copied from host memory that lives only through this call:
// pageable cudaMemcpyAsync stages it before returning.
cudaError_t launch_fp_single(const Launch &L, const Plan &p, int rpt, void *scratch, cudaStream_t st) {
  const int n = L.single.n;
  float *copies = reinterpret_cast<float *>(scratch);
  pack_single_kernel<<<dim3((n + 31) / 32, (n + 31) / 32), dim3(32, 8), 0, st>>>(L.single.buf[L.in_buf], copies, n);
  Launch Lt = L;
  Lt.single.pack = reinterpret_cast<float4 *>(copies);
  if (p.slab.ok) {
    CUtensorMap *dmap = reinterpret_cast<CUtensorMap *>(reinterpret_cast<char *>(scratch) +
                                                        fp_single_scratch_bytes(p) - sizeof(CUtensorMap));
    CUtensorMap hmap;
    // (a descriptor the driver refuses reads as "not supported", a launch
    // configuration it refuses as "invalid argument")
    if (encode_pack_tmap(&hmap, copies, n, 1, p.slab.wbox, p.slab.rows)) return cudaErrorNotSupported;
    cudaError_t e = cudaMemcpyAsync(dmap, &hmap, sizeof(hmap), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    Lt.single.tmap = dmap;
    return launch_fp_slab(Lt, 1, p.slab.ncta, p.slab.views * p.slab.rays,
                          slab_smem_bytes(1, p.slab.rows, p.slab.wbox), st);
  }
  Lt.tr = 1;
  return launch_fp(Lt, AT_GEOM_FAN, rpt, fp_ctas(L.single, rpt), st);
}

// Forward projection of a batch of fan-beam / ray-table scans without groups:
// each scan's input copied row-major and transposed into its pack buffer (over
// the pixel-pass CTAs of Lpix), then the slab projector (`slab`: every plan has
// slab tables of one CTA shape) or the L1 walk with RPT rays per thread.
// Returns the number of launches.
int launch_fp_tr(const Launch &L, const Launch &Lpix, int rpt, int nctas, int pix_nctas, const SlabLaunch *slab,
                 cudaStream_t st) {
  fp_pack_kernel<<<pix_nctas, 256, 0, st>>>(Lpix, 0);
  if (slab) {
    if (launch_fp_slab(L, 1, nctas, slab->threads, slab->smem[1], st) != cudaSuccess) return -1;
    return 2;
  }
  Launch Lt = L;
  Lt.tr = 1;
  launch_fp(Lt, AT_GEOM_FAN, rpt, nctas, st);
  return 2;
}

// Back projection of a batch whose scans sharing a plan are grouped: the max
// |r| pass, the members' sinograms interleaved (over the sinogram-pass CTAs
// of Lsino), then each group's runs walked once: groups of three or four over
// L's CTAs, pairs and scans alone over Lsmall's.  Returns the number of
// launches.
int launch_bp_group(const Launch &L, const Launch &Lsino, const Launch &Lsmall, int nctas, int sino_nctas,
                    int small_nctas, cudaStream_t st) {
  int n = 2;
  Launch La = L;  // the max |r| pass: one CTA per part, never queued
  La.queue = nullptr;
  sino_absmax_kernel<<<L.nscans * kBpMaxParts, 256, 0, st>>>(La);
  fp_pack_kernel<<<sino_nctas, 256, 0, st>>>(Lsino, 1);
  static int resg[3] = {0, 0, 0}, ress[3] = {0, 0, 0};
  auto group = [&](auto kern, int m) {
    launch_maybe_queued(kern, fan_bp_group_queue_kernel, resg[m], L, nctas, 256, st);
  };
  auto small = [&](auto kern, int m) {
    launch_maybe_queued(kern, fan_bp_small_queue_kernel, ress[m], Lsmall, small_nctas, 256, st);
  };
  if (L.bp_table == 1) group(fan_bp_group_kernel<1>, 1);
  else if (L.bp_table == 2) group(fan_bp_group_kernel<2>, 2);
  else group(fan_bp_group_kernel<0>, 0);
  if (Lsmall.bp_table == 1) small(fan_bp_small_kernel<1>, 1);
  else if (Lsmall.bp_table == 2) small(fan_bp_small_kernel<2>, 2);
  else small(fan_bp_small_kernel<0>, 0);
  return n + (nctas > 0) + (small_nctas > 0);
}

// Lpix / pix_nctas: the same launch over pixel-pass CTAs, for kernels whose
// epilogue runs per pixel in a second pass (cone beam)
cudaError_t launch_bp(const Launch &L, int kind, int nctas, cudaStream_t st, const Launch *Lpix, int pix_nctas) {
  if (kind == AT_GEOM_GOLDNC) {
    gc_bp_kernel<<<nctas, 256, 0, st>>>(L);
  } else if (kind == AT_GEOM_CONE) {
    if (!Lpix) return cudaErrorInvalidValue;
    sino_absmax_kernel<<<(L.scans ? L.nscans : 1) * kBpMaxParts, 256, 0, st>>>(L);
    return launch_cone_bp(L, nctas, *Lpix, pix_nctas, st);
  } else {
    Launch La = L;  // the max |r| pass: one CTA per part, never queued
    La.queue = nullptr;
    sino_absmax_kernel<<<(L.scans ? L.nscans : 1) * kBpMaxParts, 256, 0, st>>>(La);
    static int res[3] = {0, 0, 0};
    if (L.bp_table == 1) launch_maybe_queued(fan_bp_kernel<1>, fan_bp_queue_kernel, res[1], L, nctas, 256, st);
    else if (L.bp_table == 2) launch_maybe_queued(fan_bp_kernel<2>, fan_bp_queue_kernel, res[2], L, nctas, 256, st);
    else launch_maybe_queued(fan_bp_kernel<0>, fan_bp_queue_kernel, res[0], L, nctas, 256, st);
  }
  return cudaGetLastError();
}

}  // namespace medimg

namespace medimg {

size_t fp_single_scratch_bytes(const Plan &p);
cudaError_t launch_fp_single(const Launch &L, const Plan &p, int rpt, void *scratch, cudaStream_t st);

// Times the plan's forward projector variants on a zero image and keeps the
// fastest (results are bitwise identical across all of them): the L1 walk
// with 1, 2 and 4 rays per thread, and the slab projector for a few CTA
// shapes (views x rays per CTA, rows per slab).  Each variant is timed as a
// projection outside a batch, the image's copies included.
int autotune_fan(Plan &p, cudaStream_t st) {
  p.fp_rpt = 1;
  free_slab_tables(p.slab);
  if (p.kind == AT_GEOM_GOLDNC || p.kind == AT_GEOM_CONE) return AT_OK;
  float *img = nullptr, *sino = nullptr;
  void *scratch = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const auto free_temps = scope_exit([&] {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (img) cudaFreeAsync(img, st);
    if (sino) cudaFreeAsync(sino, st);
    if (scratch) cudaFreeAsync(scratch, st);
  });
  const size_t npix = (size_t)p.n * p.n, nbins = (size_t)p.nviews * p.ndets;
  AT_CUDA_TRY(cudaMallocAsync(&img, npix * sizeof(float), st));
  AT_CUDA_TRY(cudaMallocAsync(&sino, nbins * sizeof(float), st));
  AT_CUDA_TRY(cudaMallocAsync(&scratch, fp_single_scratch_bytes(p), st));
  AT_CUDA_TRY(cudaMemsetAsync(img, 0, npix * sizeof(float), st));
  Launch L;
  memset(&L, 0, sizeof(L));
  L.single.buf[0] = img;
  L.single.buf[1] = sino;
  L.nscans = 1;
  L.flow = FLOW_ALWAYS;
  L.stage = ST_NONE;
  L.in_buf = 0;
  L.out_buf = 1;
  L.aux_buf = -1;
  AT_CUDA_TRY(cudaEventCreate(&e0));
  AT_CUDA_TRY(cudaEventCreate(&e1));
  auto time_it = [&](int rpt, float &ms) -> int {
    fill_scan_plan(L.single, p);
    L.single.buf[0] = img;
    L.single.buf[1] = sino;
    AT_CUDA_TRY(launch_fp_single(L, p, rpt, scratch, st));
    AT_CUDA_TRY(cudaEventRecord(e0, st));
    for (int i = 0; i < 3; i++) AT_CUDA_TRY(launch_fp_single(L, p, rpt, scratch, st));
    AT_CUDA_TRY(cudaEventRecord(e1, st));
    AT_CUDA_TRY(cudaEventSynchronize(e1));
    AT_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    return AT_OK;
  };
  float best = 1e30f;
  int rc;
  for (int rpt : {1, 2, 4}) {
    float ms = 0.f;
    if ((rc = time_it(rpt, ms))) return rc;
    if (ms < best) {
      best = ms;
      p.fp_rpt = rpt;
    }
  }
  // slab shapes: views x rays per CTA (at most 512 threads), rows per slab
  const int shapes[][3] = {{4, 128, 16}, {2, 128, 16}, {4, 128, 8}, {8, 64, 16}, {4, 64, 16}, {2, 128, 32}};
  int pick = -1;
  for (int i = 0; i < (int)(sizeof(shapes) / sizeof(shapes[0])); i++) {
    if ((rc = build_slab_tables(p, shapes[i][0], shapes[i][1], shapes[i][2], st))) return rc;
    if (!p.slab.ok) continue;
    float ms = 0.f;
    if (time_it(p.fp_rpt, ms)) {
      // a shape the device refuses (shared memory, descriptor): skip it; a
      // fault would be sticky and fail the next call
      cudaGetLastError();
      AT_CUDA_TRY(cudaStreamSynchronize(st));
      continue;
    }
    if (ms < best) {
      best = ms;
      pick = i;
    }
  }
  if (pick >= 0) {
    if ((rc = build_slab_tables(p, shapes[pick][0], shapes[pick][1], shapes[pick][2], st))) return rc;
  } else {
    free_slab_tables(p.slab);
  }
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  return AT_OK;
}

}  // namespace medimg

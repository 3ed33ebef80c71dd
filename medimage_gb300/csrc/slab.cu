// slab.cu -- fan-beam / ray-table forward projection with the image staged in
// shared memory by TMA.
//
// The gathers of the ray walk (one pixel per Siddon segment) are the forward
// projector's cost: through L1 a warp's 32 neighbouring rays touch a dozen
// cache lines per step, and the L1 pipe processes about one line per cycle.
// Here a CTA owns `views` consecutive views x `rays` adjacent detectors.  Its
// rays run closer to one image axis; it reads the copy of the image (row-major
// or transposed, both in the scan's pack buffer) in which that axis is the row
// index, so at any step the warp's rays lie side by side along a row.  The
// rows are cut into slabs of `rows` rows.  Thread 0 loads each slab's band of
// columns (the columns the CTA's rays cross there, from the plan's tables)
// into shared memory with one cp.async.bulk.tensor per slab, double-buffered
// on two mbarriers.  Every thread walks its ray exactly as the L1 kernel does
// (same decision bits, crossing formula, per-word partial sums and Kahan
// folds, so the sums are bitwise the same), reading pixels from the staged
// slab, and pauses when its ray steps out of the slab's far edge; after a
// barrier the buffer is refilled two slabs ahead.  A group of scans sharing
// the plan is staged as one float2 / float4 per pixel, so one walk feeds every
// member.  CTAs holding a ray that leaves the grid (the reference traces such
// segments for rays along the far edge) walk through L1 with the L1 kernel's
// index checks instead.
//
// Every mbarrier wait is bounded: past the limit the CTA records a timeout in
// g_slab_timeouts and returns without its outputs; host calls report it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "epilogue.cuh"
#include "mbar.cuh"
#include "solver.h"

namespace medimg {

__device__ unsigned g_slab_timeouts;

namespace {

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

template <int G>
struct Elem;
template <>
struct Elem<1> {
  using T = float;
};
template <>
struct Elem<2> {
  using T = float2;
};
template <>
struct Elem<4> {
  using T = float4;
};

template <int G>
__device__ __forceinline__ void fma_elem(float (&part)[G], float wt, const typename Elem<G>::T &v) {
  if constexpr (G == 1) {
    part[0] = fmaf(wt, v, part[0]);
  } else if constexpr (G == 2) {
    part[0] = fmaf(wt, v.x, part[0]);
    part[1] = fmaf(wt, v.y, part[1]);
  } else {
    part[0] = fmaf(wt, v.x, part[0]);
    part[1] = fmaf(wt, v.y, part[1]);
    part[2] = fmaf(wt, v.z, part[2]);
    part[3] = fmaf(wt, v.w, part[3]);
  }
}

template <int G>
__device__ __forceinline__ typename Elem<G>::T zero_elem() {
  if constexpr (G == 1) return 0.f;
  else if constexpr (G == 2) return make_float2(0.f, 0.f);
  else return make_float4(0.f, 0.f, 0.f, 0.f);
}

}  // namespace

// G members per walk: 1 (a scan alone), 2 (a pair, float2) or 4 (three or four
// members, float4).  Block = views x rays threads, one ray each.
template <int G>
__global__ void __launch_bounds__(512, 2) fan_fp_slab_kernel(const Launch L) {
  using T = typename Elem<G>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + ((8 - (smem_u32(smem) & 7u)) & 7u));
  const int scan = L.scans ? find_scan(L.prefix, L.nscans, blockIdx.x) : 0;
  const ScanDev &S = scan_of(L, scan);
  // the group's members and which of them this launch serves (read again for
  // the epilogue, so that they hold no registers through the walk)
  auto members = [&](const ScanDev *(&M)[G], bool(&act)[G]) {
    const int nm = L.scans ? S.nmem : 1;
    bool any = false;
#pragma unroll
    for (int m = 0; m < G; m++) {
      M[m] = L.scans ? &L.scans[S.mem[m < nm ? m : 0]] : &L.single;
      act[m] = m < nm && flow_active(*M[m], L.flow);
      any |= act[m];
    }
    return any;
  };
  {
    const ScanDev *M[G];
    bool act[G];
    if (!members(M, act)) return;  // the same for the whole CTA
  }
  const int local_cta = blockIdx.x - (L.scans ? __ldg(L.prefix + scan) : 0);
  const int RC = S.slab_rays, SH = S.slab_rows, WB = S.slab_wbox;
  const uint4 ci = __ldg(S.slab_cta + local_cta);
  const unsigned flags = ci.y;
  const int vg = local_cta / S.slab_ndb, db = local_cta % S.slab_ndb;
  const int view = vg * S.slab_views + (int)threadIdx.x / RC;
  const int det = db * RC + (int)threadIdx.x % RC;
  const bool valid = view < S.nviews && det < S.ndets;
  int nseg = 0, x0 = 0, y0 = 0, sx = 1, sy = 1;
  float ax = 0.f, ay = 0.f, lx = 0.f, ly = 0.f;
  const uint32_t *wp = S.bits;
  if (valid) {
    const uint4 *hp = reinterpret_cast<const uint4 *>(S.rays + (size_t)view * S.ndets + det);
    const uint4 h0 = __ldg(hp), h1 = __ldg(hp + 1);
    nseg = (int)h0.y;
    x0 = (int)(h0.z & 0xffffu);
    y0 = (int)(h0.z >> 16);
    sx = (h0.w & 1u) ? 1 : -1;
    sy = (h0.w & 2u) ? 1 : -1;
    ax = __uint_as_float(h1.x);
    ay = __uint_as_float(h1.y);
    lx = __uint_as_float(h1.z);
    ly = __uint_as_float(h1.w);
    wp = S.bits + __ldg(S.blk_word + view * S.nbpv + det / kRayBlock) + det % kRayBlock;
  }
  float acc[G], comp[G], part[G];
#pragma unroll
  for (int m = 0; m < G; m++) acc[m] = comp[m] = part[m] = 0.f;
  float cx = 0.f, cy = 0.f, prev = 0.f;
  const T *__restrict__ pack = reinterpret_cast<const T *>(S.pack);
  if (flags & (kSlabFallback | kSlabEmpty)) {
    // gathers through L1 from the row-major copy, with the L1 kernel's checks
    // (a pixel is read when its linear index lies in the image)
    const unsigned npix = (unsigned)(S.n * S.n);
    int idx = x0 * S.n + y0;
    const int stx = sx * S.n, sty = sy;
    for (int k0 = 0; k0 < nseg; k0 += 32) {
      uint32_t wb = __ldg(wp + (size_t)(k0 >> 5) * kRayBlock);
      const int nk = min(32, nseg - k0);
      for (int t = 0; t < nk; t++) {
        const bool bx = wb & 1u;
        wb >>= 1;
        const float nx = fmaf(cx, lx, ax), ny = fmaf(cy, ly, ay);
        const float cur = bx ? nx : ny;
        const float wt = cur - prev;
        prev = cur;
        const T v = (unsigned)idx < npix ? pack[idx] : zero_elem<G>();
        fma_elem<G>(part, wt, v);
        idx += bx ? stx : sty;
        cx += bx ? 1.f : 0.f;
        cy += bx ? 0.f : 1.f;
      }
#pragma unroll
      for (int m = 0; m < G; m++) {
        kahan_add(acc[m], comp[m], part[m]);
        part[m] = 0.f;
      }
    }
  } else {
    const bool tr = flags & kSlabTransposed;
    const int dir = (flags & kSlabDown) ? -1 : 1;
    const int first = (int)(ci.x & 0xffffu), last = (int)(ci.x >> 16);
    const int nsl = (last - first) * dir + 1;
    const size_t buf_bytes = ((size_t)SH * WB * sizeof(T) + 127) & ~(size_t)127;
    // TMA destinations on 128-byte boundaries, whatever the dynamic region's base
    unsigned char *buf_base = smem + ((128 - (smem_u32(smem) & 127u)) & 127u) + 128;
    const unsigned box_bytes = (unsigned)(SH * WB * sizeof(T));
    const CUtensorMap *map = S.tmap;
    const int row_base = tr ? S.n : 0;
    const int16_t *wlo_row = S.slab_wlo + (size_t)local_cta * S.slab_nslab;
    auto issue = [&](int i) {
      const int s = first + dir * i;
      uint64_t *b = bar + (i & 1);
      mbar_expect_tx(b, box_bytes);
      void *dst = buf_base + (i & 1) * buf_bytes;
      const int col = __ldg(wlo_row + s), row = row_base + s * SH;
      if constexpr (G == 4) tma_load_3d(dst, map, 0, col, row, b);
      else tma_load_2d(dst, map, col, row, b);
    };
    if (threadIdx.x == 0) {
      asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
      mbar_init(bar, 1);
      mbar_init(bar + 1, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      issue(0);
      if (nsl > 1) issue(1);
    }
    // walk coordinates in the copy: u = row (along the rays), w = column
    int u = tr ? y0 : x0, w = tr ? x0 : y0;
    const int su = tr ? sy : sx, sw = tr ? sx : sy;
    const uint32_t ubit = tr ? 0u : 1u;  // decision bit of a step along u (1 = an x crossing)
    const int du = su * WB, dw = sw;
    int k = 0, b = 0;
    uint32_t word = nseg > 0 ? __ldg(wp) : 0u;
    int myslab = nseg > 0 ? u / SH : INT_MIN;
    bool timed_out = false;
    for (int i = 0; i < nsl; i++) {
      const int s = first + dir * i;
      if (!mbar_wait(bar + (i & 1), (unsigned)((i >> 1) & 1))) timed_out = true;
      if (!timed_out && k < nseg && myslab == s) {
        const T *tile = reinterpret_cast<const T *>(buf_base + (i & 1) * buf_bytes);
        const int row0 = s * SH;
        const int wlo = __ldg(wlo_row + s);
        int off = (u - row0) * WB + (w - wlo);
        int uleft = su > 0 ? row0 + SH - u : u - row0 + 1;  // u steps before the ray leaves the slab
        // Word by word: the decision bits say how many of the word's segments
        // stay in the slab (up to and including the uleft-th step along u),
        // so each run is walked without per-step exit checks.
        while (k < nseg && uleft > 0) {
          const int navail = min(32 - b, nseg - k);
          const uint32_t wb = word >> b;
          const uint32_t vmask = navail == 32 ? 0xffffffffu : ((1u << navail) - 1u);
          uint32_t um = (ubit ? wb : ~wb) & vmask;  // the steps along u among them
          const int cu = __popc(um);
          int nrun = navail;
          if (cu >= uleft) {  // leaves the slab at its uleft-th u step: find that bit
            int need = uleft, pos = 0;
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
              const int c = __popc(um & ((1u << sh) - 1u));
              if (c < need) {
                need -= c;
                um >>= sh;
                pos += sh;
              }
            }
            nrun = pos + 1;
            uleft = 0;
          } else {
            uleft -= cu;
          }
          uint32_t wr = wb;
          for (int t = 0; t < nrun; t++) {
            const bool bx = wr & 1u;
            wr >>= 1;
            const float nx = fmaf(cx, lx, ax), ny = fmaf(cy, ly, ay);
            const float cur = bx ? nx : ny;
            const float wt = cur - prev;
            prev = cur;
            fma_elem<G>(part, wt, tile[off]);
            off += ((uint32_t)bx == ubit) ? du : dw;
            cx += bx ? 1.f : 0.f;
            cy += bx ? 0.f : 1.f;
          }
          k += nrun;
          b += nrun;
          if (b == 32 || k == nseg) {  // a word ends: fold its sum (as the L1 kernel does)
#pragma unroll
            for (int m = 0; m < G; m++) {
              kahan_add(acc[m], comp[m], part[m]);
              part[m] = 0.f;
            }
            if (b == 32) {
              b = 0;
              if (k < nseg) word = __ldg(wp + (size_t)(k >> 5) * kRayBlock);
            }
          }
        }
        if (k < nseg) {  // stepped out through the far edge: into the next slab
          const int lrow = su > 0 ? SH : -1;
          w = wlo + (off - lrow * WB);
          u = row0 + lrow;
          myslab += su;
        }
      }
      if (__syncthreads_or(timed_out)) {
        timed_out = true;
        break;
      }
      if (threadIdx.x == 0 && i + 2 < nsl) {
        // the buffer's generic-proxy reads are done (barrier above); order
        // them before the async-proxy refill
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(i + 2);
      }
    }
    if (timed_out) {
      if (threadIdx.x == 0) {
        atomicAdd(&g_slab_timeouts, 1u);
        // let the loads in flight land before the CTA's shared memory goes away
        mbar_wait(bar, 0u);
        mbar_wait(bar + 1, 0u);
      }
      return;  // no outputs: the host reports the timeout
    }
  }
  const ScanDev *M[G];
  bool act[G];
  members(M, act);
  const int ncta = L.scans ? __ldg(L.prefix + scan + 1) - __ldg(L.prefix + scan) : gridDim.x;
  FF s0[G];
#pragma unroll
  for (int m = 0; m < G; m++) s0[m] = ff_zero();
  if (valid) {
    const int bin = view * S.ndets + det;
#pragma unroll
    for (int m = 0; m < G; m++)
      if (act[m]) fp_epilogue(*M[m], L, bin, acc[m] - comp[m], s0[m]);
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

// ---------------------------------------------------------------------------
// launch
// ---------------------------------------------------------------------------
size_t slab_smem_bytes(int G, int rows, int wbox) {
  const size_t esz = sizeof(float) * (size_t)G;
  return 256 + 2 * (((size_t)rows * wbox * esz + 127) & ~(size_t)127);
}

namespace {
// Raises the kernel's dynamic shared memory limit to what a launch needs
// (once per size; the limit is the device's opt-in maximum less the kernel's
// static shared memory).  Returns cudaErrorInvalidValue for a size beyond it.
template <int G>
cudaError_t launch_slab_g(const Launch &L, int nctas, int threads, size_t smem, cudaStream_t st) {
  static std::mutex mu;
  static size_t granted = 48 * 1024;  // every kernel may take 48 KB without opting in
  if (smem > granted) {
    std::lock_guard<std::mutex> lk(mu);
    if (smem > granted) {
      int dev = 0, optin = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      cudaFuncAttributes fa{};
      if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fan_fp_slab_kernel<G>);
      if (e != cudaSuccess) return e;
      if (smem + fa.sharedSizeBytes > (size_t)optin) return cudaErrorInvalidValue;
      e = cudaFuncSetAttribute(fan_fp_slab_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      granted = smem;
    }
  }
  fan_fp_slab_kernel<G><<<nctas, threads, smem, st>>>(L);
  return cudaGetLastError();
}
}  // namespace

// G: 1, 2 or 4 (the launch's group form).  The launch's scans share one CTA
// shape (threads = views x rays); `smem` covers the largest slab buffer pair
// among them.
cudaError_t launch_fp_slab(const Launch &L, int G, int nctas, int threads, size_t smem, cudaStream_t st) {
  if (nctas <= 0) return cudaSuccess;
  if (G == 4) return launch_slab_g<4>(L, nctas, threads, smem, st);
  if (G == 2) return launch_slab_g<2>(L, nctas, threads, smem, st);
  return launch_slab_g<1>(L, nctas, threads, smem, st);
}

int slab_ctas(const ScanDev &S) {
  return ((S.nviews + S.slab_views - 1) / S.slab_views) * S.slab_ndb;
}

// TMA descriptor of a pack buffer: n x n pixels, row-major rows then the
// transposed copy's rows (2n rows), G floats per pixel; box = the plan's slab
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_pack_tmap(CUtensorMap *out, const void *pack, int n, int G, int wbox, int rows) {
  static std::once_flag once;
  static EncodeTiledFn encode = nullptr;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<EncodeTiledFn>(fn);
  });
  if (!encode) return set_error(AT_ECUDA, "TMA: cuTensorMapEncodeTiled is not available from the driver");
  std::memset(out, 0, sizeof(*out));
  CUresult r;
  if (G == 4) {
    const cuuint64_t dims[3] = {4, (cuuint64_t)n, 2 * (cuuint64_t)n};
    const cuuint64_t strides[2] = {16, 16 * (cuuint64_t)n};
    const cuuint32_t box[3] = {4, (cuuint32_t)wbox, (cuuint32_t)rows};
    const cuuint32_t es[3] = {1, 1, 1};
    r = encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void *>(pack), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {
    const cuuint64_t dims[2] = {(cuuint64_t)n, 2 * (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)n * (G == 2 ? 8 : 4)};
    const cuuint32_t box[2] = {(cuuint32_t)wbox, (cuuint32_t)rows};
    const cuuint32_t es[2] = {1, 1};
    r = encode(out, G == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
               const_cast<void *>(pack), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  if (r != CUDA_SUCCESS) return set_error(AT_ECUDA, "TMA: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return AT_OK;
}

// slab timeouts recorded since the last call (and clears the record)
int slab_timeouts(unsigned *out) {
  unsigned v = 0, zero = 0;
  AT_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_slab_timeouts, sizeof(v)));
  if (v) AT_CUDA_TRY(cudaMemcpyToSymbol(g_slab_timeouts, &zero, sizeof(zero)));
  *out = v;
  return AT_OK;
}

// Bounded waits of the slab projector that ran out since the last call:
// AT_ECUDA then, as those CTAs left their outputs void.  Called after a
// synchronisation.
int check_wait_timeouts() {
  unsigned n = 0;
  const int rc = slab_timeouts(&n);
  if (rc) return rc;
  if (n)
    return set_error(AT_ECUDA, "slab projector: shared-memory copies did not arrive within the wait limit (" +
                                   std::to_string(n) + " CTAs); their results are void");
  return AT_OK;
}

// ---------------------------------------------------------------------------
// plan tables
// ---------------------------------------------------------------------------
// One thread per CTA: the copy its rays run along, from the ray nearest the
// CTA's middle that crosses the image (lenx > leny: the ray crosses more y
// planes, so it runs closer to the y axis: the transposed copy), and the
// direction of travel along that copy's rows.
__global__ void slab_cta_kernel(int nviews, int ndets, int views, int rays, int ndb, int ncta, const RayHdr *hdr,
                                unsigned *flags) {
  const int cta = blockIdx.x * blockDim.x + threadIdx.x;
  if (cta >= ncta) return;
  const int vg = cta / ndb, db = cta % ndb;
  const int v0 = vg * views, v1 = min(nviews, v0 + views), d0 = db * rays, d1 = min(ndets, d0 + rays);
  const int vm = (v0 + v1) / 2, dm = (d0 + d1) / 2;
  unsigned f = kSlabEmpty;
  // rays in order of distance from the middle ray
  for (int r = 0; r < (v1 - v0) * (d1 - d0) && (f & kSlabEmpty); r++) {
    const int v = v0 + (vm - v0 + r / (d1 - d0)) % (v1 - v0);
    const int d = d0 + (dm - d0 + r % (d1 - d0)) % (d1 - d0);
    const RayHdr h = hdr[(size_t)v * ndets + d];
    if (h.nseg == 0) continue;
    const bool tr = h.lenx > h.leny;
    const bool down = tr ? !(h.sgn & 2) : !(h.sgn & 1);
    f = (tr ? kSlabTransposed : 0u) | (down ? kSlabDown : 0u);
  }
  flags[cta] = f;
}

// One thread per ray: the band of columns its pixels occupy in each slab of
// its CTA's copy (running min / max, flushed at each slab change); marks the
// CTA for the L1 path if a pixel leaves the grid or the ray steps along the
// rows against the CTA's direction.
__global__ void slab_extent_kernel(int n, int nviews, int ndets, int nbpv, int views, int rays, int ndb, int rows,
                                   int nslab, const RayHdr *hdr, const uint32_t *bits, const uint32_t *blk_word,
                                   const unsigned *flags, unsigned *fallback, int *lo, int *hi) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= nviews * ndets) return;
  const RayHdr h = hdr[ray];
  if (h.nseg == 0) return;
  const int view = ray / ndets, det = ray % ndets;
  const int cta = (view / views) * ndb + det / rays;
  const unsigned f = flags[cta];
  const bool tr = f & kSlabTransposed;
  const int dir = (f & kSlabDown) ? -1 : 1;
  const uint32_t *wp = bits + blk_word[view * nbpv + det / kRayBlock] + (det % kRayBlock);
  int x = h.xy0 & 0xffff, y = h.xy0 >> 16;
  const int sx = (h.sgn & 1) ? 1 : -1, sy = (h.sgn & 2) ? 1 : -1;
  const int su = tr ? sy : sx;
  bool bad = false;
  int cur = -1, mn = INT_MAX, mx = INT_MIN;
  uint32_t word = 0;
  for (int k = 0; k < h.nseg; k++) {
    if ((k & 31) == 0) word = wp[(size_t)(k >> 5) * kRayBlock];
    const int u = tr ? y : x, w = tr ? x : y;
    if ((unsigned)x >= (unsigned)n || (unsigned)y >= (unsigned)n) {
      bad = true;
    } else {
      const int s = u / rows;
      if (s != cur) {
        if (cur >= 0) {
          atomicMin(lo + (size_t)cta * nslab + cur, mn);
          atomicMax(hi + (size_t)cta * nslab + cur, mx);
        }
        cur = s;
        mn = INT_MAX;
        mx = INT_MIN;
      }
      mn = min(mn, w);
      mx = max(mx, w);
    }
    const bool xs = (word >> (k & 31)) & 1u;
    if (xs == !tr && su != dir) bad = true;  // a step along the rows, against the CTA's direction
    if (xs) x += sx;
    else y += sy;
  }
  if (cur >= 0) {
    atomicMin(lo + (size_t)cta * nslab + cur, mn);
    atomicMax(hi + (size_t)cta * nslab + cur, mx);
  }
  if (bad) atomicOr(fallback + cta, 1u);
}

void free_slab_tables(SlabPlan &s) {
  cudaFree(s.cta_d);
  cudaFree(s.wlo_d);
  s = SlabPlan{};
}

void retire_slab_tables(Plan &p) {
  if (p.slab.cta_d || p.slab.wlo_d) p.retired_slabs.push_back(p.slab);
  p.slab = SlabPlan{};
}

// Builds the tables of one CTA shape into p.slab, replacing (freeing) the
// tables there; p.slab.ok = 0 when the shape does not fit.
int build_slab_tables(Plan &p, int views, int rays, int rows, cudaStream_t st) {
  free_slab_tables(p.slab);
  if (p.kind != AT_GEOM_FAN && p.kind != AT_GEOM_RAYS) return AT_OK;
  // rows of the pack buffer must start on 16-byte boundaries (floats: n % 4)
  if (p.n % 4 != 0 || views < 1 || rays < 1 || kRayBlock % rays != 0 || views * rays > 512 || rows < 1 ||
      rows > 256)
    return AT_OK;
  const int nviews = p.nviews, ndets = p.ndets, n = p.n;
  const int ndb = (ndets + rays - 1) / rays;
  const int ncta = ((nviews + views - 1) / views) * ndb;
  const int nslab = (n + rows - 1) / rows;
  const size_t cells = (size_t)ncta * nslab;
  unsigned *flags = nullptr, *fb = nullptr;
  int *lo = nullptr, *hi = nullptr;
  const auto free_temps = scope_exit([&] {
    cudaFree(flags);
    cudaFree(fb);
    cudaFree(lo);
    cudaFree(hi);
  });
  AT_CUDA_TRY(cudaMalloc(&flags, sizeof(unsigned) * ncta));
  AT_CUDA_TRY(cudaMalloc(&fb, sizeof(unsigned) * ncta));
  AT_CUDA_TRY(cudaMalloc(&lo, sizeof(int) * cells));
  AT_CUDA_TRY(cudaMalloc(&hi, sizeof(int) * cells));
  AT_CUDA_TRY(cudaMemsetAsync(fb, 0, sizeof(unsigned) * ncta, st));
  AT_CUDA_TRY(cudaMemsetAsync(lo, 0x7f, sizeof(int) * cells, st));  // 0x7f7f7f7f: above any column
  AT_CUDA_TRY(cudaMemsetAsync(hi, 0xff, sizeof(int) * cells, st));  // -1: below any column
  slab_cta_kernel<<<(ncta + 127) / 128, 128, 0, st>>>(nviews, ndets, views, rays, ndb, ncta, p.rays_d, flags);
  AT_CUDA_TRY(cudaGetLastError());
  const int nrays = nviews * ndets;
  slab_extent_kernel<<<(nrays + 127) / 128, 128, 0, st>>>(n, nviews, ndets, p.nblocks_per_view, views, rays, ndb,
                                                         rows, nslab, p.rays_d, p.bits_d, p.blk_word_d, flags, fb,
                                                         lo, hi);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<unsigned> hf(ncta), hfb(ncta);
  std::vector<int> hlo(cells), hhi(cells);
  AT_CUDA_TRY(cudaMemcpyAsync(hf.data(), flags, sizeof(unsigned) * ncta, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(hfb.data(), fb, sizeof(unsigned) * ncta, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(hlo.data(), lo, sizeof(int) * cells, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(hhi.data(), hi, sizeof(int) * cells, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<uint4> cta(ncta);
  std::vector<int16_t> wlo(cells, 0);
  int wbox = 4, nfb = 0;
  for (int c = 0; c < ncta; c++) {
    unsigned f = hf[c];
    int s0 = INT_MAX, s1 = INT_MIN;
    for (int s = 0; s < nslab; s++) {
      const size_t i = (size_t)c * nslab + s;
      if (hlo[i] > hhi[i]) continue;  // no pixel of the CTA in this slab (staged, never read)
      s0 = std::min(s0, s);
      s1 = std::max(s1, s);
      const int w0 = hlo[i] & ~3;
      wlo[i] = (int16_t)w0;
      wbox = std::max(wbox, hhi[i] - w0 + 1);
    }
    if (hfb[c]) {
      f |= kSlabFallback;
      nfb++;
    }
    if (s0 > s1) f |= kSlabEmpty;
    const bool down = f & kSlabDown;
    const int first = (f & kSlabEmpty) ? 0 : (down ? s1 : s0), last = (f & kSlabEmpty) ? 0 : (down ? s0 : s1);
    cta[c] = make_uint4((unsigned)first | ((unsigned)last << 16), f, 0u, 0u);
  }
  wbox = (wbox + 3) & ~3;
  if (wbox > 256) return AT_OK;  // wider than one TMA box: this shape does not fit
  SlabPlan &sp = p.slab;
  AT_CUDA_TRY(cudaMalloc(&sp.cta_d, sizeof(uint4) * ncta));
  AT_CUDA_TRY(cudaMalloc(&sp.wlo_d, sizeof(int16_t) * cells));
  AT_CUDA_TRY(cudaMemcpyAsync(sp.cta_d, cta.data(), sizeof(uint4) * ncta, cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaMemcpyAsync(sp.wlo_d, wlo.data(), sizeof(int16_t) * cells, cudaMemcpyHostToDevice, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  sp.views = views;
  sp.rays = rays;
  sp.rows = rows;
  sp.wbox = wbox;
  sp.nslab = nslab;
  sp.ndb = ndb;
  sp.ncta = ncta;
  sp.fallback = nfb;
  sp.ok = 1;
  return AT_OK;
}

}  // namespace medimg

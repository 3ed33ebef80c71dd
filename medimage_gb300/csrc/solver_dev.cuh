// solver_dev.cuh -- device-side state of a batch of scans and the control
// logic of the AT iteration (origin/GoldenC/src/main.c:81-360), shared by the
// projector kernels (which carry fused epilogues) and the pixel-pass kernels.
//
// Every kernel of the solver takes the whole batch.  A CTA belongs to exactly
// one scan (per-scan CTA ranges come from a prefix table), returns at once if
// that scan's step is no longer active, reduces its partial sums in FP64 and
// writes them to the scan's partial array; the last CTA of the scan to arrive
// sums the partials in a fixed order (deterministic) and runs the scalar part
// of the step (line searches, exit tests) on the device.
#pragma once

#include <cstdint>

#include "at_internal.h"

namespace medimg {

// image-shaped buffers, then sinogram-shaped buffers
enum Buf : int {
  B_F = 0,  // f (the image result; also update buffer 0)
  B_U1,     // update buffer 1
  B_V,      // edge field v
  B_D,      // d (image-step gradient / edge-step direction)
  B_P0,     // CG direction p, ping
  B_P1,     // CG direction p, pong
  B_NN,     // |grad f|^2 for the edge step
  B_NIMG,
  B_G = B_NIMG,  // sinogram data g
  B_R,           // residual r
  B_Q,           // q = A p
  B_AF,          // A f   (linear mode)
  B_AD,          // A d   (linear mode)
  B_NBUF
};

// what a kernel launch belongs to: gates it on the scan's control flags
enum Flow : int { FLOW_ALWAYS = 0, FLOW_IMAGE = 1, FLOW_EDGE = 2, FLOW_ENABLED = 3 };

// stages whose reductions end in a scalar update
enum Stage : int {
  ST_NONE = 0,
  ST_FP0,   // A(update): E_data, r = g - Af                       main.c:101-104,126-129
  ST_BP0,   // A^T r + stencil: E_smooth -> AT_f_old               main.c:110-139
  ST_PP0,   // p = d: nV, <p,d>                                    main.c:141-166
  ST_FPQ,   // q = A p: |q|^2 -> c1                                main.c:146,163-167
  ST_UPD,   // update += c1 p (+median): maxCP, exits              main.c:169-191
  ST_FPA,   // A(update): E_data; r -= c1 q                        main.c:193-197,217-219
  ST_BPD,   // A^T r + stencil: E_smooth -> AT_f_new, revert test  main.c:199-216,225-239
  ST_FPD,   // A d: <Ad,q> -> c2                                   main.c:240-245
  ST_PP,    // p = d + c2 p: nV, <p,d>, trace, k++                 main.c:247-251,148-162
  ST_SQ,    // linear mode: q = Ad + c2 q: |q|^2 -> c1
  ST_SA,    // linear mode: Af += c1 q, r -= c1 q: E_data
  ST_E1,    // edge: d, nD, sum n d^2, nNablaD -> c                main.c:294-329
  ST_E2,    // edge: v = clamp(v + c d): maxCD, exits              main.c:332-354
};

struct Ctl {
  int enabled;      // scan takes part in launches at all
  int img_active;   // image step running
  int edge_active;  // edge step running
  int k;            // inner iteration of the running step (1-based)
  int outer;        // outer iteration (1-based)
  int final_u;      // update buffer holding the image-step result (0 = F, 1 = U1)
  int exit_reason;  // last exit: 1 maxIt, 2 tolerance, 3 instability
  int trace_n;      // records written
  unsigned arrive;  // CTA arrival counter of the current kernel
  unsigned maxbits; // running max of a non-negative float (as bits)
  int iter_image, iter_edge, median_every, mode;
  double alpha, beta, eps;
  double at_old, e_data, nv, pd, normap, c1, c2;
  double nd, c;
};

constexpr int kTraceCap = 4096;  // records per scan (10 doubles each)
constexpr int kBpMaxParts = 64;  // CTAs of the max |r| pass per scan
constexpr int kBpMaxSplit = 8;   // most CTAs one back-projection tile is split over
constexpr int kGroupMax = 4;     // most scans of one plan whose projections share a walk
constexpr int kPixRows = 32;     // rows of a pixel-pass CTA's tile (32 columns; a multiple of 8)
constexpr int kFpGroupThreads = 128;  // CTA size of the grouped forward projector (<= 128)

struct ScanDev {
  int kind, n, nviews, ndets;
  int nz;                          // image slices (1 for 2D); npix = nz * n * n
  int npix, nbins, nbpv, offgrid;  // offgrid: the plan traces segments off the grid
  // cone beam (n = nx = ny; ndets = ndx * ndy)
  int ndx, ndy, half_rows, half_cols;
  float voxel, pitch, sod, sdd;
  const float2 *cone_trig;  // per view: cos, sin
  // fan plan
  const RayHdr *rays;
  const uint32_t *bits;
  const uint32_t *blk_word;
  const uint8_t *blk_off;  // per 128-ray block: a ray leaves the grid
  const uint4 *run;          // back-projection runs grouped by 16x16 tile
  const int32_t *tile_off;   // [tile * nvb + view block]
  // the plan's pixel table (Plan::pt_*), and which launches gather from it
  // instead of walking tile runs: bit0 single scans, bit1 groups
  const uint32_t *pt_meta;
  const float *pt_w;
  const int64_t *pt_woff;
  int pt_use;
  int ntiles_y, nvb, bp_term_bits;
  float pixel_mm;
  // goldnc plan
  const GcSeg *gc_seg;
  const int32_t *gc_pair_off;
  const GcEntry *gc_ent;
  const int32_t *gc_pix_off;
  // back-projection scratch: per-part max |r| of the input sinogram, and (when
  // a tile's view blocks are split over bp_split CTAs) exact 64-bit pixel sums
  // and per-tile arrival counters, both left zero by the kernel
  float *bpmax;                // [kBpMaxParts]
  unsigned long long *bp_acc;  // [npix]
  int *bp_cnt;                 // [ntiles]
  // cone beam: 32-bit sums of one chunk of views (folded into bp_acc between
  // chunks), and the views per chunk, few enough that no voxel's chunk sum
  // can overflow 32 bits
  int *bp_acc32;               // [npix] volume layout (y contiguous)
  int *bp_acc32x;              // [npix] x contiguous: (z*n + y)*n + x
  int bp_vchunk;
  int bp_split;                // CTAs per tile (>= 1)
  float4 *pack;                // [max(2*n*n, nbins)] fan/ray plans: a group's projector inputs, interleaved
  // slab forward projector (fan / ray plans with slab tables): the plan's
  // CTA shape and tables, and the TMA descriptor of this scan's pack buffer
  // (lead scans: one float, float2 or float4 per pixel, row-major rows then
  // transposed rows)
  int slab_views, slab_rays, slab_rows, slab_wbox, slab_nslab, slab_ndb;
  const uint4 *slab_cta;
  const int16_t *slab_wlo;
  const CUtensorMap *tmap;
  // scans of a batch that share this scan's plan and are projected together
  // with it: nmem members (scan indices, this one first) on the lead; 0 on
  // the others, which get no projector CTAs of their own
  int nmem;
  int mem[kGroupMax];
  // state
  float *buf[B_NBUF];
  Ctl *ctl;
  double *partials;  // >= max CTAs of any kernel for this scan x 4 sums
  double *trace;     // kTraceCap x 10
};

// One launch over the batch.  prefix[s]..prefix[s+1] are scan s's CTAs.
struct Launch {
  ScanDev single;        // used when scans == nullptr (plain projector calls)
  const ScanDev *scans;
  const int *prefix;
  int nscans;
  int flow;
  int stage;
  int in_buf, out_buf, aux_buf;  // buffer ids (meaning depends on the kernel)
  int k;                         // inner iteration this launch belongs to
  int flag;                      // kernel-specific (median this iteration, first pass, ...)
  int chunk;                     // cone back projection: the chunk of views this launch adds
  int chunks;                    // cone back projection: chunks of the launch's largest scan (host side)
  int group;                     // projector launches: largest group of scans sharing a plan
  int tr;                        // forward projection: the scans' pack buffers hold transposed inputs
  int bp_table;                  // fan back projection: 0 walk tile runs, 1 gather from pixel tables,
                                 // 2 each CTA as its scan's plan says (ScanDev::pt_use)
  // persistent launches (projectors of a batch): a grid sized to the resident
  // CTAs pulls work units (the CTA indices of the ordinary launch) from a
  // queue; order[i] is the i-th unit handed out (all units of the costlier
  // scans first), queue[0] the next position, queue[1] the CTAs done.  The
  // last CTA to finish resets both, so the launch can be replayed.
  unsigned *queue;
  const int *order;
  int units;
};

// Runs body(unit) for every unit of a persistent launch, one unit per CTA at a
// time (the unit index stands for blockIdx.x of the ordinary launch).
template <typename Body>
__device__ __forceinline__ void persistent_loop(const Launch &L, Body body) {
  __shared__ int s_unit;
  while (true) {
    __syncthreads();  // the previous unit's shared memory is free, s_unit read
    if (threadIdx.x == 0) {
      const unsigned i = atomicAdd(L.queue, 1u);
      s_unit = i < (unsigned)L.units ? __ldg(L.order + i) : -1;
    }
    __syncthreads();
    const int unit = s_unit;
    if (unit < 0) break;
    body(unit);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(L.queue + 1, 1u) == gridDim.x - 1) {  // every CTA has stopped pulling
      L.queue[0] = 0u;
      L.queue[1] = 0u;
      __threadfence();
    }
  }
}

// Launch shape of the slab forward projector over a batch whose plans all
// have slab tables of one CTA shape: threads per CTA, and dynamic shared
// memory per group form (index 0: three or four members, float4; 1: a scan
// alone, float; 2: a pair, float2), the largest over the batch's scans.
struct SlabLaunch {
  int threads;
  size_t smem[3];
};

__device__ __forceinline__ int find_scan(const int *prefix, int nscans, int cta) {
  int lo = 0, hi = nscans;  // prefix[lo] <= cta < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= cta) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ const ScanDev &scan_of(const Launch &L, int s) {
  return L.scans ? L.scans[s] : L.single;
}

__device__ __forceinline__ bool flow_active(const ScanDev &S, int flow) {
  if (flow == FLOW_ALWAYS) return true;
  const volatile Ctl *c = S.ctl;
  if (!c->enabled) return false;
  if (flow == FLOW_ENABLED) return true;
  if (flow == FLOW_IMAGE) return c->img_active != 0;
  return c->edge_active != 0;
}

// ---- float-float sums ------------------------------------------------------
// The energy and inner-product reductions are FP64 at the warp level and up,
// but GB300's FP64 pipe runs at a small fraction of its FP32 rate, and FP64
// arithmetic per element made the pixel passes FP64-bound.  Per-element terms
// are therefore formed in FP32 (products of two floats exactly, as hi + lo by
// one FMA; non-negative terms as one rounded float) and summed across the
// warp as unevaluated float pairs with error-free additions (Knuth's TwoSum),
// about 44 bits; the warp total is converted to FP64 once.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_zero() { return FF{0.f, 0.f}; }
__device__ __forceinline__ FF ff_of(float x) { return FF{x, 0.f}; }
// a * b exactly
__device__ __forceinline__ FF ff_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return FF{p, fmaf(a, b, -p)};
}
// s + e == a + b exactly (TwoSum)
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return FF{s, e};
}
// x + y, renormalised; commutative bit for bit, so a xor butterfly leaves
// the same total in every lane
__device__ __forceinline__ FF ff_add(FF x, FF y) {
  const FF s = ff_two_sum(x.hi, y.hi);
  const float lo = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  const float hi = __fadd_rn(s.hi, lo);
  return FF{hi, __fsub_rn(lo, __fsub_rn(hi, s.hi))};
}
__device__ __forceinline__ void ff_acc(FF &a, FF x) { a = ff_add(a, x); }
__device__ __forceinline__ double warp_sum_ff(FF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const FF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = ff_add(v, w);
  }
  return (double)v.hi + (double)v.lo;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void trace_push(const ScanDev &S, int step, int k, int exit_reason, double s0, double s1,
                                           double s2, double s3, double s4, double s5) {
  Ctl *c = S.ctl;
  const int i = c->trace_n;
  if (i >= kTraceCap) return;
  double *r = S.trace + (size_t)i * 10;
  r[0] = c->outer;
  r[1] = step;
  r[2] = k;
  r[3] = exit_reason;
  r[4] = s0;
  r[5] = s1;
  r[6] = s2;
  r[7] = s3;
  r[8] = s4;
  r[9] = s5;
  c->trace_n = i + 1;
}

// Scalar part of a step, run by one thread of the last CTA.
__device__ inline void finalize_stage(const ScanDev &S, const Launch &L, const double *s) {
  Ctl *c = S.ctl;
  const int k = L.k;
  switch (L.stage) {
    case ST_FP0:
      c->e_data = s[0];
      break;
    case ST_BP0:
      c->at_old = c->e_data + s[0];
      break;
    case ST_PP0:
      c->nv = s[0];
      c->pd = s[1];
      break;
    case ST_FPQ:
    case ST_SQ:
      c->normap = s[0];
      c->c1 = c->pd / (c->normap + c->alpha * c->nv);  // main.c:167
      break;
    case ST_UPD: {
      const float maxcp = __uint_as_float(c->maxbits);
      c->maxbits = 0u;
      const int next = (k & 1) ? 1 : 0;  // update buffer written at iteration k
      if (k == c->iter_image) {          // main.c:184-187
        trace_push(S, 0, k, 1, c->at_old, c->nv, c->pd, c->normap, c->c1, 0.0);
        c->final_u = next;
        c->exit_reason = 1;
        c->img_active = 0;
      } else if ((double)maxcp < 1e-5) {  // main.c:188-191
        trace_push(S, 0, k, 2, c->at_old, c->nv, c->pd, c->normap, c->c1, 0.0);
        c->final_u = next;
        c->exit_reason = 2;
        c->img_active = 0;
      }
      break;
    }
    case ST_FPA:
    case ST_SA:
      c->e_data = s[0];
      break;
    case ST_BPD: {
      const double at_new = c->e_data + s[0];
      if (1.1 * c->at_old < at_new && 1 < k) {  // main.c:209-215: keep the pre-step image
        trace_push(S, 0, k, 3, c->at_old, c->nv, c->pd, c->normap, c->c1, 0.0);
        c->final_u = (k & 1) ? 0 : 1;
        c->exit_reason = 3;
        c->img_active = 0;
      } else {
        c->at_old = at_new;
      }
      break;
    }
    case ST_FPD:
      c->c2 = -s[0] / c->normap;  // main.c:245
      break;
    case ST_PP:
      trace_push(S, 0, k, 0, c->at_old, c->nv, c->pd, c->normap, c->c1, c->c2);
      c->nv = s[0];
      c->pd = s[1];
      c->k = k + 1;
      break;
    case ST_E1: {
      const double nD = s[0], tmp = s[1], nNablaD = s[2];
      c->nd = nD;
      c->c = nD / (c->alpha * tmp + c->beta * c->eps * nNablaD + (c->beta / (4 * c->eps)) * nD);  // main.c:329
      break;
    }
    case ST_E2: {
      const float maxcd = __uint_as_float(c->maxbits);
      c->maxbits = 0u;
      if (k == c->iter_edge) {  // main.c:346-349
        trace_push(S, 1, k, 1, c->nd, c->c, (double)maxcd, 0, 0, 0);
        c->exit_reason = 1;
        c->edge_active = 0;
      } else if ((double)maxcd < 1e-5) {  // main.c:351-354
        trace_push(S, 1, k, 2, c->nd, c->c, (double)maxcd, 0, 0, 0);
        c->exit_reason = 2;
        c->edge_active = 0;
      } else {
        trace_push(S, 1, k, 0, c->nd, c->c, (double)maxcd, 0, 0, 0);
        c->k = k + 1;
      }
      break;
    }
    default:
      break;
  }
}

// Block-level reduction of NS sums (float-float per thread, FP64 from the warp
// totals on; blockDim.x a multiple of 32, <= 1024), partial write, and the
// last-CTA finalize.  Must be reached by every thread of the CTA.
// `local_cta`/`ncta` index the CTA within its scan.
template <int NS>
__device__ void reduce_and_finalize(const ScanDev &S, const Launch &L, const FF *v, int local_cta, int ncta) {
  __shared__ double red[32][NS > 0 ? NS : 1];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (NS > 0) {
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const double w = warp_sum_ff(v[i]);
      if (lane == 0) red[warp][i] = w;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int i = 0; i < NS; i++) {
        double a = 0;
        for (int w = 0; w < nw; w++) a += red[w][i];
        S.partials[(size_t)local_cta * NS + i] = a;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(&S.ctl->arrive, 1u);
    last = (t == (unsigned)ncta - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double acc[NS > 0 ? NS : 1];
#pragma unroll
  for (int i = 0; i < NS; i++) acc[i] = 0.0;
  if (NS > 0) {
    // L2 loads (the partials of other CTAs, published by their fences),
    // several in flight; the sums keep their order
#pragma unroll 8
    for (int c = threadIdx.x; c < ncta; c += blockDim.x)
#pragma unroll
      for (int i = 0; i < NS; i++) acc[i] += __ldcg(S.partials + (size_t)c * NS + i);
#pragma unroll
    for (int i = 0; i < NS; i++) {
      const double w = warp_sum_d(acc[i]);
      if (lane == 0) red[warp][i] = w;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[NS > 0 ? NS : 1];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      double a = 0;
      for (int w = 0; w < nw; w++) a += red[w][i];
      tot[i] = a;
    }
    S.ctl->arrive = 0u;
    finalize_stage(S, L, tot);
    __threadfence();
  }
}

// reduce_and_finalize<1> for the members of a projector group at once (member
// m active when bit m of `act` is set): one barrier pair for all members, the
// members' partial writes and arrival tickets taken by threads 0..G-1 side by
// side.  Each member's sum is formed in exactly the order of
// reduce_and_finalize<1>, so results do not depend on the grouping.
template <int G>
__device__ __forceinline__ void reduce_and_finalize_group(const ScanDev *const (&M)[G], unsigned act, const Launch &L,
                                          const FF (&v)[G], int local_cta, int ncta) {
  __shared__ double red[32][G];
  __shared__ bool last[G];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int m = 0; m < G; m++) {
    const double w = warp_sum_ff(v[m]);
    if (lane == 0) red[warp][m] = w;
  }
  __syncthreads();
  // thread m takes member m (static member indices keep M[] in registers)
#pragma unroll
  for (int m = 0; m < G; m++) {
    if (threadIdx.x != m) continue;
    bool is_last = false;
    if ((act >> m) & 1u) {
      double a = 0;
      for (int w = 0; w < nw; w++) a += red[w][m];
      const ScanDev &S = *M[m];
      S.partials[local_cta] = a;
      __threadfence();
      const unsigned t = atomicAdd(&S.ctl->arrive, 1u);
      is_last = (t == (unsigned)ncta - 1);
    }
    last[m] = is_last;
  }
  __syncthreads();
  // the members this CTA arrived last for (the same for every thread), all in
  // one pass: each member's partials are summed in the same order as alone
  unsigned lm = 0;
#pragma unroll
  for (int m = 0; m < G; m++) lm |= last[m] ? 1u << m : 0u;
  if (!lm) return;
  __threadfence();
  double acc[G];
#pragma unroll
  for (int m = 0; m < G; m++) acc[m] = 0.0;
#pragma unroll 4
  for (int c = threadIdx.x; c < ncta; c += blockDim.x)
#pragma unroll
    for (int m = 0; m < G; m++)
      if ((lm >> m) & 1u) acc[m] += __ldcg(M[m]->partials + c);
  double w[G];
#pragma unroll
  for (int m = 0; m < G; m++) w[m] = warp_sum_d(acc[m]);
  __syncthreads();  // red[][] is free again
  if (lane == 0)
#pragma unroll
    for (int m = 0; m < G; m++) red[warp][m] = w[m];
  __syncthreads();
  // thread m finishes member m (static member indices keep M[] in registers)
#pragma unroll
  for (int m = 0; m < G; m++) {
    if (threadIdx.x != m || !((lm >> m) & 1u)) continue;
    double a = 0;
    for (int ww = 0; ww < nw; ww++) a += red[ww][m];
    double tot[1] = {a};
    const ScanDev &S = *M[m];
    S.ctl->arrive = 0u;
    finalize_stage(S, L, tot);
    __threadfence();
  }
  __syncthreads();
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned *addr, float x) {
  atomicMax(addr, __float_as_uint(x));
}

}  // namespace medimg

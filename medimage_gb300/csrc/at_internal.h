// at_internal.h -- types shared by the engine's translation units.
//
// Layout of a fan-beam plan in HBM (one per geometry, built once on the GPU):
//   rays   : RayHdr[nviews*ndets]      32 B per ray (start pixel, segment count,
//                                        FP32 boundary parameters)
//   bits   : uint32 decision words      1 bit per Siddon segment (1 = the ray
//                                        crosses an x plane, 0 = a y plane),
//                                        block-interleaved: block b (128 rays of
//                                        one view) stores word w of ray i at
//                                        bits[blk_word[b] + w*128 + i]
//   blk_word: uint32[nblocks+1]         word offset of each 128-ray block
//   blk_off : uint8 [nblocks]           1 if a ray of the block has segments
//                                        off the grid (no unchecked fast path)
// GoldenC plan: traced walks of proj.c as explicit FP32 segments (CSR by
// (alpha, raynum) pair) plus the transposed list (CSC by pixel) for the gather.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda.h>  // CUtensorMap (the descriptor type only; no driver calls are linked)
#include <cuda_runtime.h>

#include "../../include/at_engine.h"

namespace medimg {

constexpr int kRayBlock = 128;  // rays per decision-bit block (one view)
constexpr int kBpTile = 16;     // back-projection tile edge (pixels)
constexpr int kBpViewBlock = 64;  // views whose contributions share one 32-bit accumulator
constexpr int kPtChunk = 16;      // views per chunk of a pixel-table stream (prefetched as one)

// Per-ray header.  Boundary parameters are relative to the ray's entry
// lambda_min (mm): the k-th x-plane crossing is at fmaf(k, lenx, ax), the k-th
// y-plane crossing at fmaf(k, leny, ay); a segment's weight is the difference
// of consecutive crossings.
struct __align__(16) RayHdr {
  int32_t pix0;   // x0*n + y0 of the first pixel
  int32_t nseg;   // segments the reference's loop emits
  int32_t xy0;    // x0 | (y0 << 16)
  int32_t sgn;    // bit0: signx > 0, bit1: signy > 0
  float ax, ay, lenx, leny;
};
static_assert(sizeof(RayHdr) == 32, "RayHdr must stay 32 bytes");

struct GcSeg {   // one GoldenC walk segment
  int32_t pix;   // Y*512 + X (tile-global, symmetry 0 frame)
  float w;
};
struct GcEntry { // transposed entry at a symmetry-0 pixel
  int32_t pair;  // (alpha-1)*384 + raynum
  float w;
};

// Forward projection through shared-memory slabs (slab.cu).  A CTA owns
// `views` consecutive views x `rays` adjacent detectors; its rays run closer to
// one image axis, and it reads the image copy (row-major, or transposed) in
// which that axis is the row index.  The rows are cut into slabs of `rows`
// rows; the CTA stages each slab's band of columns in shared memory by TMA
// (double-buffered) and every thread walks its ray through the slab from
// there, pausing at the slab's far edge.
struct SlabPlan {
  int ok = 0;      // tables built: the fan / ray-table forward projector uses slabs
  int views = 0;   // views per CTA
  int rays = 0;    // adjacent detectors per view per CTA (a divisor of 128)
  int rows = 0;    // image rows per slab
  int wbox = 0;    // staged columns per slab: the TMA box width, a multiple of 4
  int nslab = 0;   // slabs of one copy: ceil(n / rows)
  int ndb = 0;     // CTAs per view group: ceil(ndets / rays)
  int ncta = 0;    // CTAs of one projection
  int fallback = 0;  // CTAs that gather through L1 instead (rays off the grid)
  uint4 *cta_d = nullptr;     // per CTA: x = first slab | last slab << 16 (in walk order), y = kSlab* flags
  int16_t *wlo_d = nullptr;   // [ncta][nslab]: first staged column of each slab (a multiple of 4)
};
constexpr unsigned kSlabTransposed = 1u;  // the CTA reads the transposed copy
constexpr unsigned kSlabDown = 2u;        // its rays run towards decreasing rows
constexpr unsigned kSlabFallback = 4u;    // a ray leaves the grid or runs against the others: gather through L1
constexpr unsigned kSlabEmpty = 8u;       // no ray of the CTA crosses the image

struct Plan {
  int kind = AT_GEOM_FAN;
  at_fan_geometry geom{};
  int n = 0, nviews = 0, ndets = 0;
  int nz = 1;  // image slices (a cone-beam volume has nz > 1)
  // cone beam: the geometry and, per view, cos and sin of its angle (FP32,
  // from the host libm as in the reference's rotate_2d)
  at_cone_geometry cone{};
  float2 *cone_trig_d = nullptr;
  int cone_bp_views = 0;  // views per back-projection chunk (32-bit voxel sums cannot overflow)
  int64_t rays = 0, segments = 0, offgrid = 0, device_bytes = 0;
  int max_segments = 0;
  int fp_rpt = 1;  // rays per thread of the forward projector (autotuned)
  int alpha_fp32 = 0;  // fan / ray plans traced in FP32 (the plain form) instead of FP64
  SlabPlan slab;       // fan / ray plans: the slab forward projector's tables
  // tables replaced by at_plan_set_forward_variant, kept until the plan is
  // destroyed: batches built earlier still point at them
  std::vector<SlabPlan> retired_slabs;
  // fan
  RayHdr *rays_d = nullptr;
  uint32_t *bits_d = nullptr;
  uint32_t *blk_word_d = nullptr;
  uint8_t *blk_off_d = nullptr;
  int nblocks_per_view = 0, nblocks = 0;
  // back projection: one entry per (ray, 16x16 tile) run of the traversal,
  // grouped by tile, longest runs first.  Entry = {ray, k_in | nk << 14 |
  // cx_in << 19, the run's decision bits (bit j = segment k_in + j; a run in a
  // 16x16 tile has at most 31 segments), tile-local x | y << 4 | signx << 8 |
  // signy << 9 | previous step was an x-step << 10}: the run starts at step
  // k_in after cx_in x-crossings and covers nk segments
  uint4 *run_d = nullptr;
  int32_t *tile_off_d = nullptr;  // [ntiles * nvb + 1]: runs of (tile, view block)
  int ntiles_y = 0, ntiles = 0, nvb = 0;
  int bp_term_bits = 24;           // fixed-point bits of one back-projection term
  int64_t nruns = 0;
  // back projection by pixel: the traversal's transpose, stored.  A stream is
  // one warp's 4x8 pixel block of a 16x16 tile (stream = tile * 8 + warp;
  // warp = (x%16)/4 * 2 + (y%16)/8, lane = (x%4) * 8 + y%8).  Per (stream,
  // view, lane) one word d0 | n << 15 | pre << 21: the rays of that view
  // crossing the pixel are bins view*ndets + d0 .. + n-1, and their weights
  // (0 for a ray between them that misses the pixel) sit at pt_w[view's
  // first weight in the stream + pre + k], pre = the lane's position among
  // the warp's weights of that view.  pt_woff[stream * (nch + 1) + c]: the
  // first weight of chunk c (views c*kPtChunk ..) in the stream, nch chunks.  Weights are the forward
  // walk's FP32 segment lengths bit for bit, so each fixed-point term, and
  // each pixel's integer sum, equals the tile-run back projector's.
  uint32_t *pt_meta_d = nullptr;
  float *pt_w_d = nullptr;
  int64_t *pt_woff_d = nullptr;
  int64_t pt_entries = 0, pt_bytes = 0;
  int bp_table = 0;  // launches that back-project from the table: bit0 single scans, bit1 groups
  // goldnc
  GcSeg *gc_seg_d = nullptr;
  int32_t *gc_pair_off_d = nullptr;  // [17280+1]
  GcEntry *gc_ent_d = nullptr;
  int32_t *gc_pix_off_d = nullptr;   // [512*512+1]
  ~Plan();
};

// error state (thread-local message + status)
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);
#define AT_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return ::medimg::cuda_error(_e, #expr); \
  } while (0)

// Runs f when the enclosing scope ends, on every return path: a function's
// device temporaries are released when an AT_CUDA_TRY returns early as well
// as on success.  cudaFree(nullptr) does nothing, so temporaries not yet
// allocated are harmless.
template <typename F>
struct ScopeExit {
  F f;
  ~ScopeExit() { f(); }
};
template <typename F>
ScopeExit<F> scope_exit(F f) {
  return ScopeExit<F>{f};
}

// host-side geometry tables with the reference's libm expressions
void fan_tables(const at_fan_geometry &g, double *scos, double *ssin, double *dcos, double *dsin);
int validate_fan(const at_fan_geometry &g);
int validate_cone(const at_cone_geometry &g);
void cone_trig(const at_cone_geometry &g, float2 *trig);  // per view (cos, sin)
int build_cone_plan(Plan &p, cudaStream_t st);
int cone_trace_ray(const Plan &p, int64_t ray, int32_t *h_pix, float *h_w, int32_t cap, int32_t *n_out);

// plan construction (plan.cu)
int build_fan_plan(Plan &p, cudaStream_t st, const double *h_ends = nullptr);  // h_ends: [rays][4] for AT_GEOM_RAYS
int validate_rays(int n, double pixel_mm, int nviews, int ndets, const double *h_ends);
int build_goldnc_plan(Plan &p, cudaStream_t st);
int autotune_fan(Plan &p, cudaStream_t st);
// slab forward projector (slab.cu): tables for one CTA shape; 0 and p.slab.ok
// = 0 when the shape does not fit (staged band wider than a TMA box, or the
// grid's rows not 16-byte multiples)
int build_slab_tables(Plan &p, int views, int rays, int rows, cudaStream_t st);
void free_slab_tables(SlabPlan &s);
void retire_slab_tables(Plan &p);  // moves p.slab to p.retired_slabs
// pixel table for the back projector (ptable.cu): AT_OK with p.pt_meta_d null
// when the plan's shape does not fit the table's fields (more than 32767
// detectors, 63 rays of one view through a pixel, 2047 weights of one warp's
// pixels in one view) or the table would exceed max_bytes
int build_pixel_table(Plan &p, int64_t max_bytes, cudaStream_t st);
void free_pixel_table(Plan &p);
// AT_ECUDA when a bounded wait of the slab projector ran out since the last
// call (its CTAs' outputs are void); called after a synchronisation
int check_wait_timeouts();

}  // namespace medimg

struct at_plan {
  medimg::Plan p;
};

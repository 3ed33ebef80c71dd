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

#include <cuda_runtime.h>

#include "../../include/at_engine.h"

namespace medimg {

constexpr int kRayBlock = 128;  // rays per decision-bit block (one view)
constexpr int kBpTile = 16;     // back-projection tile edge (pixels)
constexpr int kBpViewBlock = 64;  // views whose contributions share one 32-bit accumulator

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

struct Plan {
  int kind = AT_GEOM_FAN;
  at_fan_geometry geom{};
  int n = 0, nviews = 0, ndets = 0;
  int nz = 1;  // image slices (a cone-beam volume has nz > 1)
  // cone beam: the geometry and, per view, cos and sin of its angle (FP32,
  // from the host libm as in the reference's rotate_2d)
  at_cone_geometry cone{};
  float2 *cone_trig_d = nullptr;
  int64_t rays = 0, segments = 0, offgrid = 0, device_bytes = 0;
  int max_segments = 0;
  int fp_rpt = 1;  // rays per thread of the forward projector (autotuned)
  int alpha_fp32 = 0;  // fan / ray plans traced in FP32 (the plain form) instead of FP64
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

}  // namespace medimg

struct at_plan {
  medimg::Plan p;
};

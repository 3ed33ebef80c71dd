// ptable.cu -- the fan-beam plan's pixel table: its traversal stored by pixel,
// for a back projector that gathers each pixel's terms instead of adding them
// with shared-memory reductions.
//
// A back-projection term is round(w * r * 2^s) for a segment of weight w (the
// forward walk's FP32 crossing difference) on a ray with residual r.  Stored
// bit for bit, the weights give every term exactly as the tile-run walk makes
// it, and a pixel's sum of integers does not depend on the order of its terms.
// The layout is in at_internal.h (Plan::pt_*).
//
// Built once per plan on the GPU in four passes over the plan:
//   range : walk every ray; per (pixel, view) the smallest and one past the
//           largest detector whose ray crosses the pixel (32-bit atomics)
//   meta  : one warp per stream walks the views: counts, each lane's place
//           among the warp's weights (a warp scan), the views' offsets
//   base  : the streams' first weights (a scan on the host; a few thousand)
//   fill  : walk every ray again and store each segment's weight
#include <algorithm>
#include <vector>

#include "at_internal.h"

namespace medimg {

namespace {

struct PtWalk {
  int n, nviews, ndets, nbpv, ntiles_y;
  const RayHdr *hdr;
  const uint32_t *bits;
  const uint32_t *blk_word;
};

// (stream, lane) of pixel (x, y); the cell of (pixel, view) is
// (stream * nviews + view) * 32 + lane
__device__ __forceinline__ size_t pt_cell(const PtWalk &P, int x, int y, int view) {
  const int tile = (x >> 4) * P.ntiles_y + (y >> 4);
  const int warp = ((x & 15) >> 2) * 2 + ((y & 15) >> 3);
  const int lane = ((x & 3) << 3) | (y & 7);
  return ((size_t)(tile * 8 + warp) * P.nviews + view) * 32 + lane;
}

// Every in-grid segment of a ray with its weight, as the back projector's
// walk computes it: the k-th crossing is fmaf(k, len, a) of its axis, and a
// segment's weight the difference of the crossings that bound it.
template <typename F>
__device__ __forceinline__ void pt_walk(const PtWalk &P, int ray, F &&emit) {
  const RayHdr h = P.hdr[ray];
  const int view = ray / P.ndets, det = ray - view * P.ndets;
  const uint32_t *wp = P.bits + P.blk_word[view * P.nbpv + det / kRayBlock] + (det % kRayBlock);
  int x = h.xy0 & 0xffff, y = h.xy0 >> 16;
  const int sx = (h.sgn & 1) ? 1 : -1, sy = (h.sgn & 2) ? 1 : -1;
  float cxf = 0.f, cyf = 0.f, prev = 0.f;
  uint32_t word = 0;
  for (int k = 0; k < h.nseg; k++) {
    if ((k & 31) == 0) word = wp[(size_t)(k >> 5) * kRayBlock];
    const bool bx = (word >> (k & 31)) & 1u;
    const float nx = fmaf(cxf, h.lenx, h.ax), ny = fmaf(cyf, h.leny, h.ay);
    const float cur = bx ? nx : ny;
    const float wt = cur - prev;
    prev = cur;
    if ((unsigned)x < (unsigned)P.n && (unsigned)y < (unsigned)P.n) emit(x, y, view, det, wt);
    if (bx) {
      x += sx;
      cxf += 1.f;
    } else {
      y += sy;
      cyf += 1.f;
    }
  }
}

__global__ void pt_range_kernel(const PtWalk P, uint32_t *dmin, uint32_t *dend) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= P.nviews * P.ndets) return;
  pt_walk(P, ray, [&](int x, int y, int view, int det, float) {
    const size_t c = pt_cell(P, x, y, view);
    atomicMin(dmin + c, (uint32_t)det);
    atomicMax(dend + c, (uint32_t)det + 1u);
  });
}

// One warp per stream (8 per CTA).  meta is written over dmin, cell by cell.
__global__ void __launch_bounds__(256) pt_meta_kernel(int nstreams, int nviews, int nch, uint32_t *meta,
                                                      const uint32_t *dend, uint32_t *voff, int64_t *woff,
                                                      int64_t *stream_total, int *bad) {
  const int stream = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (stream >= nstreams) return;
  int64_t run = 0;
  bool wrong = false;
  for (int v = 0; v < nviews; v++) {
    if (v % kPtChunk == 0 && lane == 0) woff[(size_t)stream * (nch + 1) + v / kPtChunk] = run;
    const size_t c = ((size_t)stream * nviews + v) * 32 + lane;
    const uint32_t e = dend[c], s = meta[c];
    const uint32_t n = e ? e - s : 0u, d0 = e ? s : 0u;
    wrong |= d0 > 0x7fffu || n > 63u;
    uint32_t inc = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const uint32_t pre = inc - n, total = __shfl_sync(0xffffffffu, inc, 31);
    wrong |= pre > 2047u;
    meta[c] = (d0 & 0x7fffu) | ((n & 63u) << 15) | ((pre & 2047u) << 21);
    if (lane == 0) voff[(size_t)stream * nviews + v] = (uint32_t)run;
    run += total;
  }
  if (lane == 0) {
    woff[(size_t)stream * (nch + 1) + nch] = run;
    stream_total[stream] = run;
  }
  if (__any_sync(0xffffffffu, wrong) && lane == 0) atomicOr(bad, 1);
}

__global__ void pt_base_kernel(int nstreams, int nch, const int64_t *base, int64_t *woff) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nstreams * (nch + 1)) return;
  woff[i] += base[i / (nch + 1)];
}

__global__ void pt_fill_kernel(const PtWalk P, const uint32_t *meta, const uint32_t *voff, const int64_t *base,
                               float *w) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= P.nviews * P.ndets) return;
  pt_walk(P, ray, [&](int x, int y, int view, int det, float wt) {
    const size_t c = pt_cell(P, x, y, view);
    const size_t stream = c / ((size_t)P.nviews * 32);
    const uint32_t m = meta[c];
    const int d0 = (int)(m & 0x7fffu), pre = (int)(m >> 21);
    w[base[stream] + voff[stream * P.nviews + view] + pre + (det - d0)] = wt;
  });
}

}  // namespace

void free_pixel_table(Plan &p) {
  cudaFree(p.pt_meta_d);
  cudaFree(p.pt_w_d);
  cudaFree(p.pt_woff_d);
  p.device_bytes -= p.pt_bytes;
  p.pt_meta_d = nullptr;
  p.pt_w_d = nullptr;
  p.pt_woff_d = nullptr;
  p.pt_entries = p.pt_bytes = 0;
  p.bp_table = 0;
}

int build_pixel_table(Plan &p, int64_t max_bytes, cudaStream_t st) {
  if (p.pt_meta_d) return AT_OK;
  if ((p.kind != AT_GEOM_FAN && p.kind != AT_GEOM_RAYS) || !p.run_d || p.ndets > 0x7fff) return AT_OK;
  const int nstreams = p.ntiles * 8;
  const int nch = (p.nviews + kPtChunk - 1) / kPtChunk;
  const size_t ncell = (size_t)nstreams * p.nviews * 32;
  // at least one weight per segment: give up early on what cannot fit
  if ((int64_t)(ncell * 4 + p.segments * 4) > max_bytes) return AT_OK;
  uint32_t *meta = nullptr, *dend = nullptr, *voff = nullptr;
  int64_t *woff = nullptr, *stotal = nullptr, *base_d = nullptr;
  float *w = nullptr;
  int *bad_d = nullptr;
  bool keep = false;
  const auto free_temps = scope_exit([&] {
    cudaFree(dend);
    cudaFree(voff);
    cudaFree(stotal);
    cudaFree(base_d);
    cudaFree(bad_d);
    if (!keep) {
      cudaFree(meta);
      cudaFree(woff);
      cudaFree(w);
    }
  });
  AT_CUDA_TRY(cudaMalloc(&meta, ncell * sizeof(uint32_t)));
  AT_CUDA_TRY(cudaMalloc(&dend, ncell * sizeof(uint32_t)));
  AT_CUDA_TRY(cudaMalloc(&voff, (size_t)nstreams * p.nviews * sizeof(uint32_t)));
  AT_CUDA_TRY(cudaMalloc(&woff, (size_t)nstreams * (nch + 1) * sizeof(int64_t)));
  AT_CUDA_TRY(cudaMalloc(&stotal, (size_t)nstreams * sizeof(int64_t)));
  AT_CUDA_TRY(cudaMalloc(&base_d, (size_t)nstreams * sizeof(int64_t)));
  AT_CUDA_TRY(cudaMalloc(&bad_d, sizeof(int)));
  AT_CUDA_TRY(cudaMemsetAsync(meta, 0xff, ncell * sizeof(uint32_t), st));
  AT_CUDA_TRY(cudaMemsetAsync(dend, 0, ncell * sizeof(uint32_t), st));
  AT_CUDA_TRY(cudaMemsetAsync(bad_d, 0, sizeof(int), st));
  const PtWalk P{p.n, p.nviews, p.ndets, p.nblocks_per_view, p.ntiles_y, p.rays_d, p.bits_d, p.blk_word_d};
  const int nrays = p.nviews * p.ndets, tpb = 128;
  pt_range_kernel<<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(P, meta, dend);
  AT_CUDA_TRY(cudaGetLastError());
  pt_meta_kernel<<<(nstreams + 7) / 8, 256, 0, st>>>(nstreams, p.nviews, nch, meta, dend, voff, woff, stotal,
                                                     bad_d);
  AT_CUDA_TRY(cudaGetLastError());
  std::vector<int64_t> tot(nstreams), base(nstreams);
  int bad = 0;
  AT_CUDA_TRY(cudaMemcpyAsync(tot.data(), stotal, sizeof(int64_t) * nstreams, cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(&bad, bad_d, sizeof(int), cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  if (bad) return AT_OK;
  int64_t entries = 0;
  for (int s = 0; s < nstreams; s++) {
    base[s] = entries;
    entries += tot[s];
  }
  const int64_t bytes = (int64_t)(ncell * 4 + (size_t)nstreams * (nch + 1) * 8) + entries * 4;
  if (bytes > max_bytes) return AT_OK;
  cudaFree(dend);  // the largest temporary, before the weights are allocated
  dend = nullptr;
  AT_CUDA_TRY(cudaMalloc(&w, (size_t)(entries + 4) * sizeof(float)));
  AT_CUDA_TRY(cudaMemsetAsync(w, 0, (size_t)(entries + 4) * sizeof(float), st));
  AT_CUDA_TRY(cudaMemcpyAsync(base_d, base.data(), sizeof(int64_t) * nstreams, cudaMemcpyHostToDevice, st));
  const int nwoff = nstreams * (nch + 1);
  pt_base_kernel<<<(nwoff + 255) / 256, 256, 0, st>>>(nstreams, nch, base_d, woff);
  AT_CUDA_TRY(cudaGetLastError());
  pt_fill_kernel<<<(nrays + tpb - 1) / tpb, tpb, 0, st>>>(P, meta, voff, base_d, w);
  AT_CUDA_TRY(cudaGetLastError());
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  keep = true;
  p.pt_meta_d = meta;
  p.pt_w_d = w;
  p.pt_woff_d = woff;
  p.pt_entries = entries;
  p.pt_bytes = bytes;
  p.device_bytes += bytes;
  return AT_OK;
}

}  // namespace medimg

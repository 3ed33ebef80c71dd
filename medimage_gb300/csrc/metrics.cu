// metrics.cu -- image quality on the GPU: PSNR and SSIM.
//
// PSNR = 10 log10(peak^2 / MSE), the measure of the reference's PSNR.m
// (msbeam/CPU_OpenMP/PSNR.m:1-12; that script fixes peak = 256, callers pass
// their own peak or let it default to max(ref)).
// SSIM is the structural similarity index of Wang, Bovik, Sheikh and
// Simoncelli (IEEE TIP 2004), with the defaults the reference's ssim_index.m
// uses: an 11x11 Gaussian window of sigma 1.5, K1 = 0.01, K2 = 0.03, the
// window applied only where it fits inside the image, and the mean of the
// resulting map.  Sums are FP64.
#include <cmath>
#include <cstring>
#include <mutex>

#include "at_internal.h"

namespace medimg {
namespace {

constexpr int kWin = 11;
__constant__ double c_window[kWin * kWin];

__device__ __forceinline__ unsigned float_key(float f) {  // order-preserving float -> uint
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void psnr_partial_kernel(const float *x, const float *ref, int64_t n, double *part_sum, unsigned *part_max) {
  double s = 0.0;
  unsigned mx = 0u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = (double)x[i] - (double)ref[i];
    s += d * d;
    mx = max(mx, float_key(ref[i]));
  }
  __shared__ double ss[32];
  __shared__ unsigned sm[32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    ss[threadIdx.x >> 5] = s;
    sm[threadIdx.x >> 5] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    unsigned m = 0u;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a += ss[w];
      m = max(m, sm[w]);
    }
    part_sum[blockIdx.x] = a;
    part_max[blockIdx.x] = m;
  }
}

__global__ void ssim_partial_kernel(const float *x, const float *y, int h, int w, double c1, double c2,
                                    double *part) {
  const int ow = w - kWin + 1, oh = h - kWin + 1;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)ow * oh;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / ow), c = (int)(i % ow);
    double mx = 0, my = 0, sxx = 0, syy = 0, sxy = 0;
    for (int a = 0; a < kWin; a++)
      for (int b = 0; b < kWin; b++) {
        const double g = c_window[a * kWin + b];
        const double xv = x[(size_t)(r + a) * w + c + b], yv = y[(size_t)(r + a) * w + c + b];
        mx += g * xv;
        my += g * yv;
        sxx += g * xv * xv;
        syy += g * yv * yv;
        sxy += g * xv * yv;
      }
    const double vx = sxx - mx * mx, vy = syy - my * my, cxy = sxy - mx * my;
    acc += ((2 * mx * my + c1) * (2 * cxy + c2)) / ((mx * mx + my * my + c1) * (vx + vy + c2));
  }
  __shared__ double ss[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) ss[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) a += ss[k];
    part[blockIdx.x] = a;
  }
}

constexpr int kBlocks = 512, kThreads = 256;

}  // namespace

// device scratch of one PSNR evaluation (partial sums and maxima)
size_t psnr_scratch_bytes() { return kBlocks * (sizeof(double) + sizeof(unsigned)); }

// PSNR of d_x against d_ref (n values) on `st` with caller-owned scratch of
// psnr_scratch_bytes(); peak <= 0 takes max(ref).  Waits for the stream.
int psnr_with_scratch(const float *d_x, const float *d_ref, int64_t n, double peak, void *scratch, double *h_psnr,
                      cudaStream_t st) {
  double *psum = reinterpret_cast<double *>(scratch);
  unsigned *pmax = reinterpret_cast<unsigned *>(psum + kBlocks);
  psnr_partial_kernel<<<kBlocks, kThreads, 0, st>>>(d_x, d_ref, n, psum, pmax);
  AT_CUDA_TRY(cudaGetLastError());
  double hs[kBlocks];
  unsigned hm[kBlocks];
  AT_CUDA_TRY(cudaMemcpyAsync(hs, psum, sizeof(hs), cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaMemcpyAsync(hm, pmax, sizeof(hm), cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  double sum = 0.0;
  unsigned m = 0u;
  for (int b = 0; b < kBlocks; b++) {
    sum += hs[b];
    m = hm[b] > m ? hm[b] : m;
  }
  const unsigned u = (m & 0x80000000u) ? (m & 0x7fffffffu) : ~m;
  float maxref;
  std::memcpy(&maxref, &u, sizeof(float));
  const double pk = peak > 0 ? peak : (double)maxref;
  const double mse = sum / (double)n;
  *h_psnr = mse == 0.0 ? INFINITY : 10.0 * std::log10(pk * pk / mse);
  return AT_OK;
}

}  // namespace medimg

using namespace medimg;

#define AT_API extern "C" __attribute__((visibility("default")))

AT_API int at_psnr(const float *d_x, const float *d_ref, int64_t n, double peak, double *h_psnr, void *stream) {
  if (!d_x || !d_ref || !h_psnr || n <= 0) return set_error(AT_EINVAL, "at_psnr: bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  void *scratch = nullptr;
  const auto free_temps = scope_exit([&] {
    if (scratch) cudaFreeAsync(scratch, st);
  });
  AT_CUDA_TRY(cudaMallocAsync(&scratch, psnr_scratch_bytes(), st));
  return psnr_with_scratch(d_x, d_ref, n, peak, scratch, h_psnr, st);
}

AT_API int at_ssim(const float *d_x, const float *d_ref, int32_t h, int32_t w, double dynamic_range, double *h_ssim,
                   void *stream) {
  if (!d_x || !d_ref || !h_ssim || h < kWin || w < kWin || !(dynamic_range > 0))
    return set_error(AT_EINVAL, "at_ssim: bad argument (images must be at least 11 x 11)");
  // the constant-memory window, once per device
  static std::mutex mu;
  static bool window_ready[64] = {};
  int dev = 0;
  AT_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 0 || dev >= 64) return set_error(AT_EINVAL, "at_ssim: device index out of range");
  if (!window_ready[dev]) {
    double g[kWin * kWin], tot = 0.0;
    for (int a = 0; a < kWin; a++)
      for (int b = 0; b < kWin; b++) {
        const double da = a - (kWin - 1) / 2.0, db = b - (kWin - 1) / 2.0;
        g[a * kWin + b] = std::exp(-(da * da + db * db) / (2.0 * 1.5 * 1.5));
        tot += g[a * kWin + b];
      }
    for (double &v : g) v /= tot;
    AT_CUDA_TRY(cudaMemcpyToSymbol(c_window, g, sizeof(g)));
    window_ready[dev] = true;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const double c1 = (0.01 * dynamic_range) * (0.01 * dynamic_range);
  const double c2 = (0.03 * dynamic_range) * (0.03 * dynamic_range);
  double *part = nullptr;
  const auto free_part = scope_exit([&] {
    if (part) cudaFreeAsync(part, st);
  });
  AT_CUDA_TRY(cudaMallocAsync(&part, sizeof(double) * kBlocks, st));
  ssim_partial_kernel<<<kBlocks, kThreads, 0, st>>>(d_x, d_ref, h, w, c1, c2, part);
  AT_CUDA_TRY(cudaGetLastError());
  double hp[kBlocks];
  AT_CUDA_TRY(cudaMemcpyAsync(hp, part, sizeof(hp), cudaMemcpyDeviceToHost, st));
  AT_CUDA_TRY(cudaStreamSynchronize(st));
  double s = 0.0;
  for (double v : hp) s += v;
  *h_ssim = s / ((double)(h - kWin + 1) * (w - kWin + 1));
  return AT_OK;
}

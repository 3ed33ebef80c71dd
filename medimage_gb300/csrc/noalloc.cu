// noalloc.cu -- forward projection with the fused residual and data-term
// energy, for callers that may not allocate device memory.
//
// Who needs it: programs whose device memory belongs to someone else's pool
// (a host framework with its own caching allocator and a fixed budget, where a
// stray cudaMalloc fragments or overruns that budget), and loops that cannot
// afford cudaMalloc/cudaFree at all because those calls synchronise the device
// and stall every other stream.  Such a caller brings its own input and output
// buffers; the only device memory this entry point needs beyond them -- the
// per-CTA partial sums and the arrival counter of the fused FP64 reduction --
// lives in one fixed array compiled into the library.
//
// The array has a stated size (kScratchBytes).  Every GPU that loads the
// library holds it until the process exits.  Calls share it and it keeps the
// previous call's contents, so each call clears the part that must start at
// zero; two calls whose work overlaps on the GPU (different streams, no
// ordering between them) race on it and must not be issued.
//
// The array's device address is looked up once per device, by the first call
// made on that device with the device current (cudaGetSymbolAddress); that
// first call should therefore happen before any stream capture begins.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "solver.h"

namespace medimg {

int fp_ctas(const ScanDev &S, int rpt);
cudaError_t launch_fp(const Launch &L, int kind, int rpt, int nctas, cudaStream_t st);

namespace {

constexpr size_t kScratchBytes = 256 * 1024;
constexpr size_t kCtlBytes = (sizeof(Ctl) + 255) & ~size_t(255);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices];

// device address of g_noalloc_scratch on the current device
int scratch_address(void **out) {
  int dev = 0;
  AT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(AT_EINVAL, "no-alloc forward: device index out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return AT_OK;
}

}  // namespace
}  // namespace medimg

using namespace medimg;

extern "C" __attribute__((visibility("default"))) int at_forward_residual_noalloc(const at_plan *plan,
                                                                                   const float *d_img,
                                                                                   const float *d_g, float *d_r,
                                                                                   double *d_energy, void *stream) {
  if (!plan || !d_img || !d_g || !d_r || !d_energy)
    return set_error(AT_EINVAL, "at_forward_residual_noalloc: null argument");
  const Plan &p = plan->p;
  Launch L;
  std::memset(&L, 0, sizeof(L));
  fill_scan_plan(L.single, p);
  const int rpt = p.fp_rpt;  // the plan's autotuned forward-projector variant
  const int nctas = fp_ctas(L.single, rpt);
  const size_t need = kCtlBytes + sizeof(double) * (size_t)nctas;
  if (need > kScratchBytes) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "at_forward_residual_noalloc: this geometry's forward projection runs %d CTAs and needs %zu "
                  "bytes of scratch; the fixed no-alloc array holds %zu bytes",
                  nctas, need, kScratchBytes);
    return set_error(AT_EINVAL, msg);
  }
  void *base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  Ctl *ctl = (Ctl *)base;
  // the reduction's arrival counter and result must start from zero
  AT_CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st));
  L.single.buf[B_F] = const_cast<float *>(d_img);
  L.single.buf[B_G] = const_cast<float *>(d_g);
  L.single.buf[B_R] = d_r;
  L.single.ctl = ctl;
  L.single.partials = (double *)((char *)base + kCtlBytes);
  L.nscans = 1;
  L.flow = FLOW_ALWAYS;
  L.stage = ST_FP0;  // r = g - A img, energy = sum (A img - g)^2 in FP64
  L.in_buf = B_F;
  L.out_buf = B_R;
  L.aux_buf = -1;
  const cudaError_t e = launch_fp(L, p.kind, rpt, nctas, st);
  if (e != cudaSuccess) return cuda_error(e, "no-alloc forward projection launch");
  AT_CUDA_TRY(cudaMemcpyAsync(d_energy, &ctl->e_data, sizeof(double), cudaMemcpyDeviceToDevice, st));
  return AT_OK;
}

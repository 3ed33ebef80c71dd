// at_step.cu -- pixel and sinogram passes of the AT iteration
// (origin/GoldenC/src/main.c:81-390) for a batch of scans.
//
// Pixel passes use tiles of kPixRows x 32 pixels (x rows, y columns; 256
// threads, each taking kPixRows / 8 rows of the tile, 8 apart), so a CTA's
// fixed costs (control-block reads, its reduction, fence and arrival ticket)
// are spread over several pixels per thread; a volume (nz > 1 slices, the
// cone beam) has the tiles of each slice in turn.
// On volumes the stencils gain the z neighbours (gradients, Laplacian,
// smoothness energy); the median stays GoldenC's 3x3 within each slice.  Each
// pass fuses the elementwise update with the reductions the next scalar step
// needs; neighbours of freshly computed values are recomputed from their
// inputs instead of being re-read, so no pass waits on another one.
#include <cuda_runtime.h>

#include "solver_dev.cuh"

namespace medimg {

struct PixCoord {
  int x, y, z, i, base;  // base: index of the slice's first pixel
  bool inside;
};

// this thread's pixel in row group j (0 <= j < kPixRows / 8) of the CTA's tile
__device__ __forceinline__ PixCoord pix_of(int n, int local_cta, int j) {
  const int tiles_y = (n + 31) >> 5, tiles = ((n + kPixRows - 1) / kPixRows) * tiles_y;
  PixCoord c;
  c.z = local_cta / tiles;
  const int t = local_cta % tiles;
  c.x = (t / tiles_y) * kPixRows + j * 8 + (threadIdx.x >> 5);
  c.y = (t % tiles_y) * 32 + (threadIdx.x & 31);
  c.inside = c.x < n && c.y < n;
  c.base = c.z * n * n;
  c.i = c.base + c.x * n + c.y;
  return c;
}

// f(c) for each of this thread's pixels
template <typename F>
__device__ __forceinline__ void for_my_pixels(int n, int local_cta, F &&f) {
#pragma unroll
  for (int j = 0; j < kPixRows / 8; j++) f(pix_of(n, local_cta, j));
}

#define AT_SCAN_PROLOGUE                                                              \
  const int scan = find_scan(L.prefix, L.nscans, blockIdx.x);                         \
  const ScanDev &S = L.scans[scan];                                                   \
  if (!flow_active(S, L.flow)) return;                                                \
  const int cta0 = __ldg(L.prefix + scan);                                            \
  const int ncta = __ldg(L.prefix + scan + 1) - cta0;                                 \
  const int local_cta = blockIdx.x - cta0;                                            \
  (void)ncta;

__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// max over the CTA into the scan's control block, one atomic per CTA (the
// scan's CTAs all add to one address).  Thread 0's atomic precedes its fence
// and arrival ticket in reduce_and_finalize, so the last CTA sees every CTA's
// maximum.  Must be reached by every thread of the CTA.
__device__ __forceinline__ void cta_max_to_ctl(const ScanDev &S, float x) {
  __shared__ float wm[32];
  x = warp_max_f(x);
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = wm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, wm[w]);
    if (m > 0.f) atomic_max_nonneg(&S.ctl->maxbits, m);
  }
}

__device__ __forceinline__ void sort2(float &a, float &b) {
  const float lo = fminf(a, b), hi = fmaxf(a, b);
  a = lo;
  b = hi;
}
__device__ __forceinline__ float med3(float a, float b, float c) {
  return fmaxf(fminf(a, b), fminf(fmaxf(a, b), c));
}

// Median of a 3x3 window: sort each row, then the median of nine is the median
// of (largest row minimum, median of row medians, smallest row maximum).
__device__ __forceinline__ float median9(float r0[3], float r1[3], float r2[3]) {
  float *rows[3] = {r0, r1, r2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float *r = rows[k];
    sort2(r[0], r[1]);
    sort2(r[1], r[2]);
    sort2(r[0], r[1]);
  }
  const float a = fmaxf(fmaxf(r0[0], r1[0]), r2[0]);
  const float b = med3(r0[1], r1[1], r2[1]);
  const float c = fminf(fminf(r0[2], r1[2]), r2[2]);
  return med3(a, b, c);
}

// update_next = update_cur + c1 p, 3x3 median (zero padding) when flag is set;
// maxCP = max |c1 p|.  main.c:169-191, 366-390.
__global__ void __launch_bounds__(256) upd_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const int n = S.n;
  const float *__restrict__ u = S.buf[L.aux_buf];
  const float *__restrict__ p = S.buf[L.in_buf];
  float *__restrict__ out = S.buf[L.out_buf];
  const float c1 = (float)S.ctl->c1;
  float cp = 0.f;
  for_my_pixels(n, local_cta, [&](const PixCoord &c) {
      if (!c.inside) return;
      const float pc = p[c.i];
      cp = fmaxf(cp, fabsf(c1 * pc));
      if (!L.flag) {
        out[c.i] = fmaf(c1, pc, u[c.i]);
      } else {
        float w[3][3];
  #pragma unroll
        for (int dx = -1; dx <= 1; dx++)
  #pragma unroll
          for (int dy = -1; dy <= 1; dy++) {
            const int xx = c.x + dx, yy = c.y + dy;
            float val = 0.f;
            if (xx >= 0 && xx < n && yy >= 0 && yy < n) {
              const int j = c.base + xx * n + yy;
              val = fmaf(c1, p[j], u[j]);
            }
            w[dx + 1][dy + 1] = val;
          }
        out[c.i] = median9(w[0], w[1], w[2]);
      }
  });
  cta_max_to_ctl(S, cp);
  reduce_and_finalize<0>(S, L, nullptr, local_cta, ncta);
}

// p_new = d + c2 p_old (p_new = d on the first pass), nV = sum over all pixels
// (v^2 + 0.01 eps^2) |backward grad p_new|^2 (p zero-padded), pd = <p_new, d>.
// main.c:141-162, 247-250.
__global__ void __launch_bounds__(256) pp_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const int n = S.n;
  const float *__restrict__ d = S.buf[B_D];
  const float *__restrict__ po = S.buf[L.in_buf];
  const float *__restrict__ v = S.buf[B_V];
  float *__restrict__ pn = S.buf[L.out_buf];
  const bool first = L.flag != 0;
  const float c2 = first ? 0.f : (float)S.ctl->c2;
  const float eps2 = (float)(0.01 * S.ctl->eps * S.ctl->eps);
  FF sums[2] = {ff_zero(), ff_zero()};
  for_my_pixels(n, local_cta, [&](const PixCoord &c) {
    if (!c.inside) return;
    auto pnew = [&](int j) -> float { return first ? d[j] : fmaf(c2, po[j], d[j]); };
    const float dc = d[c.i];
    const float pc = pnew(c.i);
    pn[c.i] = pc;
    const float pu = c.x > 0 ? pnew(c.i - n) : 0.f;
    const float pl = c.y > 0 ? pnew(c.i - 1) : 0.f;
    const float vv = v[c.i];
    const float a = pc - pu, b = pc - pl;  // non-negative terms, rounded in FP32
    if (S.nz == 1) {
      ff_acc(sums[0], ff_of(fmaf(vv, vv, eps2) * fmaf(a, a, b * b)));
    } else {
      const float pf = c.z > 0 ? pnew(c.i - n * n) : 0.f;
      const float cz = pc - pf;
      ff_acc(sums[0], ff_of(fmaf(vv, vv, eps2) * fmaf(a, a, fmaf(b, b, cz * cz))));
    }
    ff_acc(sums[1], ff_prod(pc, dc));  // exact
  });
  reduce_and_finalize<2>(S, L, sums, local_cta, ncta);
}

// F = U1 when the image step ended in update buffer 1.
__global__ void __launch_bounds__(256) commit_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  if (S.ctl->final_u != 1) return;
  for_my_pixels(S.n, local_cta, [&](const PixCoord &c) {
    if (c.inside) S.buf[B_F][c.i] = S.buf[B_U1][c.i];
  });
}

// |grad f|^2 with central differences, f zero-padded (main.c:296-298).
__global__ void __launch_bounds__(256) edge_init_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const int n = S.n;
  const float *__restrict__ f = S.buf[B_F];
  for_my_pixels(n, local_cta, [&](const PixCoord &c) {
    if (!c.inside) return;
    const float fd = c.x + 1 < n ? f[c.i + n] : 0.f, fu = c.x > 0 ? f[c.i - n] : 0.f;
    const float fr = c.y + 1 < n ? f[c.i + 1] : 0.f, fl = c.y > 0 ? f[c.i - 1] : 0.f;
    const float gx = 0.5f * (fd - fu), gy = 0.5f * (fr - fl);
    if (S.nz == 1) {
      S.buf[B_NN][c.i] = gx * gx + gy * gy;
    } else {
      const int nn = n * n;
      const float fb = c.z + 1 < S.nz ? f[c.i + nn] : 0.f, ff = c.z > 0 ? f[c.i - nn] : 0.f;
      const float gz = 0.5f * (fb - ff);
      S.buf[B_NN][c.i] = gx * gx + gy * gy + gz * gz;
    }
  });
}

// d = -(alpha v n - beta eps lap/4 v + beta (v-1)/(4 eps)), v one-padded
// (main.c:299-309); sums nD, sum n d^2, nNablaD (d zero-padded, main.c:314-328).
__global__ void __launch_bounds__(256) edge_d_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const int n = S.n;
  const float *__restrict__ v = S.buf[B_V];
  const float *__restrict__ nn = S.buf[B_NN];
  const Ctl *ct = S.ctl;
  const float alpha = (float)ct->alpha, beq = (float)(ct->beta * ct->eps);
  const float b4 = (float)(ct->beta / (4 * ct->eps));
  FF sums[3] = {ff_zero(), ff_zero(), ff_zero()};
  for_my_pixels(n, local_cta, [&](const PixCoord &c) {
    if (c.inside && S.nz == 1) {
      auto vat = [&](int xx, int yy) -> float {
        return (xx >= 0 && xx < n && yy >= 0 && yy < n) ? v[xx * n + yy] : 1.f;
      };
      auto dat = [&](int xx, int yy) -> float {
        if (xx < 0 || xx >= n || yy < 0 || yy >= n) return 0.f;
        const float vc = v[xx * n + yy];
        const float lap = 0.25f * (vat(xx + 1, yy) + vat(xx, yy + 1) - 4.f * vc + vat(xx - 1, yy) + vat(xx, yy - 1));
        const float g = alpha * vc * nn[xx * n + yy] - beq * lap + b4 * (vc - 1.f);
        return -g;
      };
      const float dc = dat(c.x, c.y);
      S.buf[B_D][c.i] = dc;
      // non-negative terms, rounded in FP32 (d^2 exactly)
      ff_acc(sums[0], ff_prod(dc, dc));
      ff_acc(sums[1], ff_of(nn[c.i] * (dc * dc)));
      const float gx = 0.5f * (dat(c.x + 1, c.y) - dat(c.x - 1, c.y));
      const float gy = 0.5f * (dat(c.x, c.y + 1) - dat(c.x, c.y - 1));
      ff_acc(sums[2], ff_of(fmaf(gx, gx, gy * gy)));
    } else if (c.inside) {
      // volumes: six-neighbour Laplacian scaled by 1/6, central differences in z
      const int nz = S.nz;
      auto vat = [&](int zz, int xx, int yy) -> float {
        return (zz >= 0 && zz < nz && xx >= 0 && xx < n && yy >= 0 && yy < n) ? v[(zz * n + xx) * n + yy] : 1.f;
      };
      auto dat = [&](int zz, int xx, int yy) -> float {
        if (zz < 0 || zz >= nz || xx < 0 || xx >= n || yy < 0 || yy >= n) return 0.f;
        const int j = (zz * n + xx) * n + yy;
        const float vc = v[j];
        const float lap = (1.f / 6.f) * (vat(zz, xx + 1, yy) + vat(zz, xx, yy + 1) + vat(zz + 1, xx, yy) - 6.f * vc +
                                        vat(zz, xx - 1, yy) + vat(zz, xx, yy - 1) + vat(zz - 1, xx, yy));
        const float g = alpha * vc * nn[j] - beq * lap + b4 * (vc - 1.f);
        return -g;
      };
      const float dc = dat(c.z, c.x, c.y);
      S.buf[B_D][c.i] = dc;
      ff_acc(sums[0], ff_prod(dc, dc));
      ff_acc(sums[1], ff_of(nn[c.i] * (dc * dc)));
      const float gx = 0.5f * (dat(c.z, c.x + 1, c.y) - dat(c.z, c.x - 1, c.y));
      const float gy = 0.5f * (dat(c.z, c.x, c.y + 1) - dat(c.z, c.x, c.y - 1));
      const float gz = 0.5f * (dat(c.z + 1, c.x, c.y) - dat(c.z - 1, c.x, c.y));
      ff_acc(sums[2], ff_of(fmaf(gx, gx, fmaf(gy, gy, gz * gz))));
    }
  });
  reduce_and_finalize<3>(S, L, sums, local_cta, ncta);
}

// v = clamp(v + c d, 0, 1); maxCD = max |c d| (main.c:332-344).
__global__ void __launch_bounds__(256) edge_upd_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const float cc = (float)S.ctl->c;
  float cd = 0.f;
  float *v = S.buf[B_V];
  const float *dd = S.buf[B_D];
  for_my_pixels(S.n, local_cta, [&](const PixCoord &c) {
    if (!c.inside) return;
    const float step = cc * dd[c.i];
    cd = fmaxf(cd, fabsf(step));
    v[c.i] = fminf(fmaxf(v[c.i] + step, 0.f), 1.f);
  });
  cta_max_to_ctl(S, cd);
  reduce_and_finalize<0>(S, L, nullptr, local_cta, ncta);
}

// linear mode: q = Ad + c2 q with |q|^2 (ST_SQ) or Af += c1 q, r -= c1 q with
// E_data (ST_SA).  256 bins per CTA.
__global__ void __launch_bounds__(256) sino_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  const int b = local_cta * 256 + threadIdx.x;
  FF s[1] = {ff_zero()};
  if (b < S.nbins) {
    float *q = S.buf[B_Q];
    if (L.stage == ST_SQ) {
      const float qn = fmaf((float)S.ctl->c2, q[b], S.buf[B_AD][b]);
      q[b] = qn;
      s[0] = ff_prod(qn, qn);
    } else {
      const float c1 = (float)S.ctl->c1;
      const float qb = q[b];
      const float af = fmaf(c1, qb, S.buf[B_AF][b]);
      S.buf[B_AF][b] = af;
      S.buf[B_R][b] = S.buf[B_R][b] - c1 * qb;
      const float dv = af - S.buf[B_G][b];
      s[0] = ff_prod(dv, dv);
    }
  }
  reduce_and_finalize<1>(S, L, s, local_cta, ncta);
}

// f = 0, v = 1 (main.c:36-40).
__global__ void __launch_bounds__(256) init_state_kernel(const Launch L) {
  AT_SCAN_PROLOGUE
  for_my_pixels(S.n, local_cta, [&](const PixCoord &c) {
    if (!c.inside) return;
    S.buf[B_F][c.i] = 0.f;
    S.buf[B_V][c.i] = 1.f;
  });
}

// step boundaries: flag 0 = begin image step, 1 = begin edge step.
__global__ void flags_kernel(const ScanDev *scans, int nscans, int mode) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nscans) return;
  Ctl *c = scans[s].ctl;
  if (!c->enabled) return;
  c->arrive = 0u;
  c->maxbits = 0u;
  c->k = 1;
  if (mode == 0) {
    c->outer += 1;
    c->img_active = 1;
    c->final_u = 0;
  } else {
    c->edge_active = 1;
  }
}

cudaError_t launch_pixel(int which, const Launch &L, int nctas, cudaStream_t st) {
  switch (which) {
    case 0: upd_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 1: pp_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 2: commit_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 3: edge_init_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 4: edge_d_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 5: edge_upd_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 6: sino_kernel<<<nctas, 256, 0, st>>>(L); break;
    case 7: init_state_kernel<<<nctas, 256, 0, st>>>(L); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_flags(const ScanDev *scans, int nscans, int mode, cudaStream_t st) {
  flags_kernel<<<(nscans + 63) / 64, 64, 0, st>>>(scans, nscans, mode);
  return cudaGetLastError();
}

}  // namespace medimg

namespace medimg {

// Standalone 3x3 median with zero padding (main.c:366-390), out of place.
__global__ void __launch_bounds__(256) median_kernel(const float *__restrict__ in, float *__restrict__ out, int n) {
  const int y = blockIdx.x * 32 + (threadIdx.x & 31);
  const int x = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= n || y >= n) return;
  float w[3][3];
#pragma unroll
  for (int dx = -1; dx <= 1; dx++)
#pragma unroll
    for (int dy = -1; dy <= 1; dy++) {
      const int xx = x + dx, yy = y + dy;
      w[dx + 1][dy + 1] = (xx >= 0 && xx < n && yy >= 0 && yy < n) ? in[xx * n + yy] : 0.f;
    }
  out[x * n + y] = median9(w[0], w[1], w[2]);
}

cudaError_t launch_median(const float *in, float *out, int n, cudaStream_t st) {
  dim3 grid((n + 31) / 32, (n + 7) / 8);
  median_kernel<<<grid, 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

}  // namespace medimg

namespace medimg {

__global__ void fill_kernel(float *p, float v, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

cudaError_t launch_fill(float *p, float v, size_t n, cudaStream_t st) {
  fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
  return cudaGetLastError();
}

}  // namespace medimg

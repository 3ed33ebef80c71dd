// epilogue.cuh -- the solver's fused projector epilogues, shared by the 2D
// (project.cu) and 3D (cone.cu) projectors.
#pragma once

#include "solver_dev.cuh"

namespace medimg {

// ---------------------------------------------------------------------------
// epilogues
// ---------------------------------------------------------------------------
// Sums are float-float (FF): squares and products of floats are exact;
// val - g is rounded once to FP32 before it is squared.
__device__ __forceinline__ void fp_epilogue(const ScanDev &S, const Launch &L, int bin, float val, FF &s0) {
  switch (L.stage) {
    case ST_FP0: {  // r = g - Af ; E_data
      const float g = S.buf[B_G][bin];
      const float rr = g - val;
      S.buf[B_R][bin] = rr;
      ff_acc(s0, ff_prod(rr, rr));
      if (L.aux_buf >= 0) S.buf[L.aux_buf][bin] = val;
      break;
    }
    case ST_FPQ:  // q = A p ; |q|^2
      S.buf[B_Q][bin] = val;
      ff_acc(s0, ff_prod(val, val));
      break;
    case ST_FPA: {  // E_data ; r -= c1 q
      const float g = S.buf[B_G][bin];
      const float dv = val - g;
      ff_acc(s0, ff_prod(dv, dv));
      const float c1 = (float)S.ctl->c1;
      S.buf[B_R][bin] = S.buf[B_R][bin] - c1 * S.buf[B_Q][bin];
      if (L.aux_buf >= 0) S.buf[L.aux_buf][bin] = val;
      break;
    }
    case ST_FPD:  // <A d, q>
      ff_acc(s0, ff_prod(val, S.buf[B_Q][bin]));
      if (L.aux_buf >= 0) S.buf[L.aux_buf][bin] = val;
      break;
    default:
      S.buf[L.out_buf][bin] = val;
      break;
  }
}

__device__ __forceinline__ bool stage_reduces(int stage) {
  return stage == ST_FP0 || stage == ST_FPQ || stage == ST_FPA || stage == ST_FPD || stage == ST_BP0 ||
         stage == ST_BPD;
}

// d = A^T r + alpha * div-stencil (main.c:112-125, 226-239) and the smoothness
// energy over the interior (main.c:135-139, 203-208), for an image (z = 0,
// nz = 1) or slice z of a volume.
__device__ __forceinline__ void bp_epilogue(const ScanDev &S, const Launch &L, int z, int x, int y, float val,
                                            FF &s0) {
  const int n = S.n;
  const int i = (z * n + x) * n + y;
  if (L.stage != ST_BP0 && L.stage != ST_BPD) {
    S.buf[L.out_buf][i] = val;
    return;
  }
  const float *u = S.buf[L.aux_buf];  // the update the stencil acts on
  const float *v = S.buf[B_V];
  const Ctl *c = S.ctl;
  const float alpha = (float)c->alpha;
  const float eps2 = (float)(0.01 * c->eps * c->eps);
  const float Pc = v[i];
  const float Pu = x > 0 ? v[i - n] : 1.f;
  const float Pl = y > 0 ? v[i - 1] : 1.f;
  const float Tc = u[i];
  const float Td = x + 1 < n ? u[i + n] : 0.f;
  const float Tr = y + 1 < n ? u[i + 1] : 0.f;
  const float Tu = x > 0 ? u[i - n] : 0.f;
  const float Tl = y > 0 ? u[i - 1] : 0.f;
  const float Pc2 = Pc * Pc;
  if (S.nz == 1) {
    const float st = Pc2 * (Td - Tc) + Pc2 * (Tr - Tc) - Pu * Pu * (Tc - Tu) - Pl * Pl * (Tc - Tl) +
                     eps2 * (Td + Tr - 4.f * Tc + Tu + Tl);
    S.buf[B_D][i] = val + alpha * st;
    if (x >= 1 && x <= n - 2 && y >= 1 && y <= n - 2) {
      const float a = Tc - Tu, b = Tc - Tl;  // a non-negative term, rounded in FP32
      ff_acc(s0, ff_of(alpha * (Pc2 + eps2) * fmaf(a, a, b * b)));
    }
    return;
  }
  // volumes: the same stencil with the z neighbours (u zero-padded, v
  // one-padded), the energy over the interior in z as well
  const int nn = n * n;
  const float Pf = z > 0 ? v[i - nn] : 1.f;
  const float Tb = z + 1 < S.nz ? u[i + nn] : 0.f;
  const float Tf = z > 0 ? u[i - nn] : 0.f;
  const float st = Pc2 * (Td - Tc) + Pc2 * (Tr - Tc) + Pc2 * (Tb - Tc) - Pu * Pu * (Tc - Tu) -
                   Pl * Pl * (Tc - Tl) - Pf * Pf * (Tc - Tf) + eps2 * (Td + Tr + Tb - 6.f * Tc + Tu + Tl + Tf);
  S.buf[B_D][i] = val + alpha * st;
  if (x >= 1 && x <= n - 2 && y >= 1 && y <= n - 2 && z >= 1 && z <= S.nz - 2) {
    const float a = Tc - Tu, b = Tc - Tl, cz = Tc - Tf;
    ff_acc(s0, ff_of(alpha * (Pc2 + eps2) * fmaf(a, a, fmaf(b, b, cz * cz))));
  }
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
  const float y = x - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

}  // namespace medimg

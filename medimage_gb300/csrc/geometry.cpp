// geometry.cpp -- host-side geometry tables and validation.
//
// Built with -ffp-contract=off so the trig arguments are rounded exactly as in
// the reference (x86-64 and aarch64 alike); the FP64 traversal on the GPU
// starts from these values.
#include <cmath>
#include <string>

#include "at_internal.h"

namespace medimg {

// helical/rebin/src/ms2d.cpp:43-54: source angle table (degrees -> cos/sin)
// and the equiangular detector table with OFF_CENTER.
void fan_tables(const at_fan_geometry &g, double *scos, double *ssin, double *dcos, double *dsin) {
  for (int v = 0; v < g.nviews; v++) {
    const double angle = g.view0_deg + v * g.view_step_deg;
    scos[v] = std::cos(angle / 180.0 * M_PI);
    ssin[v] = std::sin(angle / 180.0 * M_PI);
  }
  const double per_rad = g.det_pitch_deg * M_PI / 180.;
  const int half = g.ndets / 2;
  for (int j = -half; j < half; ++j) {
    dcos[j + half] = std::cos((j + g.off_center) * per_rad + M_PI);
    dsin[j + half] = std::sin((j + g.off_center) * per_rad + M_PI);
  }
}

int validate_fan(const at_fan_geometry &g) {
  if (g.n < 8 || g.n > 8191) return set_error(AT_EINVAL, "fan geometry: n must be in [8, 8191]");
  if (g.nviews < 1 || g.nviews > 65536) return set_error(AT_EINVAL, "fan geometry: nviews must be in [1, 65536]");
  if (g.ndets < 2 || g.ndets > 49152 || (g.ndets & 1))
    return set_error(AT_EINVAL, "fan geometry: ndets must be even and in [2, 49152]");
  if (!(g.pixel_mm > 0) || !(g.sdd_mm > g.sod_mm) || !(g.det_pitch_deg > 0))
    return set_error(AT_EINVAL, "fan geometry: need pixel_mm > 0, sdd_mm > sod_mm, det_pitch_deg > 0");
  const double r = g.n * g.pixel_mm * std::sqrt(2.0) / 2.0;
  if (!(g.sod_mm > r * 1.0001))
    return set_error(AT_EINVAL, "fan geometry: the source circle must lie outside the image");
  const double half_fan_rad = (g.ndets / 2 + std::fabs(g.off_center)) * g.det_pitch_deg * M_PI / 180.0;
  if (half_fan_rad >= M_PI / 2) return set_error(AT_EINVAL, "fan geometry: fan angle must stay below 180 degrees");
  if ((int64_t)g.nviews * g.ndets > (1ll << 31) / 2) return set_error(AT_EINVAL, "fan geometry: too many rays");
  return AT_OK;
}

int validate_rays(int n, double pixel_mm, int nviews, int ndets, const double *h_ends) {
  if (n < 8 || n > 8191) return set_error(AT_EINVAL, "ray table: n must be in [8, 8191]");
  if (nviews < 1 || nviews > 65536) return set_error(AT_EINVAL, "ray table: nviews must be in [1, 65536]");
  if (ndets < 1 || ndets > 49152) return set_error(AT_EINVAL, "ray table: ndets must be in [1, 49152]");
  if (!(pixel_mm > 0) || !std::isfinite(pixel_mm)) return set_error(AT_EINVAL, "ray table: need pixel_mm > 0");
  if ((int64_t)nviews * ndets > (1ll << 31) / 2) return set_error(AT_EINVAL, "ray table: too many rays");
  // the traversal indexes cells as doubles divided by the pixel size; end
  // points far outside the grid would overflow the int cell index
  const double lim = 1e6 * n * pixel_mm;
  for (int64_t r = 0; r < (int64_t)nviews * ndets; r++) {
    const double *e = h_ends + 4 * r;
    for (int k = 0; k < 4; k++)
      if (!std::isfinite(e[k]) || std::fabs(e[k]) > lim)
        return set_error(AT_EINVAL, "ray table: end point not finite or too far from the grid");
    if (e[0] == e[2] && e[1] == e[3]) return set_error(AT_EINVAL, "ray table: source and detector coincide");
  }
  return AT_OK;
}

// industry3d/src/tracing.cpp:57 and utility.cpp:84: theta =
// (float)alpha/NPROJ*2*PI with the product by PI in double, then the float
// overloads of cos and sin (cosf, sinf)
void cone_trig(const at_cone_geometry &g, float2 *trig) {
  constexpr double kPi = 3.1415926535897932385;  // ct3d.h:8
  for (int a = 0; a < g.nproj; a++) {
    const float t = (float)a / (float)g.nproj * 2;
    const float theta = (float)((double)t * kPi);
    trig[a] = make_float2(std::cos(theta), std::sin(theta));
  }
}

int validate_cone(const at_cone_geometry &g) {
  if (g.nx != g.ny) return set_error(AT_EINVAL, "cone geometry: nx must equal ny");
  if (g.nx < 8 || g.nx > 4096 || g.nz < 1 || g.nz > 4096)
    return set_error(AT_EINVAL, "cone geometry: nx in [8, 4096], nz in [1, 4096]");
  if ((int64_t)g.nx * g.ny * g.nz > 2147483647ll) return set_error(AT_EINVAL, "cone geometry: volume above 2^31 voxels");
  if (g.nproj < 1 || g.ndx < 1 || g.ndy < 1) return set_error(AT_EINVAL, "cone geometry: need nproj, ndx, ndy >= 1");
  if ((int64_t)g.nproj * g.ndx * g.ndy > 2147483647ll) return set_error(AT_EINVAL, "cone geometry: above 2^31 rays");
  if (!(g.voxel_mm > 0) || !(g.pitch_mm > 0) || !std::isfinite(g.voxel_mm) || !std::isfinite(g.pitch_mm))
    return set_error(AT_EINVAL, "cone geometry: need voxel_mm > 0 and pitch_mm > 0");
  if (!(g.sod_mm > 0) || !(g.sdd_mm > g.sod_mm) || !std::isfinite(g.sdd_mm))
    return set_error(AT_EINVAL, "cone geometry: need 0 < sod_mm < sdd_mm");
  const double half_diag = 0.5 * g.voxel_mm * std::sqrt(2.0 * (double)g.nx * g.nx + (double)g.nz * g.nz);
  if (!(g.sod_mm > half_diag)) return set_error(AT_EINVAL, "cone geometry: the source must lie outside the volume");
  return AT_OK;
}

}  // namespace medimg

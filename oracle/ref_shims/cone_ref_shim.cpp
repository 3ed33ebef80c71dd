// C entry points into the reference's industry3d/src/tracing.cpp and
// utility.cpp (compiled unchanged) for pinning the cone-beam restatement.
// Test infrastructure only.
#include <cstdint>

#include "ct3d.h"
#include "tracing.h"

namespace {
Parameter make(int nx, int ny, int nz, float voxel, int nproj, int ndx, int ndy, float pitch, float sod, float sdd) {
    Parameter a;
    a.NX = nx;
    a.NY = ny;
    a.NZ = nz;
    a.SAMPLESIZE = voxel;
    a.NPROJ = nproj;
    a.NDX = ndx;
    a.NDY = ndy;
    a.PIXELSIZE = pitch;
    a.SOD = sod;
    a.SDD = sdd;
    a.BEAM = "Cone";
    // the derived fields of ct3d.cpp:88-93 (that file needs Boost's JSON parser)
    a.HALFDET = ndx / 2;
    a.HALFSIZE = nx / 2.0;
    a.MAX_RAYLEN = nx * 3;
    return a;
}
}  // namespace

extern "C" void coneref_endpoints(int nx, int ny, int nz, float voxel, int nproj, int ndx, int ndy, float pitch,
                                  float sod, float sdd, int view, int row, int col, float *s, float *d) {
    Parameter a = make(nx, ny, nz, voxel, nproj, ndx, ndy, pitch, sod, sdd);
    cone(a, view, row, col, s[0], s[1], s[2], d[0], d[1], d[2]);
}

extern "C" int coneref_trace(int nx, int ny, int nz, float sx, float sy, float sz, float dx, float dy, float dz,
                             int64_t *ind, float *wgt) {
    Parameter a = make(nx, ny, nz, 1.f, 1, 2, 2, 1.f, 1.f, 2.f);
    int numb = 0;
    forward_proj(a, sx, sy, sz, dx, dy, dz, ind, wgt, numb);
    return numb;
}

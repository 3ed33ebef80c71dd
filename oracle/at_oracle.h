/*
 * at_oracle.h -- CPU oracle for the Ambrosio-Tortorelli reconstruction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is an FP64 C restatement of the reference's
 * algorithms, used as the checker for the CUDA engine.  Only tests/,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py may load it.
 * The engine never links, loads or calls it.
 *
 * What it restates (paths relative to the reference project root):
 *   - GoldenC parallel-beam projector pair A / AStar   origin/GoldenC/src/proj.c:14-397
 *   - GoldenC AT solver (image CG step, edge step,     origin/GoldenC/src/main.c:35-390
 *     3x3 median, outer alternation)
 *   - 2D fan-beam Siddon tracer                        helical/rebin/src/tracing.cpp:22-147
 *   - fan geometry tables and ray end points           helical/rebin/src/ms2d.cpp:30-62,172-183
 *
 * Parity pin: tests compare this oracle bit-for-bit with the reference's own
 * sources compiled under oracle/_ref (when the reference tree is present) and
 * with golden vectors committed under tests/golden/.
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -fPIC -shared (see
 * oracle/Makefile).  -ffp-contract=off keeps a*b+c as two rounded operations
 * on every host (x86-64 and aarch64), matching the reference built without
 * -ffast-math.
 */
#ifndef AT_ORACLE_H
#define AT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- GoldenC parallel-beam geometry (fixed) ---------------- */
#define OR_GC_N 512      /* imageHight = imageWidth   (config.h:10-11) */
#define OR_GC_DETS 767   /* projWidth                 (config.h:12)    */
#define OR_GC_VIEWS 180  /* nAlpha                    (config.h:13)    */

/* proj.c:14-204.  proj is [180][767] row-major, img is [512][512]. */
void or_gc_A(double *proj, const double *img);
/* proj.c:206-397, scatter in the reference's exact statement order. */
void or_gc_AStar(double *back, const double *proj);
/* One traced tile walk (alpha 1..45, tile 0..15, raynum 0..383) in visiting
 * order, as tile-local (ix, iy) and weight.  Returns the segment count. */
int or_gc_walk(int alpha, int tile, int raynum, int *ix, int *iy, double *w, int cap);

/* ---------------- fan-beam geometry ---------------- */
typedef struct {
    int n;                /* image n x n; pixel index = x*n + y (x slow)      */
    double pixel_mm;      /* vx = vy                                          */
    int nviews;
    int ndets;            /* even: detectors j = -ndets/2 .. ndets/2-1        */
    double sod_mm;        /* SOURCE_TO_ISO                                    */
    double sdd_mm;        /* SOURCE_TO_DET                                    */
    double det_pitch_deg; /* LENGTH_PER_DET (equiangular pitch, degrees)      */
    double off_center;    /* OFF_CENTER (detector index offset)               */
    double view0_deg;     /* source angle of view 0                           */
    double view_step_deg; /* source angle increment per view                  */
    const double *ends;   /* optional [nviews*ndets][4] (sx, sy, dx, dy) table:
                             when set, rays are taken from it (any 2D geometry,
                             the arguments of tracing.cpp:22) and the fan
                             fields above other than n, pixel_mm, nviews and
                             ndets are unused                                 */
} or_fan_geom;

/* Source/detector end points of ray (view, det), ms2d.cpp:172-183. */
void or_fan_endpoints(const or_fan_geom *g, int view, int det,
                      double *sx, double *sy, double *dx, double *dy);
/* tracing.cpp:22-147 on those end points.  ind = x*n+y, wgt in mm.  Returns
 * the segment count; *oob counts segments whose pixel lies off the grid (they
 * are still reported).  cap must be >= 2n+4. */
int or_fan_trace(const or_fan_geom *g, int view, int det, int *ind, double *wgt, int cap, int *oob);
/* Same tracer on arbitrary end points (for comparing with the reference). */
int or_fan_trace_points(int n, double pixel_mm, double sx, double sy, double dx, double dy,
                        int *ind, double *wgt, int cap);
/* Sum of segment counts over all rays (S). */
int64_t or_fan_count_segments(const or_fan_geom *g, int nthreads);
/* sino[view][det] = sum_k img[ind_k]*wgt_k, segments in tracing order. */
void or_fan_A(const or_fan_geom *g, double *sino, const double *img, int nthreads);
/* Exact transpose of or_fan_A (scatter, per-thread partial images). */
void or_fan_AT(const or_fan_geom *g, double *img, const double *sino, int nthreads);

/* ---------------- 3D cone beam (industry3d/src/tracing.cpp, or_cone.c) ---- */
typedef struct {
    int nx, ny, nz;        /* NX NY NZ; voxel index z*nx*ny + x*ny + y      */
    float voxel;           /* SAMPLESIZE (mm per voxel)                      */
    int nproj;             /* NPROJ views over 360 degrees                   */
    int ndx, ndy;          /* NDX detector rows (z), NDY columns             */
    float pitch;           /* PIXELSIZE (mm per detector cell)               */
    float sod, sdd;        /* SOD, SDD (mm)                                  */
    int half_rows;         /* HALFDET for the row axis (reference: NDX/2)    */
    int half_cols;         /* HALFDET for the column axis (reference: NDX/2) */
} or_cone_geom;

float or_cone_theta(const or_cone_geom *g, int view);
void or_cone_endpoints(const or_cone_geom *g, int view, int row, int col, float *s, float *d);
/* mark_off: report segments whose voxel lies off the grid as index -1 */
int or_cone_trace_points(int nx, int ny, int nz, float sx, float sy, float sz, float dx, float dy, float dz,
                         int64_t *ind, float *wgt, int cap, int mark_off);
int or_cone_trace(const or_cone_geom *g, int view, int row, int col, int64_t *ind, float *wgt, int cap,
                  int mark_off);
int64_t or_cone_count_segments(const or_cone_geom *g, int nthreads);
void or_cone_A(const or_cone_geom *g, double *sino, const double *vol, int nthreads);
void or_cone_AT(const or_cone_geom *g, double *vol, const double *sino, int nthreads);

/* ---------------- AT solver (GoldenC main.c restated for any projector) ---- */
enum { OR_PROJ_GOLDENC = 0, OR_PROJ_FAN = 1, OR_PROJ_CONE = 2 };
typedef struct {
    int kind;
    or_fan_geom fan;      /* used when kind == OR_PROJ_FAN */
    int nthreads;
    or_cone_geom cone;    /* used when kind == OR_PROJ_CONE (a volume, nz slices) */
} or_projector;

/* Per-iteration scalars the reference prints (main.c:251,330), recorded so
 * the engine's branch and scalar trajectory can be compared. */
typedef struct {
    int outer;            /* outer iteration, 1-based        */
    int step;             /* 0 = image step, 1 = edge step   */
    int k;                /* inner iteration, 1-based        */
    double s[6];          /* image: AT_f_old nV pSkalard normAp c1 c2 ; edge: nD c maxCD */
    int exit_reason;      /* 0 continue, 1 maxIt, 2 tol, 3 instable */
} or_trace_rec;

typedef struct {
    or_trace_rec *recs;
    int cap, count;
} or_trace;

/* main.c:81-257 */
void or_image_step(const or_projector *P, double *out, const double *g, const double *f,
                   const double *v, double alpha, double epsilon, int iter_image,
                   or_trace *tr, int outer);
/* main.c:259-360 */
/* the edge step on a volume of nz slices (nz == 1: or_edge_step) */
void or_edge_step_vol(int n, int nz, double *out, const double *f, const double *v, double alpha, double beta,
                      double epsilon, int iter_edge, or_trace *tr, int outer);
void or_edge_step(int n, double *out, const double *f, const double *v, double alpha,
                  double beta, double epsilon, int iter_edge, or_trace *tr, int outer);
/* main.c:366-390 */
void or_medfilt2(int n, double *f);
/* main.c:35-49: f = 0, v = 1, iter_alt x (image step, edge step). */
void or_solve(const or_projector *P, const double *g, double *f, double *v, double alpha,
              double beta, double epsilon, int iter_alt, int iter_image, int iter_edge,
              or_trace *tr);

/* sinogram / image sizes of a projector */
int or_proj_views(const or_projector *P);
int or_proj_dets(const or_projector *P);
int or_proj_n(const or_projector *P);
int or_proj_nz(const or_projector *P); /* slices: 1 for images */
void or_proj_A(const or_projector *P, double *sino, const double *img);
void or_proj_AT(const or_projector *P, double *img, const double *sino);

#ifdef __cplusplus
}
#endif
#endif

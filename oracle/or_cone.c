/*
 * or_cone.c -- CPU restatement of the reference's 3D cone-beam Siddon tracer
 * (TEST INFRASTRUCTURE ONLY: the checker for the engine's cone-beam
 * projectors, never linked by the engine).
 *
 * Follows industry3d/src:
 *   cone()          tracing.cpp:51-81   source / detector-cell end points
 *   rotate_2d()     utility.cpp:82-98   rotation about the z axis
 *   forward_proj()  tracing.cpp:123-307 3D lambda-parametric Siddon walk
 *   get_img_addr()  tracing.cpp:117-119 z*NX*NY + x*NY + y
 * in single precision exactly as written there (float variables, the double
 * literals 0.5, 1e-4, 1e6, 5e-2 and PI promoting where the C++ does), built
 * with -ffp-contract=off so every operation rounds as in the reference.
 *
 * The reference derives HALFDET = NDX/2 for both detector axes
 * (ct3d.cpp:90); this restatement takes the half widths of the row (z) and
 * column axes separately, which equals the reference for square detectors.
 *
 * A and A^T accumulate the FP32 segment weights in FP64 and skip segments
 * whose voxel coordinates lie off the grid (the reference would address
 * memory outside the volume there).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "at_oracle.h"

#define CONE_PI 3.1415926535897932385 /* industry3d/include/ct3d.h:8 */

static float sqrf_(float x) { return x * x; } /* utility.cpp:51 */

/* utility.cpp:82-98: d = R(theta) x, accumulated k-major from zero */
static void rotate_2d(float *x, float *y, float theta) {
    float X0 = *x, X1 = *y;
    float c = cosf(theta), s = sinf(theta);
    float R00 = c, R01 = -s, R10 = s, R11 = c;
    float d0 = 0.f, d1 = 0.f;
    d0 += R00 * X0;
    d1 += R10 * X0;
    d0 += R01 * X1;
    d1 += R11 * X1;
    *x = d0;
    *y = d1;
}

float or_cone_theta(const or_cone_geom *g, int view) {
    /* tracing.cpp:57: (float)alpha/NPROJ*2*PI, the product with PI in double */
    float a = (float)view / (float)g->nproj * 2;
    return (float)((double)a * CONE_PI);
}

/* tracing.cpp:51-81 */
void or_cone_endpoints(const or_cone_geom *g, int view, int row, int col, float *s, float *d) {
    float srcZ = 0.0f, srcX = 0.0f, srcY = -g->sod;
    float theta = or_cone_theta(g, view);
    rotate_2d(&srcX, &srcY, theta);
    float dstX = (float)((double)(col - g->half_cols) + 0.5);
    dstX *= g->pitch;
    float dstY = (g->sdd - g->sod);
    float dstZ = (float)((double)(g->half_rows - row) - 0.5);
    dstZ *= g->pitch;
    rotate_2d(&dstX, &dstY, theta);
    srcX /= g->voxel;
    srcZ /= g->voxel;
    srcY /= g->voxel;
    dstX /= g->voxel;
    dstY /= g->voxel;
    dstZ /= g->voxel;
    srcX = (float)((double)srcX + g->nx / 2.0);
    srcY = (float)((double)srcY + g->ny / 2.0);
    srcZ = (float)((double)srcZ + g->nz / 2.0);
    dstX = (float)((double)dstX + g->nx / 2.0);
    dstY = (float)((double)dstY + g->ny / 2.0);
    dstZ = (float)((double)dstZ + g->nz / 2.0);
    s[0] = srcX;
    s[1] = srcY;
    s[2] = srcZ;
    d[0] = dstX;
    d[1] = dstY;
    d[2] = dstZ;
}

#define LAMBDA(i, s, d, L) ((L) * ((float)(i) - (s)) / ((d) - (s))) /* tracing.cpp:101-103 */
#define MAXF(x, y) (((x) > (y)) ? (x) : (y))
#define MINF(x, y) (((x) < (y)) ? (x) : (y))

/* tracing.cpp:123-307 */
int or_cone_trace_points(int nx, int ny, int nz, float sx, float sy, float sz, float dx, float dy, float dz,
                         int64_t *ind, float *wgt, int cap, int mark_off) {
    int index = 0;
    float ray_x = dx - sx, ray_y = dy - sy, ray_z = dz - sz;
    float L = sqrtf(sqrf_(ray_x) + sqrf_(ray_y) + sqrf_(ray_z));
    float lambda_min = 0.0f, lambda_max = L;
    int signx = (ray_x > 0) ? 1 : -1, signy = (ray_y > 0) ? 1 : -1, signz = (ray_z > 0) ? 1 : -1;
    float absx = fabsf(ray_x), absy = fabsf(ray_y), absz = fabsf(ray_z);
    float len_x = (float)((absx > 1.e-4) ? (double)(L / absx) : 1.e6);
    float len_y = (float)((absy > 1.e-4) ? (double)(L / absy) : 1.e6);
    float len_z = (float)((absz > 1.e-4) ? (double)(L / absz) : 1.e6);
    int numb = 0;
    float tempx = (float)nx, tempy = (float)ny, tempz = (float)nz;
    float lambda0, lambdaN, temp, lambda_x, lambda_y, lambda_z;
    int v_x, v_y, v_z;

    lambda0 = LAMBDA(0, sx, dx, L);
    lambdaN = LAMBDA(tempx, sx, dx, L);
    temp = MINF(lambda0, lambdaN);
    lambda_min = MAXF(lambda_min, temp);
    if (lambda_min == temp) index = 1;
    temp = MAXF(lambda0, lambdaN);
    lambda_max = MINF(lambda_max, temp);

    lambda0 = LAMBDA(0, sy, dy, L);
    lambdaN = LAMBDA(tempy, sy, dy, L);
    temp = MINF(lambda0, lambdaN);
    lambda_min = MAXF(lambda_min, temp);
    if (lambda_min == temp) index = 2;
    temp = MAXF(lambda0, lambdaN);
    lambda_max = MINF(lambda_max, temp);

    lambda0 = LAMBDA(0, sz, dz, L);
    lambdaN = LAMBDA(tempz, sz, dz, L);
    temp = MINF(lambda0, lambdaN);
    lambda_min = MAXF(lambda_min, temp);
    if (lambda_min == temp) index = 3;
    temp = MAXF(lambda0, lambdaN);
    lambda_max = MINF(lambda_max, temp);

    if (lambda_min >= lambda_max) return 0;

    lambda0 = lambda_min;
    if (index == 1) {
        v_x = (signx == 1) ? 0 : nx - 1;
        lambda_x = lambda0 + len_x;
        v_y = (int)(sy + lambda0 * ray_y / L);
        tempy = (float)v_y;
        lambda_y = (float)((absy < 1.e-4) ? 1.e6 : (double)LAMBDA(tempy + (signy > 0), sy, dy, L));
        v_z = (int)(sz + lambda0 * ray_z / L);
        tempz = (float)v_z;
        lambda_z = (float)((absz < 1.e-4) ? 1.e6 : (double)LAMBDA(tempz + (signz > 0), sz, dz, L));
    } else if (index == 2) {
        v_y = (signy == 1) ? 0 : ny - 1;
        lambda_y = lambda0 + len_y;
        v_x = (int)(sx + lambda0 * ray_x / L);
        tempx = (float)v_x;
        lambda_x = (float)((absx < 1.e-4) ? 1.e6 : (double)LAMBDA(tempx + (signx > 0), sx, dx, L));
        v_z = (int)(sz + lambda0 * ray_z / L);
        tempz = (float)v_z;
        lambda_z = (float)((absz < 1.e-4) ? 1.e6 : (double)LAMBDA(tempz + (signz > 0), sz, dz, L));
    } else {
        v_z = (signz == 1) ? 0 : nz - 1;
        lambda_z = lambda0 + len_z;
        v_x = (int)(sx + lambda0 * ray_x / L);
        tempx = (float)v_x;
        lambda_x = (float)((absx < 1.e-4) ? 1.e6 : (double)LAMBDA(tempx + (signx > 0), sx, dx, L));
        v_y = (int)(sy + lambda0 * ray_y / L);
        tempy = (float)v_y;
        lambda_y = (float)((absy < 1.e-4) ? 1.e6 : (double)LAMBDA(tempy + (signy > 0), sy, dy, L));
    }
    while ((double)lambda0 < (double)lambda_max - 5.e-2) {
        int64_t addr = (int64_t)v_z * nx * ny + (int64_t)v_x * ny + v_y;
        if (mark_off && ((unsigned)v_x >= (unsigned)nx || (unsigned)v_y >= (unsigned)ny || (unsigned)v_z >= (unsigned)nz))
            addr = -1;
        if (lambda_x <= lambda_y && lambda_x <= lambda_z) {
            if (numb < cap) {
                ind[numb] = addr;
                wgt[numb] = lambda_x - lambda0;
            }
            ++numb;
            lambda0 = lambda_x;
            lambda_x += len_x;
            v_x += signx;
        } else if (lambda_y <= lambda_z) {
            if (numb < cap) {
                ind[numb] = addr;
                wgt[numb] = lambda_y - lambda0;
            }
            ++numb;
            lambda0 = lambda_y;
            lambda_y += len_y;
            v_y += signy;
        } else {
            if (numb < cap) {
                ind[numb] = addr;
                wgt[numb] = lambda_z - lambda0;
            }
            ++numb;
            lambda0 = lambda_z;
            lambda_z += len_z;
            v_z += signz;
        }
    }
    return numb;
}

int or_cone_trace(const or_cone_geom *g, int view, int row, int col, int64_t *ind, float *wgt, int cap,
                  int mark_off) {
    float s[3], d[3];
    or_cone_endpoints(g, view, row, col, s, d);
    return or_cone_trace_points(g->nx, g->ny, g->nz, s[0], s[1], s[2], d[0], d[1], d[2], ind, wgt, cap, mark_off);
}

static int cone_on_grid(int64_t a) { return a >= 0; } /* off-grid segments are marked -1 */

static int cone_threads(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

static int cone_cap(const or_cone_geom *g) { return 2 * (g->nx + g->ny + g->nz) + 16; }

int64_t or_cone_count_segments(const or_cone_geom *g, int nthreads) {
    int nt = cone_threads(nthreads), cap = cone_cap(g);
    int64_t total = 0;
#pragma omp parallel num_threads(nt) reduction(+ : total)
    {
        int64_t *ind = (int64_t *)malloc(sizeof(int64_t) * cap);
        float *wgt = (float *)malloc(sizeof(float) * cap);
#pragma omp for schedule(dynamic, 4)
        for (int v = 0; v < g->nproj; v++)
            for (int r = 0; r < g->ndx; r++)
                for (int c = 0; c < g->ndy; c++) total += or_cone_trace(g, v, r, c, ind, wgt, cap, 0);
        free(ind);
        free(wgt);
    }
    return total;
}

/* sino[view][row][col] = sum_k vol[ind_k] * wgt_k over the on-grid segments */
void or_cone_A(const or_cone_geom *g, double *sino, const double *vol, int nthreads) {
    int nt = cone_threads(nthreads), cap = cone_cap(g);
#pragma omp parallel num_threads(nt)
    {
        int64_t *ind = (int64_t *)malloc(sizeof(int64_t) * cap);
        float *wgt = (float *)malloc(sizeof(float) * cap);
#pragma omp for schedule(dynamic, 4)
        for (int v = 0; v < g->nproj; v++)
            for (int r = 0; r < g->ndx; r++)
                for (int c = 0; c < g->ndy; c++) {
                    int nb = or_cone_trace(g, v, r, c, ind, wgt, cap, 1);
                    double acc = 0.0;
                    for (int k = 0; k < nb; k++)
                        if (cone_on_grid(ind[k])) acc += vol[ind[k]] * (double)wgt[k];
                    sino[((int64_t)v * g->ndx + r) * g->ndy + c] = acc;
                }
        free(ind);
        free(wgt);
    }
}

/* exact transpose of or_cone_A (per-thread partial volumes, summed in order) */
void or_cone_AT(const or_cone_geom *g, double *vol, const double *sino, int nthreads) {
    int nt = cone_threads(nthreads), cap = cone_cap(g);
    const int64_t nvox = (int64_t)g->nx * g->ny * g->nz;
    double *part = (double *)calloc((size_t)nt * nvox, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *mine = part + (size_t)tid * nvox;
        int64_t *ind = (int64_t *)malloc(sizeof(int64_t) * cap);
        float *wgt = (float *)malloc(sizeof(float) * cap);
#pragma omp for schedule(static)
        for (int v = 0; v < g->nproj; v++)
            for (int r = 0; r < g->ndx; r++)
                for (int c = 0; c < g->ndy; c++) {
                    int nb = or_cone_trace(g, v, r, c, ind, wgt, cap, 1);
                    double s = sino[((int64_t)v * g->ndx + r) * g->ndy + c];
                    for (int k = 0; k < nb; k++)
                        if (cone_on_grid(ind[k])) mine[ind[k]] += s * (double)wgt[k];
                }
        free(ind);
        free(wgt);
    }
    for (int64_t i = 0; i < nvox; i++) {
        double acc = 0.0;
        for (int t = 0; t < nt; t++) acc += part[(size_t)t * nvox + i];
        vol[i] = acc;
    }
    free(part);
}

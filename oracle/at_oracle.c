/*
 * at_oracle.c -- FP64 CPU oracle (TEST INFRASTRUCTURE ONLY; see at_oracle.h).
 *
 * Every expression that feeds a comparison or a stored value is written in
 * the same evaluation order as the reference, so that with the build flags of
 * oracle/Makefile the results are bit-identical to the reference's sources
 * compiled the same way.  Citations are file:line in the reference project.
 */
#include "at_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double sq(double x) { return x * x; } /* main.c:33 and utility.cpp sqr */

static int threads_or_default(int nthreads) {
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* ========================================================================
 * GoldenC parallel-beam projector, origin/GoldenC/src/proj.c
 * ======================================================================== */
#define GC_N OR_GC_N
#define GC_LAST (OR_GC_N - 1)
#define GC_DETS OR_GC_DETS
#define GC_MID 383 /* MIDRAY, proj.c:7 */
#define GC_TILE 128 /* TILEX_L = TILEY_L, proj.c:8-9; 4x4 tiles proj.c:10-12 */

typedef struct {
    double sf, cf, hx, hy, tanphi, rtnphi;
} gc_trig;

/* proj.c:43-48 (pi written as 3.141593 in the reference) */
static void gc_trig_of(int alpha, gc_trig *t) {
    double ang = 3.141593 / 180 * alpha;
    t->sf = sin(ang);
    t->cf = cos(ang);
    t->hx = ((double)1.0) / t->sf;
    t->hy = ((double)1.0) / t->cf;
    t->tanphi = t->sf / t->cf;
    t->rtnphi = t->cf / t->sf;
}

/* Tile walk of ray (alpha, tile, raynum): proj.c:55-200.  Emits tile-local
 * (ix, iy) and weights in visiting order. */
static int gc_walk_trig(const gc_trig *t, int tile, int raynum, int *wx, int *wy, double *ww,
                        int cap) {
    const int ind = raynum - (GC_DETS / 2);
    const int col = tile % 4;
    const int dyo = GC_TILE * (tile / 4);
    double c = t->cf * ind + t->sf * ind * t->tanphi;                  /* :59 */
    c = (GC_N / 2 - dyo) - t->tanphi * (GC_N / 2 - GC_TILE * col) - c; /* :61 */
    int ix, iy, next;
    double fp, w, xc, yc;
    if (c < 0) { /* enters through the tile bottom, :66-86 */
        c = -c * t->rtnphi;
        ix = (int)c;
        iy = 0;
        fp = ((double)(ix + 1)) - c;
        ix = GC_TILE - ix - 1;
        w = t->hy * fp;
        yc = fp * t->tanphi;
        xc = -fp;
        next = 2;
    } else { /* enters through the tile side, :87-103 */
        ix = GC_TILE - 1;
        iy = (int)c;
        fp = ((double)(iy + 1)) - c;
        yc = -fp;
        w = t->hx * fp;
        xc = fp * t->rtnphi;
        next = 1;
    }
    (void)yc;
    int n = 0;
#define GC_EMIT(wt)              \
    do {                         \
        if (n < cap) {           \
            wx[n] = ix;          \
            wy[n] = iy;          \
            ww[n] = (wt);        \
        }                        \
        n++;                     \
    } while (0)
    while (ix >= 0 && ix < GC_TILE && iy >= 0 && iy < GC_TILE) { /* :104 */
        if (next == 1) {                                        /* :106-151 */
            xc -= (double)1.0;
            yc += t->tanphi;
            if (xc > 0) {
                GC_EMIT(t->hy);
                w -= t->hy;
                ix += -1;
            } else {
                GC_EMIT(w);
                w = t->hy - w;
                iy++;
                next = 2;
            }
        } else { /* :152-198 */
            yc -= 1.0;
            xc += t->rtnphi;
            if (yc > 0) {
                w -= t->hx;
                GC_EMIT(t->hx);
                iy++;
            } else {
                GC_EMIT(w);
                w = t->hx - w;
                ix += -1;
                next = 1;
            }
        }
    }
#undef GC_EMIT
    return n;
}

int or_gc_walk(int alpha, int tile, int raynum, int *ix, int *iy, double *w, int cap) {
    gc_trig t;
    gc_trig_of(alpha, &t);
    return gc_walk_trig(&t, tile, raynum, ix, iy, w, cap);
}

/* Output bin families.  A traced ray (alpha, r) writes eight symmetric bins
 * (proj.c:114-127).  For tile-global X = ix+dx, Y = iy+dy the image sample of
 * symmetry s is img[row][col] with: */
static inline void gc_sym_pixel(int s, int X, int Y, int *row, int *col) {
    switch (s) {
    case 0: *row = Y; *col = X; break;                    /* proj[a][r]             */
    case 1: *row = GC_LAST - X; *col = Y; break;          /* proj[90+a][r]          */
    case 2: *row = GC_LAST - Y; *col = GC_LAST - X; break; /* proj[a][766-r]          */
    case 3: *row = X; *col = GC_LAST - Y; break;          /* proj[90+a][766-r]      */
    case 4: *row = X; *col = Y; break;                    /* proj[90-a][r]          */
    case 5: *row = GC_LAST - Y; *col = X; break;          /* proj[180-a][r]         */
    case 6: *row = GC_LAST - X; *col = GC_LAST - Y; break; /* proj[90-a][766-r]      */
    default: *row = Y; *col = GC_LAST - X; break;         /* proj[180-a][766-r]     */
    }
}

static inline void gc_sym_bin(int s, int a, int r, int *view, int *det) {
    static const int vbase[8] = {0, 90, 0, 90, 90, 180, 90, 180};
    static const int vsign[8] = {1, 1, 1, 1, -1, -1, -1, -1};
    *view = vbase[s] + vsign[s] * a;
    *det = (s & 2) ? (GC_DETS - 1 - r) : r;
}

static inline int gc_sym_present(int s, int a, int r) {
    if ((s & 2) && r == GC_MID) return 0; /* RayNum != MIDRAY, proj.c:116 */
    if (s >= 4 && a == 45) return 0;      /* alpha != 45, proj.c:120      */
    return 1;
}

#define GC_WALK_CAP 512

void or_gc_A(double *proj, const double *img) {
    memset(proj, 0, sizeof(double) * OR_GC_VIEWS * GC_DETS); /* proj.c:15 */
    /* view 0: row sums, proj.c:17-26 */
    for (int r = 0; r < GC_DETS; r++) {
        int ind = r - (GC_DETS / 2);
        if ((ind > (GC_N / 2 - 1)) || (ind < (1 - GC_N / 2))) continue;
        int row = GC_N / 2 - 1 + ind;
        for (int x = 0; x < GC_N; x++) proj[0 * GC_DETS + r] += img[row * GC_N + x];
    }
    /* view 90: column sums, proj.c:27-36 */
    for (int r = 0; r < GC_DETS; r++) {
        int ind = r - (GC_DETS / 2);
        if ((ind > (GC_N / 2 - 1)) || (ind < (1 - GC_N / 2))) continue;
        int colx = GC_N / 2 + ind;
        for (int y = 0; y < GC_N; y++) proj[90 * GC_DETS + r] += img[y * GC_N + colx];
    }
    /* traced views.  Every bin has exactly one (alpha, r, s) source and is
     * accumulated in (tile, step) order as in the reference, so the per-bin
     * sums are bit-identical while pairs (alpha, r) run in parallel. */
#pragma omp parallel for schedule(dynamic, 16)
    for (int pair = 0; pair < 45 * (GC_MID + 1); pair++) {
        int a = 1 + pair / (GC_MID + 1);
        int r = pair % (GC_MID + 1);
        gc_trig t;
        gc_trig_of(a, &t);
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int wx[GC_WALK_CAP], wy[GC_WALK_CAP];
        double ww[GC_WALK_CAP];
        for (int tile = 0; tile < 16; tile++) {
            int ns = gc_walk_trig(&t, tile, r, wx, wy, ww, GC_WALK_CAP);
            int dxo = GC_TILE * (3 - tile % 4), dyo = GC_TILE * (tile / 4);
            for (int k = 0; k < ns; k++) {
                int X = wx[k] + dxo, Y = wy[k] + dyo;
                for (int s = 0; s < 8; s++) {
                    if (!gc_sym_present(s, a, r)) continue;
                    int row, col;
                    gc_sym_pixel(s, X, Y, &row, &col);
                    acc[s] += img[row * GC_N + col] * ww[k];
                }
            }
        }
        for (int s = 0; s < 8; s++) {
            if (!gc_sym_present(s, a, r)) continue;
            int view, det;
            gc_sym_bin(s, a, r, &view, &det);
            proj[view * GC_DETS + det] = acc[s];
        }
    }
}

void or_gc_AStar(double *back, const double *proj) {
    memset(back, 0, sizeof(double) * GC_N * GC_N); /* proj.c:207 */
    for (int r = 0; r < GC_DETS; r++) {            /* proj.c:210-219 */
        int ind = r - (GC_DETS / 2);
        if ((ind > (GC_N / 2 - 1)) || (ind < (1 - GC_N / 2))) continue;
        int row = GC_N / 2 - 1 + ind;
        for (int x = 0; x < GC_N; x++) back[row * GC_N + x] += proj[0 * GC_DETS + r];
    }
    for (int r = 0; r < GC_DETS; r++) { /* proj.c:221-230: column 255+ind, not 256+ind */
        int ind = r - (GC_DETS / 2);
        if ((ind > (GC_N / 2 - 1)) || (ind < (1 - GC_N / 2))) continue;
        int colx = GC_N / 2 - 1 + ind;
        for (int y = 0; y < GC_N; y++) back[y * GC_N + colx] += proj[90 * GC_DETS + r];
    }
    int wx[GC_WALK_CAP], wy[GC_WALK_CAP];
    double ww[GC_WALK_CAP];
    for (int a = 1; a < 46; a++) { /* proj.c:232-396, single thread, statement order */
        gc_trig t;
        gc_trig_of(a, &t);
        for (int tile = 0; tile < 16; tile++) {
            int dxo = GC_TILE * (3 - tile % 4), dyo = GC_TILE * (tile / 4);
            for (int r = 0; r < GC_MID + 1; r++) {
                int ns = gc_walk_trig(&t, tile, r, wx, wy, ww, GC_WALK_CAP);
                for (int k = 0; k < ns; k++) {
                    int X = wx[k] + dxo, Y = wy[k] + dyo;
                    for (int s = 0; s < 8; s++) {
                        if (!gc_sym_present(s, a, r)) continue;
                        int row, col, view, det;
                        gc_sym_pixel(s, X, Y, &row, &col);
                        gc_sym_bin(s, a, r, &view, &det);
                        back[row * GC_N + col] += proj[view * GC_DETS + det] * ww[k];
                    }
                }
            }
        }
    }
}

/* ========================================================================
 * Fan-beam tracer, helical/rebin/src/tracing.cpp:22-147 with the geometry of
 * helical/rebin/src/ms2d.cpp:30-62 (tables) and :172-183 (end points).
 * ======================================================================== */
static double fan_source_angle_rad(const or_fan_geom *g, int view) {
    double angle = g->view0_deg + view * g->view_step_deg;
    return angle / 180.0 * M_PI; /* ms2d.cpp:43-44 */
}

static double fan_det_angle_rad(const or_fan_geom *g, int det) {
    double per_rad = g->det_pitch_deg * M_PI / 180.; /* ms2d.cpp:51 */
    int j = det - g->ndets / 2;                      /* j = -HALFDET..HALFDET-1 */
    return (j + g->off_center) * per_rad + M_PI;     /* ms2d.cpp:53-54 */
}

void or_fan_endpoints(const or_fan_geom *g, int view, int det, double *sx, double *sy, double *dx,
                      double *dy) {
    if (g->ends) {
        const double *e = g->ends + ((int64_t)view * g->ndets + det) * 4;
        *sx = e[0];
        *sy = e[1];
        *dx = e[2];
        *dy = e[3];
        return;
    }
    double sa = fan_source_angle_rad(g, view);
    double da = fan_det_angle_rad(g, det);
    double scos = cos(sa), ssin = sin(sa), dcos = cos(da), dsin = sin(da);
    double vx = g->pixel_mm, vy = g->pixel_mm;
    int NX = g->n;
    double source_x = g->sod_mm * scos + NX * vx / 2.0; /* ms2d.cpp:173 */
    double source_y = g->sod_mm * ssin + NX * vy / 2.0; /* ms2d.cpp:174 (NX, as written) */
    *sx = source_x;
    *sy = source_y;
    *dx = g->sdd_mm * (dcos * scos - dsin * ssin) + source_x; /* :176-179 */
    *dy = g->sdd_mm * (dsin * scos + dcos * ssin) + source_y; /* :180-183 */
}

#define LAMBDA_AT(i, s, d, L) (L * ((double)(i) - (s)) / ((d) - (s))) /* tracing.cpp:9-10 */

int or_fan_trace_points(int n, double pixel_mm, double sx, double sy, double dx, double dy,
                        int *ind, double *wgt, int cap) {
    const int NX = n, NY = n;
    const double vx = pixel_mm, vy = pixel_mm;
    int index = 0;
    double ray_x = dx - sx, ray_y = dy - sy;
    double L = sqrt(sq(ray_x) + sq(ray_y));
    double lambda_min = 0.0, lambda_max = L;
    int signx = (ray_x > 0) ? 1 : -1;
    int signy = (ray_y > 0) ? 1 : -1;
    double absx = fabs(ray_x), absy = fabs(ray_y);
    double len_x = (absx > 1.e-4) ? (L / absx) * vx : 1.e6; /* :55 */
    double len_y = (absy > 1.e-4) ? (L / absy) * vy : 1.e6; /* :56 */
    int numb = 0;
    double tempx = NX * vx, tempy = NY * vy;
    double l0, lN, temp;

    l0 = LAMBDA_AT(0, sx, dx, L); /* :68-75 */
    lN = LAMBDA_AT(tempx, sx, dx, L);
    temp = (l0 < lN) ? l0 : lN;
    lambda_min = (lambda_min > temp) ? lambda_min : temp;
    if (lambda_min == temp) index = 1;
    temp = (l0 > lN) ? l0 : lN;
    lambda_max = (lambda_max < temp) ? lambda_max : temp;

    l0 = LAMBDA_AT(0, sy, dy, L); /* :77-84 */
    lN = LAMBDA_AT(tempy, sy, dy, L);
    temp = (l0 < lN) ? l0 : lN;
    lambda_min = (lambda_min > temp) ? lambda_min : temp;
    if (lambda_min == temp) index = 2;
    temp = (l0 > lN) ? l0 : lN;
    lambda_max = (lambda_max < temp) ? lambda_max : temp;

    if (lambda_min >= lambda_max) return 0; /* :86-87 */

    double lambda0 = lambda_min, lambda_x, lambda_y;
    int v_x, v_y;
    if (index == 1) { /* enters through an x plane, :91-102 */
        v_x = (signx == 1) ? 0 : NX - 1;
        lambda_x = lambda0 + len_x;
        v_y = (int)((sy + lambda0 * ray_y / L) / vy);
        tempy = v_y * vy;
        lambda_y = (absy < 1.e-4) ? 1.e6 : LAMBDA_AT(tempy + (signy > 0) * vy, sy, dy, L);
    } else { /* :104-115 */
        v_y = (signy == 1) ? 0 : NY - 1;
        lambda_y = lambda0 + len_y;
        v_x = (int)((sx + lambda0 * ray_x / L) / vx);
        tempx = v_x * vx;
        lambda_x = (absx < 1.e-4) ? 1.e6 : LAMBDA_AT(tempx + (signx > 0) * vx, sx, dx, L);
    }
    while (lambda0 < lambda_max - 5.e-2) { /* :118-146 */
        int addr = (int)((double)v_x * NY + v_y); /* get_img_addr, utility.cpp:35-37 */
        if (lambda_x <= lambda_y) {
            if (numb < cap) {
                ind[numb] = addr;
                wgt[numb] = lambda_x - lambda0;
            }
            ++numb;
            lambda0 = lambda_x;
            lambda_x += len_x;
            v_x += signx;
        } else {
            if (numb < cap) {
                ind[numb] = addr;
                wgt[numb] = lambda_y - lambda0;
            }
            ++numb;
            lambda0 = lambda_y;
            lambda_y += len_y;
            v_y += signy;
        }
    }
    return numb;
}

int or_fan_trace(const or_fan_geom *g, int view, int det, int *ind, double *wgt, int cap, int *oob) {
    double sx, sy, dx, dy;
    or_fan_endpoints(g, view, det, &sx, &sy, &dx, &dy);
    int nb = or_fan_trace_points(g->n, g->pixel_mm, sx, sy, dx, dy, ind, wgt, cap);
    if (oob) {
        int bad = 0, lim = nb < cap ? nb : cap;
        for (int k = 0; k < lim; k++)
            if (ind[k] < 0 || ind[k] >= g->n * g->n) bad++;
        *oob = bad;
    }
    return nb;
}

int64_t or_fan_count_segments(const or_fan_geom *g, int nthreads) {
    int nt = threads_or_default(nthreads);
    int64_t total = 0;
    int cap = 2 * g->n + 8;
#pragma omp parallel num_threads(nt) reduction(+ : total)
    {
        int *ind = (int *)malloc(sizeof(int) * cap);
        double *wgt = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(static)
        for (int v = 0; v < g->nviews; v++)
            for (int d = 0; d < g->ndets; d++) total += or_fan_trace(g, v, d, ind, wgt, cap, NULL);
        free(ind);
        free(wgt);
    }
    return total;
}

void or_fan_A(const or_fan_geom *g, double *sino, const double *img, int nthreads) {
    int nt = threads_or_default(nthreads);
    int cap = 2 * g->n + 8, npix = g->n * g->n;
#pragma omp parallel num_threads(nt)
    {
        int *ind = (int *)malloc(sizeof(int) * cap);
        double *wgt = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(static)
        for (int v = 0; v < g->nviews; v++)
            for (int d = 0; d < g->ndets; d++) {
                int nb = or_fan_trace(g, v, d, ind, wgt, cap, NULL);
                double acc = 0;
                for (int k = 0; k < nb; k++)
                    if (ind[k] >= 0 && ind[k] < npix) acc += img[ind[k]] * wgt[k];
                sino[(int64_t)v * g->ndets + d] = acc;
            }
        free(ind);
        free(wgt);
    }
}

void or_fan_AT(const or_fan_geom *g, double *img, const double *sino, int nthreads) {
    int nt = threads_or_default(nthreads);
    int cap = 2 * g->n + 8, npix = g->n * g->n;
    double *part = (double *)calloc((size_t)nt * npix, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *mine = part + (size_t)tid * npix;
        int *ind = (int *)malloc(sizeof(int) * cap);
        double *wgt = (double *)malloc(sizeof(double) * cap);
#pragma omp for schedule(static)
        for (int v = 0; v < g->nviews; v++)
            for (int d = 0; d < g->ndets; d++) {
                int nb = or_fan_trace(g, v, d, ind, wgt, cap, NULL);
                double s = sino[(int64_t)v * g->ndets + d];
                for (int k = 0; k < nb; k++)
                    if (ind[k] >= 0 && ind[k] < npix) mine[ind[k]] += s * wgt[k];
            }
        free(ind);
        free(wgt);
    }
    for (int i = 0; i < npix; i++) {
        double acc = 0;
        for (int t = 0; t < nt; t++) acc += part[(size_t)t * npix + i];
        img[i] = acc;
    }
    free(part);
}

/* ========================================================================
 * Projector dispatch for the solver
 * ======================================================================== */
int or_proj_views(const or_projector *P) {
    return P->kind == OR_PROJ_FAN ? P->fan.nviews : P->kind == OR_PROJ_CONE ? P->cone.nproj : OR_GC_VIEWS;
}
int or_proj_dets(const or_projector *P) {
    return P->kind == OR_PROJ_FAN ? P->fan.ndets : P->kind == OR_PROJ_CONE ? P->cone.ndx * P->cone.ndy : OR_GC_DETS;
}
int or_proj_n(const or_projector *P) {
    return P->kind == OR_PROJ_FAN ? P->fan.n : P->kind == OR_PROJ_CONE ? P->cone.nx : OR_GC_N;
}
int or_proj_nz(const or_projector *P) { return P->kind == OR_PROJ_CONE ? P->cone.nz : 1; }

void or_proj_A(const or_projector *P, double *sino, const double *img) {
    if (P->kind == OR_PROJ_CONE) or_cone_A(&P->cone, sino, img, P->nthreads);
    else if (P->kind == OR_PROJ_FAN) or_fan_A(&P->fan, sino, img, P->nthreads);
    else or_gc_A(sino, img);
}

void or_proj_AT(const or_projector *P, double *img, const double *sino) {
    if (P->kind == OR_PROJ_CONE) or_cone_AT(&P->cone, img, sino, P->nthreads);
    else if (P->kind == OR_PROJ_FAN) or_fan_AT(&P->fan, img, sino, P->nthreads);
    else or_gc_AStar(img, sino);
}

/* ========================================================================
 * AT solver, origin/GoldenC/src/main.c.  Padded arrays of the reference are
 * replaced by accessors that return the same padding values (0 or 1), which
 * leaves every arithmetic operation unchanged.
 * ======================================================================== */
static void trace_push(or_trace *tr, int outer, int step, int k, const double *s, int ns, int exit_reason) {
    if (!tr || tr->count >= tr->cap) return;
    or_trace_rec *r = &tr->recs[tr->count++];
    r->outer = outer;
    r->step = step;
    r->k = k;
    for (int i = 0; i < 6; i++) r->s[i] = i < ns ? s[i] : 0.0;
    r->exit_reason = exit_reason;
}

/* value of a (n+2)x(n+2) padded copy of a at padded coordinates (i, j) */
static inline double pad_at(const double *a, int n, int i, int j, double fill) {
    if (i < 1 || j < 1 || i > n || j > n) return fill;
    return a[(i - 1) * n + (j - 1)];
}

/* d += alpha * div-stencil, main.c:112-125 (also :226-239).  u zero-padded,
 * v one-padded. */
static void image_gradient_stencil(int n, double *d, const double *u, const double *v, double alpha,
                                   double epsilon) {
    for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j) {
            double Pc = pad_at(v, n, i, j, 1.0), Pu = pad_at(v, n, i - 1, j, 1.0),
                   Pl = pad_at(v, n, i, j - 1, 1.0);
            double Tc = pad_at(u, n, i, j, 0.0), Td = pad_at(u, n, i + 1, j, 0.0),
                   Tr = pad_at(u, n, i, j + 1, 0.0), Tu = pad_at(u, n, i - 1, j, 0.0),
                   Tl = pad_at(u, n, i, j - 1, 0.0);
            d[(i - 1) * n + (j - 1)] +=
                alpha * (+sq(Pc) * (Td - Tc) + sq(Pc) * (Tr - Tc) - sq(Pu) * (Tc - Tu) -
                         sq(Pl) * (Tc - Tl) + 0.01 * sq(epsilon) * (Td + Tr - 4 * Tc + Tu + Tl));
        }
}

/* alpha * sum over the interior (v^2 + 0.01 eps^2) |backward grad u|^2,
 * main.c:135-139 (and :203-208), added onto acc in row-major order. */
static double smooth_energy(int n, double acc, const double *u, const double *v, double alpha,
                            double epsilon) {
    for (int i = 2; i <= n - 1; ++i)
        for (int j = 2; j <= n - 1; ++j) {
            double P = pad_at(v, n, i, j, 1.0);
            double Tc = pad_at(u, n, i, j, 0.0), Tu = pad_at(u, n, i - 1, j, 0.0),
                   Tl = pad_at(u, n, i, j - 1, 0.0);
            acc += alpha * (sq(P) + 0.01 * sq(epsilon)) * (sq(Tc - Tu) + sq(Tc - Tl));
        }
    return acc;
}

void or_medfilt2(int n, double *f) {
    double *pf = (double *)malloc(sizeof(double) * n * n);
    memcpy(pf, f, sizeof(double) * n * n);
    for (int i = 1; i <= n; ++i)
        for (int j = 1; j <= n; ++j) {
            double t[9];
            t[0] = pad_at(pf, n, i, j, 0.0);
            t[1] = pad_at(pf, n, i - 1, j - 1, 0.0);
            t[2] = pad_at(pf, n, i - 1, j, 0.0);
            t[3] = pad_at(pf, n, i - 1, j + 1, 0.0);
            t[4] = pad_at(pf, n, i, j + 1, 0.0);
            t[5] = pad_at(pf, n, i + 1, j + 1, 0.0);
            t[6] = pad_at(pf, n, i + 1, j, 0.0);
            t[7] = pad_at(pf, n, i + 1, j - 1, 0.0);
            t[8] = pad_at(pf, n, i, j - 1, 0.0);
            for (int p = 0; p < 9; ++p) /* main.c:385-387 */
                for (int q = p + 1; q < 9; ++q)
                    if (t[p] > t[q]) {
                        double s = t[p];
                        t[p] = t[q];
                        t[q] = s;
                    }
            f[(i - 1) * n + (j - 1)] = t[4];
        }
    free(pf);
}

/* ---- volumes (nz > 1 slices; the cone beam).  Not in the reference: GoldenC
 * is 2D.  The same functional with the z neighbours added to every
 * stencil: backward differences in z in the smoothness term and its energy
 * (interior in z as well), central differences in z in the edge step, a
 * six-neighbour Laplacian scaled by 1/6 (GoldenC's 4-neighbour one is scaled
 * by 1/4), and GoldenC's 3x3 median within each slice. ---- */
static inline double pad3(const double *a, int n, int nz, int k, int i, int j, double fill) {
    if (k < 1 || k > nz || i < 1 || j < 1 || i > n || j > n) return fill;
    return a[((size_t)(k - 1) * n + (i - 1)) * n + (j - 1)];
}

static void image_gradient_stencil3(int n, int nz, double *d, const double *u, const double *v, double alpha,
                                    double epsilon) {
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= n; ++i)
            for (int j = 1; j <= n; ++j) {
                double Pc = pad3(v, n, nz, k, i, j, 1.0), Pu = pad3(v, n, nz, k, i - 1, j, 1.0),
                       Pl = pad3(v, n, nz, k, i, j - 1, 1.0), Pf = pad3(v, n, nz, k - 1, i, j, 1.0);
                double Tc = pad3(u, n, nz, k, i, j, 0.0), Td = pad3(u, n, nz, k, i + 1, j, 0.0),
                       Tr = pad3(u, n, nz, k, i, j + 1, 0.0), Tb = pad3(u, n, nz, k + 1, i, j, 0.0),
                       Tu = pad3(u, n, nz, k, i - 1, j, 0.0), Tl = pad3(u, n, nz, k, i, j - 1, 0.0),
                       Tf = pad3(u, n, nz, k - 1, i, j, 0.0);
                d[((size_t)(k - 1) * n + (i - 1)) * n + (j - 1)] +=
                    alpha * (sq(Pc) * (Td - Tc) + sq(Pc) * (Tr - Tc) + sq(Pc) * (Tb - Tc) - sq(Pu) * (Tc - Tu) -
                             sq(Pl) * (Tc - Tl) - sq(Pf) * (Tc - Tf) +
                             0.01 * sq(epsilon) * (Td + Tr + Tb - 6 * Tc + Tu + Tl + Tf));
            }
}

static double smooth_energy3(int n, int nz, double acc, const double *u, const double *v, double alpha,
                             double epsilon) {
    for (int k = 2; k <= nz - 1; ++k)
        for (int i = 2; i <= n - 1; ++i)
            for (int j = 2; j <= n - 1; ++j) {
                double P = pad3(v, n, nz, k, i, j, 1.0);
                double Tc = pad3(u, n, nz, k, i, j, 0.0), Tu = pad3(u, n, nz, k, i - 1, j, 0.0),
                       Tl = pad3(u, n, nz, k, i, j - 1, 0.0), Tf = pad3(u, n, nz, k - 1, i, j, 0.0);
                acc += alpha * (sq(P) + 0.01 * sq(epsilon)) * (sq(Tc - Tu) + sq(Tc - Tl) + sq(Tc - Tf));
            }
    return acc;
}

static double nv3(int n, int nz, const double *p, const double *v, double epsilon) {
    double nV = 0;
    for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= n; ++i)
            for (int j = 1; j <= n; ++j) {
                double Pv = pad3(v, n, nz, k, i, j, 1.0);
                double Tc = pad3(p, n, nz, k, i, j, 0.0), Tu = pad3(p, n, nz, k, i - 1, j, 0.0),
                       Tl = pad3(p, n, nz, k, i, j - 1, 0.0), Tf = pad3(p, n, nz, k - 1, i, j, 0.0);
                nV += (sq(Pv) + 0.01 * sq(epsilon)) * (sq(Tc - Tu) + sq(Tc - Tl) + sq(Tc - Tf));
            }
    return nV;
}

void or_image_step(const or_projector *P, double *out, const double *g, const double *f,
                   const double *v, double alpha, double epsilon, int iter_image, or_trace *tr,
                   int outer) {
    const int n = or_proj_n(P), nz = or_proj_nz(P);
    const int nb = or_proj_views(P) * or_proj_dets(P);
    const int np = nz * n * n;
    double *update = malloc(sizeof(double) * np), *d = malloc(sizeof(double) * np);
    double *p = malloc(sizeof(double) * np), *temp = malloc(sizeof(double) * np);
    double *Af = malloc(sizeof(double) * nb), *r = malloc(sizeof(double) * nb);
    double *q = malloc(sizeof(double) * nb), *Ad = malloc(sizeof(double) * nb);
    double AT_f_old, nV, c_1, AT_f_new, pSkalard, normAp, AdSkalarAp, c_2;

    memcpy(update, f, sizeof(double) * np); /* :87-89 */
    or_proj_A(P, Af, update);               /* :101 */
    for (int i = 0; i < nb; i++) r[i] = g[i] - Af[i];
    or_proj_AT(P, d, r); /* :110 */
    if (nz == 1) image_gradient_stencil(n, d, update, v, alpha, epsilon);
    else image_gradient_stencil3(n, nz, d, update, v, alpha, epsilon);
    AT_f_old = 0; /* :126-139 */
    for (int i = 0; i < nb; i++) AT_f_old += sq(Af[i] - g[i]);
    AT_f_old = nz == 1 ? smooth_energy(n, AT_f_old, update, v, alpha, epsilon)
                      : smooth_energy3(n, nz, AT_f_old, update, v, alpha, epsilon);
    memcpy(p, d, sizeof(double) * np); /* :141-143 */

    for (int k = 1; k <= iter_image; ++k) { /* :145 */
        or_proj_A(P, q, p);
        nV = 0; /* :152-158, over all pixels */
        if (nz > 1) nV = nv3(n, nz, p, v, epsilon);
        else
        for (int i = 1; i <= n; ++i)
            for (int j = 1; j <= n; ++j) {
                double Pv = pad_at(v, n, i, j, 1.0);
                double Tc = pad_at(p, n, i, j, 0.0), Tu = pad_at(p, n, i - 1, j, 0.0),
                       Tl = pad_at(p, n, i, j - 1, 0.0);
                nV += (sq(Pv) + 0.01 * sq(epsilon)) * (sq(Tc - Tu) + sq(Tc - Tl));
            }
        pSkalard = 0;
        for (int i = 0; i < np; i++) pSkalard += p[i] * d[i];
        normAp = 0;
        for (int i = 0; i < nb; i++) normAp += sq(q[i]);
        c_1 = pSkalard / (normAp + alpha * nV); /* :167 */

        memcpy(temp, update, sizeof(double) * np);
        double maxCP = 0;
        for (int i = 0; i < np; i++) { /* :173-178 */
            update[i] += c_1 * p[i];
            double CP = fabs(c_1 * p[i]);
            if (maxCP < CP) maxCP = CP;
        }
        if (k % ((int)(iter_image / 2 + 0.0001)) == 0) /* :180-182, each slice */
            for (int z = 0; z < nz; z++) or_medfilt2(n, update + (size_t)z * n * n);

        double sc[6] = {AT_f_old, nV, pSkalard, normAp, c_1, 0.0};
        if (k == iter_image) { /* :184-187 */
            trace_push(tr, outer, 0, k, sc, 5, 1);
            break;
        }
        if (maxCP < 1e-5) { /* :188-191 */
            trace_push(tr, outer, 0, k, sc, 5, 2);
            break;
        }
        or_proj_A(P, Af, update); /* :193-208 */
        AT_f_new = 0;
        for (int i = 0; i < nb; i++) AT_f_new += sq(Af[i] - g[i]);
        AT_f_new = nz == 1 ? smooth_energy(n, AT_f_new, update, v, alpha, epsilon)
                           : smooth_energy3(n, nz, AT_f_new, update, v, alpha, epsilon);
        if (1.1 * AT_f_old < AT_f_new && 1 < k) { /* :209-215 */
            memcpy(update, temp, sizeof(double) * np);
            trace_push(tr, outer, 0, k, sc, 5, 3);
            break;
        }
        AT_f_old = AT_f_new;
        for (int i = 0; i < nb; i++) r[i] -= c_1 * q[i]; /* :217-219 */
        or_proj_AT(P, d, r);                             /* :225 */
        if (nz == 1) image_gradient_stencil(n, d, update, v, alpha, epsilon);
        else image_gradient_stencil3(n, nz, d, update, v, alpha, epsilon);
        or_proj_A(P, Ad, d); /* :240-245 */
        AdSkalarAp = 0;
        for (int i = 0; i < nb; i++) AdSkalarAp += Ad[i] * q[i];
        c_2 = -AdSkalarAp / normAp;
        for (int i = 0; i < np; i++) p[i] = d[i] + c_2 * p[i]; /* :247-250 */
        double sc2[6] = {AT_f_old, nV, pSkalard, normAp, c_1, c_2};
        trace_push(tr, outer, 0, k, sc2, 6, 0);
    }
    memcpy(out, update, sizeof(double) * np);
    free(update); free(d); free(p); free(temp); free(Af); free(r); free(q); free(Ad);
}

void or_edge_step(int n, double *out, const double *f, const double *v, double alpha, double beta,
                  double epsilon, int iter_edge, or_trace *tr, int outer) {
    const int np = n * n;
    double *update = malloc(sizeof(double) * np), *temp = malloc(sizeof(double) * np);
    double *d = malloc(sizeof(double) * np), *nn = malloc(sizeof(double) * np);
    double nNablaD, nD, c;
    memcpy(update, v, sizeof(double) * np); /* :265-267 */
    for (int k = 1; k <= iter_edge; ++k) {  /* :287 */
        memcpy(temp, update, sizeof(double) * np);
        for (int i = 1; i <= n; ++i) /* :294-305; f zero-padded, temp one-padded */
            for (int j = 1; j <= n; ++j) {
                double dx = 0.5 * (pad_at(f, n, i + 1, j, 0.0) - pad_at(f, n, i - 1, j, 0.0));
                double dy = 0.5 * (pad_at(f, n, i, j + 1, 0.0) - pad_at(f, n, i, j - 1, 0.0));
                double nij = sq(dx) + sq(dy);
                double Tc = pad_at(temp, n, i, j, 1.0);
                double lap = 0.25 * (pad_at(temp, n, i + 1, j, 1.0) + pad_at(temp, n, i, j + 1, 1.0) -
                                     4 * Tc + pad_at(temp, n, i - 1, j, 1.0) +
                                     pad_at(temp, n, i, j - 1, 1.0));
                double gij = alpha * Tc * nij - beta * epsilon * lap + beta * (Tc - 1) / (4 * epsilon);
                nn[(i - 1) * n + (j - 1)] = nij;
                d[(i - 1) * n + (j - 1)] = -gij; /* :307-309 */
            }
        nNablaD = 0; /* :314-318, d zero-padded */
        for (int i = 1; i <= n; ++i)
            for (int j = 1; j <= n; ++j)
                nNablaD = nNablaD + sq(0.5 * (pad_at(d, n, i + 1, j, 0.0) - pad_at(d, n, i - 1, j, 0.0))) +
                          sq(0.5 * (pad_at(d, n, i, j + 1, 0.0) - pad_at(d, n, i, j - 1, 0.0)));
        nD = 0;
        for (int i = 0; i < np; i++) nD += sq(d[i]);
        double tmp = 0;
        for (int i = 0; i < np; i++) tmp += nn[i] * sq(d[i]);
        c = nD / (alpha * tmp + beta * epsilon * nNablaD + (beta / (4 * epsilon)) * nD); /* :329 */
        double maxCD = 0;
        for (int i = 0; i < np; i++) { /* :332-338 */
            update[i] = temp[i] + c * d[i];
            double CD = fabs(c * d[i]);
            if (CD > maxCD) maxCD = CD;
        }
        for (int i = 0; i < np; i++) { /* :340-344 */
            if (update[i] > 1) update[i] = 1;
            if (update[i] < 0) update[i] = 0;
        }
        double sc[3] = {nD, c, maxCD};
        if (k == iter_edge) {
            trace_push(tr, outer, 1, k, sc, 3, 1);
            break;
        }
        if (maxCD < 1e-5) {
            trace_push(tr, outer, 1, k, sc, 3, 2);
            break;
        }
        trace_push(tr, outer, 1, k, sc, 3, 0);
    }
    memcpy(out, update, sizeof(double) * np);
    free(update); free(temp); free(d); free(nn);
}

void or_edge_step_vol(int n, int nz, double *out, const double *f, const double *v, double alpha, double beta,
                      double epsilon, int iter_edge, or_trace *tr, int outer) {
    if (nz == 1) {
        or_edge_step(n, out, f, v, alpha, beta, epsilon, iter_edge, tr, outer);
        return;
    }
    const size_t np = (size_t)nz * n * n;
    double *update = malloc(sizeof(double) * np), *temp = malloc(sizeof(double) * np);
    double *d = malloc(sizeof(double) * np), *nn = malloc(sizeof(double) * np);
    double nNablaD, nD, c;
    memcpy(update, v, sizeof(double) * np);
    for (int k = 1; k <= iter_edge; ++k) {
        memcpy(temp, update, sizeof(double) * np);
        for (int z = 1; z <= nz; ++z)
            for (int i = 1; i <= n; ++i)
                for (int j = 1; j <= n; ++j) {
                    double dx = 0.5 * (pad3(f, n, nz, z, i + 1, j, 0.0) - pad3(f, n, nz, z, i - 1, j, 0.0));
                    double dy = 0.5 * (pad3(f, n, nz, z, i, j + 1, 0.0) - pad3(f, n, nz, z, i, j - 1, 0.0));
                    double dz = 0.5 * (pad3(f, n, nz, z + 1, i, j, 0.0) - pad3(f, n, nz, z - 1, i, j, 0.0));
                    double nij = sq(dx) + sq(dy) + sq(dz);
                    double Tc = pad3(temp, n, nz, z, i, j, 1.0);
                    double lap = (1.0 / 6.0) * (pad3(temp, n, nz, z, i + 1, j, 1.0) + pad3(temp, n, nz, z, i, j + 1, 1.0) +
                                                pad3(temp, n, nz, z + 1, i, j, 1.0) - 6 * Tc +
                                                pad3(temp, n, nz, z, i - 1, j, 1.0) + pad3(temp, n, nz, z, i, j - 1, 1.0) +
                                                pad3(temp, n, nz, z - 1, i, j, 1.0));
                    double gij = alpha * Tc * nij - beta * epsilon * lap + beta * (Tc - 1) / (4 * epsilon);
                    size_t idx = ((size_t)(z - 1) * n + (i - 1)) * n + (j - 1);
                    nn[idx] = nij;
                    d[idx] = -gij;
                }
        nNablaD = 0;
        for (int z = 1; z <= nz; ++z)
            for (int i = 1; i <= n; ++i)
                for (int j = 1; j <= n; ++j)
                    nNablaD = nNablaD + sq(0.5 * (pad3(d, n, nz, z, i + 1, j, 0.0) - pad3(d, n, nz, z, i - 1, j, 0.0))) +
                              sq(0.5 * (pad3(d, n, nz, z, i, j + 1, 0.0) - pad3(d, n, nz, z, i, j - 1, 0.0))) +
                              sq(0.5 * (pad3(d, n, nz, z + 1, i, j, 0.0) - pad3(d, n, nz, z - 1, i, j, 0.0)));
        nD = 0;
        for (size_t i = 0; i < np; i++) nD += sq(d[i]);
        double tmp = 0;
        for (size_t i = 0; i < np; i++) tmp += nn[i] * sq(d[i]);
        c = nD / (alpha * tmp + beta * epsilon * nNablaD + (beta / (4 * epsilon)) * nD);
        double maxCD = 0;
        for (size_t i = 0; i < np; i++) {
            update[i] = temp[i] + c * d[i];
            double CD = fabs(c * d[i]);
            if (CD > maxCD) maxCD = CD;
        }
        for (size_t i = 0; i < np; i++) {
            if (update[i] > 1) update[i] = 1;
            if (update[i] < 0) update[i] = 0;
        }
        double sc[3] = {nD, c, maxCD};
        if (k == iter_edge) {
            trace_push(tr, outer, 1, k, sc, 3, 1);
            break;
        }
        if (maxCD < 1e-5) {
            trace_push(tr, outer, 1, k, sc, 3, 2);
            break;
        }
        trace_push(tr, outer, 1, k, sc, 3, 0);
    }
    memcpy(out, update, sizeof(double) * np);
    free(update); free(temp); free(d); free(nn);
}

void or_solve(const or_projector *P, const double *g, double *f, double *v, double alpha,
              double beta, double epsilon, int iter_alt, int iter_image, int iter_edge,
              or_trace *tr) {
    const int n = or_proj_n(P), nz = or_proj_nz(P), np = nz * n * n;
    memset(f, 0, sizeof(double) * np); /* main.c:36-40 */
    for (int i = 0; i < np; i++) v[i] = 1.0;
    for (int it = 1; it <= iter_alt; ++it) { /* main.c:43-47 */
        or_image_step(P, f, g, f, v, alpha, epsilon, iter_image, tr, it);
        or_edge_step_vol(n, nz, v, f, v, alpha, beta, epsilon, iter_edge, tr, it);
    }
}

/*
 * or_msbeam.c -- CPU restatement of the reference's OpenMP row-action AT
 * solver, msbeam/CPU_OpenMP (TEST INFRASTRUCTURE ONLY; the CPU comparator
 * timed beside the GPU engine, never linked by the engine).
 *
 * Follows msbeam/CPU_OpenMP/src:
 *   posit / wray      proj.c:53-211   parallel-beam ray tracer (float)
 *   A                 proj.c:14-32    forward projection used for the data
 *   minIMAGE          main.c:213-261  one gradient step of f on a ray's pixels
 *   minEDGE           main.c:263-301  one gradient step of v on a ray's pixels
 *   MSbeam            main.c:364-394  ALL_ITER sweeps, OpenMP over views
 *   phantom           main.c:92-181   the built-in circle and bar phantom
 * with the constants of proto.h:4-17.  The arithmetic keeps the reference's
 * float/double mix expression by expression, so a single-threaded run is
 * bit-identical to the reference built without -ffast-math; with several
 * threads the updates race exactly as the reference's do (main.c:377).
 */
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MS_IMG 512   /* IMGSIZE */
#define MS_NPROJ 180 /* NPROJ   */
#define MS_NRAY 768  /* NRAY    */
#define MS_ALPHA 10
#define MS_BETA 0.35
#define MS_EPS 0.001
#define MS_FTOL 1e-8
#define MS_GRIDTOL 1e-2
#define MS_PI 3.14159265359
#define MS_MIDRAY 384

static float msq(float x) { return x * x; } /* utility.c:5 */

/* proj.c:53-65 */
static void ms_posit(int np, int nr, float *ax, float *ay, float *mx, float *my) {
    float sinth = sin(MS_PI / MS_NPROJ * np);
    float costh = cos(MS_PI / MS_NPROJ * np);
    int ind = nr - MS_MIDRAY;
    int rwidth = 1;
    float tmp_length = (float)ind * rwidth;
    *ax = -sinth * tmp_length;
    *ay = costh * tmp_length;
    *mx = costh;
    *my = sinth;
}

/* proj.c:67-211 */
int or_ms_wray(int np, int nr, int *line, float *weight) {
    float sorx, sory, cf, sf, rcosphi, tanphi, rtnphi, c, fp, w, yc;
    int ix, iy, incx, incy, index, next, flip, flipxy, numb = 0;
    ms_posit(np, nr, &sorx, &sory, &cf, &sf);
    if (sf < -MS_FTOL) {
        sf = -sf;
        cf = -cf;
    }
    flip = 0;
    if (sf * cf < -MS_FTOL * MS_FTOL) {
        flip = 1;
        cf = -cf;
    }
    if (flip > 0) sorx = -sorx;
    if (fabs(sf) <= MS_FTOL) sf = (sf < 0) ? -MS_FTOL * MS_FTOL : MS_FTOL * MS_FTOL;
    if (fabs(cf) <= MS_FTOL) cf = (cf < 0) ? -MS_FTOL * MS_FTOL : MS_FTOL * MS_FTOL;
    if (fabs(cf) > MS_FTOL) tanphi = sf / cf;
    else tanphi = 1 / (MS_FTOL * MS_FTOL);
    if (fabs(sf) > MS_FTOL) rtnphi = cf / sf;
    else rtnphi = 1 / (MS_FTOL * MS_FTOL);
    flipxy = 0;
    if (tanphi > 1 + MS_FTOL) {
        flipxy = 1;
        tanphi = 1 / tanphi;
        rtnphi = 1 / rtnphi;
        sf = sory;
        sory = sorx;
        sorx = sf;
    }
    rcosphi = (sqrt(1 + tanphi * tanphi));
    sory += MS_IMG / 2.0;
    sorx += MS_IMG / 2.0;
    c = sory - sorx * tanphi;
    if ((c - MS_IMG) >= MS_GRIDTOL) return 0;
    if (c < -MS_GRIDTOL) {
        c = -c * rtnphi;
        if ((c - MS_IMG) >= MS_GRIDTOL) return 0;
        ix = (int)c;
        iy = 0;
        fp = ((float)(ix + 1)) - c;
        yc = fp * tanphi;
        yc += -1.0;
    } else {
        ix = 0;
        iy = (int)c;
        fp = ((float)(iy + 1)) - c;
        yc = -fp;
        yc += tanphi;
    }
    next = (yc >= 0) ? 1 : 2;
    if (flipxy > 0) {
        index = iy + ix * MS_IMG;
        incx = MS_IMG;
        incy = 1;
        if (flip > 0) {
            index = MS_IMG - 1 - iy + ix * MS_IMG;
            incx = MS_IMG;
            incy = -1;
        }
    } else {
        index = iy * MS_IMG + ix;
        incx = 1;
        incy = MS_IMG;
        if (flip > 0) {
            index = MS_IMG - 1 - ix + iy * MS_IMG;
            incx = -1;
            incy = MS_IMG;
        }
    }
    for (;;) {
        if (next == 1) {
            if (iy + 1 >= MS_IMG || ix < 0) return numb;
            w = rcosphi * (1 - yc * rtnphi);
            weight[numb] = w;
            line[numb] = index;
            ++numb;
            iy++;
            index += incy;
            if (ix + 1 >= MS_IMG) return numb;
            w = rcosphi * (yc * rtnphi);
            weight[numb] = w;
            line[numb] = index;
            ++numb;
            ix++;
            index += incx;
            yc += tanphi - 1.0;
            next = (yc >= 0) ? 1 : 2;
        } else {
            if (iy >= MS_IMG || ix + 1 >= MS_IMG || ix < 0) return numb;
            w = rcosphi;
            weight[numb] = w;
            line[numb] = index;
            ++numb;
            ix++;
            index += incx;
            yc += tanphi;
            next = (yc >= 0) ? 1 : 2;
        }
    }
}

/* proj.c:14-32 */
void or_ms_A(float *g, const float *f) {
    int line[MS_IMG * 2];
    float weight[MS_IMG * 2];
    for (int i = 0; i < MS_NPROJ * MS_NRAY; ++i) g[i] = 0;
    for (int np = 0; np < MS_NPROJ; ++np)
        for (int nr = 0; nr < MS_NRAY; ++nr) {
            int numb = or_ms_wray(np, nr, line, weight);
            for (int i = 0; i < numb; ++i) g[np * MS_NRAY + nr] += f[line[i]] * weight[i];
        }
}

/* main.c:213-261 */
static void ms_min_image(const float *g, float *f, const float *v, float lambda, int np, int nr, const int *line,
                         const float *weight, int numb) {
    float d[MS_IMG * 2];
    float Af = 0.;
    for (int i = 0; i < numb; ++i) Af += f[line[i]] * weight[i];
    Af -= g[np * MS_NRAY + nr];
    for (int i = 0; i < numb; ++i) {
        int ind = line[i];
        int x = ind / MS_IMG, y = ind % MS_IMG;
        float tmp = 0., lap = 0.;
        if (x + 1 < MS_IMG) tmp += msq(v[ind]) * (f[ind + MS_IMG] - f[ind]);
        else tmp += msq(v[ind]) * (0 - f[ind]);
        if (y + 1 < MS_IMG) tmp += msq(v[ind]) * (f[ind + 1] - f[ind]);
        else tmp += msq(v[ind]) * (0 - f[ind]);
        if (x - 1 >= 0) tmp -= msq(v[ind - MS_IMG]) * (f[ind] - f[ind - MS_IMG]);
        else tmp -= (f[ind] - 0);
        if (y - 1 >= 0) tmp -= msq(v[ind - 1]) * (f[ind] - f[ind - 1]);
        else tmp -= (f[ind] - 0);
        if (x + 1 < MS_IMG) lap += f[ind + MS_IMG];
        if (y + 1 < MS_IMG) lap += f[ind + 1];
        if (x - 1 >= 0) lap += f[ind - MS_IMG];
        if (y - 1 >= 0) lap += f[ind - 1];
        lap -= 4 * f[ind];
        d[i] = -Af * weight[i] + MS_ALPHA * (tmp + msq(MS_EPS) * lap);
    }
    for (int i = 0; i < numb; ++i) {
        int ind = line[i];
        f[ind] += lambda * d[i];
        if (f[ind] < 0) f[ind] = 0;
    }
}

/* main.c:263-301 */
static void ms_min_edge(const float *f, float *v, float lambda, const int *line, int numb) {
    float d[MS_IMG * 2];
    for (int i = 0; i < numb; ++i) {
        int ind = line[i];
        int x = ind / MS_IMG, y = ind % MS_IMG;
        float a = 0., b = 0., c = 0.;
        if (x - 1 >= 0) a += msq(f[ind] - f[ind - MS_IMG]);
        else a += msq(f[ind] - 0);
        if (y - 1 >= 0) a += msq(f[ind] - f[ind - 1]);
        else a += msq(f[ind] - 0);
        a *= v[ind];
        b = v[ind] - 1;
        if (x + 1 < MS_IMG) c += v[ind + MS_IMG];
        if (y + 1 < MS_IMG) c += v[ind + 1];
        if (x - 1 >= 0) c += v[ind - MS_IMG];
        if (y - 1 >= 0) c += v[ind - 1];
        c -= 4 * v[ind];
        d[i] = -MS_ALPHA * a - MS_BETA / (4 * MS_EPS) * b + MS_BETA * MS_EPS * c;
    }
    for (int i = 0; i < numb; ++i) {
        int ind = line[i];
        v[ind] += lambda * d[i];
        if (v[ind] < 0) v[ind] = 0;
        if (v[ind] > 1) v[ind] = 1;
    }
}

/* main.c:364-394: f = 0, v = 1, lambda = 1e-3, `iters` sweeps over all rays
 * (views in parallel), lambda <- lambda / (1 + 500 lambda) after each. */
void or_ms_solve(const float *g, float *f, float *v, int iters, int nthreads) {
    for (int i = 0; i < MS_IMG * MS_IMG; ++i) {
        f[i] = 0.;
        v[i] = 1.;
    }
    float lambda = 0.001;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int it = 1; it <= iters; ++it) {
#pragma omp parallel for
        for (int j = 0; j < MS_NPROJ; ++j)
            for (int k = 0; k < MS_NRAY; ++k) {
                int line[MS_IMG * 2];
                float weight[MS_IMG * 2];
                int numb = or_ms_wray(j, k, line, weight);
                ms_min_image(g, f, v, lambda, j, k, line, weight, numb);
                ms_min_edge(f, v, lambda, line, numb);
            }
        lambda = lambda / (1 + 500 * lambda);
    }
}

/* The same sweeps with one thread in the order the GPU row-action mode runs
 * them: for each view, the rays nr = phase, phase + phases, ... for phase =
 * 0 .. phases-1.  phases = 1 is the reference's own one-thread order. */
void or_ms_solve_phased(const float *g, float *f, float *v, int iters, int phases) {
    for (int i = 0; i < MS_IMG * MS_IMG; ++i) {
        f[i] = 0.;
        v[i] = 1.;
    }
    float lambda = 0.001;
    int line[MS_IMG * 2];
    float weight[MS_IMG * 2];
    for (int it = 1; it <= iters; ++it) {
        for (int j = 0; j < MS_NPROJ; ++j)
            for (int ph = 0; ph < phases; ++ph)
                for (int k = ph; k < MS_NRAY; k += phases) {
                    int numb = or_ms_wray(j, k, line, weight);
                    ms_min_image(g, f, v, lambda, j, k, line, weight, numb);
                    ms_min_edge(f, v, lambda, line, numb);
                }
        lambda = lambda / (1 + 500 * lambda);
    }
}

/* main.c:92-181: unit-pixel circle/bar phantom, values 0..3 */
void or_ms_phantom(float *f) {
    memset(f, 0, sizeof(float) * MS_IMG * MS_IMG);
    struct { float cx, cy, r, val; } discs[] = {
        {0, 0, 180.0f, 1}, {80, 80, 30.0f, 2}, {-80, 80, 30.0f, 2.5f}, {80, -80, 30.0f, 2.25f}, {-80, -80, 30.0f, 3}};
    for (int k = 0; k < 5; k++)
        for (int i = 0; i < MS_IMG; ++i)
            for (int j = 0; j < MS_IMG; ++j) {
                float x = i - 255.5, y = j - 255.5;
                float dis = sqrt(msq(x - discs[k].cx) + msq(y - discs[k].cy));
                if (dis <= discs[k].r) f[i * MS_IMG + j] = discs[k].val;
            }
    for (int i = 0; i < MS_IMG; ++i) /* ring, main.c:127-132 */
        for (int j = 0; j < MS_IMG; ++j) {
            float x = i - 255.5, y = j - 255.5;
            float dis = sqrt(msq(x) + msq(y - 120));
            if (29 <= dis && dis <= 30.0) f[i * MS_IMG + j] = 1.25;
        }
    /* two bar patterns, main.c:135-179: rows in pairs, alternating column ranges */
    const int starts[2] = {165, 340};
    for (int s = 0; s < 2; s++)
        for (int p = 0; p < 7; p++) {
            int r0 = starts[s] + 2 * p;
            int c0 = (p % 2 == 0) ? 238 : 256, c1 = (p % 2 == 0) ? 256 : 274;
            for (int i = r0; i <= r0 + 1; ++i)
                for (int j = c0; j < c1; ++j) f[i * MS_IMG + j] = 2;
        }
}

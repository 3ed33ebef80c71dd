/*
 * at_engine.h -- native C-ABI of the GB300 Ambrosio-Tortorelli CT engine.
 *
 * Plain C types only: pointers, sizes and status codes.  Every call returns 0
 * on success or a negative AT_E* code; at_last_error() then holds a message.
 * Pointers named d_* are device (HBM) pointers; h_* are host pointers.
 * `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 *
 * Reference interfaces these entry points replace (paths relative to the
 * reference project root):
 *   at_forward / at_forward_host      A(proj, orig)             origin/GoldenC/src/proj.c:14-204
 *                                     fan-beam forward_proj     helical/rebin/src/tracing.cpp:22-147
 *   at_back / at_back_host            AStar(back, proj)         origin/GoldenC/src/proj.c:206-397
 *   at_solver_run / at_reconstruct_*  MumfordShah(alpha,beta,eps) origin/GoldenC/src/main.c:35-49
 *                                     with minimize_in_IMAGE_variable main.c:81-257 and
 *                                     minimize_in_EDGE_variable main.c:259-360
 *   at_fan_geometry                   NX NY vx vy NDETECTOR NPROJ SOURCE_TO_ISO SOURCE_TO_DET
 *                                     LENGTH_PER_DET OFF_CENTER  helical/rebin/src/main.h:16-47
 *   at_params                         ALPHA BETA EPSILON _IterAlt _IterImage _IterEdge
 *                                     origin/GoldenC/src/config.h:6-17
 * The GoldenC link-level symbols themselves (A, AStar, ...) are declared in
 * goldnc.h and exported by the same library.
 */
#ifndef AT_ENGINE_H
#define AT_ENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define AT_OK 0
#define AT_EINVAL (-1)   /* bad argument or geometry                    */
#define AT_ECUDA (-2)    /* CUDA runtime error                          */
#define AT_ENOMEM (-3)   /* device or host allocation failed            */
#define AT_ESTATE (-4)   /* call not valid in the object's current state */
#define AT_EBUDGET (-5)  /* request does not fit the admission budget   */
#define AT_ETIMEOUT (-6) /* a bounded device wait gave up               */

/* geometry kinds */
#define AT_GEOM_GOLDNC 0 /* GoldenC parallel beam: 512x512, 180 views x 767 detectors */
#define AT_GEOM_FAN 1    /* 2D fan beam with an equiangular detector                */
#define AT_GEOM_RAYS 2   /* 2D rays given one by one by their end points            */
#define AT_GEOM_CONE 3   /* 3D cone beam with a flat detector (industry3d)          */

/* 2D fan-beam geometry, the parameters of helical/rebin (main.h:16-47,
 * ms2d.cpp:30-62,172-183).  Image n x n, pixel index x*n + y (x slow),
 * image spans [0, n*pixel_mm]^2; source of view k at angle
 * view0_deg + k*view_step_deg around the image centre at sod_mm; detector j
 * (j = -ndets/2 .. ndets/2-1) at angle (j + off_center)*det_pitch_deg + 180
 * degrees from the source, sdd_mm away.  ndets must be even. */
typedef struct at_fan_geometry {
    int32_t n;
    double pixel_mm;
    int32_t nviews;
    int32_t ndets;
    double sod_mm;
    double sdd_mm;
    double det_pitch_deg;
    double off_center;
    double view0_deg;
    double view_step_deg;
} at_fan_geometry;

/* 3D cone-beam geometry, the parameters of industry3d (ct3d.h:17-56,
 * ct3d.cpp:49-77) with its cone() of tracing.cpp:51-81: volume nz x nx x ny
 * voxels of voxel_mm (SAMPLESIZE), voxel index z*nx*ny + x*ny + y; view a of
 * nproj at 2*pi*a/nproj about the z axis, source at distance sod_mm (SOD),
 * flat detector of ndx rows (z) x ndy columns of pitch_mm (PIXELSIZE) at
 * sdd_mm (SDD) from the source; cell (row, col) centred at
 * ((col - half_cols + 0.5)*pitch, (half_rows - row - 0.5)*pitch).  The
 * reference sets both half widths to NDX/2 (ct3d.cpp:90); they are separate
 * here so non-square detectors are centred.  Sinogram [nproj][ndx][ndy].
 * The engine needs nx == ny. */
typedef struct at_cone_geometry {
    int32_t nx, ny, nz;
    float voxel_mm;
    int32_t nproj;
    int32_t ndx, ndy;
    float pitch_mm;
    float sod_mm, sdd_mm;
    int32_t half_rows, half_cols;
} at_cone_geometry;

/* AT functional weights and iteration counts (config.h:6-8,15-17).
 * mode 0 ("exact") makes every projection the reference makes (29 forward and
 * 10 back projections per outer iteration at iter_image = 10).  mode 1
 * ("linear") replaces the forward projections that linearity of A makes
 * redundant (A(p_new) = A(d) + c2 A(p_old), A(f + c1 p) = A f + c1 A p when no
 * median step intervened) by sinogram updates. */
typedef struct at_params {
    double alpha;
    double beta;
    double epsilon;
    int32_t iter_alt;
    int32_t iter_image; /* >= 2 (the reference divides by iter_image/2) */
    int32_t iter_edge;
    int32_t mode;
} at_params;

typedef struct at_plan at_plan;     /* device-resident projector plan of one geometry */
typedef struct at_solver at_solver; /* device-resident state of a batch of scans      */

typedef struct at_plan_stats {
    int32_t kind;
    int32_t n, nviews, ndets;
    int64_t rays;          /* rays traced                                      */
    int64_t segments;      /* S: ray-pixel segments summed over all rays        */
    int64_t offgrid;       /* segments the reference traces off the pixel grid */
    int64_t device_bytes;  /* plan memory in HBM                               */
    int32_t max_segments;  /* longest ray                                      */
    int32_t fp_rays_per_thread; /* forward-projector variant the autotuner chose */
    int64_t bp_runs;       /* (ray, 16x16 tile) runs the back projector walks   */
    int32_t nz;            /* image slices (1 for 2D plans)                      */
    /* forward projector through shared-memory slabs (fan / ray plans), when the
     * autotuner chose it over the L1 walk: CTA shape (views x adjacent
     * detectors), rows per slab, staged columns per slab, and the CTAs that
     * gather through L1 because a ray leaves the grid; all 0 otherwise */
    int32_t slab_views, slab_rays, slab_rows, slab_wbox, slab_fallback_ctas;
    /* back projection from the pixel table (at_plan_set_back_variant): the
     * launches that use it (bit0 single scans, bit1 groups of scans sharing
     * the plan), the table's bytes in HBM and its weights; 0 without one */
    int32_t bp_table_use;
    int64_t bp_table_bytes, bp_table_weights;
} at_plan_stats;

const char *at_last_error(void);
int at_device_info(char *name, int name_len, int *sm_count, size_t *hbm_bytes);

/* ---- plans ---- */
int at_plan_create_fan(const at_fan_geometry *geom, at_plan **out);
/* at_plan_create_fan with a choice of traversal arithmetic.  AT_ALPHA_FP64 is
 * the reference's: forward_proj's lambda entry/exit, start pixel and crossing
 * merge in double (helical/rebin/src/tracing.cpp:39-146), so the traversed
 * pixel sequence is the reference's bit for bit; at_plan_create_fan uses it.
 * AT_ALPHA_FP32 runs the same steps in single precision throughout (the plain
 * form): no FP64 anywhere on the GPU, and the traversal may depart from the
 * reference's where two crossings nearly tie.  Kept to measure the precision
 * of each form against an FP64 oracle. */
#define AT_ALPHA_FP64 0
#define AT_ALPHA_FP32 1
int at_plan_create_fan_ex(const at_fan_geometry *geom, int32_t alpha_precision, at_plan **out);
int at_plan_create_goldnc(at_plan **out);
/* 3D cone beam, traced on the fly with the reference's FP32 walk
 * (industry3d/src/tracing.cpp:123-307); nothing per ray is stored. */
int at_plan_create_cone(const at_cone_geometry *geom, at_plan **out);
/* Any 2D geometry as a table of rays: h_endpoints[(view*ndets + det)*4 + 0..3]
 * = (sx, sy, dx, dy) in mm, the arguments of the reference tracer
 * forward_proj(sx, sy, dx, dy, ...) (helical/rebin/src/tracing.cpp:22-147);
 * same image frame as at_fan_geometry (x*n + y, image on [0, n*pixel_mm]^2).
 * Covers non-uniform view tables (ms2d.cpp:30-62) and parallel beams
 * (msbeam/CPU_OpenMP/src/proj.c:53-65).  The table is copied. */
int at_plan_create_rays(int32_t n, double pixel_mm, int32_t nviews, int32_t ndets, const double *h_endpoints,
                        at_plan **out);
/* Pins the forward projector of a fan-beam or ray-table plan, in place of the
 * autotuner's choice (results are bitwise the same for every variant):
 * views = rays = rows = 0 selects the walk that gathers through L1;
 * otherwise the slab projector with CTAs of `views` consecutive views x
 * `rays` adjacent detectors (rays divides 128, views * rays <= 512) and slabs
 * of `rows` image rows.  AT_EINVAL if the shape does not fit this plan (the
 * staged band wider than 256 columns, or an image edge not a multiple of 4).
 * Solvers, projection sets and servers made before the call keep the variant
 * they were made with (the plan keeps its earlier tables until it is
 * destroyed).  Not thread-safe against concurrent calls on the same plan.
 * The forward projector of the reference
 * (helical/rebin/src/tracing.cpp:22-147 applied per ray) has no such knob. */
int at_plan_set_forward_variant(at_plan *plan, int32_t views, int32_t rays, int32_t rows);
/* Selects the back projector of a fan-beam or ray-table plan for launches of
 * single scans (use bit0) and of groups of scans that share the plan (bit1):
 * a set bit gathers each pixel's terms from the plan's pixel table (the
 * traversal stored by pixel and view, with each segment's FP32 weight; built
 * on the first call that asks for it, about 4 bytes per segment plus 4 per
 * pixel and view), a clear bit walks the (ray, 16x16 tile) runs.  Results
 * are bitwise the same either way: both add the same fixed-point terms.
 * AT_EINVAL for a mask outside 0..3 or a plan the table's fields cannot hold
 * (more than 32767 detectors, or 63 rays of one view through one pixel).
 * Solvers, projection sets and servers made before the call keep the variant
 * they were made with; the table stays until the plan is destroyed.  Not
 * thread-safe against concurrent calls on the same plan.  The reference's
 * back projector (helical/rebin/src/tracing.cpp:22-147, transposed per ray)
 * has no such knob. */
int at_plan_set_back_variant(at_plan *plan, int32_t use);
void at_plan_destroy(at_plan *plan);
/* Launch form of the projectors of batches (solvers, projection sets, server
 * groups) made after the call, fan-beam and ray-table plans: 0 = one CTA per
 * work unit (the default), 1 = persistent, a grid of the resident CTAs pulling
 * (scan, view, ray block) and (scan, pixel tile) units from a queue, the
 * costlier scans' units first.  Results are bitwise the same.  On GB300 the
 * persistent form measured 8-9 % slower (C2, 16 slices; C3): a CTA's finished
 * warps wait at each unit's end while the hardware scheduler would start a new
 * CTA beside them.  The reference has no batched form (its only GPU code,
 * industry3d/cuda/main.cu:530-537, relaunches one kernel per iteration). */
int at_set_batch_launch_mode(int32_t persistent);
int at_plan_get_stats(const at_plan *plan, at_plan_stats *out);
/* Traversal of one ray as the device plan stores it: pixel indices and FP32
 * weights in visiting order.  For AT_GEOM_GOLDNC, (view, det) address the
 * traced walk (alpha = view 1..45, raynum = det 0..383) and pixel indices are
 * row*512+col of the tile-global walk (symmetry 0), all 16 tiles in order. */
int at_plan_trace_ray(const at_plan *plan, int32_t view, int32_t det, int32_t *h_pix, float *h_w,
                      int32_t cap, int32_t *n_out);

/* ---- projectors (FP32, device buffers) ---- */
/* d_sino[view][det] = sum over the ray's segments of d_img[pixel] * weight.
 * Fan beam and ray tables take stream-ordered scratch (cudaMallocAsync) for
 * the image's transposed copy, which the walk reads where rays run closer to
 * the y axis; the sums are the same either way. */
int at_forward(const at_plan *plan, const float *d_img, float *d_sino, void *stream);
/* d_img = A^T d_sino; deterministic: each pixel is an exact integer sum of
 * fixed-point terms (no float atomics), so the result does not depend on
 * scheduling */
int at_back(const at_plan *plan, const float *d_sino, float *d_img, void *stream);
/* host-buffer forms: copy in, project, copy out, synchronise */
int at_forward_host(const at_plan *plan, const float *h_img, float *h_sino);
int at_back_host(const at_plan *plan, const float *h_sino, float *h_img);

/* ---- projection sets: several images through their plans in one launch ----
 * Batched form of at_forward / at_back (the reference projects one slice per
 * call: origin/GoldenC/src/proj.h:6-7 A and AStar).  Images whose plans are
 * the same plan object are projected together, up to four per walk of the
 * plan, with results identical to at_forward / at_back on each image.  A set
 * holds device scratch: calls on one set must not overlap on the GPU. */
typedef struct at_projset at_projset;
int at_projset_create(at_plan *const *plans, int32_t n, at_projset **out);
void at_projset_destroy(at_projset *ps);
/* d_img[i] -> d_sino[i] through plans[i], i < n */
int at_projset_forward(at_projset *ps, const float *const *d_img, float *const *d_sino, void *stream);
/* d_sino[i] -> d_img[i] */
int at_projset_back(at_projset *ps, const float *const *d_sino, float *const *d_img, void *stream);

/* ---- device memory helpers for callers without a CUDA runtime binding ---- */
int at_dev_alloc(void **d_ptr, size_t bytes);
int at_dev_free(void *d_ptr);
int at_memcpy_h2d(void *d_dst, const void *h_src, size_t bytes, void *stream);
int at_memcpy_d2h(void *h_dst, const void *d_src, size_t bytes, void *stream);
int at_stream_create(void **stream);
int at_stream_destroy(void *stream);
int at_stream_sync(void *stream);

/* ---- AT solver over a batch of scans ----
 * Every scan has its own plan (geometry), sinogram, f, v and CG state; all
 * scans advance together, one launch per kernel for the whole batch, and each
 * decides its own early exits on the device.  One outer iteration (image step
 * + edge step) is captured once as a CUDA graph and replayed. */
int at_solver_create(at_plan *const *plans, int32_t nscans, const at_params *params, at_solver **out);
void at_solver_destroy(at_solver *s);
/* Device bytes the solver would hold for these plans (admission control). */
int at_solver_footprint(at_plan *const *plans, int32_t nscans, size_t *bytes);
int at_solver_set_sino(at_solver *s, int32_t scan, const float *d_sino, void *stream);
int at_solver_set_sino_host(at_solver *s, int32_t scan, const float *h_sino, void *stream);
/* f = 0, v = 1 for all scans (main.c:36-40); called by at_solver_run. */
int at_solver_reset(at_solver *s, void *stream);
/* Runs params.iter_alt outer iterations on `stream` (asynchronous). */
int at_solver_run(at_solver *s, void *stream);
/* Runs `count` outer iterations without resetting (for interleaving). */
int at_solver_step(at_solver *s, int32_t count, void *stream);
int at_solver_get(at_solver *s, int32_t scan, float *d_f, float *d_v, void *stream);
int at_solver_get_host(at_solver *s, int32_t scan, float *h_f, float *h_v, void *stream);
/* Scalar trajectory of one scan: records of {outer, step, k, exit, s[6]} as
 * doubles (10 per record), the scalars the reference prints (main.c:251,330). */
int at_solver_trace(at_solver *s, int32_t scan, double *h_recs, int32_t cap, int32_t *n_out);
/* Kernel launches one outer iteration makes (graph node count). */
int at_solver_launches_per_outer(const at_solver *s, int32_t *n);

/* One call, host buffers: sinogram in, f and v out (H2D, solve, D2H). */
int at_reconstruct_host(const at_plan *plan, const at_params *params, const float *h_sino, float *h_f,
                        float *h_v);

/* ---- image quality on the GPU (device buffers, result to the host) ----
 * PSNR = 10 log10(peak^2 / MSE) as msbeam/CPU_OpenMP/PSNR.m:1-12 computes it
 * (that script fixes peak = 256); peak <= 0 selects max(ref).
 * SSIM with the defaults of msbeam/CPU_OpenMP/ssim_index.m: 11x11 Gaussian
 * window of sigma 1.5, K1 = 0.01, K2 = 0.03, valid window positions, mean of
 * the map; dynamic_range is its L. */
int at_psnr(const float *d_x, const float *d_ref, int64_t n, double peak, double *h_psnr, void *stream);
int at_ssim(const float *d_x, const float *d_ref, int32_t h, int32_t w, double dynamic_range, double *h_ssim,
            void *stream);

/* ---- row-action AT: msbeam/CPU_OpenMP on the GPU ----
 * msbeam's algorithm (msbeam/CPU_OpenMP/src/main.c:213-394): per ray, one
 * gradient step of the image (minIMAGE) and one of the edge field (minEDGE) on
 * the ray's pixels, sweeping all rays of its parallel beam (proj.c:53-211:
 * view k at pi*k/nproj, ray r at offset r - nray/2 pixels) with a step that
 * shrinks after each sweep.  The reference races over views with OpenMP; here
 * the rays of a view that are `phases` apart run together (they share no
 * pixel or neighbour) and views and phases follow one another, so the result
 * is deterministic.  Images n x n, sinograms [nproj][nray], nslices of each
 * side by side. */
typedef struct at_rowaction at_rowaction;
typedef struct at_rowaction_params {
    float alpha;        /* ALPHA (proto.h:8; 10)                                   */
    double beta;        /* BETA (0.35)                                             */
    double epsilon;     /* EPSILON (0.001)                                         */
    float lambda0;      /* first step (main.c:371; 0.001)                          */
    float lambda_decay; /* after a sweep lambda <- lambda/(1 + decay*lambda) (500) */
    int32_t sweeps;     /* ALL_ITER (10)                                           */
    int32_t phases;     /* >= 3; 4 by default                                      */
} at_rowaction_params;
/* traces msbeam's rays once (wray, bit-identical) and keeps them on the device */
int at_rowaction_create(int32_t n, int32_t nproj, int32_t nray, at_rowaction **out);
void at_rowaction_destroy(at_rowaction *ra);
int at_rowaction_segments(const at_rowaction *ra, int64_t *segments);
/* pixels (index y*n + x as msbeam addresses them) and weights of one ray */
int at_rowaction_trace(const at_rowaction *ra, int32_t view, int32_t ray, int32_t *h_pix, float *h_w, int32_t cap,
                       int32_t *n_out);
/* msbeam's projection A (proj.c:14-32) on the same traces: d_g = A d_f */
int at_rowaction_forward(const at_rowaction *ra, int32_t nslices, const float *d_f, float *d_g, void *stream);
/* f = 0, v = 1, then the sweeps (main.c:364-394); device buffers on `stream`.
 * The run is captured once as a CUDA graph and replayed while the slice count,
 * buffers and parameters stay the same; calls on one handle run in order. */
int at_rowaction_run(const at_rowaction *ra, int32_t nslices, const float *d_g, float *d_f, float *d_v,
                     const at_rowaction_params *prm, void *stream);

/* ---- continuous-batching server ----
 * Requests are admitted into a running batch once they have arrived and
 * their device state fits the HBM budget and a slot is free; every round
 * advances all admitted requests by one outer iteration with one launch per
 * kernel for the whole mix; a finished request's f and v are copied out and
 * its slot and memory go to the next request.  Each result is independent of
 * the mix it ran in.  Reference counterpart: none (GoldenC runs one
 * reconstruction per process, main.c:51-79); each request runs MumfordShah
 * (main.c:35-49) on its own data. */
typedef struct at_server at_server;
typedef struct at_server_config {
    size_t hbm_budget_bytes;  /* device state of admitted requests (plans not counted) */
    int32_t max_active;       /* slots: requests advanced together                     */
    double alpha, beta, epsilon;
    int32_t iter_image, iter_edge, mode;
    int32_t fp_rays_per_thread; /* forward-projector variant for the whole run (0 = 1)  */
} at_server_config;
typedef struct at_server_stats {
    int64_t submitted, completed, rounds;
    double p50_latency_s, p99_latency_s, max_latency_s; /* completion - arrival */
    double slices_per_s;      /* completed / (last completion - first admitted arrival) */
    double busy_s;            /* time spent in rounds                                   */
    size_t peak_state_bytes;
    int64_t psnr_stops;       /* requests finished by their quality target before iter_alt */
} at_server_stats;
int at_server_create(const at_server_config *cfg, at_server **out);
void at_server_destroy(at_server *s);
/* Queues a request; arrival_s is relative to the server clock, which starts at
 * the first at_server_run.  The sinogram is copied; the plan must outlive it. */
int at_server_submit(at_server *s, at_plan *plan, const float *h_sino, int32_t iter_alt, double arrival_s,
                     int64_t *id);
/* Serves until every queued request is done (or max_seconds passed). */
int at_server_run(at_server *s, double max_seconds);
int at_server_result(at_server *s, int64_t id, float *h_f, float *h_v, double *latency_s, double *wait_s);
/* at_server_submit with a quality stop (the "equal PSNR" criterion of the
 * serving benchmark): after every outer iteration the server measures
 * PSNR(f, h_ref) on the GPU, 10 log10(peak^2 / MSE) as msbeam/CPU_OpenMP's
 * PSNR.m:11 (peak <= 0: max of h_ref), and finishes the request as soon as it
 * reaches target_psnr_db, or after iter_alt outer iterations.  h_ref (n x n,
 * or nz x n x n) is copied and held in HBM with the request; it counts against
 * the admission budget.  A request's result depends only on its data, so it
 * stops at the same iteration alone and in any mix. */
int at_server_submit_psnr(at_server *s, at_plan *plan, const float *h_sino, int32_t iter_alt, double arrival_s,
                          const float *h_ref, double target_psnr_db, double peak, int64_t *id);
/* Outer iterations a finished request ran, its last measured PSNR (NaN without
 * a quality stop) and whether the quality target ended it before iter_alt. */
int at_server_result_info(const at_server *s, int64_t id, int32_t *iterations, double *psnr_db,
                          int32_t *stopped_by_psnr);
int at_server_get_stats(const at_server *s, at_server_stats *out);

/* ---- forward projection that allocates no device memory ----
 * No counterpart in the reference.  For callers that may not allocate device
 * memory (their device memory belongs to another allocator's pool, or they
 * run where cudaMalloc's implicit device synchronisation is not allowed):
 * computes d_r = d_g - A d_img and *d_energy = sum (A d_img - d_g)^2 (FP64,
 * device pointer) with the forward projector and its fused reduction, taking
 * the reduction's scratch from a fixed 256 KiB array compiled into the
 * library instead of allocating it.  Plans whose forward projection needs more
 * than that (more than about 32,700 CTAs) are rejected with AT_EINVAL.  The
 * first call on a device looks up the array's address (make it before any
 * stream capture); calls share the array, so calls that overlap on the GPU
 * race and must not be issued. */
int at_forward_residual_noalloc(const at_plan *plan, const float *d_img, const float *d_g, float *d_r,
                                double *d_energy, void *stream);

#ifdef __cplusplus
}
#endif
#endif

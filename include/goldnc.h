/*
 * goldnc.h -- GoldenC drop-in symbols exported by libat_engine.so.
 *
 * Same names, signatures and semantics as the reference's origin/GoldenC
 * (fixed geometry of origin/GoldenC/src/config.h:10-13: 512x512 image,
 * 180 views x 767 detectors; row-major FP64 host arrays owned by the caller;
 * outputs fully overwritten).  The work runs on the GPU in FP32 with FP64
 * reductions; arrays are copied host<->device on every call.
 *
 * The functions return void like the reference's.  On failure they print a
 * message to stderr, leave the output untouched and set at_last_error()
 * (at_engine.h); goldnc_status() returns the last call's status code.
 */
#ifndef GOLDNC_H
#define GOLDNC_H

#ifdef __cplusplus
extern "C" {
#endif

#define GOLDNC_H_PIX 512  /* imageHight */
#define GOLDNC_W_PIX 512  /* imageWidth */
#define GOLDNC_DETS 767   /* projWidth  */
#define GOLDNC_VIEWS 180  /* nAlpha     */

/* origin/GoldenC/src/proj.h:6, proj.c:14-204 */
void A(double proj[GOLDNC_VIEWS][GOLDNC_DETS], double orig[GOLDNC_H_PIX][GOLDNC_W_PIX]);
/* origin/GoldenC/src/proj.h:7, proj.c:206-397 */
void AStar(double back[GOLDNC_H_PIX][GOLDNC_W_PIX], double proj[GOLDNC_VIEWS][GOLDNC_DETS]);
/* origin/GoldenC/src/main.c:25-27,81-257 (out may alias f or v) */
void minimize_in_IMAGE_variable(double out[GOLDNC_H_PIX][GOLDNC_W_PIX], double g[GOLDNC_VIEWS][GOLDNC_DETS],
                                double f[GOLDNC_H_PIX][GOLDNC_W_PIX], double v[GOLDNC_H_PIX][GOLDNC_W_PIX],
                                double alpha, double epsilon, int IterImage);
/* origin/GoldenC/src/main.c:28-30,259-360 (out may alias f or v) */
void minimize_in_EDGE_variable(double out[GOLDNC_H_PIX][GOLDNC_W_PIX], double f[GOLDNC_H_PIX][GOLDNC_W_PIX],
                               double v[GOLDNC_H_PIX][GOLDNC_W_PIX], double alpha, double beta,
                               double epsilon, int IterEdge);
/* origin/GoldenC/src/main.c:31,366-390 (in place) */
void medfilt2(double f[GOLDNC_H_PIX][GOLDNC_W_PIX]);
/* origin/GoldenC/src/main.c:35-49.  Works on the caller's globals
 * `double f[512][512], v[512][512], gDelta[180][767]` (as GoldenC's main.c
 * defines them), bound at load time as weak symbols; if the program does not
 * define them the call fails with AT_ESTATE.  Iteration counts are the
 * reference's defaults (_IterAlt = _IterImage = _IterEdge = 10) unless
 * goldnc_set_iterations() changed them. */
void MumfordShah(double alpha, double beta, double epsilon);

/* extensions (no reference counterpart) */
int goldnc_status(void);
void goldnc_set_iterations(int iter_alt, int iter_image, int iter_edge);

#ifdef __cplusplus
}
#endif
#endif

/*
 * mmo_diag.h -- measurement entry points of libmmo_gpu.so.
 *
 * The reference has no counterpart beyond wall-clock logging (Utls.time_it,
 * UnixJunkie/MMO src/utls.ml:7-10, and the "frames ... @ Hz" line of
 * src/lds.ml:2052-2087).  These give per-stage device times of a scoring call
 * and a measured FP32 FMA peak for roofline fractions.
 */
#ifndef MMO_DIAG_H
#define MMO_DIAG_H

#include "mmo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Record CUDA events around each stage of every scoring call (on the call's
 * stream) when on != 0. */
int mmo_set_profiling(mmo_ctx* ctx, int on);

/* Device milliseconds of the last scoring call's stages, ms[4]: ms[0] pose
 * rebuild, ms[1] pair sweep (its kernel launches only), ms[2] finishing
 * (piece reduction, intra energy and gradient, reverse kinematics), ms[3]
 * entry sort of the cut-off sweep (0 without it).  Waits for those events. */
int mmo_stage_times(mmo_ctx* ctx, float* ms);

/* Pair evaluations of the last batched scoring call: *evaluated counts the
 * (entry, protein atom) pairs the sweep computed (the cut-off sweep computes
 * 32 * entries_per_lane pairs for each protein atom a warp visits), *all the
 * pairs of the batch (poses x ligand atoms x protein atoms).  Waits for the
 * device. */
int mmo_pair_count(mmo_ctx* ctx, double* evaluated, double* all);

/* Kernels (this library's own) that the last scoring call launched. */
int mmo_last_launches(const mmo_ctx* ctx, int* kernels);

/* FP32 FMA throughput of the device: a grid of independent FMA chains timed
 * with CUDA events; *tflops = 2 * FMAs / time. */
int mmo_fp32_fma_peak(mmo_ctx* ctx, double* tflops, double* ms);

/* The last mmo_build_grids: lattice points inside the mask, (point, protein
 * atom) pairs the build kernel evaluated for them, and those within 12 A (the
 * pairs the grid values need); the pair counts are made only while
 * mmo_set_profiling is on (else 0).  Any pointer may be NULL. */
int mmo_grid_build_stats(const mmo_ctx* ctx, double* points, double* pairs_evaluated,
                         double* pairs_within_cutoff);

/* Pairs (posed ligand atom, protein atom) closer than r in the last scoring
 * call that rebuilt its poses in the library's work buffers (a batched call,
 * B > 1), counted by a brute kernel over the posed coordinates (hi + lo): the
 * roofline's second denominator, the pairs within the 12 A cutoff.  No
 * counterpart in the reference.  Synchronous. */
int mmo_diag_pairs_within(mmo_ctx* ctx, double r, double* count);

/* Accuracy check of the device's double-float sine and cosine (no
 * counterpart in the reference; the one-pose kernel takes the angles' sines
 * and cosines from it instead of the FP64 library): for n host floats x,
 * out[4 i .. 4 i + 3] = sin(x_i) hi, lo, cos(x_i) hi, lo, the values being
 * hi + lo.  Synchronous. */
int mmo_diag_sincos(mmo_ctx* ctx, int n, const float* x, float* out);

/* Failure-path check of the device-side waits (no counterpart in the
 * reference).  The sweep kernels wait for their TMA copies into shared memory
 * on an mbarrier with a bounded number of polls; a wait that gives up sets a
 * device-side error flag that mmo_sync reports as MMO_ETIMEOUT, and the CTA
 * then waits once more, with the default bound, for the copy in flight before
 * it returns, so that nothing is left waiting.  This sets the poll limit of
 * the first wait of every later launch: 0 makes it give up at once (the
 * copies still land during the second wait); polls < 0 restores the default
 * (2^22).  Results of a call whose wait gave up are not valid. */
int mmo_diag_set_wait_polls(mmo_ctx* ctx, long long polls);

#ifdef __cplusplus
}
#endif
#endif

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

/* Device milliseconds of the last scoring call's stages: ms[0] pose rebuild
 * (+ intra energy), ms[1] pair sweep (all launches), ms[2] finishing pass
 * (reduction, intra gradient, reverse kinematics).  Waits for those events. */
int mmo_stage_times(mmo_ctx* ctx, float* ms);

/* FP32 FMA throughput of the device: a grid of independent FMA chains timed
 * with CUDA events; *tflops = 2 * FMAs / time. */
int mmo_fp32_fma_peak(mmo_ctx* ctx, double* tflops, double* ms);

#ifdef __cplusplus
}
#endif
#endif

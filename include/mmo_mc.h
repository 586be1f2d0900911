/*
 * mmo_mc.h -- Monte Carlo chains in dihedral space on the GPU.
 *
 * The counterpart of Lds.simulate_lig (UnixJunkie/MMO src/lds.ml:882-995),
 * which runs one chain on the host and calls the scoring closures every step.
 * Here `chains` chains of the context's ligand in its pocket advance together:
 * each step proposes a move for every chain (rigid on even steps, one torsion
 * on odd steps, src/lds.ml:659-660,883), scores all trial poses in one batched
 * call (the MC pose map x = R (y - centroid) + t of
 * Mol.center_rotate_translate_copy, src/mol.ml:705-710) and applies the
 * Metropolis test E' <= E or U < exp(-(E' - E) / kT) in FP64
 * (src/lds.ml:931-934), with the reference's resets (hard region of interest,
 * E_inter = 0) and its step-size adaptation from sliding windows of accept /
 * reject events.  A reset (reset_run_params, src/lds.ml:652-671) puts the
 * rigid part of the pose back to the start pose and the rigid steps to their
 * initial values, clears the rigid window and sets the current and best
 * energies to +inf, so the next clean trial is accepted; the conformer, the
 * bond steps and the bond windows stay.  The energy returned for a chain
 * whose last frame was a reset is therefore +inf.  A ligand without rotatable
 * bonds makes no move on conformer frames.  Random numbers come from
 * Philox4x32-10 keyed by the seed and counted by (chain, step, draw), so a run
 * is reproducible and independent of the number of chains.  Every minimize_every steps the chains
 * run minimize_iters iterations of gradient descent on the analytic gradient
 * (a step of length eta in the max norm along -dE/d(dofs), kept and lengthened
 * x1.2 when the energy drops, else halved).  The step sequence of a block of
 * steps is captured once in a CUDA graph and replayed.
 */
#ifndef MMO_MC_H
#define MMO_MC_H

#include "mmo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { MMO_MC_UNIFORM = 0, MMO_MC_GAUSSIAN = 1 };

typedef struct mmo_mc_params {
  double kT;             /* kcal/mol (0.593 at 298 K) */
  double rot_step;       /* rad: half-width (uniform) or sigma (Gaussian) of a rigid rotation */
  double trans_step;     /* A: per axis, half-width or sigma of a translation */
  double tors_step;      /* rad: half-width or sigma of a torsion move */
  int move_law;          /* MMO_MC_UNIFORM: Move.rand_rot / rand_trans / Mol.tweak_rbond
                            (src/move.ml:14-54, src/mol.ml:635-647): an angle in [-dr, dr]
                            about Ox, Oy or Oz, a shift in [-1, 1]^3 dt, a torsion in
                            [-dr_i, dr_i]; MMO_MC_GAUSSIAN: a normal angle about a uniform
                            axis, normal shifts, a normal torsion change */
  int adapt;             /* 1: per chain, the rigid steps after every 100 rigid frames and
                            each bond's step after every 100 nrb conformer frames, x0.95 /
                            x1.05 when the acceptance over the last 100 events of that kind
                            (a sliding window, src/SW.ml:7-37) is <= 0.45 / >= 0.55, angles
                            capped at pi (src/lds.ml:586-621, 962-988) */
  int flip_every;        /* uniform law: a conformer frame whose count of earlier conformer
                            frames is a positive multiple of flip_every draws in [-pi, pi]
                            (Mol.flip_rbond, src/lds.ml:783-793); 0: never */
  int minimize_every;    /* steps between minimisations; 0: none */
  int minimize_iters;    /* gradient-descent iterations per minimisation */
  double gd_step;        /* first gradient-descent step (A or rad, max norm) */
  unsigned long long seed;
  int use_grid;          /* 1: inter energy from the precomputed grids (MMO_F_GRID, mmo_grid.h),
                            the reference's default (src/lds.ml:1963-1975); 0: pair sums */
  double roi_center[3];  /* centre of the region of interest, in the caller's frame */
  double roi_radius;     /* > 0: hard ROI (lds --hard-ROI): a trial whose ligand centre (the
                            translation of the MC pose map) lies farther than roi_radius from
                            roi_center resets the chain (src/lds.ml:908-916); <= 0: off */
  int reset_on_zero_inter; /* 1: a trial whose inter energy is exactly 0 (the ligand left
                            the pocket) resets the chain (src/lds.ml:918-927) */
  int too_long_ends_chain; /* 1: an over-long trial conformer (Mol.Too_long) ends the chain,
                            as the reference's exception ends its frame loop
                            (src/lds.ml:989-991); 0: the trial is rejected */
} mmo_mc_params;

/* Device buffers of a run.  dofs holds the start poses on entry and the final
 * poses on return ([chains][6 + nrb], the optimiser layout); E the final
 * energies.  The other pointers may be NULL; the trace buffers, when given,
 * receive every step's trial pose, its energy and what became of it. */
typedef struct mmo_mc_state {
  float* dofs;
  double* E;
  float* best_dofs;      /* [chains][6 + nrb] lowest-energy pose seen */
  double* best_E;        /* [chains] */
  int* accepted;         /* [chains] accepted Metropolis moves */
  int* status;           /* [chains] OR of the status bits (MMO_S_*) of every scored pose;
                            trial poses with a status bit set are rejected */
  int* resets;           /* [chains] resets of the chain (out of the ROI, or E_inter = 0) */
  float* trace_dofs;     /* [steps][chains][6 + nrb] the trial pose of every step */
  double* trace_E;       /* [steps][chains] its energy */
  int* trace_event;      /* [steps][chains] MMO_MC_ACCEPTED | MMO_MC_RESET | MMO_MC_STOPPED |
                            MMO_MC_BLOCKED (the trial was not clean) */
} mmo_mc_state;

enum { MMO_MC_ACCEPTED = 1, MMO_MC_RESET = 2, MMO_MC_STOPPED = 4, MMO_MC_BLOCKED = 8 };

/* Run `steps` steps of `chains` chains on `stream` (NULL: the legacy default
 * stream).  use_graph 1 captures a block of min(steps, minimize_every or 50)
 * steps (with the minimisation that ends it) once per parameter set and
 * replays it; 0 launches the same sequence directly (the results are the same
 * bit for bit).  The first call for a chain count allocates work buffers.
 * Returns MMO_EINVAL for bad arguments, MMO_ESTATE without a ligand or with a
 * capture already running on the stream. */
int mmo_mc_run(mmo_ctx* ctx, int chains, int steps, const mmo_mc_params* params,
               const mmo_mc_state* state, void* stream, int use_graph);

/* Philox4x32-10 blocks of the chains' generator, for checking it: out[i] =
 * philox(counter (i, c1, c2, 0), key (k0, k1)) for i < n, out a device array
 * of 4 n uint32. */
int mmo_philox4x32(mmo_ctx* ctx, unsigned k0, unsigned k1, unsigned c1, unsigned c2, int n,
                   unsigned* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif

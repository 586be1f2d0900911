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
 * (src/lds.ml:931-934).  Random numbers come from Philox4x32-10 keyed by the
 * seed and counted by (chain, step, draw), so a run is reproducible and
 * independent of the number of chains.  Every minimize_every steps the chains
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
  int adapt;             /* 1: per chain, step sizes x0.95 / x1.05 after each block of 100
                            moves with acceptance <= 0.45 / >= 0.55 (src/lds.ml:586-621) */
  int flip_every;        /* uniform law: every flip_every-th torsion move draws in [-pi, pi]
                            (Mol.flip_rbond); 0: never */
  int minimize_every;    /* steps between minimisations; 0: none */
  int minimize_iters;    /* gradient-descent iterations per minimisation */
  double gd_step;        /* first gradient-descent step (A or rad, max norm) */
  unsigned long long seed;
  int use_grid;          /* 1: inter energy from the precomputed grids (MMO_F_GRID, mmo_grid.h),
                            the reference's default (src/lds.ml:1963-1975); 0: pair sums */
} mmo_mc_params;

/* Device buffers of a run.  dofs holds the start poses on entry and the final
 * poses on return ([chains][6 + nrb], the optimiser layout); E the final
 * energies.  The other pointers may be NULL. */
typedef struct mmo_mc_state {
  float* dofs;
  double* E;
  float* best_dofs;      /* [chains][6 + nrb] lowest-energy pose seen */
  double* best_E;        /* [chains] */
  int* accepted;         /* [chains] accepted Metropolis moves */
  int* status;           /* [chains] OR of the status bits (MMO_S_*) of every scored pose;
                            trial poses with a status bit set are rejected */
} mmo_mc_state;

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

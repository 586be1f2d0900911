/*
 * mmo_systems.h -- ragged batches of independent (pocket, ligand) systems.
 *
 * No counterpart in the reference, which docks one ligand into one receptor
 * per run (src/lds.ml: the protein closure of src/lds.ml:1952-1979 and the
 * ligand of src/lds.ml:702-739 are fixed for the process).  Here many systems,
 * each with its own protein, ligand and number of poses, are scored by one
 * pass of the same kernels: the poses of all systems are rebuilt in one
 * launch, the (pose, ligand atom) entries of each system are grouped in one
 * launch, and one persistent launch sweeps every (system, protein piece) work
 * item.  Every pose's energy and gradient equal those of the same pose scored
 * alone through mmo_set_protein / mmo_set_ligand / mmo_score_poses_device with
 * the same settings (the cut-off sweep's results do not depend on the batch).
 *
 * Packed layout: the poses of system 0, then of system 1, ...; a pose has
 * 6 + nrb_s DOFs in the optimiser layout [x, y, z, a, b, g, tau ...]
 * (src/optim.ml:19-22), so dofs and grad are ragged rows; E and status have
 * one entry per pose.  mmo_systems_layout gives the offsets.
 */
#ifndef MMO_SYSTEMS_H
#define MMO_SYSTEMS_H

#include "mmo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mmo_system {
  /* the protein, as mmo_set_protein */
  int n_prot;
  const double *prot_x, *prot_y, *prot_z, *prot_q;
  const int* prot_anum;
  /* the ligand, as mmo_set_ligand */
  int n_lig;
  const double *lig_x, *lig_y, *lig_z, *lig_q;
  const int* lig_anum;
  const uint8_t* interacting;
  int nrb;
  const int* bond_lr;
  const int* group_offsets;
  const int* group_atoms;
  /* poses of this system in every batch (0 allowed) */
  int poses;
} mmo_system;

/* Set the context's batch of systems (replacing an earlier one; the
 * single-system protein and ligand stay as they are).  Copies every array.
 * The physics (mmo_set_physics) and the cut-off settings (mmo_set_cull,
 * mmo_set_tiles) apply to the batch as to the single system. */
int mmo_set_systems(mmo_ctx* ctx, int nsys, const mmo_system* systems);

/* Sizes of the packed layout: *total_poses, *total_dofs (floats); pose_off
 * and dof_off (each nsys + 1 ints, may be NULL) the first pose and first DOF
 * float of each system. */
int mmo_systems_layout(const mmo_ctx* ctx, int* total_poses, int* total_dofs, int* pose_off,
                       int* dof_off);

/* Score every pose of the batch on `stream` (NULL: the legacy default
 * stream): device pointers, d_grad (packed like d_dofs) with MMO_F_GRAD, flags
 * as mmo_score_poses.  Allocates work buffers on the first call for a batch
 * or plan; later calls allocate nothing and may be captured in a CUDA graph. */
int mmo_score_systems_device(mmo_ctx* ctx, const float* d_dofs, int flags, double* d_E,
                             float* d_grad, int* d_status, void* stream);

/* Autotuner of the batch's sweep: times entries per lane (1, 2, 4), piece
 * atoms (256, 512) and threads per CTA (128, 256, 512 where the registers
 * allow) on this batch and keeps the fastest as the context's settings
 * (mmo_set_cull / mmo_set_tiles).  Arguments as mmo_score_systems_device,
 * whose outputs it leaves as the chosen plan computes them; *ms (may be NULL)
 * the chosen plan's device milliseconds.  Refused inside a stream capture. */
int mmo_tune_systems(mmo_ctx* ctx, const float* d_dofs, int flags, double* d_E, float* d_grad,
                     int* d_status, void* stream, double* ms);

/* The plan of the batch's last scoring call. */
int mmo_systems_plan(const mmo_ctx* ctx, int* per_lane, int* threads, int* piece_atoms);

/* mmo_score_systems_device with host buffers (copies in and out through
 * pinned staging). */
int mmo_score_systems(mmo_ctx* ctx, const float* dofs, int flags, double* E, float* grad,
                      int* status);

#ifdef __cplusplus
}
#endif
#endif

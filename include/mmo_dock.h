/*
 * mmo_dock.h -- binding-site clients of the scorer: protein masks, clash
 * filters, exhaustive rigid docking, placement in the ROI, desolvation.
 *
 * All lattice work uses the lattice of the context's grids (mmo_grid.h), as
 * the reference keeps one simulation grid for the grids and the masks
 * (src/lds.ml:1956-1990).  Masks hold one byte per lattice point (i fastest).
 * Frames: the protein's coordinate frame, as everywhere in this ABI.
 */
#ifndef MMO_DOCK_H
#define MMO_DOCK_H

#include "mmo_grid.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- protein masks ------------------------------------------------------- */
/* Lds.vdW_volume and Lds.first_solvent_shell (src/lds.ml:149-196) of the
 * protein of mmo_set_protein on the grids' lattice: vdW volume = points within
 * radius[i] of an atom; solvent shell = points within radius[i] + r_water of an
 * atom and in no atom's volume (Const.r_H2O = 1.4 A).  radius: one per protein
 * atom in mmo_set_protein order (the .pqrs radius column, Mol.get_radius). */
int mmo_build_masks(mmo_ctx* ctx, const double* radius, double r_water);
int mmo_load_masks(mmo_ctx* ctx, const uint8_t* vdw, const uint8_t* shell);
/* host copies of the masks (either may be NULL) */
int mmo_mask_values(mmo_ctx* ctx, uint8_t* vdw, uint8_t* shell);

/* ---- clash filters --------------------------------------------------------- */
#define MMO_CLASH_INTRA 1  /* Mol.ligand_atoms_clash_fast (src/mol.ml:1077-1088): a pair at
                              topological distance >= 3 closer than 0.8 (r_i + r_j) */
#define MMO_CLASH_HEAVY 2  /* Mol.heavy_atom_clash (src/mol.ml:1170-1190): a ligand heavy atom
                              closer than 0.8 (r_i + r_j) to a protein heavy atom */
#define MMO_CLASH_GRID 4   /* Mol.protein_ligand_clash (src/mol.ml:1195-1207): a corner of an
                              atom's lattice cell in the protein's vdW volume (needs the masks) */

/* The clash tests of B poses (dofs as mmo_score_poses, flags MMO_F_RECENTER or
 * 0): out[b] = the MMO_CLASH_* bits (of `tests`) that hold.  Radii are
 * Ptable.vdW_radii by element (src/ptable.ml:41-53). */
int mmo_clash_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags, int tests,
                           int* d_out, void* stream);
int mmo_clash_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, int tests, int* out);

/* ---- rotations --------------------------------------------------------------- */
/* SO3.rotations (src/SO3.ml:18-46): the n super-Fibonacci samples of SO(3)
 * (Alexa, CVPR 2022) as row-major 3x3 matrices, R[9 n]. */
int mmo_so3_rotations(int n, double* R);

/* ---- exhaustive rigid docking ------------------------------------------------ */
typedef struct mmo_dock_spec {
  double roi_center[3];   /* the ROI sphere (ROI.from_bild) */
  double roi_radius;
  double trans_step;      /* A between positions (--ext dx,n) */
  int n_rotations;        /* super-Fibonacci rotations (--ext dx,n) */
  int topk;               /* best scores to return, 1..1024 (-top) */
  double const_intra;     /* the rigid ligand's E_intra, added to every score */
  const double* lig_radius; /* [L] ligand atom radii, or NULL: Ptable.vdW_radii */
} mmo_dock_spec;

typedef struct mmo_dock_result {
  int n_top;              /* scores returned (fewer than topk when fewer poses scored) */
  double best_score;      /* +inf when no pose was scored */
  double best_pos[3];
  int best_rot;           /* index of the best pose's rotation */
  long long positions;    /* positions inside the ROI */
  long long poses;        /* positions x rotations */
  long long scored;       /* poses scored (clash-free) */
  long long clashed;      /* poses dropped by the vdW clash test */
  double ms;              /* device milliseconds of the sweep and the selection */
} mmo_dock_result;

/* Lds.exhaustive_rigid_ligand_docking (src/lds.ml:1040-1114) with the
 * interpolated inter energy (mmo_grid.h) and the protein's vdW volume
 * (mmo_build_masks): every position of the lattice Grid.from_box(trans_step)
 * of the ROI's bounding cube inside the ROI (positions whose cell is wholly in
 * the vdW volume skipped when the ligand's centre is inside one of its atoms),
 * every rotation; a pose whose atoms touch the vdW volume is dropped, the
 * others scored const_intra + E_inter.  top_scores (ascending) and
 * top_frames (frame = rotation + n_rotations * position index, position
 * index = i + j d + k d^2, the reference's loop order; ties go to the smaller
 * frame) receive the n_top best; the ligand is the centred reference
 * conformer of mmo_set_ligand. */
int mmo_dock_exhaustive(mmo_ctx* ctx, const mmo_dock_spec* spec, double* top_scores,
                        long long* top_frames, mmo_dock_result* result);

/* ---- placement ------------------------------------------------------------- */
/* Lds.place_ligand_in_ROI (src/lds.ml:308-345): n placements of the ligand, each
 * a uniform point of the ROI (drawn in its cube, kept inside the sphere) and a
 * uniform random rotation (Move.rand_rot_full) without a heavy-atom clash with
 * the protein.  Candidates are drawn from Philox4x32-10 keyed by seed and tested
 * in parallel; the first clash-free candidate of each placement is kept.
 * dofs (host, n x (6 + nrb)) receive [x, y, z, a, b, g, 0 ...] for the MC map
 * (MMO_F_RECENTER); *trials the candidates drawn up to the kept ones.  Gives
 * MMO_ESTATE when a placement finds nothing in 100,000 candidates. */
int mmo_place_in_roi(mmo_ctx* ctx, const double center[3], double radius, int n,
                     unsigned long long seed, float* dofs, long long* trials);

/* ---- desolvation -------------------------------------------------------------- */
/* Ligand atom radii (the .pqrs radius column) for the desolvation terms. */
int mmo_set_ligand_radii(mmo_ctx* ctx, const double* radius);

/* Lds.protein_desolv (src/lds.ml:204-233): per point of the protein's solvent
 * shell inside the ROI, C vol sum_j (q_j / d^2)^2 over the protein atoms within
 * 12 A (C = (1/4 - 1/78.5) / (8 pi)); kept in the context; out (host, one per
 * lattice point, may be NULL) receives a copy. */
int mmo_protein_desolv(mmo_ctx* ctx, const double center[3], double radius, double* out);

/* Lds.desolvation_penalty (src/lds.ml:236-267) of B poses (flags
 * MMO_F_RECENTER or 0): over the points of both solvent shells (the protein's
 * and the pose's, the pose's from the radii of mmo_set_ligand_radii and
 * r_water), prot[b] = the sum of the protein's contributions, lig[b] = C vol
 * sum of sum_j (q_j / d^2)^2 over the ligand atoms within 12 A.  status[b] bit
 * 1: the pose's box of lattice points is too large (both 0). */
int mmo_desolvation_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags,
                                 double r_water, double* d_prot, double* d_lig, int* d_status,
                                 void* stream);
int mmo_desolvation_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, double r_water,
                          double* prot, double* lig, int* status);

#ifdef __cplusplus
}
#endif
#endif

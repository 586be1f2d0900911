/*
 * mmo_grid.h -- precomputed interaction grids and the interpolated inter energy.
 *
 * The reference's default inter-energy path (src/lds.ml:1963-1975, unless
 * --no-interp): one float32 lattice per ligand atom type, a type being an
 * (element, partial charge) pair of the ligand (Mol.get_all_vdW_elec_types,
 * src/mol.ml:295-304).  The value of type l at lattice point p is
 *   E_l(p) = min(max_E, K sum_i w(r) q_i q_l / r + sum_i w(r) D_il ((x_il/r)^12 - 2 (x_il/r)^6)),
 * the shifted 12 A energy of a one-atom ligand of type l at p
 * (Lds.pre_calculate_FF_components_grid, src/lds.ml:452-469, summing
 * Mol.ene_inter_UFF_shifted_grid, src/mol.ml:964-989), r = max(|p - r_i|,
 * 0.01 A), over the protein atoms within 12 A; points outside the mask sphere
 * hold 0 (Lds.bitmask_ROI_only, src/lds.ml:269-305: the ROI's outer radius
 * plus 24 A).  Scoring with MMO_F_GRID replaces the pair sums by
 *   E_inter = sum_j trilin(E_{type j}, x_j)
 * (Mol.ene_inter_UFF_interp, src/mol.ml:1010-1020, G3D.trilin,
 * src/G3D.ml:97-157), and the gradient by the derivative of that trilinear
 * form.  The physics switches of mmo_set_physics (dielectric, mixing) apply
 * to the build; the interpolation has none.
 *
 * Lattice: value[l][k][j][i] (i fastest, as the reference's .ba1 files,
 * Grid.idx_of_ijk src/grid.ml) at origin + step (i, j, k).  The reference's
 * lattice has its lowest point at 0 of the simulation box (Grid.from_box,
 * src/grid.ml:40-52: ceil(length / step) + 1 points per axis).
 */
#ifndef MMO_GRID_H
#define MMO_GRID_H

#include <stddef.h>

#include "mmo_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mmo_grid_spec {
  double step;            /* A between lattice points (Params.grid_step = 0.5) */
  int nx, ny, nz;         /* lattice points per axis, each >= 2 */
  double origin[3];       /* point (0, 0, 0) in the frame of the protein's coordinates */
  double mask_center[3];  /* points at distance >= mask_radius hold 0 ... */
  double mask_radius;     /* ... unless mask_radius <= 0 (no mask: every point computed) */
  double max_E;           /* cap of every value (Params.max_E = 100000) */
  int ntypes;             /* ligand atom types, 1..128 */
  const int* type_anum;   /* [ntypes] atomic numbers */
  const double* type_q;   /* [ntypes] partial charges */
} mmo_grid_spec;

/* Compute the grids of spec on the GPU from the protein of mmo_set_protein and
 * keep them in the context (replacing earlier grids).  Returns when they are
 * done; *ms (may be NULL) the build kernel's device milliseconds. */
int mmo_build_grids(mmo_ctx* ctx, const mmo_grid_spec* spec, double* ms);

/* Launch shape of the build kernel: lattice points per lane (1, 2, or 4 under
 * geometric mixing, where 2 is used instead otherwise; 0 the automatic
 * choice).  The values do not depend on it. */
int mmo_set_grid_build(mmo_ctx* ctx, int points_per_lane);

/* Load grids computed elsewhere (the reference's .ba1 files, one per type, in
 * type order): values holds ntypes * nz * ny * nx floats.  mask_center,
 * mask_radius and max_E of spec are not used. */
int mmo_load_grids(mmo_ctx* ctx, const mmo_grid_spec* spec, const float* values);

/* Copy the context's grids to the host array values (ntypes * nz * ny * nx). */
int mmo_grid_values(mmo_ctx* ctx, float* values);

/* The context's grids: sizes (any pointer may be NULL) and the device array. */
int mmo_grid_dims(const mmo_ctx* ctx, int* ntypes, int* nx, int* ny, int* nz);
int mmo_grid_device(const mmo_ctx* ctx, const float** d_values);

/* Plain drop-in for the closure Mol.ene_inter_UFF_interp grid ff_comps
 * (src/lds.ml:1975, src/mol.ml:1010-1020): the interpolated inter energy of
 * one ligand (any n <= 128 atoms) at the given coordinates, its atoms typed by
 * (element, charge) among the grid types (MMO_EINVAL for an atom of no grid
 * type).  *status (may be NULL) receives MMO_S_OFF_GRID when a corner of an
 * atom's cell is off the lattice (that atom adds 0). */
int mmo_ene_inter_grid(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                       const double* q, const int* anum, double* out, int* status);

/* Type of each atom of the ligand of mmo_set_ligand among the grid types
 * (out[n]); MMO_EINVAL when an atom's (element, charge) is not a grid type,
 * which also makes MMO_F_GRID scoring fail. */
int mmo_grid_atom_types(mmo_ctx* ctx, int* out);

#ifdef __cplusplus
}
#endif
#endif

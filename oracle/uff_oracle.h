/*
 * uff_oracle.h -- FP64 CPU oracle for the MMO UFF scoring hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA path is compared
 * against, and the CPU baseline that bench.py times.  Nothing in the shipped
 * library (mmo_gb300/) links, imports or calls it.
 *
 * It restates, in double precision and in the reference's summation order, the
 * OCaml code of UnixJunkie/MMO (paths relative to that project):
 *   src/UFF.ml:10-51        per-element (x_i, D_i), geometric-mean pair table
 *   src/UFF.ml:25, const.ml:18   elec weight 332.0637 / 4.0
 *   src/FF.ml:11-20         pow6, shift_12A
 *   src/math.ml:58-62       non_zero_dist (r >= 0.01 A)
 *   src/math.ml:48-56       dihedral_angle (pinned by src/tests.ml:10-54)
 *   src/rot.ml:52-66        r_xyz = Rz(g) Ry(b) Rx(a)
 *   src/rot.ml:121-146      of_axis_angle (Rodrigues)
 *   src/mol.ml:576-591      radius / check_elongation_exn (Too_long above 12 A)
 *   src/mol.ml:610-631      rotate_bond
 *   src/mol.ml:705-710      center_rotate_translate_copy (MC pose map)
 *   src/mol.ml:796-818      ene_inter_UFF_global_brute
 *   src/mol.ml:822-849      ene_inter_UFF_shifted_brute
 *   src/mol.ml:853-877      ene_intra_UFFNB_shifted_brute_DEPRECATED
 *   src/mol.ml:881-903      ene_intra_UFFNB_brute
 *   src/mol.ml:928-960      ene_inter_UFF_shifted_bst (12 A neighbour sum)
 *   src/optim.ml:64-80      apply_config (torsions in order, Too_long, r_xyz, +t)
 *   src/lds.ml:1118-1136    approx_local_gradient (central finite differences)
 *   src/lds.ml:882-995      simulate_lig frames (moves, resets, Metropolis,
 *                           sliding-window step adaptation; src/SW.ml:7-37)
 *
 * Parity status: the reference ships no golden energies or gradients and its
 * OCaml toolchain is absent, so energy parity is UNPINNED against the reference
 * itself.  The oracle is pinned by known-answer tests derived from the formulas
 * (LJ minimum -D_ij at r = x_ij, switch values, Coulomb pair, exclusions) and by
 * the reference's only numeric test vectors (src/tests.ml:10-54, dihedral
 * angles), which also pin rotate_bond through the dihedral it changes.
 */
#ifndef MMO_UFF_ORACLE_H
#define MMO_UFF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* physics switches; 0 is the reference behaviour */
typedef struct {
  int dielectric; /* 0: eps = 4 (UFF.ml:25); 1: eps = 4 r                        */
  int mixing;     /* 0: geometric mean of x and D (UFF.ml:47-48); 1: Lorentz-Berthelot */
  int inter_form; /* 0: shifted, 12 A (mol.ml:822-849); 1: global (mol.ml:796-818)   */
  int intra_form; /* 0: plain (mol.ml:881-903); 1: shifted (mol.ml:853-877)         */
} orc_physics;

typedef struct {
  int n;
  const double *x, *y, *z, *q;
  const int *anum;
} orc_mol;

typedef struct {
  orc_mol m;                        /* centred reference conformer            */
  const uint8_t *interacting;       /* n*n, 1 if topological distance >= 3    */
  int nrb;                          /* rotatable bonds                         */
  const int *bond_lr;               /* 2*nrb: (left, right) per bond           */
  const int *grp_off;               /* nrb+1 offsets into grp_atoms            */
  const int *grp_atoms;             /* rotation group atoms, right end excluded */
} orc_ligand;

enum { ORC_F_INTER = 1, ORC_F_INTRA = 2, ORC_F_RECENTER = 8 };
enum { ORC_S_TOO_LONG = 1, ORC_S_NONFINITE = 2 };

double orc_elec_weight(void);
/* returns 1 and fills (x_i, D_i) when anum is a supported element, else 0 */
int orc_uff_params(int anum, double *xi, double *di);
void orc_pair_params(const orc_physics *ph, int a1, int a2, double *x_ij, double *d_ij);
double orc_shift_12A(double d);
double orc_non_zero_dist(double d);
double orc_dihedral(const double i[3], const double j[3], const double k[3], const double l[3]);

void orc_rot_xyz(double a, double b, double g, double R[9]);
void orc_rot_axis_angle(const double u[3], double theta, double R[9]);
void orc_rotate_bond(int n, double *x, double *y, double *z, int left, int right,
                     const int *grp, int ng, double alpha);

/* brute-force sums over every protein x ligand pair */
double orc_ene_inter(const orc_physics *ph, const orc_mol *prot, const orc_mol *lig);
/* elec and vdW parts separately (mol.ml:921-956); parts[0] = elec, parts[1] = vdW */
void orc_ene_inter_parts(const orc_physics *ph, const orc_mol *prot, const orc_mol *lig,
                         double parts[2]);
double orc_ene_intra(const orc_physics *ph, const orc_mol *lig, const uint8_t *interacting);

/* 12 A neighbour form through a cell grid (the BST query of mol.ml:939) */
typedef struct orc_cells orc_cells;
orc_cells *orc_cells_build(const orc_mol *prot);
void orc_cells_free(orc_cells *c);
double orc_ene_inter_cells(const orc_physics *ph, const orc_cells *c, const orc_mol *lig);

/* pose rebuild: conf = [x, y, z, a, b, g, tau_0 .. tau_{nrb-1}]
 * flags & ORC_F_RECENTER selects the MC map (centre, rotate, translate);
 * otherwise Optim.apply_config.  Returns ORC_S_TOO_LONG if the conformer's
 * enclosing radius exceeds 12 A (the reference raises Mol.Too_long). */
int orc_apply_config(const orc_ligand *lig, const double *conf, int flags,
                     double *x, double *y, double *z);

/* E_inter + E_intra of one configuration; status gets ORC_S_* bits */
double orc_score_conf(const orc_physics *ph, const orc_mol *prot, const orc_cells *cells,
                      const orc_ligand *lig, const double *conf, int flags, int *status);

/* dE/dconf by central differences with per-DOF steps eps (lds.ml:1118-1136) */
void orc_grad_fd(const orc_physics *ph, const orc_mol *prot, const orc_cells *cells,
                 const orc_ligand *lig, const double *conf, int flags, const double *eps,
                 double *grad);

/* analytic FP64 gradient (reverse mode through the rigid map and the torsion
 * chain); returns E and fills grad[6+nrb].  Also fills dE/dxyz of the final
 * atoms when gxyz != NULL (3*n, interleaved). */
double orc_grad_analytic(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                         const double *conf, int flags, double *grad, double *gxyz,
                         int *status);

/* condition scales of one configuration: returns S = sum over pairs of
 * w (|elec| + D (x/r)^12 + 2 D (x/r)^6) and fills grad_abs[6+nrb] with the sum of |terms| that
 * orc_grad_analytic adds into each gradient component (pair terms split into
 * their parts, products and cross products bounded by their absolute values).  An evaluation in a precision with unit round-off u is
 * accurate to about u times these scales, whatever the cancellation. */
double orc_grad_scale(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                      const double *conf, int flags, double *grad_abs);

/* batch over poses on nthreads host threads.  dofs: B x (6+nrb) float32 (the
 * GPU input format, widened exactly).  mode 0: energy; 1: energy + analytic
 * gradient; 2: energy + central-difference gradient with eps (the reference's
 * method); 3: the condition scales of orc_grad_scale (E gets S, grad gets the
 * per-component scales).  use_cells selects the 12 A neighbour form for E_inter. */
void orc_score_batch(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                     int B, const float *dofs, int flags, int mode, const double *eps,
                     int use_cells, int nthreads, double *E, double *grad, int *status);

/* Philox4x32-10 block: out = philox(ctr, key) */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Monte Carlo chains (src/lds.ml:882-995): replay of a GPU trace of `steps`
 * frames of B chains from the start poses (float32 [B][6+nrb], the MC pose
 * map), frame by frame: each proposal is recomputed and compared bit for bit
 * with the GPU's trial (gpu_trial [steps][B][6+nrb]); each outcome (the
 * event bits of mmo_mc_state.trace_event) is decided from FP64 energies and
 * compared with the GPU's (gpu_event [steps][B]); outcomes within
 * e_tol max(|E|, S) of their threshold are ambiguous and follow the GPU.
 * gpu_E [steps][B] is compared with the FP64 trial energy. */
typedef struct {
  double kT, rot, trans, tors; /* kT (kcal/mol), initial steps (rad, A, rad) */
  int law;                     /* 0: uniform (src/move.ml), 1: Gaussian */
  int adapt, flip_every;
  uint64_t seed;               /* Philox key: low word, high word */
  double roi_c[3], roi_r;      /* hard ROI; roi_r <= 0: off */
  int reset_zero;              /* reset on E_inter = 0 */
  int too_long_ends;           /* an over-long trial conformer ends the chain */
} orc_mc_params;

typedef struct {
  long proposals, proposal_mismatch; /* trial poses compared, not bit-equal */
  long decisions, decision_mismatch; /* outcomes compared, different and unambiguous */
  long ambiguous;                    /* outcomes within the tolerance of their threshold */
  long resets, adapt_events;         /* resets and step-size adaptations of the replay */
  double max_rel_err_E;              /* max |E_gpu - E64| / max(|E64|, S) of scored trials */
} orc_mc_stats;

void orc_mc_replay(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                   const orc_mc_params *p, int B, const float *start, int steps,
                   const float *gpu_trial, const double *gpu_E, const int *gpu_event,
                   double e_tol, int nthreads, orc_mc_stats *out);

/* The same chains run by the oracle alone (FP64 outcomes), writing the trace
 * in the GPU's layout: trial [steps][B][6+nrb], E and event [steps][B]. */
void orc_mc_run(const orc_physics *ph, const orc_mol *prot, const orc_ligand *lig,
                const orc_mc_params *p, int B, const float *start, int steps, float *trial,
                double *E, int *event, int nthreads, orc_mc_stats *out);

/* precomputed interaction grids (src/lds.ml:452-469, src/mol.ml:964-989) and
 * their trilinear interpolation (src/G3D.ml:97-157, src/mol.ml:1010-1020) */
void orc_grid_point(const orc_physics *ph, const orc_mol *prot, const double p[3], int ntypes,
                    const int *type_anum, const double *type_q, double max_E, double *out);
double orc_trilin(double step, int nx, int ny, int nz, const float *v, const double p[3],
                  int *off);
void orc_grid_points(const orc_physics *ph, const orc_mol *prot, int n, const double *pts,
                     int ntypes, const int *type_anum, const double *type_q, double max_E,
                     int nthreads, double *out, double *scale);
double orc_ene_inter_interp(double step, int nx, int ny, int nz, const float *grids, int n,
                            const double *x, const double *y, const double *z, const int *type,
                            int *off);

/* lattice of the grids: point (i, j, k) at o + step (i, j, k) */
typedef struct {
  double step;
  int nx, ny, nz;
  double o[3];
} orc_lattice;

/* masks, clash tests, SO(3) samples, exhaustive docking, desolvation
 * (src/lds.ml:149-267, 1040-1114; src/mol.ml:1077-1219; src/G3D.ml:159-213;
 * src/SO3.ml:18-46; src/ptable.ml:41-80) */
double orc_vdw_radius(int anum);
double orc_clash2(int a1, int a2);
void orc_atom_bitmask_set(const orc_lattice *g, const double p[3], double radius, uint8_t b,
                          uint8_t *mask);
void orc_masks(const orc_lattice *g, int n, const double *x, const double *y, const double *z,
               const double *radius, double r_w, uint8_t *vdw, uint8_t *shell);
int orc_clash_or(const orc_lattice *g, const uint8_t *mask, const double p[3]);
int orc_clash_and(const orc_lattice *g, const uint8_t *mask, const double p[3]);
int orc_protein_ligand_clash(const orc_lattice *g, const uint8_t *vdw, int n, const double *x,
                             const double *y, const double *z);
int orc_center_occupied(int n, const double *x, const double *y, const double *z,
                        const double *radius);
int orc_heavy_atom_clash(const orc_mol *prot, int n, const double *x, const double *y,
                         const double *z, const int *anum);
int orc_intra_clash(int n, const double *x, const double *y, const double *z, const int *anum,
                    const uint8_t *interacting);
void orc_so3_rotation(int n, int i, double R[9]);
void orc_dock_scores(const orc_lattice *g, const float *grids, const uint8_t *vdw,
                     const orc_mol *lig, const int *lig_type, const double *lig_radius,
                     const double roi_c[3], double roi_r, double trans_step, int nrot,
                     const double *R, double const_intra, int dims[3], double *scores);
double orc_desolv_constant(void);
void orc_protein_desolv(const orc_lattice *g, const orc_mol *prot, const uint8_t *shell,
                        const double roi_c[3], double roi_r, double *out);
void orc_desolvation_penalty(const orc_lattice *g, const double *prot_contrib,
                             const uint8_t *prot_shell, int n, const double *x, const double *y,
                             const double *z, const double *q, const double *radius, double r_w,
                             double out[2]);

#ifdef __cplusplus
}
#endif
#endif

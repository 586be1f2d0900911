/*
 * mmo_gpu.h -- C ABI of the GB300 UFF scoring library (libmmo_gpu.so).
 *
 * Drop-in for the force-field scoring calls of UnixJunkie/MMO (paths inside
 * that project).  MMO scores a ligand through OCaml closures of type
 * Mol.t -> float:
 *   ene_inter = Mol.ene_inter_UFF_shifted_bst prot_bst prot   (src/lds.ml:1952-1955)
 *   ene_intra = Mol.ene_intra_UFFNB_brute                      (src/lds.ml:702-712)
 * called once per Monte Carlo frame (src/lds.ml:900-905), per NLopt objective
 * evaluation (src/lds.ml:1246-1251) and 2(6 + n) more times per numerical
 * gradient (src/lds.ml:1118-1136).  The functions below replace those calls:
 * the plain ones one call for one call, the batched one many poses (and the
 * analytic gradient) per call.
 *
 * Conventions: every function returns MMO_OK (0) or a negative MMO_E* code;
 * mmo_last_error() gives a message.  Host pointers unless the name ends in
 * _device.  Energies are kcal/mol in FP64; coordinates in Angstrom.  A context
 * owns one GPU and one CUDA stream and is not thread-safe; create it after any
 * fork() (MMO forks its workers, src/lds.ml:2009,2050).
 */
#ifndef MMO_GPU_H
#define MMO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define MMO_OK 0
#define MMO_EINVAL (-1)       /* bad argument (size, pointer, flag)             */
#define MMO_ECUDA (-2)        /* CUDA runtime error                              */
#define MMO_ENOMEM (-3)       /* device or pinned allocation failed              */
#define MMO_ESTATE (-4)       /* protein or ligand not set                       */
#define MMO_EELEMENT (-5)     /* atomic number not in the UFF table (UFF.ml:10-22) */
#define MMO_ETIMEOUT (-6)     /* a bounded device-side wait gave up              */

/* ---- physics switches (mmo_set_physics) ---------------------------------- */
#define MMO_DIEL_CONST 0      /* eps = 4: K q_i q_j / r, K = 332.0637/4 (UFF.ml:25) */
#define MMO_DIEL_DIST 1       /* eps = 4 r: K q_i q_j / r^2                       */
#define MMO_MIX_GEOMEAN 0     /* x_ij = sqrt(x_i x_j), D_ij = sqrt(D_i D_j) (UFF.ml:47-48) */
#define MMO_MIX_LB 1          /* x_ij = (x_i + x_j)/2, D_ij = sqrt(D_i D_j)       */
#define MMO_INTER_SHIFTED 0   /* (1-(r/12)^2)^2 switch, 12 A cut: -ff BrL / Bst (mol.ml:822-849, 928-960) */
#define MMO_INTER_GLOBAL 1    /* no switch, no cut: -ff BrG (mol.ml:796-818)      */
#define MMO_INTRA_PLAIN 0     /* no switch, no cut (mol.ml:881-903)               */
#define MMO_INTRA_SHIFTED 1   /* switch + 12 A cut (mol.ml:853-877)               */

/* ---- mmo_score_poses flags ------------------------------------------------ */
#define MMO_F_INTER 1         /* add the ligand-protein energy                    */
#define MMO_F_INTRA 2         /* add the intra-ligand energy                      */
#define MMO_F_GRAD 4          /* also dE/d[x, y, z, a, b, g, tau_0 ..]            */
#define MMO_F_RECENTER 8      /* MC pose map (mol.ml:705-710) instead of Optim.apply_config (optim.ml:64-80) */
#define MMO_F_GRID 16         /* with MMO_F_INTER: the inter energy interpolated from the
                                 precomputed grids (mmo_grid.h, mol.ml:1010-1020) */

/* ---- per-pose status bits ------------------------------------------------- */
#define MMO_S_TOO_LONG 1      /* enclosing radius > 12 A: Mol.Too_long (mol.ml:587-591) */
#define MMO_S_NONFINITE 2     /* energy is not finite                             */
#define MMO_S_OFF_GRID 4      /* MMO_F_GRID: an atom's lattice cell falls off the grids; its
                                 inter term is 0 (the reference reads out of bounds) */

typedef struct mmo_ctx mmo_ctx;

/* Last error message of ctx (or of the last failed mmo_ctx_create when ctx is NULL). */
const char* mmo_last_error(const mmo_ctx* ctx);

/* Open a context on CUDA device `device`.  Replaces nothing in MMO: it holds
 * what the partial applications of src/lds.ml:1952-1979 close over. */
int mmo_ctx_create(int device, mmo_ctx** out);
int mmo_ctx_destroy(mmo_ctx* ctx);

/* Physics switches; the default (all 0) is the reference's behaviour. */
int mmo_set_physics(mmo_ctx* ctx, int dielectric, int mixing, int inter_form, int intra_form);

/* Upload the rigid protein once: Mol.receptor_of_pqrs_file (mol.ml:412-417)
 * plus the partial application `ff0 prot` (lds.ml:1967).  anum = atomic
 * numbers (Mol.t.elt_a). */
int mmo_set_protein(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                    const double* q, const int* anum);

/* Upload the ligand once: the fields of Mol.t that a .pqrs ligand carries
 * (pqrs.ml:41-87, mol.ml:384-402).  xs/ys/zs: centred reference conformer;
 * interacting: n*n bytes, 1 where the topological distance is >= 3
 * (mol.ml:203-208); bond_lr: 2*nrb (left, right) atoms of each rotatable bond;
 * group_offsets[nrb+1] / group_atoms: each bond's rotation group with its right
 * end excluded (pqrs.ml:343-351).  Replaces the per-ligand set-up of
 * ene_intra_builder (lds.ml:702-712).  n <= 128, nrb <= 32. */
int mmo_set_ligand(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                   const double* q, const int* anum, const uint8_t* interacting, int nrb,
                   const int* bond_lr, const int* group_offsets, const int* group_atoms);

/* Plain drop-in for Mol.ene_inter_UFF_shifted_bst / _shifted_brute /
 * _global_brute (mol.ml:796-849, 928-960) on the protein of mmo_set_protein:
 * one ligand (any n <= 128 atoms) per call, energy into *out; one launch (the
 * pair partials, and their total from the last block). */
int mmo_ene_inter(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                  const double* q, const int* anum, double* out);

/* The same sum with its two parts kept apart, as
 * Mol.ene_inter_UFF_shifted_bst_components (mol.ml:920-957) keeps them for
 * rescoring functions: *elec the electrostatic part (elec_weight_protein
 * applied), *vdw the van der Waals part; *elec + *vdw is mmo_ene_inter's
 * energy up to rounding.  One launch. */
int mmo_ene_inter_parts(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                        const double* q, const int* anum, double* elec, double* vdw);

/* Plain drop-in for Mol.ene_intra_UFFNB_brute (mol.ml:881-903) on the ligand
 * of mmo_set_ligand, at the given coordinates.  One launch. */
int mmo_ene_intra(mmo_ctx* ctx, const double* xs, const double* ys, const double* zs,
                  double* out);

/* Score B poses of the ligand of mmo_set_ligand.  dofs: B x (6 + nrb) floats,
 * the config vector [x, y, z, a, b, g, tau_0 ..] of optim.ml:19-22 rebuilt by
 * Optim.apply_config (optim.ml:64-80) or, with MMO_F_RECENTER, by the MC map
 * centre-rotate-translate (mol.ml:705-710) with R = r_xyz(a, b, g).
 * E_out[B] (FP64): E_inter and/or E_intra as flags select.  grad_out (null
 * unless MMO_F_GRAD): B x (6 + nrb) floats, the analytic gradient replacing
 * approx_local_gradient (lds.ml:1118-1136).  status_out[B] (nullable):
 * MMO_S_* bits.  B = 1 with the inter term is one kernel launch (the
 * one-pose path: rebuild, pair sums and finish fused).  Page-locked
 * buffers (cudaHostAlloc / cudaHostRegister) are read and written by DMA
 * directly; other host memory goes through the context's staging buffers. */
int mmo_score_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, double* E_out,
                    float* grad_out, int* status_out);

/* The posed coordinates of B poses (the pose map of mmo_score_poses alone:
 * Optim.apply_config, optim.ml:64-80, or with MMO_F_RECENTER the MC map,
 * mol.ml:705-710; other flags are ignored): xyz_out B x L x 3 doubles in the
 * input frame, from the kernel's float-pair coordinates; status_out[B]
 * (nullable): MMO_S_TOO_LONG as Optim.apply_config raises Mol.Too_long.  The
 * coordinates a caller writes out as a pose (.xyz, .pqrs). */
int mmo_posed_coords(mmo_ctx* ctx, int B, const float* dofs, int flags, double* xyz_out,
                     int* status_out);

/* As mmo_score_poses with device pointers, queued on `stream` (a
 * cudaStream_t; NULL is the legacy default stream) without synchronising;
 * mmo_sync() waits and reports device-side errors.  Calls on one context
 * share its scratch buffers, so they must all go to one stream. */
int mmo_score_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E,
                           float* d_grad, int* d_status, void* stream);

/* Allocation-free variant of mmo_score_poses_device (no counterpart in the
 * reference).  For callers that cannot allocate device memory while they
 * score: real-time loops that may not stall on the allocator, and hosts whose
 * device memory is owned by another allocator (a framework's caching
 * allocator, or a fixed arena reserved up front).  The
 * caller passes every input and output as device pointers; the call's work
 * buffers come from a static 32 MiB device array that every GPU loading this
 * library holds until the process exits, so this function calls no cudaMalloc
 * or cudaFree.  It always runs the full pair sweep (not the cut-off sweep of
 * mmo_set_cull, whose work buffers are larger).  A call needs 32*B*L bytes,
 * with MMO_F_GRAD another 32*B*L + 48*B*nrb + 32*B, and 8*B*L (24*B*L with
 * MMO_F_GRAD) per protein chunk; a batch that does not fit with one chunk
 * per shared-memory slice of the protein is rejected with MMO_EINVAL and a
 * message naming the sizes (4,096 poses of a 48-atom ligand fit, with the
 * gradient).  The first call on a device looks up the array's device address
 * with that device current; make that first call before any stream capture.
 * All calls share the one array, so calls that overlap on the GPU (other
 * streams, other contexts on the same device) race: serialise them on one
 * stream.  Device-side wait timeouts are reported by mmo_sync. */
int mmo_score_poses_noalloc(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E,
                            float* d_grad, int* d_status, void* stream);

/* Wait for `stream` (a cudaStream_t; NULL is the legacy default stream) and
 * report, then clear, the device-side error flag of the device-pointer calls
 * (MMO_ETIMEOUT). */
int mmo_sync(mmo_ctx* ctx, void* stream);

/* Tile shape of the batched pair kernels: poses per lane (1, 2, 4) and
 * protein chunks per pose (0: automatic) of the full sweep, and threads per
 * CTA (256, 512, 768, 1024; the full sweep runs at most 512, the cut-off
 * sweep at most 768, 512 or 256 for 1, 2 or 4 entries per lane).  Setting 0
 * for all restores the automatic choice. */
int mmo_set_tiles(mmo_ctx* ctx, int poses_per_lane, int threads, int chunks);

/* Cut-off sweep of the shifted form for batches (the counterpart of
 * Mol.ene_inter_UFF_shifted_bst, UnixJunkie/MMO src/mol.ml:928-962, which
 * visits only the protein atoms within 12 A of each ligand atom).  mode 0:
 * automatic, used for batches of 2 or more poses under the shifted form, the
 * protein staged in shared memory when it fits (about 6,500 atoms) and read
 * from global memory otherwise; mode 1: off, every pair is evaluated; mode 2:
 * the cut-off sweep with the protein always read from global memory.
 * row_spacing: (y, z) spacing of the protein's row index in A (<= 0: 3; a
 * change rebuilds the index); piece_atoms: protein atoms per work item (0:
 * 256); entries_per_lane: 1, 2, 4 (0: 2). */
int mmo_set_cull(mmo_ctx* ctx, int mode, double row_spacing, int piece_atoms,
                 int entries_per_lane);

/* Autotuner of the batched pair sweep (no counterpart in the reference).
 * Times launch plans on this batch and keeps the fastest as the context's
 * settings (mmo_set_cull, mmo_set_tiles): under the shifted form the cut-off
 * sweep's row spacing (2, 3, 4 A), entries per lane (1, 2, 4) and piece
 * size (256, 512 atoms) against the full sweep's poses per lane (1, 2, 4) and
 * protein chunks (4 to 24); under the global form the full sweep's plans.
 * Arguments as mmo_score_poses_device, whose outputs it leaves as computed by
 * the chosen plan.  With a cache file (mmo_set_tune_cache) a plan recorded
 * there for the same shape (poses, ligand atoms, torsions, protein atoms,
 * physics, gradient) is applied without timing (*ms = -1) and a timed one is
 * appended.  Each candidate runs 4 times; the call synchronises the stream.
 * Refused inside a stream capture (MMO_ESTATE).  *ms (may be NULL): device
 * milliseconds of one call with the chosen plan. */
int mmo_tune(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E, float* d_grad,
             int* d_status, void* stream, double* ms);

/* File of tuned plans for mmo_tune, one line per shape; NULL or "" for none. */
int mmo_set_tune_cache(mmo_ctx* ctx, const char* path);

/* Plan of the last batched call: *path 1 for the cut-off sweep with the
 * protein in shared memory, 2 for the cut-off sweep reading it from global
 * memory, 0 for the full sweep; entries (or poses) per lane; threads per CTA; piece atoms (or
 * protein chunks per pose); the row spacing of the protein index. */
int mmo_get_plan(const mmo_ctx* ctx, int* path, int* per_lane, int* threads,
                 int* piece_or_chunks, double* row_spacing);

/* Number of SMs of the context's device (for callers that size batches). */
int mmo_device_sms(const mmo_ctx* ctx, int* out);

#ifdef __cplusplus
}
#endif
#endif

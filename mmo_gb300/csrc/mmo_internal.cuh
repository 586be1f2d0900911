// mmo_internal.cuh -- device data layout, launch plans and shared helpers of
// the GB300 (sm_103a) UFF scoring library.  Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mmo {

constexpr int kMaxLig = 128;    // ligand atoms per system (4 per lane in a warp)
constexpr int kSlots = kMaxLig / 32;
constexpr int kMaxTors = 32;    // rotatable bonds per ligand
constexpr int kNTypes = 12;     // UFF elements of src/UFF.ml:10-22
constexpr int kSliceAtoms = 6912;   // protein atoms resident in shared memory per launch (32 B each)
constexpr float kCut2 = 144.0f;     // 12 A cutoff, squared (const.ml:12-14)
constexpr float kMinR2 = 1e-4f;     // (0.01 A)^2, Math.non_zero_dist (math.ml:58-62)

// Coordinates are carried as unevaluated float pairs hi + lo (hi = fl(v),
// lo = fl(v - hi)), so a pair difference (x_hi - p_hi) + (x_lo - p_lo) is
// accurate to about one float ulp of |d| however close the atoms are: the
// r^-12 term turns a coordinate error delta into a relative energy error of
// about 12 delta / r, which plain floats (delta ~ 1e-6 A at 16 A) cannot keep
// below 1e-5 for clashing contacts.
//
// Protein in HBM: atoms sorted by UFF type so that the pair parameters are
// constant over each run; (x, y, z) are relative to the frame origin and w is
// K * q with K = 332.0637 / 4.
struct DevProtein {
  const float4* atoms;    // [P][2]: (x_hi, y_hi, z_hi, K q), (x_lo, y_lo, z_lo, 0)
  const uint8_t* type;    // [P] type index, for the plain kernel
  const int* runs;        // [2 * kNTypes + 1]: run_start[nruns + 1], then run_type[nruns]
  int P;
  int nruns;
};

// Pair parameters (x_ij^2, D_ij) for every type pair, passed by value so that
// warp-uniform lookups hit the constant bank.
struct PairTable {
  float2 xd[kNTypes * kNTypes];
};

// The same pairs for the batched sweep: (X = D^(1/3) x^2, 1/D (0 when D = 0),
// x^2, D).
struct PairTable4 {
  float4 v[kNTypes * kNTypes];
};

// Ligand topology and reference conformer in HBM.
struct DevLigand {
  int L, nrb, npairs;
  // 1 when the rotation groups are nested or disjoint with each axis moving
  // rigidly with the groups that contain it (rotatable bonds that are
  // bridges, groups on one side: mol_graph.ml:126-192).  Then a torsion turns
  // its group rigidly about its final axis, and the intra-ligand term (which
  // is rigid-invariant) enters the gradient only through pairs that straddle
  // a group boundary.
  int nested;
  float ilh, ill;           // 1 / L as a double-float (hi, lo), rounded from FP64
  const float4* ref;        // [L] (x, y, z, q) centred conformer, rounded to float
  const double* ref64;      // [L][3] the same conformer in double
  const float2* ref2;       // [L][3] the same conformer as float pairs (hi, lo)
  const int* type;          // [L] type index
  const float* q;           // [L] partial charge
  const int2* bonds;        // [nrb] (left, right) rotation axis
  const uint32_t* gmask;    // [nrb][kSlots] group bitmask, bit (a & 31) of word (a >> 5)
  const int2* pair_ij;      // [npairs] interacting pairs i < j (mol.ml:203-208)
  const float4* pair_par;   // [npairs] (x^2, D, K q_i q_j, the bits of the torsions whose
                            // group holds exactly one of the two atoms)
  const uint32_t* amask;    // [L] bit t set when the atom is in rotation group t
  const float2* tax;        // [nrb][6] unit axis (centre - left) and centre of each
                            // torsion in the reference conformer, double-float
  const int* tord;          // [nrb] torsions by group size, smallest first
  const uint32_t* ramask;   // [L] bit k set when the atom is in the group of tord[k]
  const int* grp_off;       // [nrb + 1] rotation groups as CSR
  const int* grp_atoms;
  const int* nb_off;        // [L + 1] both-direction CSR of the same pairs
  const int* nb_idx;        // partner atom
  const float4* nb_par;     // (x^2, D, K q_i q_j, 0)
  const int* seg_of_atom;   // [L] rank of the atom's type among the ligand's types
};

// Per-pose work buffers, pose-major so the warp-per-pose kernels read them
// contiguously.  C = protein chunks per pose.
// Polls of a bounded mbarrier wait on a TMA copy.  The first wait of a sweep
// kernel takes its limit from the launch (first_wait_polls, this value unless
// mmo_diag_set_wait_polls changed it); a wait that gives up sets kErrTimeout,
// and the kernel then waits once more with this limit for the copy in flight
// before its CTA returns.
constexpr uint32_t kWaitPollsDefault = 1u << 22;

struct Scratch {
  float4* X;       // [B][L][2] posed coordinates in the device frame, hi then lo
  double* Epart;   // [B][C][L] inter energy partial per chunk and ligand atom
  float4* Gpart;   // [B][C][L] dE/dX partial per chunk and ligand atom
  float4* Y;       // [B][L][2] coordinates after the torsions, before the rigid map, hi then
                   // lo (gradient only)
  float4* rec;     // [B][nrb][3] torsion records (c hi, cos), (u, sin), (1/|a|, c lo)
                   // (gradient only)
  float4* cen;     // [B][2] centroid of Y, hi then lo (gradient only)
  int C;
  uint32_t first_wait_polls = kWaitPollsDefault;  // polls of the full sweep's first TMA wait
  // the cut-off sweep's entry binning, done by the rebuild when binning != 0:
  // entry e = b L + j of pose b, ligand atom j goes to bin seg_of_atom[j]
  // kCullBins + its Hilbert cell, rank[e] its place in the bin (hist counts)
  int binning = 0;
  unsigned* hist = nullptr;
  int* bin = nullptr;
  int* rank = nullptr;
  const int* seg_of_atom = nullptr;
  float glo[3] = {0.f, 0.f, 0.f};
  float ginv = 0.f;
};

struct PoseIO {
  const float* dofs;  // [B][6 + nrb] optimiser layout (optim.ml:19-22)
  double* E;          // [B]
  float* grad;        // [B][6 + nrb] or null
  int* status;        // [B]
  int* err;           // device-side error flag (kErr* bits)
  int zero_err;       // the rebuild kernel clears *err first
  int B;
  float ox, oy, oz;   // frame origin subtracted from the translation
  double* E_inter;    // [B] the inter part of E, or null
};

enum : int { kFlagInter = 1, kFlagIntra = 2, kFlagGrad = 4, kFlagRecenter = 8 };
enum : int { kStatusTooLong = 1, kStatusNonFinite = 2, kStatusOffGrid = 4 };
enum : int { kErrTimeout = 1 };

struct Physics {
  int dielectric;  // 0: eps = 4; 1: eps = 4 r
  int mixing;      // 0: geometric mean; 1: Lorentz-Berthelot
  int inter_form;  // 0: shifted 12 A; 1: global
  int intra_form;  // 0: plain; 1: shifted 12 A
};

// Launch plan of the batched pair kernel (chosen by the tuner).
struct PairPlan {
  int kp;        // poses per lane: 1, 2 or 4
  int threads;   // threads per CTA: 256 or 512
  int C;         // protein chunks per pose
  int blocks;    // persistent grid size
};

// ---- cut-off sweep (shifted form) ----------------------------------------
// The shifted form is exactly 0 beyond 12 A (s = max(1 - r^2/144, 0)), and
// in a pocket most ligand-protein pairs lie beyond it.  The cut-off sweep
// groups the (pose, ligand atom) entries of a batch by ligand type and by
// position, bounds each group of 32 * KP entries by a box, and visits only the
// protein atoms within 12 A of the box, found through a row index of the
// protein.  Pairs it skips have r^2 > kCullR2, where the switched term and its
// derivative are exactly 0 in FP32, and it accumulates in a fixed order over
// fixed pieces of the protein, so an entry's result does not depend on which
// entries share its group.
constexpr int kCullGrid = 32;                                   // entry binning cells per axis
constexpr int kCullBins = kCullGrid * kCullGrid * kCullGrid;    // cells in Hilbert order
constexpr float kCullR2 = 145.0f;  // visit radius^2: 1 - r^2/144 < 0 in FP32 beyond it
// protein type row of the cut-off sweep's null pair partner: (X, 1/D, c1) all 0
constexpr int kNullTypeRow = kNTypes;
constexpr int kCullFlush = 256;    // protein atoms per FP32 partial before the FP64 add

// The protein ordered in rows of a (y, z) grid of spacing h: row order (iz, iy)
// with empty rows dropped, atoms in a row sorted by x.
struct DevCull {
  const float4* atoms;       // [P][2]: (x_hi, y_hi, z_hi, K q), (x_lo, y_lo, z_lo, w): w holds the
                             // int bits of type * kNTypes * 16, the byte offset of the type's
                             // row in the shared pair table
  const int* row_start;      // [nrows + 1]
  const float4* row_box;     // [nrows] (y_min, y_max, z_min, z_max) of the row's atoms
  const int* row_flush;      // [nrows] end (exclusive) of the row's flush block: the FP32
                             // partials go into the FP64 sums after row row_flush[r] - 1
  const float4* pairs;       // [npairs][4] the cut-off sweep's layout of the same rows: atoms
                             // in pairs, negated coordinates (see pair_step_ab)
  const int* pair_start;     // [nrows + 1] first pair of each row
  int P, nrows, npairs;
  float glo[3];              // entry binning grid origin and cells per A
  float ginv;
};

// Per-call description of the entry groups: the entries of ligand type
// segment t fill slots [off[t], off[t] + n[t]), the segment padded to a
// multiple of the group size G = 32 * kp.
struct CullSegs {
  int nseg;
  int G;
  int off[kNTypes + 1];
  int n[kNTypes];
  int type[kNTypes];
};

struct CullScratch {
  unsigned* hist;        // [nseg * kCullBins] counts, then slot cursors
  int* bin;              // [B * L] entry -> bin
  int* rank;             // [B * L] entry -> rank in its bin
  float4* Xs;            // [slots][2] entries in slot order: (x, y, z hi, q), (x, y, z lo, 0)
  int* order;            // [slots] slot -> entry b * L + j
  double* Ep;            // [npieces][slots] energy per protein piece
  float4* Gp;            // [npieces][slots] -dE/dX (scaled) per protein piece
  unsigned* queue;       // work counter of the sweep
  unsigned long long* pairs;  // pair evaluations of the sweep (32 * KP per visited atom)
  int* arrive;           // [groups] pieces of the group done
  uint8_t* vis;          // [groups][npieces] 1: the piece came within 12 A of the group
  double* Eout;          // [B * L] inter energy per entry (Scratch::Epart, one chunk)
  float4* Gout;          // [B * L] dE/dX per entry (Scratch::Gpart, one chunk)
  const int* seg_of_atom;  // [L] ligand atom -> type segment
  const int* piece_row;  // [npieces + 1] first row of each protein piece
  const float4* pbox;    // [npieces][2] bounding box of each piece's atoms (lo, hi)
  int* gcount;           // [groups] pieces within reach of each group (the broad phase)
  int* glist;            // [groups][npieces] those pieces, ascending
  int2* items;           // [groups * npieces] (group, piece) work items; queue[1] counts them
  int slots, npieces;
  uint32_t first_wait_polls = kWaitPollsDefault;  // polls of the sweep's first TMA wait
};

// threads per CTA of the cut-off sweep: the register budget of KP entries per
// lane (each entry value held in both halves of a register pair)
constexpr int cull_max_threads(int kp) { return kp == 1 ? 768 : (kp == 2 ? 512 : 256); }

struct CullPlan {
  int kp, threads, blocks;
  int piece_atoms;
  int smem;              // dynamic shared memory of the sweep
  int global;            // 1: protein records read from global memory (L1 / L2), 0: the whole
                         // protein staged in shared memory
};

// ---- ragged batch of systems ----------------------------------------------
// Many (pocket, ligand) systems, each with its own number of poses, scored in
// one pass.  Per system s the poses are consecutive ([pose0, pose0 + poses)),
// and so are its entries (pose-major, L_s per pose), torsion records (nrb_s
// per pose) and DOF rows (6 + nrb_s floats per pose).  Proteins are packed one
// after the other in row-index order; the cut-off sweep works on pieces of one
// protein (a few hundred atoms, whole rows) staged per CTA.
constexpr int kSysGrid = 8;                      // binning cells per axis per system
constexpr int kSysCells = kSysGrid * kSysGrid * kSysGrid;
constexpr int kSysSortMax = 16384;               // entries one sort CTA holds

struct SysInfo {
  int pose0, ent0, rec0, dof0;   // first global pose, entry, torsion record, DOF float
  int poses, L, nrb, nseg;       // poses, ligand atoms, torsions, ligand type segments
  int piece0, npieces;           // the system's protein pieces
  int group0, ngroups;           // the system's entry groups (cut-off sweep)
  int seg0;                      // first (system, type) segment in the segment table
  int vis0;                      // first piece flag: group-major [ngroups][npieces]
  long long part0;               // first piece partial: [ngroups][npieces][G]
  float ox, oy, oz;              // frame origin (centroid of the protein)
  float glo[3], ginv;            // binning grid: origin, cells per A
};

struct SysBlk {                  // a block's system and its system-local poses [p0, p0 + n)
  int sys, p0, n, pad;
};

struct SysGroup {                // a group of G slots of one (system, type) segment
  int slot0, s_end, ltype, sys;
};

struct DevSystems {
  const SysInfo* info;           // [nsys]
  const DevLigand* lig;          // [nsys] descriptors into the packed ligand blob
  const SysBlk* rblk;            // rebuild blocks (32 / TPP poses each)
  const SysBlk* fblk;            // finishing blocks (4 poses each)
  const int4* piece;             // [npieces] (atom0, atom1, row0, row1), packed indices
  const int2* item;              // [nitems] (system, piece) work items of the sweep
  const SysGroup* group;         // [ngroups]
  const int* seg_slot;           // [nsegs] first slot of each (system, type) segment
  const float4* pairs;           // [pairs][4] packed proteins, row order, as DevCull::pairs
  const int* row_start;          // [rows + 1] packed pair index of each row's first pair
  const float4* row_box;         // [rows]
  const int* flush_end;          // [rows] packed row index ending the row's flush block
  int nsys, B, nitems, ngroups, G;
  int Lmax, nrbmax, piece_pairs_max, piece_rows_max;
};

// ---- the one-pose path in one launch (kernels_pose.cu, k_one_pose) --------
struct GridLook {
  double o[3], inv;        // lattice origin (device frame), 1 / step
  int nx, ny, nz;
  float oh[3], ol[3];      // the origin as float pairs
  float invh, invl;        // 1 / step as a float pair
};

constexpr int kOneChunk = 128;  // protein atoms per CTA of the one-pose kernel
// threads in flight the pose rebuild aims for (threads per pose x poses)
constexpr long kRebuildThreadsInFlight = 160000;
// dynamic shared memory of a rebuild block of ppb poses (rebuild_pose's layout)
inline size_t rebuild_smem(int L, int nrb, int ppb) {
  return sizeof(float2) * 3 * (size_t)L * ppb + sizeof(float4) * (size_t)ppb * (3 + kMaxTors) +
         sizeof(float2) * 12 * (size_t)ppb * nrb;
}

struct OneScratch {
  float2* E;          // [npair][L] inter energy of each pair CTA's protein atoms per
                      // ligand atom (double-float: hi, lo)
  float4* G;          // [npair][L] dE/dX of the same
  float* intra;       // [kMaxTors + 2] the intra CTA's torsion terms, then its energy
  unsigned* arrive;   // CTAs done; the last one clears it
  int npair;          // pair CTAs (kOneChunk protein atoms each; 1 with the grids)
  int with_intra;     // 1: CTA 0 takes the intra terms (nested groups with MMO_F_INTRA)
  // MMO_F_GRID: the one pair CTA looks the inter energy up in the grids
  int grid;
  GridLook gl;
  const float* grids;
  const int* grid_lt;  // [L] grid type of each ligand atom
  int* gstat;          // MMO_S_OFF_GRID from the lookup CTA
};

// ---- Monte Carlo chains (kernels_mc.cu) ----------------------------------
enum : int { kMcUniform = 0, kMcGaussian = 1 };
constexpr int kMcCounts = 3;   // per chain: step, rigid frames, conformer frames
constexpr int kMcBlock = 100;  // adaptation period and sliding-window length (params.ml:29)
constexpr int kMcWin = 8;      // ints per sliding window: 4 words of event bits, head, length,
                               // accepts, padding
// trace events of a step (mmo_mc_state.trace_event)
enum : int { kMcAccepted = 1, kMcReset = 2, kMcStopped = 4, kMcBlocked = 8 };

struct MCDev {
  float* cur;       // [B][nd] current poses (optimiser layout)
  float* trial;     // [B][nd] proposed poses
  float* start;     // [B][6] rigid part of the start pose (the reset target)
  double* E_cur;    // [B]
  double* E_trial;  // [B]
  double* Ei_trial; // [B] inter energy of the trial pose
  float* G_cur;     // [B][nd] gradient at the current pose (minimiser)
  float* G_trial;   // [B][nd]
  int* st_trial;    // [B] status bits of the trial pose
  float* best;      // [B][nd] lowest-energy pose seen
  double* E_best;   // [B]
  double* steps;    // [B][2 + nrb] rotation (rad), translation (A), per-bond torsion step (rad)
  int* cnt;         // [B][kMcCounts] counters
  int* win;         // [B][1 + nrb][kMcWin] sliding windows: rigid moves, then one per bond
  int* moved;       // [B] bond of the last conformer move; -1 rigid move, -2 no move
  int* accepted;    // [B] accepted moves
  int* resets;      // [B] resets (out of the ROI, or E_inter = 0)
  int* stopped;     // [B] 1: the chain ended (an over-long trial conformer)
  int* status_or;   // [B] OR of the status bits of every scored pose
  float* eta;       // [B] gradient-descent step
};

struct MCParams {
  double kT;        // kcal/mol
  double rot, trans, tors;  // initial step sizes
  double roi_c[3], roi_r;   // hard region of interest (roi_r <= 0: off)
  float gd_step;
  int law;          // kMcUniform (Move.rand_*) or kMcGaussian
  int adapt;        // step-size adaptation from the sliding windows
  int flip_every;   // uniform law: every flip_every-th conformer move in [-pi, pi]
  int reset_zero;   // 1: a trial with E_inter exactly 0 resets the chain
  int too_long_ends;  // 1: an over-long trial conformer ends the chain
  uint32_t key0, key1;
  int B, nd, nrb;
  int trace_steps;  // steps of the trace buffers (0: no trace)
  float* trace_dofs;     // [trace_steps][B][nd] trial poses
  double* trace_E;       // [trace_steps][B] trial energies
  int* trace_event;      // [trace_steps][B] kMc* bits
};

// ---- precomputed interaction grids (kernels_grid.cu) --------------------
// One float32 lattice per ligand atom type (element, charge), x fastest:
// value[type][k][j][i] at the point o + step (i, j, k) of the device frame.
constexpr int kGridElems = kNTypes;  // distinct ligand elements of one set of grids
constexpr int kGridTileX = 4, kGridTileY = 4;  // lattice points per warp tile along x, y
                                                // (2 kp along z)

struct GridBuild {
  const int3* tiles;       // [ntiles] 4 x 4 x 2 kp point tiles that meet the mask sphere
  const float* type_qf;    // [ntypes] charge of each grid type
  const int* type_elem;    // [ntypes] rank of the type's element among the grid elements
  int ntiles, ntypes, nelem;
  int kp;                  // lattice points per lane: 1 or 2
  int nx, ny, nz;
  double o[3], step;       // lattice point (0, 0, 0) in the device frame, spacing
  double mc[3], mr2;       // mask sphere (device frame); points outside hold 0
  float max_Ef;            // cap of every value (rounded to float, as the values are)
  float2 el[kNTypes * kGridElems];  // [protein type][grid element] (D^(1/3) x^2, 1/D)
                                    // (1/D := 0 when D = 0); with fact, [protein type][0] =
                                    // (sqrt(D) x^6, sqrt(D) x^3)
  int fact;                         // 1: geometric mixing, the factorised vdW sums
  float4 elf[kGridElems];           // with fact, per grid element (sqrt(D), 2 x^3, x^6, 0)
  unsigned long long* pairs;  // [2] (point, atom) pairs evaluated for masked points, and
                              // those within 12 A (may be null)
};


// ---- lattice masks, clash tests, exhaustive docking, placement and
// desolvation (kernels_dock.cu) --------------------------------------------
enum : int { kClashIntra = 1, kClashHeavy = 2, kClashGrid = 4 };
constexpr int kDockBlock = 256;           // threads of a docking block
constexpr int kDockPerBlock = 2048;       // poses a docking block scores and sorts
constexpr int kDockMaxK = 1024;           // largest top-k
constexpr float kHeavyClashMax = 3.52f;   // 0.8 (2.2 + 2.2): the largest clash distance

// protein masks on the grids' lattice (Lds.vdW_volume, Lds.first_solvent_shell)
struct MaskBuild {
  const float* radius;     // [P] radius of each protein atom, row order
  int nx, ny, nz;
  double o[3], step;       // lattice point (0, 0, 0) in the device frame
  float r_w, r_max;        // water radius, largest atom radius
};

struct ClashArgs {
  GridLook g;                       // the masks' lattice (device frame)
  const uint8_t* vdw;               // [points] protein vdW volume, or null
  uint8_t heavy[kNTypes];           // 1 for the types of heavy atoms (anum > 1)
  float clash2[kNTypes * kNTypes];  // (0.8 (r_i + r_j))^2 by UFF type; NaN without radii
  int tests;                        // kClash* bits
};

struct DockArgs {
  const double* ref;        // [L][3] centred reference conformer
  const int* lig_type;      // [L] grid type of each atom
  const float* grids;       // [ntypes][nz][ny][nx]
  GridLook g;               // grids' lattice (device frame)
  const uint8_t* vcell;     // [points] cell masks of the vdW volume (k_cell_masks)
  const double* rot;        // [nrot][9] rotations, row-major
  float* off;               // [nrot][L][6] rotated atoms in lattice units, float pairs
  float4* pcell;            // [npos][2] position: fraction hi (x, y, z, bits of cell x), lo
  int* pcell_k;             // [npos][2] position: cells y, z
  const int* pos_idx;       // [npos] index of each position in the position lattice
  int L, npos, nrot, pdim;  // positions: pdim points per axis
  int rtile;                // rotations per CTA tile (a power of 2 dividing kDockPerBlock)
  double p0[3], pstep;      // position lattice origin (device frame), spacing
  int center_occ;           // the ligand's centre is inside one of its atoms
  double const_intra;
  int k;
  unsigned long long* cand;    // [blocks][k][2] (sortable score, frame)
  unsigned long long* counts;  // [2] poses scored, poses rejected by the clash test
};

struct PlaceArgs {
  const double* ref;        // [L][3]
  const int* type;          // [L] UFF type
  const int* slot_id;       // [slots] placement index of each launch slot
  int L, slots, per_slot, c0;  // candidates c0 .. c0 + per_slot - 1 of every slot
  double c[3], r;           // ROI (device frame)
  uint32_t key0, key1;
  float* out;               // [slots][per_slot][7]: (x, y, z, a, b, g) device frame, ok
};

struct DesolvBuild {
  const int3* tiles;        // [ntiles] 4 x 4 x 2 tiles meeting the ROI
  const uint8_t* shell;     // [points] protein solvent shell
  int ntiles, nx, ny, nz;
  double o[3], step;
  double c[3], r2;          // ROI (device frame)
  double scale;             // C vol / K^2 (the atoms carry K q)
};

struct DesolvPose {
  const float4* X;          // [B][L][2] posed atoms (hi, lo)
  const float* q;           // [L]
  const double* radius;     // [L]
  const uint8_t* shell;     // [points] protein solvent shell
  const double* contrib;    // [points] protein desolvation per point
  GridLook g;
  double step;
  float r_w;
  int L, B, cap;            // cap: lattice points of a pose's box the shared masks hold
  double scale;             // C vol
  double* prot;             // [B]
  double* lig;              // [B]
  int* status;              // [B] bit 1: the box exceeded cap
};

// ---- launchers (defined in the .cu files) --------------------------------
cudaError_t launch_k_mc_init(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_mc_start(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_mc_propose(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_mc_accept(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_gd_begin(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_gd_propose(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_gd_accept(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_k_gd_take(const MCDev& s, const MCParams& p, cudaStream_t st);
cudaError_t launch_philox(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, int n, uint4* out,
                          cudaStream_t st);
// ragged batch of systems (kernels_pose.cu, kernels_cull.cu)
cudaError_t launch_sys_rebuild(const DevSystems& S, int nblk, int tpp, const PoseIO& io,
                               const Scratch& s, int flags, cudaStream_t st);
cudaError_t launch_sys_finish(const DevSystems& S, int nblk, const PoseIO& io, const Scratch& s,
                              int flags, const Physics& ph, cudaStream_t st);
cudaError_t launch_sys_sort(const DevSystems& S, const Scratch& s, const CullScratch& cs,
                            int smem, cudaStream_t st);
cudaError_t launch_sys_pairs(const DevSystems& S, const float4* tab, const CullScratch& cs,
                             int kp, int threads, int blocks, int smem, int flags,
                             const Physics& ph, int* d_err, cudaStream_t st);
int sys_pairs_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem);
int sys_pairs_smem(int piece_pairs_max, int piece_rows_max, int threads);
cudaError_t launch_rebuild(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                           cudaStream_t st);
cudaError_t launch_pairs_batched(const DevProtein& prot, const float4* tab,
                                 const DevLigand& lig, const Scratch& s, int B, int flags,
                                 const Physics& ph, const PairPlan& plan, int* d_err,
                                 cudaStream_t st);
// Eout (with its arrival counter): the total of all partials, by the last block
cudaError_t launch_pairs_plain(const DevProtein& prot, const PairTable& tab, const float4* X,
                               const float* lig_q, const int* lig_type, int L, int C,
                               double* Epart, float4* Gpart, int grad, const Physics& ph,
                               cudaStream_t st, double* Eout = nullptr,
                               unsigned* arrive = nullptr);
int one_pose_smem(int L, int nrb);  // static + dynamic shared memory of k_one_pose, bytes
// *stage: 1 when the shared-memory attribute call failed, 2 the launch
cudaError_t launch_one_pose(const DevLigand& lig, const DevProtein& prot, const float4* tab4,
                            const PoseIO& io, const Scratch& s, const OneScratch& os, int flags,
                            const Physics& ph, cudaStream_t st, int* stage);
cudaError_t launch_finish(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                          const Physics& ph, cudaStream_t st);
// the inter energy's two parts for one ligand: Eout[0] electrostatic, Eout[1]
// van der Waals (Epart: 2 C L partials), one launch
cudaError_t launch_pairs_parts(const DevProtein& prot, const PairTable& tab, const float4* X,
                               const float* lig_q, const int* lig_type, int L, int C,
                               double* Epart, const Physics& ph, cudaStream_t st, double* Eout,
                               unsigned* arrive);
cudaError_t launch_intra_plain(const DevLigand& lig, const float4* X, int form, int dielectric,
                               double* out, cudaStream_t st);
int pairs_batched_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem_bytes);
// entry sort of the cut-off sweep: bin, scan, scatter (hist must be zeroed)
cudaError_t launch_cull_sort(const Scratch& s, const float* lig_q, int B, int L,
                             const CullSegs& seg, const CullScratch& cs, cudaStream_t st);
cudaError_t launch_pairs_cull(const DevCull& cull, const float4* tab, const CullSegs& seg,
                              const CullScratch& cs, int flags, const Physics& ph,
                              const CullPlan& plan, int* d_err, cudaStream_t st);
int cull_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem_bytes,
                    bool glob);
int cull_smem_bytes(int npairs, int nrows, int threads, bool glob, int kp);
cudaError_t launch_grid_build(const DevCull& cull, const GridBuild& gb, int dielectric,
                              float* grids, cudaStream_t st);
// one ligand of n <= kMaxLig atoms in one launch: its energy and status
cudaError_t launch_grid_inter_one(const GridLook& g, const float4* X, int n,
                                  const int* atom_type, const float* grids, double* Eout,
                                  int* status, cudaStream_t st);
cudaError_t launch_grid_inter(const GridLook& g, const float4* X, int n, int L,
                              const int* atom_type, const float* grids, double* Epart,
                              float4* Gpart, int* status, int grad, cudaStream_t st);
cudaError_t launch_masks(const DevCull& cull, const MaskBuild& mb, const double* radius64,
                         uint8_t* vdw, uint8_t* shell, cudaStream_t st);
cudaError_t launch_clash(const DevLigand& lig, const float4* X, int B, const DevCull& cull,
                         const ClashArgs& ca, int* out, cudaStream_t st);
cudaError_t launch_cell_masks(const GridLook& g, const uint8_t* mask, uint8_t* cell,
                              cudaStream_t st);
cudaError_t launch_dock(const DockArgs& a, int blocks, cudaStream_t st);
cudaError_t launch_topk_merge(const unsigned long long* in, int n, int k, unsigned long long* out,
                              cudaStream_t st);
cudaError_t launch_place(const PlaceArgs& a, const DevCull& cull, const ClashArgs& ca,
                         cudaStream_t st);
cudaError_t launch_prot_desolv(const DevCull& cull, const DesolvBuild& db, double* out,
                               cudaStream_t st);
cudaError_t launch_desolv_pose(const DesolvPose& d, cudaStream_t st);
cudaError_t launch_fma_peak(int sms, int iters, float* out, cudaStream_t st, double* flops);
cudaError_t launch_df_sincos(const float* x, int n, float4* out, cudaStream_t st);
cudaError_t launch_count_within(const float4* X, int n, const float4* atoms, int P, float r2cut,
                                unsigned long long* out, cudaStream_t st);

// ---- device helpers ------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC 2011): counter c, key (k0, k1)
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
  }
  return c;
}

// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double u01(uint32_t a, uint32_t b) {
  return (double)(((uint64_t)a << 21) ^ (uint64_t)(b >> 11)) * (1.0 / 9007199254740992.0);
}

// pair difference a - b of two hi/lo coordinate pairs
__device__ __forceinline__ float split_diff(float ah, float al, float bh, float bl) {
  return (ah - bh) + (al - bl);
}

// 1 / x from the reciprocal instruction (about one ulp; x >= 1e-4 here, so
// flushing subnormals changes nothing).  The pair terms take 1 / r^2 from it
// instead of squaring the reciprocal square root, whose error the squaring
// doubles and the r^-12 and r^-14 terms of a close contact multiply six- and
// sevenfold again.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// (hi, lo) = (ch + cl) + v as a normalised float pair: TwoSum of ch and v
// (Knuth), the low parts added, then Fast2Sum
__device__ __forceinline__ void dadd_into(float ch, float cl, float v, float& hi, float& lo) {
  const float s = ch + v;
  const float bb = s - ch;
  const float e = (ch - (s - bb)) + (v - bb);
  const float t = e + cl;
  hi = s + t;
  lo = t - (hi - s);
}

// One UFF nonbonded pair, FP32.  d = ligand - partner.  FORM 0: shifted by
// (1 - (r/12)^2)^2 and cut at 12 A (mol.ml:836-845); FORM 1: unshifted
// (mol.ml:811-815, 894-900).  DIEL 0: K qq / r; DIEL 1: K qq / r^2.  The
// distance is clamped at 0.01 A (math.ml:58-62), where the derivative is 0.
// acc += E_pair; with GRAD, g += dE_pair/dd.
template <bool GRAD, int DIEL, int FORM>
__device__ __forceinline__ void uff_pair(float dx, float dy, float dz, float x2, float D,
                                         float qq, float& acc, float& gx, float& gy,
                                         float& gz) {
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float r2c = fmaxf(r2, kMinR2);
  const float ir = rsqrtf(r2c);
  const float ir2 = rcp_approx(r2c);
  const float p2 = x2 * ir2;
  const float p6 = p2 * p2 * p2;
  const float Dp6 = D * p6;
  // explicit fused forms: the energy rounds the same in every kernel variant
  const float el = DIEL == 0 ? qq * ir : qq * ir2;
  const float e = fmaf(Dp6, p6 - 2.0f, el);
  float s = 1.0f, w = 1.0f;
  if (FORM == 0) {
    s = fmaxf(fmaf(r2c, -1.0f / 144.0f, 1.0f), 0.0f);
    w = s * s;
  }
  acc = fmaf(w, e, acc);
  if (GRAD) {
    // 2 dE/dr2: w (2 dLJ/dr2 + 2 dEl/dr2) + 2 dw/dr2 * e
    const float t = fmaf(-12.0f, Dp6 * (p6 - 1.0f), DIEL == 0 ? -el : -2.0f * el);
    float g = w * t * ir2;
    if (FORM == 0) g = fmaf(s * (-1.0f / 36.0f), e, g);
    g = r2 < kMinR2 ? 0.0f : g;
    gx = fmaf(g, dx, gx);
    gy = fmaf(g, dy, gy);
    gz = fmaf(g, dz, gz);
  }
}

// The electrostatic and van der Waals parts of uff_pair's energy, each with
// the switch weight, into el_acc and lj_acc (mol.ml:945-953)
template <int DIEL, int FORM>
__device__ __forceinline__ void uff_pair_parts(float dx, float dy, float dz, float x2, float D,
                                               float qq, float& el_acc, float& lj_acc) {
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float r2c = fmaxf(r2, kMinR2);
  const float ir = rsqrtf(r2c);
  const float ir2 = rcp_approx(r2c);
  const float p2 = x2 * ir2;
  const float p6 = p2 * p2 * p2;
  const float el = DIEL == 0 ? qq * ir : qq * ir2;
  float w = 1.0f;
  if (FORM == 0) {
    const float s = fmaxf(fmaf(r2c, -1.0f / 144.0f, 1.0f), 0.0f);
    w = s * s;
  }
  el_acc = fmaf(w, el, el_acc);
  lj_acc = fmaf(w, (D * p6) * (p6 - 2.0f), lj_acc);
}

// Energy e and the scalar g of one pair's gradient, dE_pair/dd = g d (the
// terms of uff_pair, from one reciprocal square root).
template <int DIEL, int FORM>
__device__ __forceinline__ void uff_pair_eg(float dx, float dy, float dz, float x2, float D,
                                            float qq, float& e_out, float& g_out) {
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float r2c = fmaxf(r2, kMinR2);
  const float ir = rsqrtf(r2c);
  const float ir2 = rcp_approx(r2c);
  const float p2 = x2 * ir2;
  const float p6 = p2 * p2 * p2;
  const float Dp6 = D * p6;
  const float el = DIEL == 0 ? qq * ir : qq * ir2;
  const float e = fmaf(Dp6, p6 - 2.0f, el);
  float s = 1.0f, w = 1.0f;
  if (FORM == 0) {
    s = fmaxf(fmaf(r2c, -1.0f / 144.0f, 1.0f), 0.0f);
    w = s * s;
  }
  const float t = fmaf(-12.0f, Dp6 * (p6 - 1.0f), DIEL == 0 ? -el : -2.0f * el);
  float g = w * t * ir2;
  if (FORM == 0) g = fmaf(s * (-1.0f / 36.0f), e, g);
  e_out = w * e;
  g_out = r2 < kMinR2 ? 0.0f : g;
}

// One pair: ligand atom (hi/lo) against protein atom p (hi, K q) / pl (lo).
// With Dp6 = (X / r^2)^3 = D p6 (X = D^(1/3) x^2) and p6 = Dp6 / D:
//   lj = Dp6 (Dp6 / D - 2),  e = lj + el,
//   -(2 dE/dr2 unswitched) r2     = e - Dp6 (10 - 11 p6)        (eps = 4)
//   -(2 dE/dr2 unswitched) r2 / 2 = e - Dp6 (4 - 5 p6)          (eps = 4 r)
// so nt below is -t (eps 4) or -t/2 (eps 4r) and g accumulates -dE/dd or
// -dE/dd / 2 (the caller rescales); (c1, c0) = (11/D, -10) or (5/D, -4).
// mn tracks the smallest r2 for the 0.01 A clamp check.
template <bool GRAD, int DIEL, int FORM, bool MASK = false>
__device__ __forceinline__ void pair_step(float xh, float yh, float zh, float xl, float yl,
                                          float zl, float4 p, float4 pl, float qq, float X,
                                          float invD, float c1, float c0, float& acc, float& gx,
                                          float& gy, float& gz, float& mn) {
  const float dx = (xh - p.x) + (xl - pl.x);
  const float dy = (yh - p.y) + (yl - pl.y);
  const float dz = (zh - p.z) + (zl - pl.z);
  const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  const float r2c = fmaxf(r2, kMinR2);
  const float ir = rsqrtf(r2c);
  const float ir2 = rcp_approx(r2c);
  const float P = X * ir2;
  const float Dp6 = (P * P) * P;
  const float lj = Dp6 * fmaf(Dp6, invD, -2.0f);
  const float e = fmaf(qq, DIEL == 0 ? ir : ir2, lj);
  float s = 1.0f;
  if (FORM == 0) {
    s = fmaxf(fmaf(r2c, -1.0f / 144.0f, 1.0f), 0.0f);
    acc = fmaf(s * s, e, acc);
  } else {
    acc += e;
  }
  if (GRAD) {
    const float nt = fmaf(Dp6, fmaf(Dp6, c1, c0), e);
    const float na = nt * ir2;
    float g = na;
    if (FORM == 0) g = s * fmaf(s, na, e * (DIEL == 0 ? 1.0f / 36.0f : 1.0f / 72.0f));
    if (MASK) g = r2 < kMinR2 ? 0.0f : g;  // clamped distance: derivative 0
    mn = fminf(mn, r2);
    gx = fmaf(g, dx, gx);
    gy = fmaf(g, dy, gy);
    gz = fmaf(g, dz, gz);
  }
}

// both halves of a packed FP32 operand
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }

// One entry (the same values in both halves) against a pair of protein atoms
// (a, b) of the cut-off sweep's layout, on the packed FP32 instructions:
// a0 = (-x_hi a, -x_hi b, -y_hi a, -y_hi b), a1 = (-z_hi a, -z_hi b, Kq a, Kq b),
// a2, a3 the lo halves (a3.zw: type offsets), (X, 1/D, c1) of a and b.  Each
// half is pair_step's arithmetic in its order; the half of atom a accumulates
// the even atoms of a row, that of b the odd ones.  A packed instruction does
// two FP32 operations on the FMA pipes in one issue slot, and the atoms' values
// come in pairs from shared memory, so nothing is broadcast in the loop.
__device__ __forceinline__ float2 lo_pair(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi_pair(float4 v) { return make_float2(v.z, v.w); }
template <bool GRAD, int DIEL, int FORM, bool MASK = false>
__device__ __forceinline__ void pair_step_ab(float2 xh, float2 yh, float2 zh, float2 xl,
                                             float2 yl, float2 zl, float2 q, float4 a0, float4 a1,
                                             float4 a2, float4 a3, float2 X, float2 invD,
                                             float2 c1, float c0, float2& acc, float2& gx,
                                             float2& gy, float2& gz, float& mn) {
  const float2 dx = __fadd2_rn(__fadd2_rn(xh, lo_pair(a0)), __fadd2_rn(xl, lo_pair(a2)));
  const float2 dy = __fadd2_rn(__fadd2_rn(yh, hi_pair(a0)), __fadd2_rn(yl, hi_pair(a2)));
  const float2 dz = __fadd2_rn(__fadd2_rn(zh, lo_pair(a1)), __fadd2_rn(zl, lo_pair(a3)));
  const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
  const float2 r2c = make_float2(fmaxf(r2.x, kMinR2), fmaxf(r2.y, kMinR2));
  const float2 ir = make_float2(rsqrtf(r2c.x), rsqrtf(r2c.y));
  const float2 ir2 = make_float2(rcp_approx(r2c.x), rcp_approx(r2c.y));
  const float2 P = __fmul2_rn(X, ir2);
  const float2 Dp6 = __fmul2_rn(__fmul2_rn(P, P), P);
  const float2 lj = __fmul2_rn(Dp6, __ffma2_rn(Dp6, invD, bc2(-2.0f)));
  const float2 qq = __fmul2_rn(hi_pair(a1), q);
  const float2 e = __ffma2_rn(qq, DIEL == 0 ? ir : ir2, lj);
  float2 s = bc2(1.0f);
  if (FORM == 0) {
    const float2 t = __ffma2_rn(r2c, bc2(-1.0f / 144.0f), bc2(1.0f));
    s = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));
    acc = __ffma2_rn(__fmul2_rn(s, s), e, acc);
  } else {
    acc = __fadd2_rn(acc, e);
  }
  if (GRAD) {
    const float2 nt = __ffma2_rn(Dp6, __ffma2_rn(Dp6, c1, bc2(c0)), e);
    const float2 na = __fmul2_rn(nt, ir2);
    float2 g = na;
    if (FORM == 0)
      g = __fmul2_rn(s, __ffma2_rn(s, na,
                                   __fmul2_rn(e, bc2(DIEL == 0 ? 1.0f / 36.0f : 1.0f / 72.0f))));
    if (MASK) {  // clamped distance: derivative 0
      g.x = r2.x < kMinR2 ? 0.0f : g.x;
      g.y = r2.y < kMinR2 ? 0.0f : g.y;
    }
    mn = fminf(mn, fminf(r2.x, r2.y));
    gx = __ffma2_rn(g, dx, gx);
    gy = __ffma2_rn(g, dy, gy);
    gz = __ffma2_rn(g, dz, gz);
  }
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D bulk copy global -> shared through the TMA engine; 16-byte aligned
// addresses and a size that is a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait on an mbarrier phase: returns false after max_iter polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_iter) {
  for (uint32_t it = 0; it < max_iter; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Index of cell (x, y, z) of the 32^3 binning grid along a 3-D Hilbert curve
// (J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc. 707, 2004:
// axes to transposed index, then the bits interleaved).  Consecutive slots in
// Hilbert order stay closer together than in Morton order, so the groups'
// boxes are smaller.
template <int kBits = 5>
__device__ __forceinline__ uint32_t hilbert_cell(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t X[3] = {x, y, z};
  for (uint32_t Q = 1u << (kBits - 1); Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;
      } else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  X[2] ^= X[1];
  uint32_t t = 0;
  for (uint32_t Q = 1u << (kBits - 1); Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  uint32_t k = 0;
#pragma unroll
  for (int b = kBits - 1; b >= 0; --b)
#pragma unroll
    for (int i = 0; i < 3; ++i) k = (k << 1) | (((X[i] ^ t) >> b) & 1u);
  return k;
}

__device__ __forceinline__ int grid_cell(float v, float lo, float inv) {
  // NaN converts to 0; the clamp keeps infinities and far entries on the grid
  return min(max(__float2int_rd((v - lo) * inv), 0), kCullGrid - 1);
}

// Lattice coordinate u = (x - o) / step of a float-pair coordinate on one axis,
// as a cell i = floor(u) and a fraction w in [0, 1), in float-pair arithmetic
// (TwoDiff of the high parts, the product's error by FMA); false unless the
// cell's high corner is on the lattice (0 <= u < n - 1).
__device__ __forceinline__ bool lattice_cell(float xh, float xl, float oh, float ol, float ih,
                                             float il, int n, int& i, float& w) {
  const float dh = __fsub_rn(xh, oh);
  const float bp = __fsub_rn(dh, xh), ap = __fsub_rn(dh, bp);
  const float de = __fadd_rn(__fsub_rn(xh, ap), __fsub_rn(-oh, bp));
  const float dl = __fadd_rn(de, __fsub_rn(xl, ol));
  const float uh = __fmul_rn(dh, ih);
  const float ul = __fadd_rn(fmaf(dh, ih, -uh), fmaf(dh, il, __fmul_rn(dl, ih)));
  if (!(uh > -2.0f && uh < (float)n + 1.0f)) return false;  // also NaN
  const float f = floorf(uh);
  float frac = __fadd_rn(__fsub_rn(uh, f), ul);
  int k = (int)f;
  if (frac < 0.f) {
    frac = __fadd_rn(frac, 1.f);
    --k;
  } else if (frac >= 1.f) {
    frac = __fsub_rn(frac, 1.f);
    ++k;
  }
  if (frac >= 1.f) frac = 0.99999994f;
  i = k;
  w = frac;
  return k >= 0 && k <= n - 2;
}

// One thread per entry: E = trilin of the atom's type grid at the atom, and
// dE/dx (the derivative of the trilinear form), into Epart / Gpart.  The
// lattice coordinate in float pairs; weights, values and the interpolation
// in FP32 (the values are float32, as the reference's .ba1 grids).  A corner
// off the lattice (the reference reads out of bounds) sets MMO_S_OFF_GRID and
// the entry adds 0.
// the trilinear value (and gradient) of the type grid `type` at the entry's
// position; false when a corner is off the lattice (E = 0 then)
template <bool GRAD>
__device__ __forceinline__ bool grid_entry(const GridLook& g, float4 h, float4 l, int type,
                                           const float* __restrict__ grids, float& E, float& gx,
                                           float& gy, float& gz) {
  int i0, j0, k0;
  float wx, wy, wz;
  const bool ok = lattice_cell(h.x, l.x, g.oh[0], g.ol[0], g.invh, g.invl, g.nx, i0, wx) &
                  lattice_cell(h.y, l.y, g.oh[1], g.ol[1], g.invh, g.invl, g.ny, j0, wy) &
                  lattice_cell(h.z, l.z, g.oh[2], g.ol[2], g.invh, g.invl, g.nz, k0, wz);
  E = gx = gy = gz = 0.f;
  if (ok) {
    const size_t nx = g.nx, nxy = (size_t)g.nx * g.ny;
    const float* v = grids + (size_t)type * nxy * g.nz + i0 + j0 * nx + k0 * nxy;
    const float a = v[0], b = v[1], c = v[1 + nx], d = v[nx];
    const float ee = v[nxy], f = v[1 + nxy], gg = v[1 + nx + nxy], hh = v[nx + nxy];
    const float hx = 1.f - wx, hy = 1.f - wy, hz = 1.f - wz;
    const float c00 = fmaf(b, wx, a * hx), c10 = fmaf(c, wx, d * hx);
    const float c01 = fmaf(f, wx, ee * hx), c11 = fmaf(gg, wx, hh * hx);
    const float c0 = fmaf(c10, wy, c00 * hy), c1 = fmaf(c11, wy, c01 * hy);
    E = fmaf(c1, wz, c0 * hz);
    if (GRAD) {
      const float inv = g.invh;
      gx = inv * (hz * fmaf(c - d, wy, (b - a) * hy) + wz * fmaf(gg - hh, wy, (f - ee) * hy));
      gy = inv * (hz * (c10 - c00) + wz * (c11 - c01));
      gz = inv * (c1 - c0);
    }
  }
  return ok;
}

// Double-float arithmetic: a value is an unevaluated pair h + l of floats
// (|l| <= ulp(h) / 2), about 48 significant bits, on the FP32 pipe (GB300's
// FP64 rate is 1/64 of its FP32 rate).  ts / qts are the error-free sums
// (TwoSum, and Fast2Sum for |a| >= |b|); the products take their error by FMA.
__device__ __forceinline__ float2 df_of(double x) {
  const float h = __double2float_rn(x);
  return make_float2(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ float2 qts(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 ts(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp)));
}
__device__ __forceinline__ float2 dadd(float2 a, float2 b) {
  const float2 s = ts(a.x, b.x);
  return qts(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 dneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 dsub(float2 a, float2 b) { return dadd(a, dneg(b)); }
__device__ __forceinline__ float2 dmul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  return qts(p, fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p))));
}
// a0 b0 + a1 b1 + a2 b2 + c
__device__ __forceinline__ float2 ddot3c(float2 a0, float2 b0, float2 a1, float2 b1, float2 a2,
                                         float2 b2, float2 c) {
  return dadd(dadd(dadd(dmul(a0, b0), dmul(a1, b1)), dmul(a2, b2)), c);
}
__device__ __forceinline__ float2 dshfl_xor(float2 a, int o) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, o), __shfl_xor_sync(0xffffffffu, a.y, o));
}
__device__ __forceinline__ bool dgt(float2 a, float2 b) {
  return a.x > b.x || (a.x == b.x && a.y > b.y);
}
// s += x for a double-float running sum s (TwoSum on the high part)
__device__ __forceinline__ void acc2(float2& s, float x) {
  const float2 t = ts(s.x, x);
  s.x = t.x;
  s.y = __fadd_rn(s.y, t.y);
}

// sin and cos of a float angle x as double-floats, on the FP32 pipe (the FP64
// library sincos runs at GB300's FP64 rate).  Cody-Waite reduction:
// k = rint(2 x / pi), r = x - k pi/2 with pi/2 split in three floats (the
// first with 8 significant bits, so k * kHalfPi1 is exact for |k| < 2^16);
// then the Taylor series of sin r and cos r on |r| <= pi/4 + (rounding of k),
//   sin r = r (1 - z/3! + z^2/5! - ...),  cos r = 1 - z/2! + z^2/4! - ...,
// z = r^2, summed by Horner's scheme with the five leading steps in
// double-float and the tail (below 3e-8 of the result from z^5 on) in FP32;
// the last terms kept are z^8 / 17! and z^9 / 18! (the next ones are below
// 1e-18).  Absolute error below 1e-14 (the double-float operations), plus
// |k| 6e-17 from pi / 2 rounded to double (4e-13 at |x| = 1e4); |x| >= 1e5
// takes the FP64 library function.
constexpr double kHalfPi = 1.5707963267948966;  // pi / 2 rounded to double
constexpr float kHalfPi1 = 1.5703125f;          // 201 / 128
constexpr float kHalfPi2 = (float)(kHalfPi - 1.5703125);
constexpr float kHalfPi3 = (float)(kHalfPi - 1.5703125 - (double)(float)(kHalfPi - 1.5703125));
constexpr double inv_fact(int m) {
  double f = 1.0;
  for (int i = 2; i <= m; ++i) f *= i;
  return 1.0 / f;
}
// 1 / m! rounded at compile time: hi, and the lo of the double-float
#define MMO_INV_FACT(m)                                 \
  constexpr float kIF##m##h = (float)inv_fact(m);       \
  constexpr float kIF##m##l = (float)(inv_fact(m) - (double)(float)inv_fact(m));
MMO_INV_FACT(2)
MMO_INV_FACT(3)
MMO_INV_FACT(4)
MMO_INV_FACT(5)
MMO_INV_FACT(6)
MMO_INV_FACT(7)
MMO_INV_FACT(8)
MMO_INV_FACT(9)
MMO_INV_FACT(10)
MMO_INV_FACT(11)
MMO_INV_FACT(12)
MMO_INV_FACT(13)
MMO_INV_FACT(14)
MMO_INV_FACT(15)
MMO_INV_FACT(16)
MMO_INV_FACT(17)
MMO_INV_FACT(18)
#undef MMO_INV_FACT

__device__ __forceinline__ void df_sincos(float x, float2& s, float2& c) {
  if (!(fabsf(x) < 1e5f)) {  // (also NaN and infinities)
    double sd, cd;
    sincos((double)x, &sd, &cd);
    s = df_of(sd);
    c = df_of(cd);
    return;
  }
  const float k = rintf(x * 0.63661977236758134f);  // 2 / pi
  float2 r = ts(x, -k * kHalfPi1);                   // k kHalfPi1 exact
  const float p2 = k * kHalfPi2;
  r = dsub(r, make_float2(p2, fmaf(k, kHalfPi2, -p2)));
  r = dsub(r, make_float2(k * kHalfPi3, 0.f));
  const float2 z = dmul(r, r);
  const float zf = z.x;
  // sin: tail from z^5 in FP32, then z^4 / 9!, -z^3 / 7!, z^2 / 5!, -z / 3!, 1
  const float ts5 = fmaf(fmaf(fmaf(kIF17h, zf, -kIF15h), zf, kIF13h), zf, -kIF11h);
  float2 hs = make_float2(ts5, 0.f);
  hs = dadd(dmul(hs, z), make_float2(kIF9h, kIF9l));
  hs = dadd(dmul(hs, z), make_float2(-kIF7h, -kIF7l));
  hs = dadd(dmul(hs, z), make_float2(kIF5h, kIF5l));
  hs = dadd(dmul(hs, z), make_float2(-kIF3h, -kIF3l));
  hs = dadd(dmul(hs, z), make_float2(1.f, 0.f));
  const float2 sr = dmul(r, hs);
  // cos: tail from z^5 in FP32, then z^4 / 8!, -z^3 / 6!, z^2 / 4!, -z / 2!, 1
  const float tc5 = fmaf(fmaf(fmaf(fmaf(-kIF18h, zf, kIF16h), zf, -kIF14h), zf, kIF12h), zf, -kIF10h);
  float2 hc = make_float2(tc5, 0.f);
  hc = dadd(dmul(hc, z), make_float2(kIF8h, kIF8l));
  hc = dadd(dmul(hc, z), make_float2(-kIF6h, -kIF6l));
  hc = dadd(dmul(hc, z), make_float2(kIF4h, kIF4l));
  hc = dadd(dmul(hc, z), make_float2(-kIF2h, -kIF2l));
  const float2 cr = dadd(dmul(hc, z), make_float2(1.f, 0.f));
  switch (((int)k) & 3) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = dneg(sr); break;
    case 2: s = dneg(sr); c = dneg(cr); break;
    default: s = dneg(cr); c = sr; break;
  }
}
#endif

}  // namespace mmo

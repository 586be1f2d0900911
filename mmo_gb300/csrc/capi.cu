// capi.cu -- the extern "C" boundary of libmmo_gpu.so (include/mmo_gpu.h):
// context, uploads of the protein and the ligand into their HBM layouts,
// the plain drop-in calls and the batched pose scorer.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/mmo_diag.h"
#include "../../include/mmo_gpu.h"
#include "../../include/mmo_dock.h"
#include "../../include/mmo_grid.h"
#include "../../include/mmo_mc.h"
#include "../../include/mmo_systems.h"
#include "mmo_internal.cuh"

using namespace mmo;

namespace {

// src/UFF.ml:10-22: (anum, x_i, D_i); index in this table = device type index
struct UffRow {
  int anum;
  double xi, di;
};
constexpr UffRow kUff[kNTypes] = {{0, 0.0, 0.0},      {1, 2.886, 0.044},  {6, 3.851, 0.105},
                                  {7, 3.660, 0.069},  {8, 3.500, 0.060},  {9, 3.364, 0.050},
                                  {12, 3.021, 0.111}, {15, 4.147, 0.305}, {16, 4.035, 0.274},
                                  {17, 3.947, 0.227}, {35, 4.189, 0.251}, {53, 4.500, 0.339}};
constexpr double kElec = 332.0637 / 4.0;  // UFF.ml:25, const.ml:18

int type_of(int anum) {
  for (int t = 0; t < kNTypes; ++t)
    if (kUff[t].anum == anum) return t;
  return -1;
}

// (x_ij^2, D_ij) in double, rounded once
void pair_xd(int mixing, int t1, int t2, double* x2, double* d) {
  const double x1 = kUff[t1].xi, xb = kUff[t2].xi;
  if (mixing == MMO_MIX_LB) {
    const double x = 0.5 * (x1 + xb);
    *x2 = x * x;
  } else {
    *x2 = x1 * xb;  // (sqrt(x_i x_j))^2, UFF.ml:47
  }
  *d = std::sqrt(kUff[t1].di * kUff[t2].di);  // UFF.ml:48
}

char g_create_err[256] = "";

// (x, y, z) as hi/lo float pairs: dst[0] = (hi..., w), dst[1] = (lo..., 0)
void split_store(float4* dst, double x, double y, double z, float w) {
  const float xh = (float)x, yh = (float)y, zh = (float)z;
  dst[0] = make_float4(xh, yh, zh, w);
  dst[1] = make_float4((float)(x - (double)xh), (float)(y - (double)yh), (float)(z - (double)zh),
                       0.f);
}

// true for page-locked (or registered) host memory, which a copy can reach by DMA
bool host_pinned(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // not a pointer the runtime knows: ordinary host memory
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// next 16-byte aligned offset of a block of `bytes`
size_t take(size_t& off, size_t bytes) {
  const size_t o = (off + 15) & ~size_t(15);
  off = o + bytes;
  return o;
}

// pointer into `base` (or null while only sizing) for `count` T's
template <class T>
T* align_ptr(char* base, size_t& off, size_t count) {
  const size_t o = take(off, sizeof(T) * count);
  return base ? reinterpret_cast<T*>(base + o) : nullptr;
}

}  // namespace

struct mmo_ctx {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  Physics ph{0, 0, 0, 0};
  PairTable tab{};
  PairTable4 tab4{};
  float4* d_tab4 = nullptr;  // device copy of tab4
  int tile_kp = 0, tile_threads = 0, tile_chunks = 0;
  // last launch plan and the inputs it was made for
  // launch plans, one per gradient flag, and the inputs they were made for
  PairPlan plan[2] = {};
  long plan_key[2][8] = {{-1, -1, -1, -1, -1, -1, -1, -1}, {-1, -1, -1, -1, -1, -1, -1, -1}};

  // protein
  DevProtein prot{};
  void* d_prot = nullptr;
  double origin[3] = {0, 0, 0};
  float origin_f[3] = {0, 0, 0};
  // host copy in the device frame, for rebuilding the row index
  std::vector<double> pxs, pys, pzs;
  std::vector<float> pkq;
  std::vector<int> ptypes;

  // cut-off sweep of the shifted form (mmo_set_cull)
  int cull_mode = 0;        // 0: automatic, 1: off, 2: protein read from global memory
  double cull_h = 3.0;      // row spacing of the protein index, A
  int cull_piece = 0;       // protein atoms per piece, 0: automatic
  int cull_kp = 0;          // entries per lane, 0: automatic
  bool cull_ok = false;     // row index built
  bool cull_fits = false;   // the whole protein and its row index fit in shared memory
  float4* d_pbox = nullptr;  // [npieces][2] piece boxes of the cut-off sweep
  size_t capPbox = 0;
  size_t capGcnt = 0, capGlist = 0, capItems = 0;
  long cull_version = 0;    // bumped by every rebuild of the row index
  DevCull cull{};
  void* d_cull = nullptr;
  std::vector<int> cull_rows;  // host copy of row_start
  int smem_optin = 0;
  CullScratch cs{};
  CullSegs segs[2] = {};
  CullPlan cplan[2] = {};
  long cplan_key[2][11] = {{-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1},
                           {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1}};
  long piece_key[2] = {-1, -1};  // (row index version, piece atoms) of the uploaded pieces
  int npieces = 0;
  int* d_piece = nullptr;
  size_t capPiece = 0, capHist = 0, capBin = 0, capRank = 0, capXs = 0, capOrd = 0, capEp = 0,
         capGp = 0, capArr = 0, capVis = 0;
  std::string tune_cache;        // file of tuned plans (mmo_set_tune_cache)
  unsigned* d_queue = nullptr;  // [0] work counter, [2..3] pair evaluations (u64)
  bool last_cull = false;       // the last call's inter term used the cut-off sweep
  int last_grad = 0;            // the last call computed the gradient
  double last_pairs = 0;        // poses x ligand atoms x protein atoms of the last call
  int last_launches = 0;        // kernels of the last scoring call

  // ligand (host copies kept for physics changes)
  DevLigand lig{};
  void* d_lig = nullptr;
  bool has_lig = false;
  std::vector<double> lx, ly, lz, lq;
  std::vector<int> ltype, lbonds, lgoff, lgatoms;
  std::vector<uint8_t> linter;
  std::vector<int> lseg_type, lseg_count;  // ligand types present, atoms of each
  long lig_version = 0, prot_version = 0;  // bumped by every upload

  // scratch
  Scratch scr{};
  size_t capX = 0, capE = 0, capG = 0, capI = 0, capY = 0, capR = 0;
  int* d_err = nullptr;
  uint32_t first_wait_polls = kWaitPollsDefault;  // mmo_diag_set_wait_polls
  // the one-pose path (k_one_pose): per-CTA partials and the arrival count
  OneScratch one{};
  unsigned* d_plain_arrive = nullptr;  // mmo_ene_inter's arrival counter
  int last_pose_entries = 0;           // B L posed entries in scr.X from the last call
  bool one_ok = false;       // its shared memory fits (set with the ligand)
  size_t capOneE = 0, capOneG = 0;

  // stage timing (mmo_set_profiling): start, rebuilt, sorted, swept, finished
  bool profiling = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  bool ev_valid = false;

  // Monte Carlo chains (mmo_mc_run): one blob of per-chain buffers and the
  // CUDA graph of a block of steps
  void* d_mc = nullptr;
  size_t cap_mc = 0;
  cudaGraphExec_t mc_exec = nullptr;
  std::vector<long> mc_key;
  cudaEvent_t mc_ev[2] = {nullptr, nullptr};
  long epoch = 0;  // bumped whenever baked launch arguments (buffers, uploads, plans) change
  struct SysBatch* sys = nullptr;  // ragged batch of systems (mmo_set_systems)

  // precomputed interaction grids (mmo_build_grids / mmo_load_grids)
  bool grid_ok = false;
  double grid_step = 0.0;
  int grid_n[3] = {0, 0, 0};
  double grid_origin[3] = {0, 0, 0};  // lattice point (0, 0, 0) in the user's frame
  std::vector<int> grid_anum;
  std::vector<double> grid_q;
  float* d_grid = nullptr;            // [ntypes][nz][ny][nx]
  size_t cap_grid = 0;
  int* d_grid_lt = nullptr;           // [L] grid type of each ligand atom
  size_t cap_grid_lt = 0;
  std::vector<int> grid_lt;           // host copy
  bool grid_map_ok = false;
  std::string grid_map_err = "no grids: call mmo_build_grids or mmo_load_grids first";
  double grid_stats[3] = {0, 0, 0};   // last build: masked points, pairs evaluated, within 12 A
  int grid_kp_set = 0;                // lattice points per lane of the build kernel, 0: automatic

  // protein masks on the grids' lattice (mmo_build_masks / mmo_load_masks),
  // ligand radii, desolvation contributions, docking and placement scratch
  std::vector<int> cull_perm;         // row position -> mmo_set_protein index
  bool masks_ok = false;
  uint8_t* d_vdw = nullptr;           // [points]
  uint8_t* d_vcell = nullptr;         // [points] cell masks of the vdW volume (any / all corners)
  size_t cap_vcell = 0;
  uint8_t* d_shell = nullptr;         // [points]
  size_t cap_vdw = 0, cap_shell = 0;
  bool desolv_ok = false;
  double* d_desolv = nullptr;         // [points] Lds.protein_desolv
  size_t cap_desolv = 0;
  std::vector<double> lradius;        // ligand atom radii (mmo_set_ligand_radii)
  double* d_lradius = nullptr;
  size_t cap_lradius = 0;
  void* d_dock = nullptr;             // docking tables and candidates
  size_t cap_dock = 0;
  int* d_clash = nullptr;             // per-pose scratch status
  size_t cap_clash = 0;

  // host-API staging
  char* h_in = nullptr;
  char* h_out = nullptr;
  char* d_in = nullptr;
  char* d_out = nullptr;
  size_t cap_in = 0, cap_out = 0;
};

namespace {

int fail(mmo_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(mmo_ctx* c, cudaError_t e, const char* what) {
  return fail(c, e == cudaErrorMemoryAllocation ? MMO_ENOMEM : MMO_ECUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

#define MMO_CK(call, what)                                \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
  } while (0)

void rebuild_table(mmo_ctx* ctx) {
  for (int a = 0; a < kNTypes; ++a)
    for (int b = 0; b < kNTypes; ++b) {
      double x2, d;
      pair_xd(ctx->ph.mixing, a, b, &x2, &d);
      ctx->tab.xd[a * kNTypes + b] = make_float2((float)x2, (float)d);
      // packed sweep: (X / r^2)^3 = D (x / r)^6 with X = D^(1/3) x^2
      ctx->tab4.v[a * kNTypes + b] = make_float4(
          (float)(std::cbrt(d) * x2), d > 0.0 ? (float)(1.0 / d) : 0.f, (float)x2, (float)d);
    }
}

// copy the packed pair table to the device (after in-flight work on the
// context's stream)
int upload_table(mmo_ctx* ctx) {
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before table upload");
  MMO_CK(cudaMemcpy(ctx->d_tab4, ctx->tab4.v, sizeof(ctx->tab4.v), cudaMemcpyHostToDevice),
         "pair table upload");
  return MMO_OK;
}

int grow(mmo_ctx* ctx, void** p, size_t* cap, size_t bytes, const char* what) {
  if (bytes <= *cap) return MMO_OK;
  ++ctx->epoch;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  bytes = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return cuda_fail(ctx, e, what);
  *cap = bytes;
  return MMO_OK;
}

int grow_host(mmo_ctx* ctx, char** h, char** d, size_t* cap, size_t bytes) {
  if (bytes <= *cap) return MMO_OK;
  if (*h) cudaFreeHost(*h);
  if (*d) cudaFree(*d);
  *h = *d = nullptr;
  *cap = 0;
  bytes = std::max<size_t>(bytes, 4096);
  MMO_CK(cudaHostAlloc((void**)h, bytes, cudaHostAllocDefault), "pinned staging");
  MMO_CK(cudaMalloc((void**)d, bytes), "device staging");
  *cap = bytes;
  return MMO_OK;
}

int ensure_scratch(mmo_ctx* ctx, int B, int L, int C, bool grad) {
  int r;
  const size_t n = (size_t)B * C * L;
  if ((r = grow(ctx, (void**)&ctx->scr.X, &ctx->capX, sizeof(float4) * 2 * (size_t)B * L, "X")))
    return r;
  if ((r = grow(ctx, (void**)&ctx->scr.Epart, &ctx->capE, sizeof(double) * n, "Epart"))) return r;
  if (grad && (r = grow(ctx, (void**)&ctx->scr.Gpart, &ctx->capG, sizeof(float4) * n, "Gpart")))
    return r;
  if (grad) {
    const size_t nrb = std::max(1, ctx->lig.nrb);
    if ((r = grow(ctx, (void**)&ctx->scr.Y, &ctx->capY, sizeof(float4) * 2 * (size_t)B * L, "Y")))
      return r;
    if ((r = grow(ctx, (void**)&ctx->scr.rec, &ctx->capR, sizeof(float4) * 3 * (size_t)B * nrb,
                  "torsion records")))
      return r;
    if ((r = grow(ctx, (void**)&ctx->scr.cen, &ctx->capI, sizeof(float4) * 2 * (size_t)B, "centroids")))
      return r;
  }
  ctx->scr.C = C;
  return MMO_OK;
}

// Host image of a ligand's device blob and what is needed to lay it out at
// any base address.
struct LigIn {
  std::vector<double> x, y, z, q;
  std::vector<int> type, bonds, goff, gat;
  std::vector<uint8_t> inter;
};

struct LigBlob {
  std::vector<char> host;
  std::vector<int> seg_type, seg_count;
  int n = 0, nrb = 0, np = 0, nbonds = 0, ngmask = 0, ngat = 0, nnb = 0;
  bool nested = false;
};

DevLigand ligand_at(const LigBlob& B, char* b, size_t* bytes) {
  size_t off = 0;
  DevLigand L{};
  const int n = B.n, nrb = B.nrb, np = B.np;
  L.L = n;
  L.nrb = nrb;
  L.npairs = np;
  L.nested = B.nested ? 1 : 0;
  L.ilh = n > 0 ? (float)(1.0 / n) : 0.f;
  L.ill = n > 0 ? (float)(1.0 / n - (double)L.ilh) : 0.f;
  L.ref = align_ptr<float4>(b, off, n);
  L.ref64 = align_ptr<double>(b, off, 3 * (size_t)n);
  L.ref2 = align_ptr<float2>(b, off, 3 * (size_t)n);
  L.type = align_ptr<int>(b, off, n);
  L.q = align_ptr<float>(b, off, n);
  L.bonds = align_ptr<int2>(b, off, B.nbonds);
  L.gmask = align_ptr<uint32_t>(b, off, B.ngmask);
  L.pair_ij = align_ptr<int2>(b, off, std::max(np, 1));
  L.pair_par = align_ptr<float4>(b, off, std::max(np, 1));
  L.amask = align_ptr<uint32_t>(b, off, n);
  L.tax = align_ptr<float2>(b, off, 6 * (size_t)std::max(nrb, 1));
  L.tord = align_ptr<int>(b, off, std::max(nrb, 1));
  L.ramask = align_ptr<uint32_t>(b, off, n);
  L.grp_off = align_ptr<int>(b, off, nrb + 1);
  L.grp_atoms = align_ptr<int>(b, off, std::max(B.ngat, 1));
  L.nb_off = align_ptr<int>(b, off, n + 1);
  L.nb_idx = align_ptr<int>(b, off, std::max(B.nnb, 1));
  L.nb_par = align_ptr<float4>(b, off, std::max(B.nnb, 1));
  L.seg_of_atom = align_ptr<int>(b, off, n);
  if (bytes) *bytes = off;
  return L;
}

void make_ligand_blob(int mixing, const LigIn& in, LigBlob* out) {
  const int n = (int)in.x.size(), nrb = (int)in.bonds.size() / 2;
  // interacting pairs (mol.ml:203-208), i < j, in the reference's loop order
  std::vector<int2> pij;
  std::vector<float4> ppar;
  std::vector<std::vector<std::pair<int, float4>>> nb(n);
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j) {
      if (!in.inter[(size_t)i * n + j]) continue;
      double x2, d;
      pair_xd(mixing, in.type[i], in.type[j], &x2, &d);
      const float4 par = make_float4((float)x2, (float)d, (float)(kElec * in.q[i] * in.q[j]), 0.f);
      pij.push_back(make_int2(i, j));
      ppar.push_back(par);
      nb[i].push_back({j, par});
      nb[j].push_back({i, par});
    }
  std::vector<int> nb_off(n + 1, 0), nb_idx;
  std::vector<float4> nb_par;
  for (int i = 0; i < n; ++i) {
    nb_off[i + 1] = nb_off[i] + (int)nb[i].size();
    for (auto& e : nb[i]) {
      nb_idx.push_back(e.first);
      nb_par.push_back(e.second);
    }
  }
  std::vector<float4> ref(n);
  for (int i = 0; i < n; ++i)
    ref[i] = make_float4((float)in.x[i], (float)in.y[i], (float)in.z[i], (float)in.q[i]);
  std::vector<uint32_t> gmask((size_t)std::max(nrb, 1) * kSlots, 0u);
  for (int t = 0; t < nrb; ++t)
    for (int k = in.goff[t]; k < in.goff[t + 1]; ++k) {
      const int a = in.gat[k];
      gmask[(size_t)t * kSlots + (a >> 5)] |= 1u << (a & 31);
    }
  std::vector<int2> bonds(std::max(nrb, 1));
  for (int t = 0; t < nrb; ++t) bonds[t] = make_int2(in.bonds[2 * t], in.bonds[2 * t + 1]);
  // nested groups: every two groups nested or disjoint; the axis of an inner
  // group inside its outer group or on the outer axis; no axis atom of one of
  // two disjoint groups inside the other
  auto has = [&](int t, int a) { return (gmask[(size_t)t * kSlots + (a >> 5)] >> (a & 31)) & 1u; };
  auto subset = [&](int t, int u) {  // G_t subset of G_u
    for (int w = 0; w < kSlots; ++w)
      if (gmask[(size_t)t * kSlots + w] & ~gmask[(size_t)u * kSlots + w]) return false;
    return true;
  };
  auto disjoint = [&](int t, int u) {
    for (int w = 0; w < kSlots; ++w)
      if (gmask[(size_t)t * kSlots + w] & gmask[(size_t)u * kSlots + w]) return false;
    return true;
  };
  bool nested = true;
  for (int t = 0; t < nrb && nested; ++t)
    for (int u = 0; u < nrb && nested; ++u) {
      if (t == u) continue;
      const int ul = bonds[u].x, ur = bonds[u].y, tl = bonds[t].x, tr = bonds[t].y;
      if (disjoint(t, u)) {
        nested = !has(t, ul) && !has(t, ur);
      } else if (subset(u, t)) {
        nested = (has(t, ul) || ul == tl || ul == tr) && (has(t, ur) || ur == tl || ur == tr);
      } else if (!subset(t, u)) {
        nested = false;
      }
    }
  const int np = (int)pij.size();
  LigBlob& B = *out;
  B.n = n;
  B.nrb = nrb;
  B.np = np;
  B.nbonds = (int)bonds.size();
  B.ngmask = (int)gmask.size();
  B.ngat = (int)in.gat.size();
  B.nnb = (int)nb_idx.size();
  B.nested = nested;
  size_t bytes = 0;
  ligand_at(B, nullptr, &bytes);
  B.host.assign(bytes, 0);
  std::vector<char>& host = B.host;
  DevLigand H = ligand_at(B, host.data(), nullptr);
  for (int t = 0; t < nrb; ++t)
    for (int k = in.goff[t]; k < in.goff[t + 1]; ++k)
      const_cast<uint32_t*>(H.amask)[in.gat[k]] |= 1u << t;
  // the torsions whose group holds exactly one atom of the pair, as bits in the
  // pair parameters' w (unused by the pair term)
  for (int p = 0; p < np; ++p) {
    const uint32_t cross = H.amask[pij[p].x] ^ H.amask[pij[p].y];
    memcpy(&ppar[p].w, &cross, sizeof cross);
  }
  memcpy((void*)H.grp_off, in.goff.data(), sizeof(int) * (nrb + 1));
  if (!in.gat.empty())
    memcpy((void*)H.grp_atoms, in.gat.data(), sizeof(int) * in.gat.size());
  memcpy((void*)H.ref, ref.data(), sizeof(float4) * n);
  for (int i = 0; i < n; ++i) {
    double* r64 = const_cast<double*>(H.ref64) + 3 * i;
    r64[0] = in.x[i];
    r64[1] = in.y[i];
    r64[2] = in.z[i];
    float2* r2 = const_cast<float2*>(H.ref2) + 3 * i;
    for (int d = 0; d < 3; ++d) {
      const float h = (float)r64[d];
      r2[d] = make_float2(h, (float)(r64[d] - (double)h));
    }
  }
  // per torsion: the unit axis and centre in the reference conformer, and the
  // order of the groups by size (inner groups first; the one-pose kernel's
  // rotation chains for nested groups)
  {
    std::vector<int> gsz(nrb);
    for (int t = 0; t < nrb; ++t) {
      gsz[t] = in.goff[t + 1] - in.goff[t];
      const int l = bonds[t].x, c = bonds[t].y;
      double a[3] = {in.x[c] - in.x[l], in.y[c] - in.y[l], in.z[c] - in.z[l]};
      const double len = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
      const double v[6] = {a[0] / len, a[1] / len, a[2] / len, in.x[c], in.y[c], in.z[c]};
      float2* tx = const_cast<float2*>(H.tax) + 6 * t;
      for (int d = 0; d < 6; ++d) {
        const float h = (float)v[d];
        tx[d] = make_float2(h, (float)(v[d] - (double)h));
      }
    }
    std::vector<int> ord(nrb);
    for (int t = 0; t < nrb; ++t) ord[t] = t;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return gsz[a] < gsz[b]; });
    if (nrb) memcpy((void*)H.tord, ord.data(), sizeof(int) * nrb);
    for (int k = 0; k < nrb; ++k)
      for (int g = in.goff[ord[k]]; g < in.goff[ord[k] + 1]; ++g)
        const_cast<uint32_t*>(H.ramask)[in.gat[g]] |= 1u << k;
  }
  memcpy((void*)H.type, in.type.data(), sizeof(int) * n);
  for (int i = 0; i < n; ++i) const_cast<float*>(H.q)[i] = (float)in.q[i];
  memcpy((void*)H.bonds, bonds.data(), sizeof(int2) * bonds.size());
  memcpy((void*)H.gmask, gmask.data(), sizeof(uint32_t) * gmask.size());
  if (np) {
    memcpy((void*)H.pair_ij, pij.data(), sizeof(int2) * np);
    memcpy((void*)H.pair_par, ppar.data(), sizeof(float4) * np);
    memcpy((void*)H.nb_idx, nb_idx.data(), sizeof(int) * nb_idx.size());
    memcpy((void*)H.nb_par, nb_par.data(), sizeof(float4) * nb_par.size());
  }
  memcpy((void*)H.nb_off, nb_off.data(), sizeof(int) * (n + 1));
  // type segments of the cut-off sweep: the ligand's types in ascending order
  B.seg_type.clear();
  B.seg_count.clear();
  for (int t = 0; t < kNTypes; ++t) {
    const int c = (int)std::count(in.type.begin(), in.type.end(), t);
    if (!c) continue;
    for (int i = 0; i < n; ++i)
      if (in.type[i] == t) const_cast<int*>(H.seg_of_atom)[i] = (int)B.seg_type.size();
    B.seg_type.push_back(t);
    B.seg_count.push_back(c);
  }
}

int upload_ligand(mmo_ctx* ctx) {
  LigIn in;
  in.x = ctx->lx;
  in.y = ctx->ly;
  in.z = ctx->lz;
  in.q = ctx->lq;
  in.type = ctx->ltype;
  in.bonds = ctx->lbonds;
  in.goff = ctx->lgoff;
  in.gat = ctx->lgatoms;
  in.inter = ctx->linter;
  LigBlob B;
  make_ligand_blob(ctx->ph.mixing, in, &B);
  ctx->lseg_type = B.seg_type;
  ctx->lseg_count = B.seg_count;
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before ligand upload");
  if (ctx->d_lig) cudaFree(ctx->d_lig);
  ctx->d_lig = nullptr;
  MMO_CK(cudaMalloc(&ctx->d_lig, B.host.size()), "ligand blob");
  MMO_CK(cudaMemcpy(ctx->d_lig, B.host.data(), B.host.size(), cudaMemcpyHostToDevice),
         "ligand upload");
  ctx->lig = ligand_at(B, reinterpret_cast<char*>(ctx->d_lig), nullptr);
  ctx->has_lig = true;
  ctx->one_ok = one_pose_smem(ctx->lig.L, ctx->lig.nrb) <= ctx->smem_optin;
  ++ctx->lig_version;
  ++ctx->epoch;
  return MMO_OK;
}

// Row index of a protein for the cut-off sweep: rows of a (y, z) grid of
// spacing h in (iz, iy) order, empty rows dropped, each row sorted by x; a
// flush point after the row where 256 atoms have accumulated.  Coordinates are
// in the device frame (origin subtracted).
// Grid type of each ligand atom: the grid type of the atom's element and
// charge (the reference types a ligand's atoms by its unique (anum, charge)
// pairs, Mol.get_typ / Mol.get_all_vdW_elec_types, src/mol.ml:295-304).  An
// atom without a grid type leaves MMO_F_GRID scoring refused (not an error of
// the upload that found it).
int grid_map(mmo_ctx* ctx) {
  ctx->grid_map_ok = false;
  if (!ctx->grid_ok) {
    ctx->grid_map_err = "no grids: call mmo_build_grids or mmo_load_grids first";
    return MMO_OK;
  }
  if (!ctx->has_lig) {
    ctx->grid_map_err = "no ligand: call mmo_set_ligand first";
    return MMO_OK;
  }
  const int L = (int)ctx->ltype.size(), nt = (int)ctx->grid_anum.size();
  std::vector<int> lt(L, -1);
  for (int a = 0; a < L; ++a) {
    for (int l = 0; l < nt && lt[a] < 0; ++l)
      if (type_of(ctx->grid_anum[l]) == ctx->ltype[a] && ctx->grid_q[l] == ctx->lq[a]) lt[a] = l;
    if (lt[a] < 0) {
      char buf[160];
      snprintf(buf, sizeof buf, "ligand atom %d (UFF row %d, charge %.9g) has no grid type", a,
               ctx->ltype[a], ctx->lq[a]);
      ctx->grid_map_err = buf;
      return MMO_OK;
    }
  }
  int r = grow(ctx, (void**)&ctx->d_grid_lt, &ctx->cap_grid_lt, sizeof(int) * L, "grid atom types");
  if (r) return r;
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before grid type upload");
  MMO_CK(cudaMemcpy(ctx->d_grid_lt, lt.data(), sizeof(int) * L, cudaMemcpyHostToDevice),
         "grid atom type upload");
  ctx->grid_lt = lt;
  ctx->grid_map_ok = true;
  ++ctx->epoch;
  return MMO_OK;
}

// checks of a grid spec shared by the build and the load; on success the
// context's lattice, types and value array are set (values not yet written)
int grid_take_spec(mmo_ctx* ctx, const char* who, const mmo_grid_spec* sp, bool build) {
  if (!sp) return fail(ctx, MMO_EINVAL, "%s: spec is NULL", who);
  if (!(sp->step > 0) || !std::isfinite(sp->step))
    return fail(ctx, MMO_EINVAL, "%s: step must be a positive finite number", who);
  const int n[3] = {sp->nx, sp->ny, sp->nz};
  for (int d = 0; d < 3; ++d)
    if (n[d] < 2 || n[d] > (1 << 14))
      return fail(ctx, MMO_EINVAL, "%s: lattice points per axis must be in 2..16384", who);
  const size_t pts = (size_t)n[0] * n[1] * n[2];
  if (pts > (size_t)INT32_MAX)
    return fail(ctx, MMO_EINVAL, "%s: more than 2^31 - 1 lattice points", who);
  if (sp->ntypes < 1 || sp->ntypes > kMaxLig || !sp->type_anum || !sp->type_q)
    return fail(ctx, MMO_EINVAL, "%s: ntypes must be in 1..%d with both type arrays", who,
                kMaxLig);
  for (int d = 0; d < 3; ++d)
    if (!std::isfinite(sp->origin[d]))
      return fail(ctx, MMO_EINVAL, "%s: non-finite origin", who);
  if (build) {
    if (std::isnan(sp->max_E)) return fail(ctx, MMO_EINVAL, "%s: max_E is NaN", who);
    if (std::isnan(sp->mask_radius) || (sp->mask_radius > 0 && !std::isfinite(sp->mask_radius)))
      return fail(ctx, MMO_EINVAL, "%s: mask_radius must be finite (or <= 0: no mask)", who);
    for (int d = 0; d < 3; ++d)
      if (sp->mask_radius > 0 && !std::isfinite(sp->mask_center[d]))
        return fail(ctx, MMO_EINVAL, "%s: non-finite mask centre", who);
  }
  for (int l = 0; l < sp->ntypes; ++l) {
    if (type_of(sp->type_anum[l]) < 0)
      return fail(ctx, MMO_EELEMENT, "%s: type %d: element %d not in the UFF table", who, l,
                  sp->type_anum[l]);
    if (!std::isfinite(sp->type_q[l]))
      return fail(ctx, MMO_EINVAL, "%s: type %d: non-finite charge", who, l);
  }
  const bool same_lattice = ctx->grid_ok && ctx->grid_step == sp->step &&
                            ctx->grid_n[0] == n[0] && ctx->grid_n[1] == n[1] &&
                            ctx->grid_n[2] == n[2] && ctx->grid_origin[0] == sp->origin[0] &&
                            ctx->grid_origin[1] == sp->origin[1] &&
                            ctx->grid_origin[2] == sp->origin[2];
  if (!same_lattice) {  // masks live on the grids' lattice
    ctx->masks_ok = false;
    ctx->desolv_ok = false;
  }
  ctx->grid_ok = false;
  ctx->grid_map_ok = false;
  ctx->grid_map_err = "no grids: call mmo_build_grids or mmo_load_grids first";
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before grid upload");
  int r = grow(ctx, (void**)&ctx->d_grid, &ctx->cap_grid, sizeof(float) * pts * sp->ntypes,
               "grid values");
  if (r) return r;
  ctx->grid_step = sp->step;
  for (int d = 0; d < 3; ++d) {
    ctx->grid_n[d] = n[d];
    ctx->grid_origin[d] = sp->origin[d];
  }
  ctx->grid_anum.assign(sp->type_anum, sp->type_anum + sp->ntypes);
  ctx->grid_q.assign(sp->type_q, sp->type_q + sp->ntypes);
  return MMO_OK;
}

// Ptable.vdW_radii (src/ptable.ml:41-53); NaN for elements it lacks
double vdw_radius(int anum) {
  switch (anum) {
    case 1: return 1.2;
    case 6: return 1.7;
    case 7: return 1.6;
    case 8: return 1.55;
    case 9: return 1.5;
    case 12: return 2.2;
    case 15: return 1.95;
    case 16: return 1.8;
    case 17: return 1.8;
    case 35: return 1.9;
    case 53: return 2.1;
    default: return NAN;
  }
}

// the lattice of the context's grids in the device frame
GridLook grid_look(const mmo_ctx* ctx) {
  GridLook g{};
  for (int d = 0; d < 3; ++d) g.o[d] = ctx->grid_origin[d] - ctx->origin[d];
  g.inv = 1.0 / ctx->grid_step;
  for (int d = 0; d < 3; ++d) {
    g.oh[d] = (float)g.o[d];
    g.ol[d] = (float)(g.o[d] - (double)g.oh[d]);
  }
  g.invh = (float)g.inv;
  g.invl = (float)(g.inv - (double)g.invh);
  g.nx = ctx->grid_n[0];
  g.ny = ctx->grid_n[1];
  g.nz = ctx->grid_n[2];
  return g;
}

struct RowIndex {
  std::vector<float4> atoms;    // [n][2]
  std::vector<int> perm;        // [n] row position -> input index
  std::vector<int> rs;          // [nrows + 1]
  std::vector<float4> rbox;     // [nrows]
  std::vector<int> flush_end;   // [nrows]
  std::vector<float4> pairs;    // [npairs][4] the cut-off sweep's layout (build_pairs)
  std::vector<int> prs;         // [nrows + 1] first pair of each row
  float lo[3], hi[3];           // bounding box (hi parts)
};

// The partners of a row's atoms: in x order, each atom not yet taken with the
// nearest of the next few untaken atoms of its row, so that the two atoms of a
// pair are close (a pair is swept when either atom is within reach of the
// entry group's box, and the farther one's work is then mostly wasted).  Only
// the row's last untaken atom can be left without one (b = -1).
std::vector<int2> pair_row(const RowIndex& R, int a0, int a1) {
  constexpr int kLook = 6;
  std::vector<int2> out;
  std::vector<char> taken(a1 - a0, 0);
  for (int a = a0; a < a1; ++a) {
    if (taken[a - a0]) continue;
    taken[a - a0] = 1;
    const float4 p = R.atoms[2 * (size_t)a];
    int best = -1, seen = 0;
    float bd = 0.f;
    for (int b = a + 1; b < a1 && seen < kLook; ++b) {
      if (taken[b - a0]) continue;
      ++seen;
      const float4 q = R.atoms[2 * (size_t)b];
      const float d = (p.x - q.x) * (p.x - q.x) + (p.y - q.y) * (p.y - q.y) + (p.z - q.z) * (p.z - q.z);
      if (best < 0 || d < bd) {
        best = b;
        bd = d;
      }
    }
    if (best >= 0) taken[best - a0] = 1;
    out.push_back(make_int2(a, best));
  }
  return out;
}

// The cut-off sweep's copy of a row index: the atoms of each row in pairs
// (pair_row), as four float4 per pair, negated coordinates so that the sweep
// adds them: (-x_hi a, -x_hi b, -y_hi a, -y_hi b), (-z_hi a, -z_hi b, Kq a, Kq b),
// the lo halves likewise, (-z_lo a, -z_lo b, type offset a, type offset b).  An
// atom without a partner gets a null one: itself again, with charge -0 (a zero
// charge of a real atom is +0) and the null type row (all zeros), whose terms
// are exact zeros.
void build_pairs(RowIndex* io) {
  RowIndex& R = *io;
  const int nrows = (int)R.rbox.size();
  R.prs.assign(nrows + 1, 0);
  R.pairs.clear();
  for (int r = 0; r < nrows; ++r) {
    R.prs[r] = (int)(R.pairs.size() / 4);
    for (const int2 ab : pair_row(R, R.rs[r], R.rs[r + 1])) {
      const int a = ab.x, b = ab.y;
      const bool real_b = b >= 0;
      const float4 ah = R.atoms[2 * (size_t)a], al = R.atoms[2 * (size_t)a + 1];
      const float4 bh = real_b ? R.atoms[2 * (size_t)b] : ah;
      const float4 bl = real_b ? R.atoms[2 * (size_t)b + 1] : al;
      const float wa = ah.w == 0.f ? 0.f : ah.w;
      const float wb = real_b ? (bh.w == 0.f ? 0.f : bh.w) : -0.f;
      float offb = bl.w;
      if (!real_b) {
        const int nb = kNullTypeRow * kNTypes * (int)sizeof(float4);
        memcpy(&offb, &nb, sizeof nb);
      }
      R.pairs.push_back(make_float4(-ah.x, -bh.x, -ah.y, -bh.y));
      R.pairs.push_back(make_float4(-ah.z, -bh.z, wa, wb));
      R.pairs.push_back(make_float4(-al.x, -bl.x, -al.y, -bl.y));
      R.pairs.push_back(make_float4(-al.z, -bl.z, al.w, offb));
    }
  }
  R.prs[nrows] = (int)(R.pairs.size() / 4);
}

void build_rows(int n, const double* px, const double* py, const double* pz, const float* pkq,
                const int* ptypes, double h, RowIndex* out) {
  RowIndex& R = *out;
  std::vector<float> fx(n), fy(n), fz(n);
  float* lo = R.lo;
  float* hi = R.hi;
  for (int d = 0; d < 3; ++d) {
    lo[d] = 1e30f;
    hi[d] = -1e30f;
  }
  for (int i = 0; i < n; ++i) {
    fx[i] = (float)px[i];
    fy[i] = (float)py[i];
    fz[i] = (float)pz[i];
    const float v[3] = {fx[i], fy[i], fz[i]};
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], v[d]);
      hi[d] = std::max(hi[d], v[d]);
    }
  }
  long ny = 0, nz = 0;
  for (;;) {
    ny = (long)std::floor((hi[1] - lo[1]) / h) + 1;
    nz = (long)std::floor((hi[2] - lo[2]) / h) + 1;
    if (ny * nz <= (1L << 20)) break;
    h *= 1.5;
  }
  std::vector<long> key(n);
  for (int i = 0; i < n; ++i) {
    const long iy = std::min(ny - 1, (long)std::floor((fy[i] - lo[1]) / h));
    const long iz = std::min(nz - 1, (long)std::floor((fz[i] - lo[2]) / h));
    key[i] = iz * ny + iy;
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int a, int b) {
    if (key[a] != key[b]) return key[a] < key[b];
    if (fx[a] != fx[b]) return fx[a] < fx[b];
    return a < b;
  });
  R.atoms.assign(2 * (size_t)n, make_float4(0.f, 0.f, 0.f, 0.f));
  R.perm = idx;
  R.rs.clear();
  R.rbox.clear();
  std::vector<int> rflush;
  int since = 0;
  for (int k = 0; k < n; ++k) {
    const int i = idx[k];
    split_store(&R.atoms[2 * (size_t)k], px[i], py[i], pz[i], pkq[i]);
    const int tb = ptypes[i] * kNTypes * (int)sizeof(float4);
    memcpy(&R.atoms[2 * (size_t)k + 1].w, &tb, sizeof tb);
    if (k == 0 || key[i] != key[idx[k - 1]]) {
      if (k) {
        since += k - R.rs.back();
        rflush.push_back(since >= kCullFlush);
        if (since >= kCullFlush) since = 0;
      }
      R.rs.push_back(k);
      R.rbox.push_back(make_float4(1e30f, -1e30f, 1e30f, -1e30f));
    }
    float4& bx = R.rbox.back();
    bx.x = std::min(bx.x, fy[i]);
    bx.y = std::max(bx.y, fy[i]);
    bx.z = std::min(bx.z, fz[i]);
    bx.w = std::max(bx.w, fz[i]);
  }
  rflush.push_back(1);
  R.rs.push_back(n);
  const int nrows = (int)R.rbox.size();
  // flag -> end of the flush block that holds the row
  R.flush_end.assign(nrows, nrows);
  for (int r = nrows - 1, end = nrows; r >= 0; --r) {
    if (rflush[r]) end = r + 1;
    R.flush_end[r] = end;
  }
  build_pairs(&R);
}

// pieces of a row index: consecutive rows of about piece_atoms atoms, as row
// boundaries [0 .. nrows]
std::vector<int> row_pieces(const std::vector<int>& rs, int piece_atoms) {
  const int nrows = (int)rs.size() - 1;
  std::vector<int> pr{0};
  int acc = 0;
  for (int r = 0; r < nrows; ++r) {
    acc += rs[r + 1] - rs[r];
    if (acc >= piece_atoms && r + 1 < nrows) {
      pr.push_back(r + 1);
      acc = 0;
    }
  }
  pr.push_back(nrows);
  return pr;
}

int build_cull(mmo_ctx* ctx) {
  ctx->cull_ok = false;
  ctx->cull_rows.clear();
  if (ctx->d_cull) {
    MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before row index upload");
    cudaFree(ctx->d_cull);
  }
  ctx->d_cull = nullptr;
  const int n = (int)ctx->pxs.size();
  if (n <= 0) return MMO_OK;
  RowIndex R;
  build_rows(n, ctx->pxs.data(), ctx->pys.data(), ctx->pzs.data(), ctx->pkq.data(),
             ctx->ptypes.data(), ctx->cull_h > 0 ? ctx->cull_h : 3.0, &R);
  const int nrows = (int)R.rbox.size();
  size_t off = 0;
  const size_t o_atoms = take(off, sizeof(float4) * R.atoms.size());
  const size_t o_rs = take(off, sizeof(int) * R.rs.size());
  const size_t o_box = take(off, sizeof(float4) * R.rbox.size());
  const size_t o_fl = take(off, sizeof(int) * R.flush_end.size());
  const size_t o_pairs = take(off, sizeof(float4) * R.pairs.size());
  const size_t o_prs = take(off, sizeof(int) * R.prs.size());
  std::vector<char> blob(off, 0);
  memcpy(blob.data() + o_atoms, R.atoms.data(), sizeof(float4) * R.atoms.size());
  memcpy(blob.data() + o_rs, R.rs.data(), sizeof(int) * R.rs.size());
  memcpy(blob.data() + o_box, R.rbox.data(), sizeof(float4) * R.rbox.size());
  memcpy(blob.data() + o_fl, R.flush_end.data(), sizeof(int) * R.flush_end.size());
  memcpy(blob.data() + o_pairs, R.pairs.data(), sizeof(float4) * R.pairs.size());
  memcpy(blob.data() + o_prs, R.prs.data(), sizeof(int) * R.prs.size());
  MMO_CK(cudaMalloc(&ctx->d_cull, off), "protein row index");
  MMO_CK(cudaMemcpy(ctx->d_cull, blob.data(), off, cudaMemcpyHostToDevice), "row index upload");
  DevCull c{};
  char* base = reinterpret_cast<char*>(ctx->d_cull);
  c.atoms = reinterpret_cast<const float4*>(base + o_atoms);
  c.row_start = reinterpret_cast<const int*>(base + o_rs);
  c.row_box = reinterpret_cast<const float4*>(base + o_box);
  c.row_flush = reinterpret_cast<const int*>(base + o_fl);
  c.pairs = reinterpret_cast<const float4*>(base + o_pairs);
  c.pair_start = reinterpret_cast<const int*>(base + o_prs);
  c.P = n;
  c.nrows = nrows;
  c.npairs = R.prs[nrows];
  // entry binning: a cube about the protein's box, 2 A beyond it
  float side = 0.f;
  for (int d = 0; d < 3; ++d) side = std::max(side, R.hi[d] - R.lo[d]);
  side += 4.0f;
  for (int d = 0; d < 3; ++d) c.glo[d] = 0.5f * (R.lo[d] + R.hi[d]) - 0.5f * side;
  c.ginv = (float)kCullGrid / side;
  ctx->cull = c;
  ctx->cull_rows = R.rs;
  ctx->cull_perm = R.perm;
  ctx->masks_ok = false;  // built on the old protein
  ctx->desolv_ok = false;
  ++ctx->cull_version;
  ++ctx->epoch;
  // the sweep can stage the whole protein and its index in shared memory, or
  // read them from global memory (any size)
  ctx->cull_ok = true;
  // (the default plan's 512 threads with 2 entries per lane)
  ctx->cull_fits = cull_smem_bytes(c.npairs, nrows, 512, false, 2) <= ctx->smem_optin;
  return MMO_OK;
}

PairPlan make_plan(mmo_ctx* ctx, int B, bool grad);

// automatic tile plan for the batched pair kernel, cached per input shape
PairPlan plan_for(mmo_ctx* ctx, int B, bool grad) {
  const long key[8] = {B, grad, ctx->prot.P, ctx->lig.L, ctx->tile_kp, ctx->tile_threads,
                       ctx->tile_chunks, ctx->ph.dielectric * 2 + ctx->ph.inter_form};
  const int g = grad ? 1 : 0;
  if (!std::equal(key, key + 8, ctx->plan_key[g])) {
    ctx->plan[g] = make_plan(ctx, B, grad);
    std::copy(key, key + 8, ctx->plan_key[g]);
  }
  return ctx->plan[g];
}

PairPlan make_plan(mmo_ctx* ctx, int B, bool grad) {
  PairPlan p{};
  p.kp = ctx->tile_kp ? ctx->tile_kp : (B >= 4096 ? 4 : (B >= 256 ? 2 : 1));
  p.threads = std::min(ctx->tile_threads ? ctx->tile_threads : 512, 512);
  const int P = ctx->prot.P, L = ctx->lig.L;
  const int nslices = (P + kSliceAtoms - 1) / kSliceAtoms;
  const int slice_len = (P + nslices - 1) / nslices;
  const int smem = slice_len * 32;
  int bps = pairs_batched_max_blocks(p.kp, p.threads, grad, ctx->ph, smem);
  if (bps < 1) bps = 1;
  p.blocks = ctx->sms * bps;
  const long W = (long)p.blocks * (p.threads / 32);
  const long npb = (B + 32L * p.kp - 1) / (32L * p.kp);
  int best = 1;
  if (ctx->tile_chunks) {
    best = std::max(1, ctx->tile_chunks / nslices);
  } else {
    double best_cost = 1e300;
    for (int c = 1; c <= 64; ++c) {
      const long items = npb * L * c;
      const long waves = (items + W - 1) / W;
      const long len = (slice_len + c - 1) / c;
      const double cost = (double)waves * (double)(len + 48);
      if (cost < best_cost - 1e-9) {
        best_cost = cost;
        best = c;
      }
    }
  }
  p.C = best * nslices;
  const long items = npb * L * best;
  const long need = (items + p.threads / 32 - 1) / (p.threads / 32);
  if (need < p.blocks) p.blocks = (int)std::max(1L, need);
  return p;
}

// the cut-off sweep serves the shifted form of batches of 2 or more poses
bool use_cull(const mmo_ctx* ctx, int B) {
  return ctx->cull_mode != 1 && ctx->cull_ok && ctx->ph.inter_form == 0 && B >= 2 &&
         !ctx->lseg_type.empty();
}

// plan of the cut-off sweep (pieces and their boxes, type segments, grid),
// cached per input
int cull_plan_for(mmo_ctx* ctx, int B, bool grad) {
  const long key[11] = {B, grad, ctx->prot_version, ctx->lig_version, ctx->cull_kp,
                        ctx->cull_piece, ctx->tile_threads, ctx->ph.dielectric,
                        ctx->cull_version, ctx->prot.P, ctx->cull_mode};
  const int g = grad ? 1 : 0;
  if (std::equal(key, key + 11, ctx->cplan_key[g])) {
    ctx->cs.npieces = ctx->npieces;
    return MMO_OK;
  }
  CullPlan p{};
  p.kp = ctx->cull_kp ? ctx->cull_kp : 2;
  p.threads = std::min(ctx->tile_threads ? ctx->tile_threads : 1024, cull_max_threads(p.kp));
  p.piece_atoms = ctx->cull_piece ? ctx->cull_piece : 256;
  p.global = (ctx->cull_mode == 2 ||
              cull_smem_bytes(ctx->cull.npairs, ctx->cull.nrows, p.threads, false, p.kp) >
                  ctx->smem_optin)
                 ? 1
                 : 0;
  if (ctx->piece_key[0] != ctx->cull_version || ctx->piece_key[1] != p.piece_atoms) {
    const std::vector<int> pr = row_pieces(ctx->cull_rows, p.piece_atoms);
    const int np = (int)pr.size() - 1;
    // each piece's bounding box over its atoms' FP32 coordinates (the
    // broad phase's test, conservative for the sweep's per-atom test)
    std::vector<float4> pb(2 * (size_t)np);
    for (int q = 0; q < np; ++q) {
      float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
      for (int k = ctx->cull_rows[pr[q]]; k < ctx->cull_rows[pr[q + 1]]; ++k) {
        const int i = ctx->cull_perm[k];
        const float v[3] = {(float)ctx->pxs[i], (float)ctx->pys[i], (float)ctx->pzs[i]};
        for (int d = 0; d < 3; ++d) {
          lo[d] = std::min(lo[d], v[d]);
          hi[d] = std::max(hi[d], v[d]);
        }
      }
      pb[2 * q] = make_float4(lo[0], lo[1], lo[2], 0.f);
      pb[2 * q + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
    int r = grow(ctx, (void**)&ctx->d_piece, &ctx->capPiece, sizeof(int) * pr.size(),
                 "piece table");
    if (r) return r;
    if ((r = grow(ctx, (void**)&ctx->d_pbox, &ctx->capPbox, sizeof(float4) * pb.size(),
                  "piece boxes")))
      return r;
    MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before piece table upload");
    MMO_CK(cudaMemcpy(ctx->d_piece, pr.data(), sizeof(int) * pr.size(), cudaMemcpyHostToDevice),
           "piece table upload");
    MMO_CK(cudaMemcpy(ctx->d_pbox, pb.data(), sizeof(float4) * pb.size(),
                      cudaMemcpyHostToDevice),
           "piece box upload");
    ctx->npieces = np;
    ctx->piece_key[0] = ctx->cull_version;
    ctx->piece_key[1] = p.piece_atoms;
  }
  const int npieces = ctx->npieces;
  CullSegs sg{};
  sg.nseg = (int)ctx->lseg_type.size();
  sg.G = 32 * p.kp;
  sg.off[0] = 0;
  for (int t = 0; t < sg.nseg; ++t) {
    sg.n[t] = B * ctx->lseg_count[t];
    sg.type[t] = ctx->lseg_type[t];
    sg.off[t + 1] = sg.off[t] + (sg.n[t] + sg.G - 1) / sg.G * sg.G;
  }
  p.smem = cull_smem_bytes(ctx->cull.npairs, ctx->cull.nrows, p.threads, p.global != 0, p.kp);
  const int bps =
      std::max(1, cull_max_blocks(p.kp, p.threads, grad, ctx->ph, p.smem, p.global != 0));
  p.blocks = ctx->sms * bps;
  const long items = (long)sg.off[sg.nseg] / sg.G * npieces;
  const long need = (items + p.threads / 32 - 1) / (p.threads / 32);
  if (need < p.blocks) p.blocks = (int)std::max(1L, need);
  ctx->cplan[g] = p;
  ctx->segs[g] = sg;
  ctx->cs.npieces = npieces;
  std::copy(key, key + 11, ctx->cplan_key[g]);
  return MMO_OK;
}

int ensure_cull_scratch(mmo_ctx* ctx, int B, int L, bool grad) {
  int r;
  const CullSegs& sg = ctx->segs[grad ? 1 : 0];
  const size_t slots = sg.off[sg.nseg], np = ctx->cs.npieces;
  CullScratch& c = ctx->cs;
  if ((r = grow(ctx, (void**)&c.hist, &ctx->capHist, sizeof(unsigned) * sg.nseg * kCullBins,
                "entry bins")))
    return r;
  if ((r = grow(ctx, (void**)&c.bin, &ctx->capBin, sizeof(int) * (size_t)B * L, "entry bin")))
    return r;
  if ((r = grow(ctx, (void**)&c.rank, &ctx->capRank, sizeof(int) * (size_t)B * L, "entry rank")))
    return r;
  if ((r = grow(ctx, (void**)&c.Xs, &ctx->capXs, sizeof(float4) * 2 * slots, "sorted entries")))
    return r;
  if ((r = grow(ctx, (void**)&c.order, &ctx->capOrd, sizeof(int) * slots, "slot order"))) return r;
  if ((r = grow(ctx, (void**)&c.Ep, &ctx->capEp, sizeof(double) * np * slots, "piece energies")))
    return r;
  if (grad &&
      (r = grow(ctx, (void**)&c.Gp, &ctx->capGp, sizeof(float4) * np * slots, "piece gradients")))
    return r;
  const size_t groups = slots / sg.G;
  if ((r = grow(ctx, (void**)&c.arrive, &ctx->capArr, sizeof(int) * groups, "group arrivals")))
    return r;
  if ((r = grow(ctx, (void**)&c.vis, &ctx->capVis, groups * np, "piece flags"))) return r;
  if ((r = grow(ctx, (void**)&c.gcount, &ctx->capGcnt, sizeof(int) * groups, "group counts")))
    return r;
  if ((r = grow(ctx, (void**)&c.glist, &ctx->capGlist, sizeof(int) * groups * np,
                "group piece lists")))
    return r;
  if ((r = grow(ctx, (void**)&c.items, &ctx->capItems, sizeof(int2) * groups * np,
                "sweep items")))
    return r;
  c.pbox = ctx->d_pbox;
  c.Eout = ctx->scr.Epart;
  c.Gout = grad ? ctx->scr.Gpart : nullptr;
  c.queue = ctx->d_queue;
  c.pairs = reinterpret_cast<unsigned long long*>(ctx->d_queue + 2);
  c.seg_of_atom = ctx->lig.seg_of_atom;
  c.piece_row = ctx->d_piece;
  c.slots = (int)slots;
  return MMO_OK;
}

int check_dev_err(mmo_ctx* ctx, int flag) {
  if (flag & kErrTimeout)
    return fail(ctx, MMO_ETIMEOUT, "a bounded device-side wait (protein staging) gave up");
  return MMO_OK;
}

// the one-pose path's per-CTA partials: npair CTAs of kOneChunk protein atoms,
// and the intra CTA's terms
int ensure_one_scratch(mmo_ctx* ctx, int L, bool grid) {
  OneScratch& o = ctx->one;
  o.npair = grid ? 1 : std::max(1, (ctx->prot.P + kOneChunk - 1) / kOneChunk);
  int r;
  if ((r = grow(ctx, (void**)&o.E, &ctx->capOneE, sizeof(float2) * (size_t)o.npair * L,
                "one-pose partials")))
    return r;
  if ((r = grow(ctx, (void**)&o.G, &ctx->capOneG, sizeof(float4) * (size_t)o.npair * L,
                "one-pose partials")))
    return r;
  if (!o.arrive) {
    MMO_CK(cudaMalloc((void**)&o.arrive, sizeof(unsigned)), "one-pose counter");
    MMO_CK(cudaMemset(o.arrive, 0, sizeof(unsigned)), "one-pose counter");
  }
  if (!o.intra) MMO_CK(cudaMalloc((void**)&o.intra, sizeof(float) * (kMaxTors + 2)), "one-pose intra terms");
  if (!o.gstat) MMO_CK(cudaMalloc((void**)&o.gstat, sizeof(int)), "one-pose grid status");
  return MMO_OK;
}

int score_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E,
                 float* d_grad, int* d_status, int* d_err, int zero_err, cudaStream_t st,
                 double* d_E_inter = nullptr) {
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  const bool use_grid = (flags & MMO_F_INTER) && (flags & MMO_F_GRID);
  if (use_grid && !ctx->grid_map_ok)
    return fail(ctx, MMO_ESTATE, "MMO_F_GRID: %s", ctx->grid_map_err.c_str());
  if ((flags & MMO_F_INTER) && !use_grid && ctx->prot.P <= 0)
    return fail(ctx, MMO_ESTATE, "no protein: call mmo_set_protein first");
  if (B < 0 || (B > 0 && (!d_dofs || !d_E || !d_status)))
    return fail(ctx, MMO_EINVAL, "bad batch arguments");
  if ((flags & MMO_F_GRAD) && !d_grad) return fail(ctx, MMO_EINVAL, "MMO_F_GRAD needs grad_out");
  if (B == 0) return MMO_OK;
  const bool grad = flags & MMO_F_GRAD;
  const bool inter = use_grid || ((flags & MMO_F_INTER) && ctx->prot.P > 0);
  const int L = ctx->lig.L;
  const bool cull = inter && !use_grid && use_cull(ctx, B);
  ctx->last_cull = cull;
  ctx->last_grad = grad ? 1 : 0;
  ctx->last_pairs = inter && !use_grid ? (double)B * L * ctx->prot.P : 0.0;
  ctx->last_pose_entries = 0;  // set below once the rebuild has written X
  // one pose with the inter term (pair sums or the grids): the fused one-launch
  // path (k_one_pose)
  const bool one = B == 1 && inter && ctx->one_ok;
  // rebuild (which bins the entries for the cut-off sweep) + finish, and the
  // sweep: scan, scatter, broad phase, sweep (or the grid lookup)
  ctx->last_launches = one ? 1 : 2 + (cull ? 4 : (inter ? 1 : 0));
  PairPlan plan{};
  int C = 1;
  int r;
  if (inter && !use_grid) {
    if (B == 1) {
      C = one ? 1 : std::max(1, (ctx->prot.P + 255) / 256);
    } else if (cull) {
      if ((r = cull_plan_for(ctx, B, grad))) return r;
    } else {
      plan = plan_for(ctx, B, grad);
      C = plan.C;
    }
  }
  if ((r = ensure_scratch(ctx, B, L, C, grad))) return r;
  if (cull && (r = ensure_cull_scratch(ctx, B, L, grad))) return r;
  if (one && (r = ensure_one_scratch(ctx, L, use_grid))) return r;
  PoseIO io{};
  io.dofs = d_dofs;
  io.E = d_E;
  io.grad = grad ? d_grad : nullptr;
  io.status = d_status;
  io.err = d_err;
  io.zero_err = zero_err;
  io.E_inter = d_E_inter;
  io.B = B;
  io.ox = ctx->origin_f[0];
  io.oy = ctx->origin_f[1];
  io.oz = ctx->origin_f[2];
  int fl = flags & (kFlagInter | kFlagIntra | kFlagGrad | kFlagRecenter);
  if (!inter) fl &= ~kFlagInter;
  ctx->scr.first_wait_polls = ctx->first_wait_polls;
  ctx->cs.first_wait_polls = ctx->first_wait_polls;
  const bool prof = ctx->profiling;
  auto mark = [&](int k) { return prof ? cudaEventRecord(ctx->ev[k], st) : cudaSuccess; };
  if (one) {  // the whole call is the "sweep" stage of the stage timings
    MMO_CK(mark(0), "event");
    MMO_CK(mark(1), "event");
    MMO_CK(mark(2), "event");
    int stage = 0;
    ctx->one.with_intra = ctx->lig.nested && (fl & kFlagIntra) ? 1 : 0;
    ctx->one.grid = use_grid ? 1 : 0;
    if (use_grid) {
      ctx->one.gl = grid_look(ctx);
      ctx->one.grids = ctx->d_grid;
      ctx->one.grid_lt = ctx->d_grid_lt;
    }
    const cudaError_t pending = cudaGetLastError();
    if (pending != cudaSuccess)
      return cuda_fail(ctx, pending, "error left by an earlier runtime call");
    const cudaError_t e1 =
        launch_one_pose(ctx->lig, ctx->prot, ctx->d_tab4, io, ctx->scr, ctx->one, fl, ctx->ph, st,
                        &stage);
    if (e1 != cudaSuccess) {
      char what[96];
      snprintf(what, sizeof what, "one-pose kernel (%s, %d bytes of shared memory)",
               stage == 1 ? "shared-memory attribute" : "launch",
               one_pose_smem(ctx->lig.L, ctx->lig.nrb));
      return cuda_fail(ctx, e1, what);
    }
    MMO_CK(mark(3), "event");
    if (prof) {
      MMO_CK(mark(4), "event");
      ctx->ev_valid = true;
    }
    return MMO_OK;
  }
  // with the cut-off sweep the rebuild also bins the entries (k_cull_bin's
  // work), into the histogram reset just before it
  Scratch sr = ctx->scr;
  if (cull) {
    sr.binning = 1;
    sr.hist = ctx->cs.hist;
    sr.bin = ctx->cs.bin;
    sr.rank = ctx->cs.rank;
    sr.seg_of_atom = ctx->cs.seg_of_atom;
    for (int d = 0; d < 3; ++d) sr.glo[d] = ctx->cull.glo[d];
    sr.ginv = ctx->cull.ginv;
  }
  MMO_CK(mark(0), "event");
  if (cull)
    MMO_CK(cudaMemsetAsync(ctx->cs.hist, 0,
                           sizeof(unsigned) * ctx->segs[grad ? 1 : 0].nseg * kCullBins, st),
           "entry bin reset");
  MMO_CK(launch_rebuild(ctx->lig, io, sr, fl, st), "rebuild kernel");
  ctx->last_pose_entries = B * L;
  MMO_CK(mark(1), "event");
  if (cull) {
    const CullSegs& sg = ctx->segs[grad ? 1 : 0];
    MMO_CK(launch_cull_sort(ctx->scr, ctx->lig.q, B, L, sg, ctx->cs, st),
           "entry sort kernels");
    MMO_CK(mark(2), "event");
    MMO_CK(launch_pairs_cull(ctx->cull, ctx->d_tab4, sg, ctx->cs, fl, ctx->ph, ctx->cplan[grad], d_err,
                             st),
           "cut-off pair kernel");
    MMO_CK(mark(3), "event");
  } else {
    MMO_CK(mark(2), "event");
    if (use_grid) {
      MMO_CK(launch_grid_inter(grid_look(ctx), ctx->scr.X, B * L, L, ctx->d_grid_lt, ctx->d_grid,
                               ctx->scr.Epart, grad ? ctx->scr.Gpart : nullptr, d_status, grad, st),
             "grid lookup kernel");
    } else if (inter) {
      if (B == 1) {
        MMO_CK(launch_pairs_plain(ctx->prot, ctx->tab, ctx->scr.X, ctx->lig.q, ctx->lig.type, L,
                                  C, ctx->scr.Epart, ctx->scr.Gpart, grad, ctx->ph, st),
               "plain pair kernel");
      } else {
        MMO_CK(launch_pairs_batched(ctx->prot, ctx->d_tab4, ctx->lig, ctx->scr, B, fl, ctx->ph,
                                    plan, d_err, st),
               "batched pair kernel");
      }
    }
    MMO_CK(mark(3), "event");
  }
  MMO_CK(launch_finish(ctx->lig, io, ctx->scr, fl, ctx->ph, st), "finish kernel");
  if (prof) {
    MMO_CK(mark(4), "event");
    ctx->ev_valid = true;
  }
  return MMO_OK;
}

}  // namespace

// ---- ragged batch of systems ----------------------------------------------
struct SysBatch {
  struct Sys {              // one user system
    LigIn lig;
    std::vector<double> px, py, pz;  // device frame
    std::vector<float> pkq;
    std::vector<int> ptype;
    float origin[3];
    int poses;
  };
  std::vector<Sys> in;
  std::vector<int> pose_off, dof_off;  // per user system, nsys + 1
  int B = 0, D = 0;                    // poses, DOF floats
  // static layout (rebuilt when the physics or the row spacing changes)
  long built_key[2] = {-1, -1};        // (mixing, row spacing in 1e-3 A)
  std::vector<SysInfo> info;           // virtual systems: user systems cut to sort-sized pose ranges
  std::vector<int> vuser;              // virtual -> user system
  std::vector<std::vector<int>> rows;  // per user system: row starts of its row index
  std::vector<std::vector<int>> prows;  // per user system: first pair of each row
  std::vector<int> row0, pair0;        // per user system: packed row and pair offsets
  std::vector<std::vector<int>> segcount, segtype;  // per user system: ligand type segments
  std::vector<int> Ls, nrbs;
  void* d_static = nullptr;
  size_t cap_static = 0;
  DevSystems dev{};
  int E = 0, R = 0, nrblk = 0, nfblk = 0, tpp = 4, Lmax = 1, nrbmax = 0;
  double pairs_all = 0.0;  // poses x ligand atoms x protein atoms over the batch
  // plan (pieces, groups, items) for (kp, piece atoms)
  long plan_key[3] = {-1, -1, -1};
  void* d_plan = nullptr;
  size_t cap_plan = 0;
  int kp = 2, threads = 256, blocks = 0, smem = 0, sort_smem = 0, slots = 0;
  long launch_key[2][4] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}};
  int lthreads[2] = {0, 0}, lsmem[2] = {0, 0}, lblocks[2] = {0, 0};
  long long npart = 0;
  long nvis = 0;
  // work buffers
  Scratch scr{};
  CullScratch cs{};
  size_t capX = 0, capE = 0, capG = 0, capY = 0, capR = 0, capC = 0, capXs = 0, capO = 0,
         capEp = 0, capGp = 0, capA = 0, capV = 0;
};

namespace {

void sys_free(SysBatch* b) {
  if (!b) return;
  cudaFree(b->d_static);
  cudaFree(b->d_plan);
  cudaFree(b->scr.X);
  cudaFree(b->scr.Epart);
  cudaFree(b->scr.Gpart);
  cudaFree(b->scr.Y);
  cudaFree(b->scr.rec);
  cudaFree(b->scr.cen);
  cudaFree(b->cs.Xs);
  cudaFree(b->cs.order);
  cudaFree(b->cs.Ep);
  cudaFree(b->cs.Gp);
  cudaFree(b->cs.arrive);
  cudaFree(b->cs.vis);
  delete b;
}

// static layout: ligand blobs, packed proteins in row-index order, virtual
// systems and the rebuild / finishing block tables
int sys_build_static(mmo_ctx* ctx, SysBatch* S) {
  const long key[2] = {ctx->ph.mixing, (long)std::llround((ctx->cull_h > 0 ? ctx->cull_h : 3.0) * 1e3)};
  if (S->built_key[0] == key[0] && S->built_key[1] == key[1] && S->d_static) return MMO_OK;
  const int ns = (int)S->in.size();
  std::vector<LigBlob> blobs(ns);
  std::vector<RowIndex> ri(ns);
  S->rows.assign(ns, {});
  S->pair0.assign(ns + 1, 0);
  S->prows.assign(ns, {});
  S->row0.assign(ns + 1, 0);
  S->segcount.assign(ns, {});
  S->segtype.assign(ns, {});
  S->Ls.assign(ns, 0);
  S->nrbs.assign(ns, 0);
  S->Lmax = 1;
  S->nrbmax = 0;
  const double h = ctx->cull_h > 0 ? ctx->cull_h : 3.0;
  for (int u = 0; u < ns; ++u) {
    const SysBatch::Sys& sy = S->in[u];
    make_ligand_blob(ctx->ph.mixing, sy.lig, &blobs[u]);
    const int np = (int)sy.px.size();
    if (np > 0) {
      build_rows(np, sy.px.data(), sy.py.data(), sy.pz.data(), sy.pkq.data(), sy.ptype.data(), h,
                 &ri[u]);
    } else {
      ri[u].rs = {0};
      ri[u].prs = {0};
      for (int d = 0; d < 3; ++d) ri[u].lo[d] = ri[u].hi[d] = 0.f;
    }
    S->rows[u] = ri[u].rs;
    S->prows[u] = ri[u].prs;
    S->pair0[u + 1] = S->pair0[u] + (int)(ri[u].pairs.size() / 4);
    S->row0[u + 1] = S->row0[u] + (int)ri[u].rbox.size();
    S->segcount[u] = blobs[u].seg_count;
    S->segtype[u] = blobs[u].seg_type;
    S->Ls[u] = blobs[u].n;
    S->nrbs[u] = blobs[u].nrb;
    S->Lmax = std::max(S->Lmax, blobs[u].n);
    S->nrbmax = std::max(S->nrbmax, blobs[u].nrb);
  }
  // virtual systems: pose ranges of at most kSysSortMax entries
  S->info.clear();
  S->vuser.clear();
  int pose = 0, ent = 0, rec = 0, dof = 0;
  for (int u = 0; u < ns; ++u) {
    const int L = S->Ls[u], nrb = S->nrbs[u];
    const int chunk = std::max(1, kSysSortMax / L);
    const RowIndex& R = ri[u];
    float side = 0.f;
    for (int d = 0; d < 3; ++d) side = std::max(side, R.hi[d] - R.lo[d]);
    side += 4.0f;
    for (int p0 = 0; p0 < S->in[u].poses; p0 += chunk) {
      SysInfo v{};
      v.poses = std::min(chunk, S->in[u].poses - p0);
      v.pose0 = pose;
      v.ent0 = ent;
      v.rec0 = rec;
      v.dof0 = dof;
      v.L = L;
      v.nrb = nrb;
      v.nseg = (int)S->segtype[u].size();
      v.ox = S->in[u].origin[0];
      v.oy = S->in[u].origin[1];
      v.oz = S->in[u].origin[2];
      for (int d = 0; d < 3; ++d) v.glo[d] = 0.5f * (R.lo[d] + R.hi[d]) - 0.5f * side;
      v.ginv = (float)kSysGrid / side;
      pose += v.poses;
      ent += v.poses * L;
      rec += v.poses * nrb;
      dof += v.poses * (6 + nrb);
      S->info.push_back(v);
      S->vuser.push_back(u);
    }
  }
  S->E = ent;
  S->R = rec;
  S->pairs_all = 0.0;
  for (int u = 0; u < ns; ++u)
    S->pairs_all += (double)S->in[u].poses * S->Ls[u] * (double)S->in[u].px.size();
  const int nv = (int)S->info.size();
  // threads per pose of the rebuild, as launch_rebuild chooses them
  int tpp = 32;
  while (tpp > 1 && (long)S->B * (tpp / 2) >= kRebuildThreadsInFlight) tpp /= 2;
  while (tpp < 32 && rebuild_smem(S->Lmax, S->nrbmax, 128 / tpp) > 200 * 1024) tpp *= 2;
  S->tpp = tpp;
  const int ppb = 128 / tpp;
  std::vector<SysBlk> rblk, fblk;
  for (int v = 0; v < nv; ++v) {
    for (int p0 = 0; p0 < S->info[v].poses; p0 += ppb)
      rblk.push_back({v, p0, std::min(ppb, S->info[v].poses - p0), 0});
    for (int p0 = 0; p0 < S->info[v].poses; p0 += 4)
      fblk.push_back({v, p0, std::min(4, S->info[v].poses - p0), 0});
  }
  S->nrblk = (int)rblk.size();
  S->nfblk = (int)fblk.size();
  // one device blob: ligands (256-aligned each), atoms, rows, boxes, flush ends, tables
  std::vector<size_t> lig_off(ns);
  size_t off = 0;
  for (int u = 0; u < ns; ++u) {
    off = (off + 255) & ~size_t(255);
    lig_off[u] = off;
    off += blobs[u].host.size();
  }
  const int NP = S->pair0[ns], nrows = S->row0[ns];
  const size_t o_atoms = take(off, sizeof(float4) * 4 * (size_t)std::max(NP, 1));
  const size_t o_rs = take(off, sizeof(int) * (nrows + 1));
  const size_t o_box = take(off, sizeof(float4) * std::max(nrows, 1));
  const size_t o_fe = take(off, sizeof(int) * std::max(nrows, 1));
  const size_t o_info = take(off, sizeof(SysInfo) * std::max(nv, 1));
  const size_t o_lig = take(off, sizeof(DevLigand) * std::max(nv, 1));
  const size_t o_rb = take(off, sizeof(SysBlk) * std::max(S->nrblk, 1));
  const size_t o_fb = take(off, sizeof(SysBlk) * std::max(S->nfblk, 1));
  std::vector<char> host(off, 0);
  for (int u = 0; u < ns; ++u)
    memcpy(host.data() + lig_off[u], blobs[u].host.data(), blobs[u].host.size());
  float4* atoms = reinterpret_cast<float4*>(host.data() + o_atoms);
  int* rs = reinterpret_cast<int*>(host.data() + o_rs);
  float4* box = reinterpret_cast<float4*>(host.data() + o_box);
  int* fe = reinterpret_cast<int*>(host.data() + o_fe);
  for (int u = 0; u < ns; ++u) {
    const RowIndex& R = ri[u];
    if (!R.pairs.empty())
      memcpy(atoms + 4 * (size_t)S->pair0[u], R.pairs.data(), sizeof(float4) * R.pairs.size());
    const int nr = (int)R.rbox.size();
    for (int r = 0; r < nr; ++r) {
      rs[S->row0[u] + r] = S->pair0[u] + R.prs[r];
      box[S->row0[u] + r] = R.rbox[r];
      fe[S->row0[u] + r] = S->row0[u] + R.flush_end[r];
    }
  }
  rs[nrows] = NP;
  memcpy(host.data() + o_info, S->info.data(), sizeof(SysInfo) * nv);
  memcpy(host.data() + o_rb, rblk.data(), sizeof(SysBlk) * rblk.size());
  memcpy(host.data() + o_fb, fblk.data(), sizeof(SysBlk) * fblk.size());
  int r;
  if ((r = grow(ctx, &S->d_static, &S->cap_static, off, "system batch"))) return r;
  char* d = static_cast<char*>(S->d_static);
  DevLigand* ligs = reinterpret_cast<DevLigand*>(host.data() + o_lig);
  for (int v = 0; v < nv; ++v) {
    const int u = S->vuser[v];
    ligs[v] = ligand_at(blobs[u], d + lig_off[u], nullptr);
  }
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before system batch upload");
  MMO_CK(cudaMemcpy(d, host.data(), off, cudaMemcpyHostToDevice), "system batch upload");
  DevSystems& D = S->dev;
  D = DevSystems{};
  D.info = reinterpret_cast<const SysInfo*>(d + o_info);
  D.lig = reinterpret_cast<const DevLigand*>(d + o_lig);
  D.rblk = reinterpret_cast<const SysBlk*>(d + o_rb);
  D.fblk = reinterpret_cast<const SysBlk*>(d + o_fb);
  D.pairs = reinterpret_cast<const float4*>(d + o_atoms);
  D.row_start = reinterpret_cast<const int*>(d + o_rs);
  D.row_box = reinterpret_cast<const float4*>(d + o_box);
  D.flush_end = reinterpret_cast<const int*>(d + o_fe);
  D.nsys = nv;
  D.B = S->B;
  D.Lmax = S->Lmax;
  D.nrbmax = S->nrbmax;
  S->built_key[0] = key[0];
  S->built_key[1] = key[1];
  S->plan_key[0] = -1;  // the plan's tables refer to this layout
  ++ctx->epoch;
  return MMO_OK;
}

// plan: protein pieces, entry groups, segment slots, work items
int sys_build_plan(mmo_ctx* ctx, SysBatch* S, bool grad) {
  const int kp = ctx->cull_kp ? ctx->cull_kp : 2;
  const int piece_atoms = ctx->cull_piece ? ctx->cull_piece : 256;
  const long key[3] = {kp, piece_atoms, S->built_key[1]};
  const int G = 32 * kp;
  if (!(S->plan_key[0] == key[0] && S->plan_key[1] == key[1] && S->plan_key[2] == key[2])) {
    const int ns = (int)S->in.size(), nv = (int)S->info.size();
    std::vector<int4> pieces;
    std::vector<int> piece0(ns), npieces(ns);
    int amax = 1, rmax = 1;
    for (int u = 0; u < ns; ++u) {
      piece0[u] = (int)pieces.size();
      const std::vector<int>& rs = S->rows[u];
      const int nr = (int)rs.size() - 1;
      if (nr <= 0) {  // no protein: one empty piece, so that the groups still close
        pieces.push_back(make_int4(S->pair0[u], S->pair0[u], S->row0[u], S->row0[u]));
      } else {
        const std::vector<int> pr = row_pieces(rs, piece_atoms);
        const std::vector<int>& prs = S->prows[u];
        for (size_t k = 0; k + 1 < pr.size(); ++k) {
          const int a0 = S->pair0[u] + prs[pr[k]], a1 = S->pair0[u] + prs[pr[k + 1]];
          pieces.push_back(make_int4(a0, a1, S->row0[u] + pr[k], S->row0[u] + pr[k + 1]));
          amax = std::max(amax, a1 - a0);
          rmax = std::max(rmax, pr[k + 1] - pr[k]);
        }
      }
      npieces[u] = (int)pieces.size() - piece0[u];
    }
    std::vector<SysGroup> groups;
    std::vector<int> seg_slot;
    std::vector<int2> items;
    int slot = 0;
    long long part = 0;
    long vis = 0;
    for (int v = 0; v < nv; ++v) {
      SysInfo& inf = S->info[v];
      const int u = S->vuser[v];
      inf.piece0 = piece0[u];
      inf.npieces = npieces[u];
      inf.seg0 = (int)seg_slot.size();
      inf.group0 = (int)groups.size();
      for (int t = 0; t < inf.nseg; ++t) {
        const int n = inf.poses * S->segcount[u][t];
        seg_slot.push_back(slot);
        for (int g0 = 0; g0 < n; g0 += G)
          groups.push_back({slot + g0, slot + n, S->segtype[u][t], v});
        slot += (n + G - 1) / G * G;
      }
      inf.ngroups = (int)groups.size() - inf.group0;
      inf.vis0 = (int)vis;
      inf.part0 = part;
      vis += (long)inf.ngroups * inf.npieces;
      part += (long long)inf.ngroups * inf.npieces * G;
      if (inf.ngroups > 0)
        for (int k = 0; k < inf.npieces; ++k) items.push_back(make_int2(v, inf.piece0 + k));
    }
    size_t off = 0;
    const size_t o_info = take(off, sizeof(SysInfo) * std::max(nv, 1));
    const size_t o_piece = take(off, sizeof(int4) * std::max<size_t>(pieces.size(), 1));
    const size_t o_item = take(off, sizeof(int2) * std::max<size_t>(items.size(), 1));
    const size_t o_group = take(off, sizeof(SysGroup) * std::max<size_t>(groups.size(), 1));
    const size_t o_seg = take(off, sizeof(int) * std::max<size_t>(seg_slot.size(), 1));
    std::vector<char> host(off, 0);
    memcpy(host.data() + o_info, S->info.data(), sizeof(SysInfo) * nv);
    memcpy(host.data() + o_piece, pieces.data(), sizeof(int4) * pieces.size());
    memcpy(host.data() + o_item, items.data(), sizeof(int2) * items.size());
    memcpy(host.data() + o_group, groups.data(), sizeof(SysGroup) * groups.size());
    memcpy(host.data() + o_seg, seg_slot.data(), sizeof(int) * seg_slot.size());
    int r;
    if ((r = grow(ctx, &S->d_plan, &S->cap_plan, off, "system batch plan"))) return r;
    char* d = static_cast<char*>(S->d_plan);
    MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before plan upload");
    MMO_CK(cudaMemcpy(d, host.data(), off, cudaMemcpyHostToDevice), "plan upload");
    DevSystems& D = S->dev;
    D.info = reinterpret_cast<const SysInfo*>(d + o_info);  // the plan's copy holds the piece fields
    D.piece = reinterpret_cast<const int4*>(d + o_piece);
    D.item = reinterpret_cast<const int2*>(d + o_item);
    D.group = reinterpret_cast<const SysGroup*>(d + o_group);
    D.seg_slot = reinterpret_cast<const int*>(d + o_seg);
    D.nitems = (int)items.size();
    D.ngroups = (int)groups.size();
    D.G = G;
    D.piece_pairs_max = amax;
    D.piece_rows_max = rmax;
    S->kp = kp;
    S->slots = slot;
    S->npart = part;
    S->nvis = vis;
    int sort_smem = 0;
    for (const SysInfo& v : S->info)
      sort_smem = std::max(sort_smem, (int)sizeof(unsigned) * (v.nseg * kSysCells + v.poses * v.L));
    S->sort_smem = std::max(sort_smem, 16);
    std::copy(key, key + 3, S->plan_key);
    ++ctx->epoch;
  }
  // launch shape, per gradient flag (occupancy queried once per shape)
  const int g = grad ? 1 : 0;
  const int maxt = cull_max_threads(S->kp);
  const int threads = std::min(ctx->tile_threads ? ctx->tile_threads : 256, maxt);
  const long lkey[4] = {S->plan_key[0], S->plan_key[1], threads,
                        ctx->ph.dielectric * 2 + ctx->ph.inter_form};
  if (!std::equal(lkey, lkey + 4, S->launch_key[g])) {
    const int smem = sys_pairs_smem(S->dev.piece_pairs_max, S->dev.piece_rows_max, threads);
    const int bps = std::max(1, sys_pairs_max_blocks(S->kp, threads, grad, ctx->ph, smem));
    S->lthreads[g] = threads;
    S->lsmem[g] = smem;
    S->lblocks[g] = ctx->sms * bps;
    std::copy(lkey, lkey + 4, S->launch_key[g]);
  }
  S->threads = S->lthreads[g];
  S->smem = S->lsmem[g];
  S->blocks = S->lblocks[g];
  return MMO_OK;
}

int sys_scratch(mmo_ctx* ctx, SysBatch* S, bool grad, bool inter) {
  int r;
  const size_t E = std::max(S->E, 1), B = std::max(S->B, 1), R = std::max(S->R, 1);
  if ((r = grow(ctx, (void**)&S->scr.X, &S->capX, sizeof(float4) * 2 * E, "X"))) return r;
  if ((r = grow(ctx, (void**)&S->scr.Epart, &S->capE, sizeof(double) * E, "Epart"))) return r;
  if (grad) {
    if ((r = grow(ctx, (void**)&S->scr.Gpart, &S->capG, sizeof(float4) * E, "Gpart"))) return r;
    if ((r = grow(ctx, (void**)&S->scr.Y, &S->capY, sizeof(float4) * 2 * E, "Y"))) return r;
    if ((r = grow(ctx, (void**)&S->scr.rec, &S->capR, sizeof(float4) * 3 * R, "records"))) return r;
    if ((r = grow(ctx, (void**)&S->scr.cen, &S->capC, sizeof(float4) * 2 * B, "centroids"))) return r;
  }
  S->scr.C = 1;
  if (inter) {
    CullScratch& c = S->cs;
    const size_t slots = std::max(S->slots, 1);
    if ((r = grow(ctx, (void**)&c.Xs, &S->capXs, sizeof(float4) * 2 * slots, "sorted entries")))
      return r;
    if ((r = grow(ctx, (void**)&c.order, &S->capO, sizeof(int) * slots, "slot order"))) return r;
    const size_t np = (size_t)std::max<long long>(S->npart, 1);
    if ((r = grow(ctx, (void**)&c.Ep, &S->capEp, sizeof(double) * np, "piece energies"))) return r;
    if (grad && (r = grow(ctx, (void**)&c.Gp, &S->capGp, sizeof(float4) * np, "piece gradients")))
      return r;
    if ((r = grow(ctx, (void**)&c.arrive, &S->capA, sizeof(int) * std::max(S->dev.ngroups, 1),
                  "group arrivals")))
      return r;
    if ((r = grow(ctx, (void**)&c.vis, &S->capV, (size_t)std::max(S->nvis, 1L), "piece flags")))
      return r;
    c.queue = ctx->d_queue;
    c.pairs = reinterpret_cast<unsigned long long*>(ctx->d_queue + 2);
    c.Eout = S->scr.Epart;
    c.Gout = S->scr.Gpart;
  }
  return MMO_OK;
}

int score_systems(mmo_ctx* ctx, const float* d_dofs, int flags, double* d_E, float* d_grad,
                  int* d_status, int* d_err, cudaStream_t st) {
  SysBatch* S = ctx->sys;
  if (!S) return fail(ctx, MMO_ESTATE, "no systems: call mmo_set_systems first");
  if (S->B > 0 && (!d_dofs || !d_E || !d_status))
    return fail(ctx, MMO_EINVAL, "mmo_score_systems: bad arguments");
  if ((flags & MMO_F_GRAD) && S->B > 0 && !d_grad)
    return fail(ctx, MMO_EINVAL, "MMO_F_GRAD needs grad_out");
  if (S->B == 0) return MMO_OK;
  const bool grad = flags & MMO_F_GRAD;
  const bool inter = flags & MMO_F_INTER;
  int r;
  if ((r = sys_build_static(ctx, S))) return r;
  if (inter && (r = sys_build_plan(ctx, S, grad))) return r;
  if ((r = sys_scratch(ctx, S, grad, inter))) return r;
  PoseIO io{};
  io.dofs = d_dofs;
  io.E = d_E;
  io.grad = grad ? d_grad : nullptr;
  io.status = d_status;
  io.err = d_err;
  io.B = S->B;
  const int fl = flags & (kFlagInter | kFlagIntra | kFlagGrad | kFlagRecenter);
  ctx->last_cull = inter;  // the sweep counts its pair evaluations
  ctx->last_grad = grad ? 1 : 0;
  ctx->last_pairs = inter ? S->pairs_all : 0.0;
  ctx->last_launches = 2 + (inter ? 2 : 0);
  const bool prof = ctx->profiling;
  auto mark = [&](int k) { return prof ? cudaEventRecord(ctx->ev[k], st) : cudaSuccess; };
  MMO_CK(mark(0), "event");
  MMO_CK(launch_sys_rebuild(S->dev, S->nrblk, S->tpp, io, S->scr, fl, st), "system rebuild kernel");
  MMO_CK(mark(1), "event");
  if (inter) {
    MMO_CK(cudaMemsetAsync(ctx->d_queue, 0, 16, st), "work counter reset");
    MMO_CK(launch_sys_sort(S->dev, S->scr, S->cs, S->sort_smem, st), "system sort kernel");
    MMO_CK(mark(2), "event");
    S->cs.first_wait_polls = ctx->first_wait_polls;
    MMO_CK(launch_sys_pairs(S->dev, ctx->d_tab4, S->cs, S->kp, S->threads, S->blocks, S->smem,
                            fl, ctx->ph, d_err, st),
           "system pair kernel");
  } else {
    MMO_CK(mark(2), "event");
  }
  MMO_CK(mark(3), "event");
  MMO_CK(launch_sys_finish(S->dev, S->nfblk, io, S->scr, fl, ctx->ph, st), "system finish kernel");
  if (prof) {
    MMO_CK(mark(4), "event");
    ctx->ev_valid = true;
  }
  return MMO_OK;
}

}  // namespace

extern "C" {

const char* mmo_last_error(const mmo_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_err; }

int mmo_ctx_create(int device, mmo_ctx** out) {
  if (!out) return MMO_EINVAL;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || device < 0 || device >= ndev) {
    snprintf(g_create_err, sizeof g_create_err, "no CUDA device %d (%s)", device,
             e != cudaSuccess ? cudaGetErrorString(e) : "out of range");
    return e != cudaSuccess ? MMO_ECUDA : MMO_EINVAL;
  }
  mmo_ctx* ctx = new (std::nothrow) mmo_ctx();
  if (!ctx) return MMO_ENOMEM;
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device)) !=
          cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc((void**)&ctx->d_err, sizeof(int))) != cudaSuccess ||
      (e = cudaMemset(ctx->d_err, 0, sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc((void**)&ctx->d_tab4, sizeof(ctx->tab4.v))) != cudaSuccess ||
      (e = cudaMalloc((void**)&ctx->d_queue, 16)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&ctx->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                  device)) != cudaSuccess) {
    snprintf(g_create_err, sizeof g_create_err, "context set-up: %s", cudaGetErrorString(e));
    delete ctx;
    return e == cudaErrorMemoryAllocation ? MMO_ENOMEM : MMO_ECUDA;
  }
  rebuild_table(ctx);
  if (upload_table(ctx) != MMO_OK) {
    snprintf(g_create_err, sizeof g_create_err, "context set-up: %s", ctx->err.c_str());
    mmo_ctx_destroy(ctx);
    return MMO_ECUDA;
  }
  *out = ctx;
  return MMO_OK;
}

int mmo_ctx_destroy(mmo_ctx* ctx) {
  if (!ctx) return MMO_EINVAL;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_prot);
  cudaFree(ctx->d_lig);
  cudaFree(ctx->scr.X);
  cudaFree(ctx->scr.Epart);
  cudaFree(ctx->scr.Gpart);
  cudaFree(ctx->scr.Y);
  cudaFree(ctx->scr.rec);
  cudaFree(ctx->scr.cen);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  cudaFree(ctx->d_err);
  cudaFree(ctx->d_tab4);
  cudaFree(ctx->d_queue);
  cudaFree(ctx->d_cull);
  cudaFree(ctx->d_piece);
  cudaFree(ctx->d_pbox);
  cudaFree(ctx->one.E);
  cudaFree(ctx->one.G);
  cudaFree(ctx->one.arrive);
  cudaFree(ctx->one.intra);
  cudaFree(ctx->one.gstat);
  cudaFree(ctx->d_plain_arrive);
  cudaFree(ctx->cs.gcount);
  cudaFree(ctx->cs.glist);
  cudaFree(ctx->cs.items);
  cudaFree(ctx->cs.hist);
  cudaFree(ctx->cs.bin);
  cudaFree(ctx->cs.rank);
  cudaFree(ctx->cs.Xs);
  cudaFree(ctx->cs.order);
  cudaFree(ctx->cs.Ep);
  cudaFree(ctx->cs.Gp);
  cudaFree(ctx->cs.arrive);
  cudaFree(ctx->cs.vis);
  cudaFree(ctx->d_mc);
  cudaFree(ctx->d_grid);
  cudaFree(ctx->d_grid_lt);
  cudaFree(ctx->d_vdw);
  cudaFree(ctx->d_vcell);
  cudaFree(ctx->d_shell);
  cudaFree(ctx->d_desolv);
  cudaFree(ctx->d_lradius);
  cudaFree(ctx->d_dock);
  cudaFree(ctx->d_clash);
  sys_free(ctx->sys);
  if (ctx->mc_exec) cudaGraphExecDestroy(ctx->mc_exec);
  for (auto& e : ctx->mc_ev)
    if (e) cudaEventDestroy(e);
  cudaFree(ctx->d_in);
  cudaFree(ctx->d_out);
  if (ctx->h_in) cudaFreeHost(ctx->h_in);
  if (ctx->h_out) cudaFreeHost(ctx->h_out);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MMO_OK;
}

int mmo_set_physics(mmo_ctx* ctx, int dielectric, int mixing, int inter_form, int intra_form) {
  if (!ctx) return MMO_EINVAL;
  if ((dielectric | mixing | inter_form | intra_form) & ~1)
    return fail(ctx, MMO_EINVAL, "physics switches are 0 or 1");
  ++ctx->epoch;
  ctx->ph = Physics{dielectric, mixing, inter_form, intra_form};
  rebuild_table(ctx);
  if (int r = upload_table(ctx)) return r;
  if (ctx->has_lig) return upload_ligand(ctx);
  return MMO_OK;
}

int mmo_set_tiles(mmo_ctx* ctx, int kp, int threads, int chunks) {
  if (!ctx) return MMO_EINVAL;
  if (!(kp == 0 || kp == 1 || kp == 2 || kp == 4) ||
      !(threads == 0 || threads == 256 || threads == 512 || threads == 768 || threads == 1024) ||
      chunks < 0 || chunks > 4096)
    return fail(ctx, MMO_EINVAL,
                "tiles: poses_per_lane in {0,1,2,4}, threads in {0,256,512,768,1024}");
  ctx->tile_kp = kp;
  ctx->tile_threads = threads;
  ctx->tile_chunks = chunks;
  ++ctx->epoch;
  return MMO_OK;
}

int mmo_set_cull(mmo_ctx* ctx, int mode, double row_spacing, int piece_atoms,
                 int entries_per_lane) {
  if (!ctx) return MMO_EINVAL;
  if (mode < 0 || mode > 2 || piece_atoms < 0 || piece_atoms > (1 << 20) ||
      !(entries_per_lane == 0 || entries_per_lane == 1 || entries_per_lane == 2 ||
        entries_per_lane == 4) ||
      !std::isfinite(row_spacing) || (row_spacing > 0 && (row_spacing < 0.25 || row_spacing > 64)))
    return fail(ctx, MMO_EINVAL,
                "cull: mode 0, 1 or 2, row spacing in [0.25, 64] A (<= 0: default), piece atoms "
                ">= 0, entries per lane in {0,1,2,4}");
  ctx->cull_mode = mode;
  ctx->cull_piece = piece_atoms;
  ctx->cull_kp = entries_per_lane;
  ++ctx->epoch;
  const double h = row_spacing > 0 ? row_spacing : 3.0;
  if (h != ctx->cull_h) {
    ctx->cull_h = h;
    MMO_CK(cudaSetDevice(ctx->device), "set device");
    return build_cull(ctx);
  }
  return MMO_OK;
}

int mmo_device_sms(const mmo_ctx* ctx, int* out) {
  if (!ctx || !out) return MMO_EINVAL;
  *out = ctx->sms;
  return MMO_OK;
}

int mmo_set_protein(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                    const double* q, const int* anum) {
  if (!ctx) return MMO_EINVAL;
  if (n < 0 || (n > 0 && (!xs || !ys || !zs || !q || !anum)))
    return fail(ctx, MMO_EINVAL, "mmo_set_protein: bad arguments");
  std::vector<int> type(n);
  double o[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    type[i] = type_of(anum[i]);
    if (type[i] < 0)
      return fail(ctx, MMO_EELEMENT, "protein atom %d: element %d not in the UFF table", i, anum[i]);
    if (!std::isfinite(xs[i]) || !std::isfinite(ys[i]) || !std::isfinite(zs[i]) ||
        !std::isfinite(q[i]))
      return fail(ctx, MMO_EINVAL, "protein atom %d: non-finite coordinate or charge", i);
    o[0] += xs[i];
    o[1] += ys[i];
    o[2] += zs[i];
  }
  if (n > 0)
    for (int d = 0; d < 3; ++d) o[d] /= n;
  float of[3] = {(float)o[0], (float)o[1], (float)o[2]};
  // stable sort by type: runs of constant pair parameters
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return type[a] < type[b]; });
  std::vector<float4> atoms(2 * (size_t)std::max(n, 1));
  std::vector<uint8_t> ptype(std::max(n, 16), 0);
  std::vector<int> rstart, rtype;
  DevProtein P{};
  P.P = n;
  for (int k = 0; k < n; ++k) {
    const int i = idx[k];
    split_store(&atoms[2 * (size_t)k], xs[i] - (double)of[0], ys[i] - (double)of[1],
                zs[i] - (double)of[2], (float)(kElec * q[i]));
    ptype[k] = (uint8_t)type[i];
    if (k == 0 || type[i] != type[idx[k - 1]]) {
      rstart.push_back(k);
      rtype.push_back(type[i]);
    }
  }
  P.nruns = (int)rtype.size();
  rstart.push_back(n);
  std::vector<int> runs(2 * kNTypes + 1, 0);
  std::copy(rstart.begin(), rstart.end(), runs.begin());
  std::copy(rtype.begin(), rtype.end(), runs.begin() + P.nruns + 1);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before protein upload");
  if (ctx->d_prot) cudaFree(ctx->d_prot);
  ctx->d_prot = nullptr;
  size_t off = 0;
  const size_t o_atoms = take(off, sizeof(float4) * atoms.size());
  const size_t o_type = take(off, ptype.size());
  const size_t o_runs = take(off, sizeof(int) * runs.size());
  std::vector<char> blob(off, 0);
  memcpy(blob.data() + o_atoms, atoms.data(), sizeof(float4) * atoms.size());
  memcpy(blob.data() + o_type, ptype.data(), ptype.size());
  memcpy(blob.data() + o_runs, runs.data(), sizeof(int) * runs.size());
  MMO_CK(cudaMalloc(&ctx->d_prot, off), "protein");
  MMO_CK(cudaMemcpy(ctx->d_prot, blob.data(), off, cudaMemcpyHostToDevice), "protein upload");
  P.atoms = reinterpret_cast<const float4*>((char*)ctx->d_prot + o_atoms);
  P.type = reinterpret_cast<const uint8_t*>((char*)ctx->d_prot + o_type);
  P.runs = reinterpret_cast<const int*>((char*)ctx->d_prot + o_runs);
  ctx->prot = P;
  for (int d = 0; d < 3; ++d) {
    ctx->origin[d] = (double)of[d];
    ctx->origin_f[d] = of[d];
  }
  ctx->pxs.resize(n);
  ctx->pys.resize(n);
  ctx->pzs.resize(n);
  ctx->pkq.resize(n);
  ctx->ptypes.resize(n);
  for (int i = 0; i < n; ++i) {
    ctx->pxs[i] = xs[i] - (double)of[0];
    ctx->pys[i] = ys[i] - (double)of[1];
    ctx->pzs[i] = zs[i] - (double)of[2];
    ctx->pkq[i] = (float)(kElec * q[i]);
    ctx->ptypes[i] = type[i];
  }
  ++ctx->prot_version;
  ++ctx->epoch;
  return build_cull(ctx);
}

namespace {

// the checks of mmo_set_ligand, into a LigIn
int parse_ligand(mmo_ctx* ctx, const char* who, int n, const double* xs, const double* ys,
                 const double* zs, const double* q, const int* anum, const uint8_t* interacting,
                 int nrb, const int* bond_lr, const int* group_offsets, const int* group_atoms,
                 LigIn* out) {
  if (n < 1 || n > kMaxLig) return fail(ctx, MMO_EINVAL, "%s: n = %d outside 1..%d", who, n, kMaxLig);
  if (nrb < 0 || nrb > kMaxTors)
    return fail(ctx, MMO_EINVAL, "%s: nrb = %d outside 0..%d", who, nrb, kMaxTors);
  if (!xs || !ys || !zs || !q || !anum || !interacting ||
      (nrb > 0 && (!bond_lr || !group_offsets || !group_atoms)))
    return fail(ctx, MMO_EINVAL, "%s: null array", who);
  std::vector<int> type(n);
  for (int i = 0; i < n; ++i) {
    type[i] = type_of(anum[i]);
    if (type[i] < 0)
      return fail(ctx, MMO_EELEMENT, "ligand atom %d: element %d not in the UFF table", i, anum[i]);
    if (!std::isfinite(xs[i]) || !std::isfinite(ys[i]) || !std::isfinite(zs[i]) ||
        !std::isfinite(q[i]))
      return fail(ctx, MMO_EINVAL, "ligand atom %d: non-finite coordinate or charge", i);
  }
  std::vector<int> goff, gat, bonds;
  if (nrb > 0) {
    goff.assign(group_offsets, group_offsets + nrb + 1);
    if (goff[0] != 0) return fail(ctx, MMO_EINVAL, "group_offsets[0] must be 0");
    for (int t = 0; t < nrb; ++t) {
      const int l = bond_lr[2 * t], r = bond_lr[2 * t + 1];
      if (l < 0 || l >= n || r < 0 || r >= n || l == r)
        return fail(ctx, MMO_EINVAL, "rotatable bond %d: bad atoms (%d, %d)", t, l, r);
      if (goff[t + 1] < goff[t]) return fail(ctx, MMO_EINVAL, "group_offsets not monotone");
      for (int k = goff[t]; k < goff[t + 1]; ++k) {
        const int a = group_atoms[k];
        if (a < 0 || a >= n || a == r || a == l)
          return fail(ctx, MMO_EINVAL, "rotation group %d: bad atom %d", t, a);
      }
      bonds.push_back(l);
      bonds.push_back(r);
    }
    gat.assign(group_atoms, group_atoms + goff[nrb]);
  }
  out->x.assign(xs, xs + n);
  out->y.assign(ys, ys + n);
  out->z.assign(zs, zs + n);
  out->q.assign(q, q + n);
  out->type = type;
  out->bonds = bonds;
  out->goff = nrb > 0 ? goff : std::vector<int>{0};
  out->gat = gat;
  out->inter.assign(interacting, interacting + (size_t)n * n);
  return MMO_OK;
}

// the checks of mmo_set_protein; the device frame origin is the centroid
int parse_protein(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                  const double* q, const int* anum, std::vector<int>* type, float of[3]) {
  if (n < 0 || (n > 0 && (!xs || !ys || !zs || !q || !anum)))
    return fail(ctx, MMO_EINVAL, "protein: bad arguments");
  type->resize(n);
  double o[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i) {
    (*type)[i] = type_of(anum[i]);
    if ((*type)[i] < 0)
      return fail(ctx, MMO_EELEMENT, "protein atom %d: element %d not in the UFF table", i, anum[i]);
    if (!std::isfinite(xs[i]) || !std::isfinite(ys[i]) || !std::isfinite(zs[i]) ||
        !std::isfinite(q[i]))
      return fail(ctx, MMO_EINVAL, "protein atom %d: non-finite coordinate or charge", i);
    o[0] += xs[i];
    o[1] += ys[i];
    o[2] += zs[i];
  }
  if (n > 0)
    for (int d = 0; d < 3; ++d) o[d] /= n;
  for (int d = 0; d < 3; ++d) of[d] = (float)o[d];
  return MMO_OK;
}

}  // namespace

int mmo_set_ligand(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                   const double* q, const int* anum, const uint8_t* interacting, int nrb,
                   const int* bond_lr, const int* group_offsets, const int* group_atoms) {
  if (!ctx) return MMO_EINVAL;
  LigIn in;
  int r = parse_ligand(ctx, "mmo_set_ligand", n, xs, ys, zs, q, anum, interacting, nrb, bond_lr,
                       group_offsets, group_atoms, &in);
  if (r) return r;
  ctx->lx = in.x;
  ctx->ly = in.y;
  ctx->lz = in.z;
  ctx->lq = in.q;
  ctx->ltype = in.type;
  ctx->lbonds = in.bonds;
  ctx->lgoff = in.goff;
  ctx->lgatoms = in.gat;
  ctx->linter = in.inter;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  if ((r = upload_ligand(ctx))) return r;
  return grid_map(ctx);
}

namespace {

// mmo_ene_inter (parts = false: out[0] the energy) and mmo_ene_inter_parts
// (out[0] electrostatic, out[1] van der Waals): one launch each
int ene_inter_impl(mmo_ctx* ctx, const char* who, int n, const double* xs, const double* ys,
                   const double* zs, const double* q, const int* anum, bool parts, double* out) {
  if (!ctx) return MMO_EINVAL;
  if (n < 0 || n > kMaxLig || !out || (n > 0 && (!xs || !ys || !zs || !q || !anum)))
    return fail(ctx, MMO_EINVAL, "%s: bad arguments (n <= %d)", who, kMaxLig);
  const int nout = parts ? 2 : 1;
  if (n == 0 || ctx->prot.P == 0) {
    for (int k = 0; k < nout; ++k) out[k] = 0.0;
    return MMO_OK;
  }
  // staging: X[n] float4 | q[n] float | type[n] int ; output: nout C n partials | the totals
  const int C = std::max(1, (ctx->prot.P + 255) / 256);
  size_t off = 0;
  const size_t oX = take(off, sizeof(float4) * 2 * n);
  const size_t oq = take(off, sizeof(float) * n);
  const size_t ot = take(off, sizeof(int) * n);
  const size_t in_bytes = off;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  int r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_bytes);
  if (r) return r;
  r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out,
                sizeof(double) * ((size_t)nout * C * n + nout));
  if (r) return r;
  float4* hX = reinterpret_cast<float4*>(ctx->h_in + oX);
  float* hq = reinterpret_cast<float*>(ctx->h_in + oq);
  int* ht = reinterpret_cast<int*>(ctx->h_in + ot);
  for (int i = 0; i < n; ++i) {
    const int t = type_of(anum[i]);
    if (t < 0) return fail(ctx, MMO_EELEMENT, "ligand atom %d: element %d not in the UFF table", i, anum[i]);
    split_store(&hX[2 * i], xs[i] - ctx->origin[0], ys[i] - ctx->origin[1],
                zs[i] - ctx->origin[2], 0.f);
    hq[i] = (float)q[i];
    ht[i] = t;
  }
  const float4* dX = reinterpret_cast<const float4*>(ctx->d_in + oX);
  const float* dq = reinterpret_cast<const float*>(ctx->d_in + oq);
  const int* dt = reinterpret_cast<const int*>(ctx->d_in + ot);
  double* dEp = reinterpret_cast<double*>(ctx->d_out);
  double* dE = dEp + (size_t)nout * C * n;
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, in_bytes, cudaMemcpyHostToDevice, ctx->stream),
         "H2D");
  if (!ctx->d_plain_arrive) {
    MMO_CK(cudaMalloc((void**)&ctx->d_plain_arrive, sizeof(unsigned)), "arrival counter");
    MMO_CK(cudaMemset(ctx->d_plain_arrive, 0, sizeof(unsigned)), "arrival counter");
  }
  // one launch: the pair partials, and their totals from the last block
  if (parts)
    MMO_CK(launch_pairs_parts(ctx->prot, ctx->tab, dX, dq, dt, n, C, dEp, ctx->ph, ctx->stream,
                              dE, ctx->d_plain_arrive),
           "plain pair-parts kernel");
  else
    MMO_CK(launch_pairs_plain(ctx->prot, ctx->tab, dX, dq, dt, n, C, dEp, nullptr, 0, ctx->ph,
                              ctx->stream, dE, ctx->d_plain_arrive),
           "plain pair kernel");
  ctx->last_launches = 1;
  MMO_CK(cudaMemcpyAsync(ctx->h_out, dE, sizeof(double) * nout, cudaMemcpyDeviceToHost,
                         ctx->stream),
         "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  memcpy(out, ctx->h_out, sizeof(double) * nout);
  return MMO_OK;
}

}  // namespace

int mmo_ene_inter(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                  const double* q, const int* anum, double* out) {
  return ene_inter_impl(ctx, "mmo_ene_inter", n, xs, ys, zs, q, anum, false, out);
}

int mmo_ene_inter_parts(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                        const double* q, const int* anum, double* elec, double* vdw) {
  if (ctx && (!elec || !vdw)) return fail(ctx, MMO_EINVAL, "mmo_ene_inter_parts: null output");
  double two[2];
  const int r = ene_inter_impl(ctx, "mmo_ene_inter_parts", n, xs, ys, zs, q, anum, true, two);
  if (r == MMO_OK) {
    *elec = two[0];
    *vdw = two[1];
  }
  return r;
}

int mmo_ene_intra(mmo_ctx* ctx, const double* xs, const double* ys, const double* zs,
                  double* out) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (!xs || !ys || !zs || !out) return fail(ctx, MMO_EINVAL, "mmo_ene_intra: null pointer");
  const int n = ctx->lig.L;
  int r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, sizeof(float4) * 2 * n);
  if (r) return r;
  r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, sizeof(double));
  if (r) return r;
  float4* hX = reinterpret_cast<float4*>(ctx->h_in);
  // the intra term is translation-invariant: centre on atom 0 before rounding
  for (int i = 0; i < n; ++i)
    split_store(&hX[2 * i], xs[i] - xs[0], ys[i] - ys[0], zs[i] - zs[0], 0.f);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, sizeof(float4) * 2 * n, cudaMemcpyHostToDevice,
                         ctx->stream),
         "H2D");
  ctx->last_launches = 1;
  MMO_CK(launch_intra_plain(ctx->lig, reinterpret_cast<const float4*>(ctx->d_in),
                            ctx->ph.intra_form, ctx->ph.dielectric,
                            reinterpret_cast<double*>(ctx->d_out), ctx->stream),
         "intra kernel");
  MMO_CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, sizeof(double), cudaMemcpyDeviceToHost,
                         ctx->stream),
         "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  memcpy(out, ctx->h_out, sizeof(double));
  return MMO_OK;
}

// The host side of a scoring call: in_bytes of inputs to the device, run(d_in,
// d_E, d_grad, d_status, d_err) queued on the context's stream, then nE
// doubles, ngrad floats and nst ints of results back into E, grad, status
// (grad and status nullable), and the device error flag.  Page-locked caller
// buffers are copied by DMA directly, other host memory through the
// context's page-locked staging buffers.
extern "C++" {
template <class Run>
int host_call(mmo_ctx* ctx, const void* in, size_t in_bytes, double* E, size_t nE, float* grad,
              size_t ngrad, int* status, size_t nst, Run run) {
  size_t off = 0;
  take(off, sizeof(double) * nE);
  const size_t o_grad = take(off, grad ? sizeof(float) * ngrad : 0);
  const size_t o_st = take(off, sizeof(int) * nst);
  const size_t o_err = take(off, sizeof(int));
  const size_t out_bytes = off;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  int r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_bytes);
  if (r) return r;
  r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, out_bytes);
  if (r) return r;
  const bool pin_in = host_pinned(in);
  const bool pin_out =
      host_pinned(E) && (!grad || host_pinned(grad)) && (!status || host_pinned(status));
  if (!pin_in) memcpy(ctx->h_in, in, in_bytes);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, pin_in ? in : ctx->h_in, in_bytes, cudaMemcpyHostToDevice,
                         ctx->stream),
         "H2D");
  r = run(reinterpret_cast<const float*>(ctx->d_in), reinterpret_cast<double*>(ctx->d_out),
          grad ? reinterpret_cast<float*>(ctx->d_out + o_grad) : nullptr,
          reinterpret_cast<int*>(ctx->d_out + o_st), reinterpret_cast<int*>(ctx->d_out + o_err));
  if (r) return r;
  if (pin_out) {
    MMO_CK(cudaMemcpyAsync(E, ctx->d_out, sizeof(double) * nE, cudaMemcpyDeviceToHost,
                           ctx->stream),
           "D2H");
    if (grad)
      MMO_CK(cudaMemcpyAsync(grad, ctx->d_out + o_grad, sizeof(float) * ngrad,
                             cudaMemcpyDeviceToHost, ctx->stream),
             "D2H");
    if (status)
      MMO_CK(cudaMemcpyAsync(status, ctx->d_out + o_st, sizeof(int) * nst,
                             cudaMemcpyDeviceToHost, ctx->stream),
             "D2H");
    MMO_CK(cudaMemcpyAsync(ctx->h_out + o_err, ctx->d_out + o_err, sizeof(int),
                           cudaMemcpyDeviceToHost, ctx->stream),
           "D2H");
  } else {
    MMO_CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, out_bytes, cudaMemcpyDeviceToHost, ctx->stream),
           "D2H");
  }
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  if (!pin_out) {
    memcpy(E, ctx->h_out, sizeof(double) * nE);
    if (grad) memcpy(grad, ctx->h_out + o_grad, sizeof(float) * ngrad);
    if (status) memcpy(status, ctx->h_out + o_st, sizeof(int) * nst);
  }
  return check_dev_err(ctx, *reinterpret_cast<int*>(ctx->h_out + o_err));
}
}  // extern "C++"

int mmo_score_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, double* E_out,
                    float* grad_out, int* status_out) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (B < 0 || (B > 0 && (!dofs || !E_out)) || ((flags & MMO_F_GRAD) && !grad_out))
    return fail(ctx, MMO_EINVAL, "mmo_score_poses: bad arguments");
  if (B == 0) return MMO_OK;
  const int nd = 6 + ctx->lig.nrb;
  const bool grad = flags & MMO_F_GRAD;
  return host_call(ctx, dofs, sizeof(float) * (size_t)B * nd, E_out, B,
                   grad ? grad_out : nullptr, (size_t)B * nd, status_out, B,
                   [&](const float* d_in, double* d_E, float* d_grad, int* d_st, int* d_err) {
                     return score_device(ctx, B, d_in, flags, d_E, d_grad, d_st, d_err, 1,
                                         ctx->stream);
                   });
}

int mmo_posed_coords(mmo_ctx* ctx, int B, const float* dofs, int flags, double* xyz_out,
                     int* status_out) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (B < 0 || (B > 0 && (!dofs || !xyz_out)))
    return fail(ctx, MMO_EINVAL, "mmo_posed_coords: bad arguments");
  if (B == 0) return MMO_OK;
  const int L = ctx->lig.L, nd = 6 + ctx->lig.nrb;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  int r = ensure_scratch(ctx, B, L, 1, false);
  if (r) return r;
  size_t off = 0;
  const size_t o_st = take(off, sizeof(int) * B);
  const size_t o_err = take(off, sizeof(int));
  const size_t in_bytes = sizeof(float) * (size_t)B * nd, st_bytes = off;
  const size_t x_bytes = sizeof(float4) * 2 * (size_t)B * L;
  if ((r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_bytes))) return r;
  if ((r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, st_bytes + x_bytes))) return r;
  memcpy(ctx->h_in, dofs, in_bytes);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, in_bytes, cudaMemcpyHostToDevice, ctx->stream),
         "H2D");
  PoseIO io{};
  io.dofs = reinterpret_cast<const float*>(ctx->d_in);
  io.status = reinterpret_cast<int*>(ctx->d_out + o_st);
  io.err = reinterpret_cast<int*>(ctx->d_out + o_err);
  io.zero_err = 1;
  io.B = B;
  io.ox = ctx->origin_f[0];
  io.oy = ctx->origin_f[1];
  io.oz = ctx->origin_f[2];
  MMO_CK(launch_rebuild(ctx->lig, io, ctx->scr, flags & kFlagRecenter, ctx->stream),
         "rebuild kernel");
  MMO_CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, st_bytes, cudaMemcpyDeviceToHost, ctx->stream),
         "D2H");
  MMO_CK(cudaMemcpyAsync(ctx->h_out + st_bytes, ctx->scr.X, x_bytes, cudaMemcpyDeviceToHost,
                         ctx->stream),
         "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  // the posed atoms as hi + lo float pairs in the device frame -> FP64, input frame
  const float4* X = reinterpret_cast<const float4*>(ctx->h_out + st_bytes);
  for (size_t e = 0; e < (size_t)B * L; ++e) {
    const float4 h = X[2 * e], l = X[2 * e + 1];
    xyz_out[3 * e] = ((double)h.x + (double)l.x) + ctx->origin[0];
    xyz_out[3 * e + 1] = ((double)h.y + (double)l.y) + ctx->origin[1];
    xyz_out[3 * e + 2] = ((double)h.z + (double)l.z) + ctx->origin[2];
  }
  if (status_out) memcpy(status_out, ctx->h_out + o_st, sizeof(int) * B);
  return MMO_OK;
}

int mmo_score_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E,
                           float* d_grad, int* d_status, void* stream) {
  if (!ctx) return MMO_EINVAL;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  return score_device(ctx, B, d_dofs, flags, d_E, d_grad, d_status, ctx->d_err, 0, st);
}

namespace {

// One launch plan of the batched pair sweep as the tuner sets it.
struct TunePlan {
  int cull;       // 0: full sweep, 1: cut-off sweep, protein staged in shared memory, 2: cut-off
                  // sweep, protein read from global memory
  double h;       // row spacing (cut-off)
  int kp;         // entries per lane (cut-off) or poses per lane (full)
  int piece;      // protein atoms per piece (cut-off)
  int threads;
  int chunks;     // protein chunks per pose (full)
};

void apply_plan(mmo_ctx* ctx, const TunePlan& p, int* r) {
  ++ctx->epoch;
  ctx->cull_mode = p.cull == 0 ? 1 : (p.cull == 2 ? 2 : 0);
  ctx->cull_kp = p.cull ? p.kp : 0;
  ctx->cull_piece = p.cull ? p.piece : 0;
  ctx->tile_kp = p.cull ? 0 : p.kp;
  ctx->tile_chunks = p.cull ? 0 : p.chunks;
  ctx->tile_threads = p.threads;
  *r = MMO_OK;
  if (p.cull && p.h != ctx->cull_h) {
    ctx->cull_h = p.h;
    *r = build_cull(ctx);
  }
}

std::string tune_key(const mmo_ctx* ctx, int B, bool grad) {
  char k[160];
  snprintf(k, sizeof k, "%d %d %d %d %d %d %d %d %d", B, ctx->lig.L, ctx->lig.nrb, ctx->prot.P,
           ctx->ph.dielectric, ctx->ph.mixing, ctx->ph.inter_form, ctx->ph.intra_form,
           grad ? 1 : 0);
  return k;
}

bool tune_lookup(const std::string& path, const std::string& key, TunePlan* p) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return false;
  char line[512];
  bool found = false;
  while (fgets(line, sizeof line, f)) {
    const char* colon = strchr(line, ':');
    if (line[0] == '#' || !colon) continue;
    std::string k(line, colon - line);
    while (!k.empty() && k.back() == ' ') k.pop_back();
    TunePlan q{};
    double ms;
    if (k == key && sscanf(colon + 1, "%d %lf %d %d %d %d %lf", &q.cull, &q.h, &q.kp, &q.piece,
                           &q.threads, &q.chunks, &ms) == 7) {
      *p = q;  // the last line for a key wins
      found = true;
    }
  }
  fclose(f);
  return found;
}

}  // namespace

int mmo_set_tune_cache(mmo_ctx* ctx, const char* path) {
  if (!ctx) return MMO_EINVAL;
  ctx->tune_cache = path ? path : "";
  return MMO_OK;
}

int mmo_get_plan(const mmo_ctx* ctx, int* path, int* per_lane, int* threads, int* chunks_or_piece,
                 double* row_spacing) {
  if (!ctx || !path || !per_lane || !threads || !chunks_or_piece || !row_spacing)
    return MMO_EINVAL;
  const int g = ctx->last_grad;
  *path = ctx->last_cull ? 1 + ctx->cplan[g].global : 0;
  *per_lane = ctx->last_cull ? ctx->cplan[g].kp : ctx->plan[g].kp;
  *threads = ctx->last_cull ? ctx->cplan[g].threads : ctx->plan[g].threads;
  *chunks_or_piece = ctx->last_cull ? ctx->cplan[g].piece_atoms : ctx->plan[g].C;
  *row_spacing = ctx->cull_h;
  return MMO_OK;
}

int mmo_tune(mmo_ctx* ctx, int B, const float* d_dofs, int flags, double* d_E, float* d_grad,
             int* d_status, void* stream, double* ms_out) {
  if (!ctx) return MMO_EINVAL;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MMO_CK(cudaStreamIsCapturing(st, &cap), "capture status");
  if (cap != cudaStreamCaptureStatusNone)
    return fail(ctx, MMO_ESTATE, "mmo_tune times launches and cannot run inside a stream capture");
  const bool grad = flags & MMO_F_GRAD;
  const bool inter = (flags & MMO_F_INTER) && ctx->prot.P > 0;
  auto run = [&]() {
    return score_device(ctx, B, d_dofs, flags, d_E, d_grad, d_status, ctx->d_err, 0, st);
  };
  const std::string key = tune_key(ctx, B, grad);
  TunePlan best{};
  int r = MMO_OK;
  if (!ctx->tune_cache.empty() && tune_lookup(ctx->tune_cache, key, &best)) {
    apply_plan(ctx, best, &r);
    if (r || (r = run())) return r;
    if (ms_out) *ms_out = -1.0;
    return MMO_OK;
  }
  std::vector<TunePlan> cands;
  if (inter && B >= 2) {
    if (ctx->ph.inter_form == 0 && ctx->cull_ok)
      for (int mem : {1, 2}) {
        if (mem == 1 && !ctx->cull_fits) continue;  // the staged copy needs shared memory
        for (double h : {2.0, 3.0, 4.0, 5.0})
          for (int kp : {1, 2, 4})
            for (int piece : {256, 512, 1024}) {
              // the register budget's thread count, and fewer warps with more shared
              // memory left to the L1
              const int th = cull_max_threads(kp);
              cands.push_back({mem, h, kp, piece, th, 0});
              if (th >= 512) cands.push_back({mem, h, kp, piece, th - 256, 0});
            }
      }
    for (int kp : {1, 2, 4})
      for (int ch : {4, 8, 12, 16, 24}) cands.push_back({0, ctx->cull_h, kp, 0, 512, ch});
  }
  if (cands.empty()) {  // nothing to choose: the plain call
    if ((r = run())) return r;
    if (ms_out) *ms_out = -1.0;
    return MMO_OK;
  }
  cudaEvent_t a, b;
  MMO_CK(cudaEventCreate(&a), "event");
  MMO_CK(cudaEventCreate(&b), "event");
  float best_ms = 3e38f;
  for (const TunePlan& c : cands) {
    apply_plan(ctx, c, &r);
    if (r || (r = run()) || cudaStreamSynchronize(st) != cudaSuccess) continue;  // plan unusable
    float t[3];
    bool ok = true;
    for (float& v : t) {
      ok = ok && cudaEventRecord(a, st) == cudaSuccess && run() == MMO_OK &&
           cudaEventRecord(b, st) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
           cudaEventElapsedTime(&v, a, b) == cudaSuccess;
    }
    if (!ok) continue;
    std::sort(t, t + 3);
    if (t[1] < best_ms) {
      best_ms = t[1];
      best = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->err.clear();
  if (best_ms >= 3e38f) return fail(ctx, MMO_ECUDA, "mmo_tune: no launch plan ran");
  apply_plan(ctx, best, &r);
  if (r || (r = run())) return r;
  if (ms_out) *ms_out = best_ms;
  if (!ctx->tune_cache.empty()) {
    if (FILE* f = fopen(ctx->tune_cache.c_str(), "a")) {
      fprintf(f, "%s : %d %.3f %d %d %d %d %.4f\n", key.c_str(), best.cull, best.h, best.kp,
              best.piece, best.threads, best.chunks, best_ms);
      fclose(f);
    }
  }
  return MMO_OK;
}

namespace {

// per-chain buffers of mmo_mc_run in one allocation
MCDev mc_layout(char* base, int B, int nd, int nrb, size_t* bytes) {
  size_t off = 0;
  MCDev s{};
  s.cur = align_ptr<float>(base, off, (size_t)B * nd);
  s.trial = align_ptr<float>(base, off, (size_t)B * nd);
  s.start = align_ptr<float>(base, off, (size_t)B * 6);
  s.best = align_ptr<float>(base, off, (size_t)B * nd);
  s.G_cur = align_ptr<float>(base, off, (size_t)B * nd);
  s.G_trial = align_ptr<float>(base, off, (size_t)B * nd);
  s.E_cur = align_ptr<double>(base, off, B);
  s.E_trial = align_ptr<double>(base, off, B);
  s.Ei_trial = align_ptr<double>(base, off, B);
  s.E_best = align_ptr<double>(base, off, B);
  s.st_trial = align_ptr<int>(base, off, B);
  s.moved = align_ptr<int>(base, off, B);
  s.accepted = align_ptr<int>(base, off, B);
  s.resets = align_ptr<int>(base, off, B);
  s.stopped = align_ptr<int>(base, off, B);
  s.status_or = align_ptr<int>(base, off, B);
  s.steps = align_ptr<double>(base, off, (size_t)B * (2 + nrb));
  s.cnt = align_ptr<int>(base, off, (size_t)B * kMcCounts);
  s.win = align_ptr<int>(base, off, (size_t)B * (1 + nrb) * kMcWin);
  s.eta = align_ptr<float>(base, off, B);
  *bytes = off;
  return s;
}

// one block of MC steps, optionally ending with a minimisation: a fixed launch
// sequence on st (captured into a graph, or launched directly)
int mc_block(mmo_ctx* ctx, const MCDev& s, const MCParams& p, int nsteps, bool minimize,
             int iters, int flags, cudaStream_t st) {
  int r;
  for (int k = 0; k < nsteps; ++k) {
    MMO_CK(launch_k_mc_propose(s, p, st), "MC propose kernel");
    if ((r = score_device(ctx, p.B, s.trial, flags, s.E_trial, nullptr, s.st_trial, ctx->d_err, 0,
                          st, s.Ei_trial)))
      return r;
    MMO_CK(launch_k_mc_accept(s, p, st), "MC accept kernel");
  }
  if (minimize) {
    const int gf = flags | MMO_F_GRAD;
    MMO_CK(launch_k_gd_begin(s, p, st), "GD kernel");
    if ((r = score_device(ctx, p.B, s.cur, gf, s.E_trial, s.G_trial, s.st_trial, ctx->d_err, 0, st)))
      return r;
    MMO_CK(launch_k_gd_take(s, p, st), "GD kernel");
    for (int it = 0; it < iters; ++it) {
      MMO_CK(launch_k_gd_propose(s, p, st), "GD propose kernel");
      if ((r = score_device(ctx, p.B, s.trial, gf, s.E_trial, s.G_trial, s.st_trial, ctx->d_err, 0,
                            st)))
        return r;
      MMO_CK(launch_k_gd_accept(s, p, st), "GD accept kernel");
    }
  }
  return MMO_OK;
}

}  // namespace

int mmo_mc_run(mmo_ctx* ctx, int chains, int steps, const mmo_mc_params* prm,
               const mmo_mc_state* state, void* stream, int use_graph) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (chains <= 0 || steps < 0 || !prm || !state || !state->dofs || !state->E)
    return fail(ctx, MMO_EINVAL, "mmo_mc_run: bad arguments");
  if (!(prm->kT > 0) || !std::isfinite(prm->kT) || !(prm->rot_step >= 0) ||
      !(prm->trans_step >= 0) || !(prm->tors_step >= 0) || !std::isfinite(prm->rot_step) ||
      !std::isfinite(prm->trans_step) || !std::isfinite(prm->tors_step) ||
      (prm->move_law != MMO_MC_UNIFORM && prm->move_law != MMO_MC_GAUSSIAN) ||
      prm->minimize_every < 0 || prm->minimize_iters < 0 || prm->flip_every < 0 ||
      !(prm->gd_step >= 0) || !std::isfinite(prm->gd_step) ||
      !std::isfinite(prm->roi_radius) || !std::isfinite(prm->roi_center[0]) ||
      !std::isfinite(prm->roi_center[1]) || !std::isfinite(prm->roi_center[2]))
    return fail(ctx, MMO_EINVAL, "mmo_mc_run: bad parameters");
  if (steps > 0 && (state->trace_dofs || state->trace_E || state->trace_event) &&
      (long long)steps * chains > (1LL << 31) / std::max(1, 6 + ctx->lig.nrb))
    return fail(ctx, MMO_EINVAL, "mmo_mc_run: trace of %d steps x %d chains too large", steps,
                chains);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t us = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MMO_CK(cudaStreamIsCapturing(us, &cap), "capture status");
  if (cap != cudaStreamCaptureStatusNone)
    return fail(ctx, MMO_ESTATE, "mmo_mc_run: the stream is being captured");
  const int B = chains, nrb = ctx->lig.nrb, nd = 6 + nrb;
  size_t bytes = 0;
  mc_layout(nullptr, B, nd, nrb, &bytes);
  int r;
  if ((r = grow(ctx, &ctx->d_mc, &ctx->cap_mc, bytes, "MC chain buffers"))) return r;
  const MCDev s = mc_layout(static_cast<char*>(ctx->d_mc), B, nd, nrb, &bytes);
  MCParams p{};
  p.kT = prm->kT;
  p.rot = prm->rot_step;
  p.trans = prm->trans_step;
  p.tors = prm->tors_step;
  for (int k = 0; k < 3; ++k) p.roi_c[k] = prm->roi_center[k];
  p.roi_r = prm->roi_radius;
  p.reset_zero = prm->reset_on_zero_inter ? 1 : 0;
  p.too_long_ends = prm->too_long_ends_chain ? 1 : 0;
  p.trace_steps = (state->trace_dofs || state->trace_E || state->trace_event) ? steps : 0;
  p.trace_dofs = state->trace_dofs;
  p.trace_E = state->trace_E;
  p.trace_event = state->trace_event;
  p.gd_step = (float)prm->gd_step;
  p.law = prm->move_law;
  p.adapt = prm->adapt ? 1 : 0;
  p.flip_every = prm->flip_every;
  p.key0 = (uint32_t)(prm->seed & 0xffffffffu);
  p.key1 = (uint32_t)(prm->seed >> 32);
  p.B = B;
  p.nd = nd;
  p.nrb = nrb;
  if (prm->use_grid && !ctx->grid_map_ok)
    return fail(ctx, MMO_ESTATE, "mmo_mc_run: use_grid: %s", ctx->grid_map_err.c_str());
  const int flags = (prm->use_grid ? MMO_F_INTER | MMO_F_GRID
                                   : (ctx->prot.P > 0 ? MMO_F_INTER : 0)) |
                    MMO_F_INTRA | MMO_F_RECENTER;
  const bool minimize = prm->minimize_every > 0 && prm->minimize_iters > 0;
  const int block = std::max(1, std::min(steps, minimize ? prm->minimize_every : 50));
  const bool prof = ctx->profiling;
  ctx->profiling = false;  // no stage events inside a graph
  for (auto& e : ctx->mc_ev)
    if (!e) MMO_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  // work on the context's stream, ordered after the caller's stream
  cudaStream_t st = ctx->stream;
  MMO_CK(cudaEventRecord(ctx->mc_ev[0], us), "event");
  MMO_CK(cudaStreamWaitEvent(st, ctx->mc_ev[0], 0), "stream wait");
  auto body = [&]() -> int {
    MMO_CK(cudaMemcpyAsync(s.cur, state->dofs, sizeof(float) * B * nd, cudaMemcpyDeviceToDevice, st),
           "start poses");
    MMO_CK(launch_k_mc_init(s, p, st), "MC init kernel");
    int q;
    if ((q = score_device(ctx, B, s.cur, flags, s.E_cur, nullptr, s.st_trial, ctx->d_err, 0, st)))
      return q;
    MMO_CK(launch_k_mc_start(s, p, st), "MC start kernel");
    // plans and work buffers of both scorings before any capture
    if (minimize &&
        (q = score_device(ctx, B, s.cur, flags | MMO_F_GRAD, s.E_trial, s.G_trial, s.st_trial,
                          ctx->d_err, 0, st)))
      return q;
    const int nfull = steps / block, rem = steps % block;
    if (use_graph && nfull > 0) {
      std::vector<long> key = {B, block, minimize, prm->minimize_iters, flags, ctx->epoch, nd,
                               (long)(size_t)ctx->d_mc};
      const long* pw = reinterpret_cast<const long*>(&p);
      key.insert(key.end(), pw, pw + sizeof(MCParams) / sizeof(long));
      if (!ctx->mc_exec || key != ctx->mc_key) {
        if (ctx->mc_exec) cudaGraphExecDestroy(ctx->mc_exec);
        ctx->mc_exec = nullptr;
        MMO_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
        q = mc_block(ctx, s, p, block, minimize, prm->minimize_iters, flags, st);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (q) {
          if (g) cudaGraphDestroy(g);
          return q;
        }
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "end capture");
        const cudaError_t ie = cudaGraphInstantiate(&ctx->mc_exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
          ctx->mc_exec = nullptr;
          return cuda_fail(ctx, ie, "graph instantiate");
        }
        ctx->mc_key = key;
      }
      for (int i = 0; i < nfull; ++i) MMO_CK(cudaGraphLaunch(ctx->mc_exec, st), "graph launch");
    } else {
      for (int i = 0; i < nfull; ++i)
        if ((q = mc_block(ctx, s, p, block, minimize, prm->minimize_iters, flags, st))) return q;
    }
    if (rem && (q = mc_block(ctx, s, p, rem, false, 0, flags, st))) return q;
    MMO_CK(cudaMemcpyAsync(state->dofs, s.cur, sizeof(float) * B * nd, cudaMemcpyDeviceToDevice, st),
           "final poses");
    MMO_CK(cudaMemcpyAsync(state->E, s.E_cur, sizeof(double) * B, cudaMemcpyDeviceToDevice, st),
           "final energies");
    if (state->best_dofs)
      MMO_CK(cudaMemcpyAsync(state->best_dofs, s.best, sizeof(float) * B * nd,
                             cudaMemcpyDeviceToDevice, st), "best poses");
    if (state->best_E)
      MMO_CK(cudaMemcpyAsync(state->best_E, s.E_best, sizeof(double) * B, cudaMemcpyDeviceToDevice,
                             st), "best energies");
    if (state->accepted)
      MMO_CK(cudaMemcpyAsync(state->accepted, s.accepted, sizeof(int) * B,
                             cudaMemcpyDeviceToDevice, st), "accepted moves");
    if (state->status)
      MMO_CK(cudaMemcpyAsync(state->status, s.status_or, sizeof(int) * B,
                             cudaMemcpyDeviceToDevice, st), "status");
    if (state->resets)
      MMO_CK(cudaMemcpyAsync(state->resets, s.resets, sizeof(int) * B, cudaMemcpyDeviceToDevice,
                             st), "resets");
    return MMO_OK;
  };
  r = body();
  ctx->profiling = prof;
  // the caller's stream waits for the run (also after an error: nothing is left pending)
  cudaEventRecord(ctx->mc_ev[1], st);
  cudaStreamWaitEvent(us, ctx->mc_ev[1], 0);
  return r;
}

int mmo_philox4x32(mmo_ctx* ctx, unsigned k0, unsigned k1, unsigned c1, unsigned c2, int n,
                   unsigned* out, void* stream) {
  if (!ctx) return MMO_EINVAL;
  if (n < 0 || (n > 0 && !out)) return fail(ctx, MMO_EINVAL, "mmo_philox4x32: bad arguments");
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(launch_philox(k0, k1, c1, c2, n, reinterpret_cast<uint4*>(out),
                       reinterpret_cast<cudaStream_t>(stream)),
         "Philox kernel");
  return MMO_OK;
}

int mmo_sync(mmo_ctx* ctx, void* stream) {
  if (!ctx) return MMO_EINVAL;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  MMO_CK(cudaStreamSynchronize(st), "sync");
  int flag = 0;
  MMO_CK(cudaMemcpy(&flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (flag) MMO_CK(cudaMemset(ctx->d_err, 0, sizeof(int)), "clear error flag");
  return check_dev_err(ctx, flag);
}

int mmo_set_profiling(mmo_ctx* ctx, int on) {
  if (!ctx) return MMO_EINVAL;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  if (on && !ctx->ev[0])
    for (auto& e : ctx->ev) MMO_CK(cudaEventCreate(&e), "event create");
  ctx->profiling = on != 0;
  ctx->ev_valid = false;
  return MMO_OK;
}

int mmo_stage_times(mmo_ctx* ctx, float* ms) {
  if (!ctx || !ms) return MMO_EINVAL;
  if (!ctx->ev_valid) return fail(ctx, MMO_ESTATE, "no profiled scoring call yet");
  MMO_CK(cudaEventSynchronize(ctx->ev[4]), "event sync");
  MMO_CK(cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->ev[1]), "elapsed");
  MMO_CK(cudaEventElapsedTime(&ms[1], ctx->ev[2], ctx->ev[3]), "elapsed");
  MMO_CK(cudaEventElapsedTime(&ms[2], ctx->ev[3], ctx->ev[4]), "elapsed");
  MMO_CK(cudaEventElapsedTime(&ms[3], ctx->ev[1], ctx->ev[2]), "elapsed");
  return MMO_OK;
}

int mmo_last_launches(const mmo_ctx* ctx, int* kernels) {
  if (!ctx || !kernels) return MMO_EINVAL;
  *kernels = ctx->last_launches;
  return MMO_OK;
}

int mmo_pair_count(mmo_ctx* ctx, double* evaluated, double* all) {
  if (!ctx || !evaluated || !all) return MMO_EINVAL;
  *all = ctx->last_pairs;
  *evaluated = ctx->last_pairs;
  if (ctx->last_cull) {
    unsigned long long n = 0;
    MMO_CK(cudaSetDevice(ctx->device), "set device");
    MMO_CK(cudaDeviceSynchronize(), "device sync");
    MMO_CK(cudaMemcpy(&n, ctx->d_queue + 2, sizeof n, cudaMemcpyDeviceToHost), "pair count");
    *evaluated = (double)n;
  }
  return MMO_OK;
}

int mmo_diag_set_wait_polls(mmo_ctx* ctx, long long polls) {
  if (!ctx) return MMO_EINVAL;
  if (polls > 0xffffffffLL)
    return fail(ctx, MMO_EINVAL, "mmo_diag_set_wait_polls: %lld polls above 2^32 - 1", polls);
  ctx->first_wait_polls = polls < 0 ? kWaitPollsDefault : (uint32_t)polls;
  ++ctx->epoch;  // graphs captured with the old limit are rebuilt
  return MMO_OK;
}

int mmo_diag_pairs_within(mmo_ctx* ctx, double r, double* count) {
  if (!ctx || !count) return MMO_EINVAL;
  if (!(r > 0.0)) return fail(ctx, MMO_EINVAL, "mmo_diag_pairs_within: r = %g", r);
  if (ctx->last_pose_entries <= 0 || ctx->prot.P <= 0)
    return fail(ctx, MMO_ESTATE, "mmo_diag_pairs_within: no batched scoring call before it");
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  unsigned long long* d = nullptr;
  MMO_CK(cudaMalloc(&d, sizeof *d), "counter");
  unsigned long long n = 0;
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof *d, ctx->stream);
  if (e == cudaSuccess)
    e = launch_count_within(ctx->scr.X, ctx->last_pose_entries, ctx->prot.atoms, ctx->prot.P,
                            (float)(r * r), d, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&n, d, sizeof n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "mmo_diag_pairs_within");
  *count = (double)n;
  return MMO_OK;
}

int mmo_diag_sincos(mmo_ctx* ctx, int n, const float* x, float* out) {
  if (!ctx) return MMO_EINVAL;
  if (n < 0 || (n > 0 && (!x || !out)))
    return fail(ctx, MMO_EINVAL, "mmo_diag_sincos: bad arguments");
  if (n == 0) return MMO_OK;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  float* dx = nullptr;
  float4* dout = nullptr;
  cudaError_t e = cudaMalloc(&dx, sizeof(float) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(float4) * (size_t)n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dx, x, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = launch_df_sincos(dx, n, dout, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dout, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dx);
  cudaFree(dout);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "mmo_diag_sincos");
  return MMO_OK;
}

int mmo_fp32_fma_peak(mmo_ctx* ctx, double* tflops, double* ms_out) {
  if (!ctx || !tflops) return MMO_EINVAL;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  float* d = nullptr;
  MMO_CK(cudaMalloc(&d, sizeof(float)), "probe buffer");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double flops = 0.0, best = 0.0, best_ms = 0.0;
  cudaError_t e = cudaSuccess;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(a, ctx->stream);
    e = launch_fma_peak(ctx->sms, 8192, d, ctx->stream, &flops);
    cudaEventRecord(b, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess && rep > 0 && flops / (ms * 1e-3) > best) {
      best = flops / (ms * 1e-3);
      best_ms = ms;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "fma probe");
  *tflops = best * 1e-12;
  if (ms_out) *ms_out = best_ms;
  return MMO_OK;
}


int mmo_set_systems(mmo_ctx* ctx, int nsys, const mmo_system* systems) {
  if (!ctx) return MMO_EINVAL;
  if (nsys < 0 || (nsys > 0 && !systems)) return fail(ctx, MMO_EINVAL, "mmo_set_systems: bad arguments");
  SysBatch* S = new (std::nothrow) SysBatch();
  if (!S) return MMO_ENOMEM;
  S->in.resize(nsys);
  S->pose_off.assign(nsys + 1, 0);
  S->dof_off.assign(nsys + 1, 0);
  for (int u = 0; u < nsys; ++u) {
    const mmo_system& y = systems[u];
    SysBatch::Sys& sy = S->in[u];
    int r = parse_ligand(ctx, "mmo_set_systems", y.n_lig, y.lig_x, y.lig_y, y.lig_z, y.lig_q,
                         y.lig_anum, y.interacting, y.nrb, y.bond_lr, y.group_offsets,
                         y.group_atoms, &sy.lig);
    if (!r) r = parse_protein(ctx, y.n_prot, y.prot_x, y.prot_y, y.prot_z, y.prot_q, y.prot_anum,
                              &sy.ptype, sy.origin);
    if (!r && y.poses < 0) r = fail(ctx, MMO_EINVAL, "mmo_set_systems: system %d: poses < 0", u);
    if (r) {
      delete S;
      return r;
    }
    const int n = y.n_prot;
    sy.px.resize(n);
    sy.py.resize(n);
    sy.pz.resize(n);
    sy.pkq.resize(n);
    for (int i = 0; i < n; ++i) {
      sy.px[i] = y.prot_x[i] - (double)sy.origin[0];
      sy.py[i] = y.prot_y[i] - (double)sy.origin[1];
      sy.pz[i] = y.prot_z[i] - (double)sy.origin[2];
      sy.pkq[i] = (float)(kElec * y.prot_q[i]);
    }
    sy.poses = y.poses;
    S->pose_off[u + 1] = S->pose_off[u] + y.poses;
    S->dof_off[u + 1] = S->dof_off[u] + y.poses * (6 + y.nrb);
  }
  S->B = S->pose_off[nsys];
  S->D = S->dof_off[nsys];
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before replacing the systems");
  sys_free(ctx->sys);
  ctx->sys = S;
  ++ctx->epoch;
  return sys_build_static(ctx, S);
}

int mmo_tune_systems(mmo_ctx* ctx, const float* d_dofs, int flags, double* d_E, float* d_grad,
                     int* d_status, void* stream, double* ms_out) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->sys) return fail(ctx, MMO_ESTATE, "no systems: call mmo_set_systems first");
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MMO_CK(cudaStreamIsCapturing(st, &cap), "capture status");
  if (cap != cudaStreamCaptureStatusNone)
    return fail(ctx, MMO_ESTATE, "mmo_tune_systems cannot run inside a stream capture");
  auto run = [&]() { return score_systems(ctx, d_dofs, flags, d_E, d_grad, d_status, ctx->d_err, st); };
  struct Cand { int kp, piece, threads; };
  std::vector<Cand> cands;
  for (int kp : {1, 2, 4})
    for (int piece : {256, 512})
      for (int th : {128, 256, 512})
        if (th <= cull_max_threads(kp)) cands.push_back({kp, piece, th});
  cudaEvent_t a, b;
  MMO_CK(cudaEventCreate(&a), "event");
  MMO_CK(cudaEventCreate(&b), "event");
  float best_ms = 3e38f;
  Cand best{0, 0, 0};
  int r = MMO_OK;
  for (const Cand& c : cands) {
    ctx->cull_kp = c.kp;
    ctx->cull_piece = c.piece;
    ctx->tile_threads = c.threads;
    ++ctx->epoch;
    if (run() != MMO_OK || cudaStreamSynchronize(st) != cudaSuccess) continue;
    float t[3];
    bool ok = true;
    for (float& v : t)
      ok = ok && cudaEventRecord(a, st) == cudaSuccess && run() == MMO_OK &&
           cudaEventRecord(b, st) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
           cudaEventElapsedTime(&v, a, b) == cudaSuccess;
    if (!ok) continue;
    std::sort(t, t + 3);
    if (t[1] < best_ms) {
      best_ms = t[1];
      best = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  ctx->err.clear();
  if (best_ms >= 3e38f) return fail(ctx, MMO_ECUDA, "mmo_tune_systems: no launch plan ran");
  ctx->cull_kp = best.kp;
  ctx->cull_piece = best.piece;
  ctx->tile_threads = best.threads;
  ++ctx->epoch;
  if ((r = run())) return r;
  if (ms_out) *ms_out = best_ms;
  return MMO_OK;
}

int mmo_systems_plan(const mmo_ctx* ctx, int* per_lane, int* threads, int* piece_atoms) {
  if (!ctx || !per_lane || !threads || !piece_atoms) return MMO_EINVAL;
  if (!ctx->sys) return fail(const_cast<mmo_ctx*>(ctx), MMO_ESTATE, "no systems");
  *per_lane = ctx->sys->kp;
  *threads = ctx->sys->threads;
  *piece_atoms = (int)ctx->sys->plan_key[1];
  return MMO_OK;
}

int mmo_systems_layout(const mmo_ctx* ctx, int* total_poses, int* total_dofs, int* pose_off,
                       int* dof_off) {
  if (!ctx || !total_poses || !total_dofs) return MMO_EINVAL;
  const SysBatch* S = ctx->sys;
  *total_poses = S ? S->B : 0;
  *total_dofs = S ? S->D : 0;
  if (S && pose_off) std::copy(S->pose_off.begin(), S->pose_off.end(), pose_off);
  if (S && dof_off) std::copy(S->dof_off.begin(), S->dof_off.end(), dof_off);
  return MMO_OK;
}

int mmo_score_systems_device(mmo_ctx* ctx, const float* d_dofs, int flags, double* d_E,
                             float* d_grad, int* d_status, void* stream) {
  if (!ctx) return MMO_EINVAL;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  return score_systems(ctx, d_dofs, flags, d_E, d_grad, d_status, ctx->d_err,
                       reinterpret_cast<cudaStream_t>(stream));
}

int mmo_score_systems(mmo_ctx* ctx, const float* dofs, int flags, double* E, float* grad,
                      int* status) {
  if (!ctx) return MMO_EINVAL;
  SysBatch* S = ctx->sys;
  if (!S) return fail(ctx, MMO_ESTATE, "no systems: call mmo_set_systems first");
  const int B = S->B, D = S->D;
  const bool g = flags & MMO_F_GRAD;
  if (B > 0 && (!dofs || !E || (g && !grad))) return fail(ctx, MMO_EINVAL, "mmo_score_systems: bad arguments");
  if (B == 0) return MMO_OK;
  return host_call(ctx, dofs, sizeof(float) * (size_t)D, E, B, g ? grad : nullptr, D, status, B,
                   [&](const float* d_in, double* d_E, float* d_grad, int* d_st, int* d_err) {
                     MMO_CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream), "error flag");
                     return score_systems(ctx, d_in, flags, d_E, d_grad, d_st, d_err, ctx->stream);
                   });
}

// ---- precomputed interaction grids ------------------------------------------
int mmo_build_grids(mmo_ctx* ctx, const mmo_grid_spec* spec, double* ms) {
  if (!ctx) return MMO_EINVAL;
  if (ctx->prot.P <= 0 || !ctx->d_cull)
    return fail(ctx, MMO_ESTATE, "mmo_build_grids: no protein: call mmo_set_protein first");
  int r = grid_take_spec(ctx, "mmo_build_grids", spec, true);
  if (r) return r;
  const int nt = spec->ntypes, nx = spec->nx, ny = spec->ny, nz = spec->nz;
  // the distinct elements of the types, in order of first appearance
  std::vector<int> elems, type_elem(nt);
  for (int l = 0; l < nt; ++l) {
    const int t = type_of(spec->type_anum[l]);
    const auto it = std::find(elems.begin(), elems.end(), t);
    type_elem[l] = (int)(it - elems.begin());
    if (it == elems.end()) elems.push_back(t);
  }
  GridBuild gb{};
  gb.ntypes = nt;
  gb.nelem = (int)elems.size();
  gb.nx = nx;
  gb.ny = ny;
  gb.nz = nz;
  gb.step = spec->step;
  gb.max_Ef = (float)spec->max_E;
  for (int d = 0; d < 3; ++d) {
    gb.o[d] = spec->origin[d] - ctx->origin[d];
    gb.mc[d] = spec->mask_center[d] - ctx->origin[d];
  }
  const bool masked = spec->mask_radius > 0;
  gb.mr2 = masked ? spec->mask_radius * spec->mask_radius : HUGE_VAL;
  gb.fact = ctx->ph.mixing == MMO_MIX_GEOMEAN;
  if (gb.fact) {
    // x_ij = sqrt(x_i x_j), D_ij = sqrt(D_i D_j) (UFF.ml:47-48): the vdW terms
    // factor into protein-side sums shared by every element
    for (int pt = 0; pt < kNTypes; ++pt) {
      const double x = kUff[pt].xi, sd = std::sqrt(kUff[pt].di);
      gb.el[pt * kGridElems] = make_float2((float)(sd * std::pow(x, 6)), (float)(sd * x * x * x));
    }
    for (int e = 0; e < gb.nelem; ++e) {
      const double x = kUff[elems[e]].xi;
      gb.elf[e] = make_float4((float)std::sqrt(kUff[elems[e]].di), (float)(2.0 * x * x * x),
                              (float)std::pow(x, 6), 0.f);
    }
  } else {
    for (int pt = 0; pt < kNTypes; ++pt)
      for (int e = 0; e < gb.nelem; ++e) {
        double x2, d;
        pair_xd(ctx->ph.mixing, pt, elems[e], &x2, &d);
        // (X, 1/D), X = D^(1/3) x^2: (X / r^2)^3 = D (x / r)^6
        gb.el[pt * kGridElems + e] =
            make_float2((float)(std::cbrt(d) * x2), d > 0.0 ? (float)(1.0 / d) : 0.f);
      }
  }
  // the point tiles that meet the mask sphere (and the points inside it)
  std::vector<int3> tiles;
  double npts = masked ? 0.0 : (double)nx * ny * nz;
  // the counting variant of the kernel (profiling) has one point per lane
  gb.kp = ctx->profiling ? 1 : (ctx->grid_kp_set ? ctx->grid_kp_set : 2);
  if (gb.kp == 4 && !gb.fact) gb.kp = 2;  // 4 points per lane: the factorised kernel only
  const int TX = kGridTileX, TY = kGridTileY, TZ = 2 * gb.kp;
  for (int tz = 0; tz < (nz + TZ - 1) / TZ; ++tz)
    for (int ty = 0; ty < (ny + TY - 1) / TY; ++ty)
      for (int tx = 0; tx < (nx + TX - 1) / TX; ++tx) {
        if (masked) {
          const int lo[3] = {TX * tx, TY * ty, TZ * tz};
          const int hi[3] = {std::min(TX * tx + TX - 1, nx - 1), std::min(TY * ty + TY - 1, ny - 1),
                             std::min(TZ * tz + TZ - 1, nz - 1)};
          double d2 = 0.0;
          for (int d = 0; d < 3; ++d) {
            const double a = gb.o[d] + spec->step * lo[d], b = gb.o[d] + spec->step * hi[d];
            const double c = gb.mc[d];
            const double g = c < a ? a - c : (c > b ? c - b : 0.0);
            d2 += g * g;
          }
          if (!(d2 < gb.mr2)) continue;
          for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
              for (int i = lo[0]; i <= hi[0]; ++i) {
                const double px = gb.o[0] + spec->step * i - gb.mc[0];
                const double py = gb.o[1] + spec->step * j - gb.mc[1];
                const double pz = gb.o[2] + spec->step * k - gb.mc[2];
                npts += px * px + py * py + pz * pz < gb.mr2;
              }
        }
        tiles.push_back(make_int3(tx, ty, tz));
      }
  gb.ntiles = (int)tiles.size();
  size_t off = 0;
  const size_t o_cnt = take(off, 2 * sizeof(unsigned long long));
  const size_t o_tiles = take(off, sizeof(int3) * std::max<size_t>(tiles.size(), 1));
  const size_t o_q = take(off, sizeof(float) * nt);
  const size_t o_el = take(off, sizeof(int) * nt);
  std::vector<char> blob(off, 0);
  if (!tiles.empty()) memcpy(blob.data() + o_tiles, tiles.data(), sizeof(int3) * tiles.size());
  for (int l = 0; l < nt; ++l) {
    const float qf = (float)spec->type_q[l];
    memcpy(blob.data() + o_q + sizeof(float) * l, &qf, sizeof qf);
  }
  memcpy(blob.data() + o_el, type_elem.data(), sizeof(int) * nt);
  char* d_blob = nullptr;
  MMO_CK(cudaMalloc((void**)&d_blob, off), "grid build tables");
  cudaError_t e = cudaMemcpy(d_blob, blob.data(), off, cudaMemcpyHostToDevice);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  gb.tiles = reinterpret_cast<const int3*>(d_blob + o_tiles);
  gb.type_qf = reinterpret_cast<const float*>(d_blob + o_q);
  gb.type_elem = reinterpret_cast<const int*>(d_blob + o_el);
  // pair counts only under mmo_set_profiling (a separate instantiation of the kernel)
  gb.pairs = ctx->profiling ? reinterpret_cast<unsigned long long*>(d_blob + o_cnt) : nullptr;
  const size_t bytes = sizeof(float) * (size_t)nx * ny * nz * nt;
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_grid, 0, bytes, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], ctx->stream);
  if (e == cudaSuccess) e = launch_grid_build(ctx->cull, gb, ctx->ph.dielectric, ctx->d_grid,
                                              ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  unsigned long long cnt[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(cnt, d_blob + o_cnt, sizeof cnt, cudaMemcpyDeviceToHost);
  for (auto& v : ev)
    if (v) cudaEventDestroy(v);
  cudaFree(d_blob);
  ctx->grid_stats[0] = npts;
  ctx->grid_stats[1] = (double)cnt[0];
  ctx->grid_stats[2] = (double)cnt[1];
  if (e != cudaSuccess) return cuda_fail(ctx, e, "grid build");
  if (ms) *ms = t;
  ctx->grid_ok = true;
  ++ctx->epoch;
  return grid_map(ctx);
}

int mmo_set_grid_build(mmo_ctx* ctx, int points_per_lane) {
  if (!ctx) return MMO_EINVAL;
  if (points_per_lane < 0 || points_per_lane > 4 || points_per_lane == 3)
    return fail(ctx, MMO_EINVAL, "mmo_set_grid_build: points_per_lane must be 0, 1, 2 or 4");
  ctx->grid_kp_set = points_per_lane;
  return MMO_OK;
}

int mmo_load_grids(mmo_ctx* ctx, const mmo_grid_spec* spec, const float* values) {
  if (!ctx) return MMO_EINVAL;
  if (!values) return fail(ctx, MMO_EINVAL, "mmo_load_grids: values is NULL");
  int r = grid_take_spec(ctx, "mmo_load_grids", spec, false);
  if (r) return r;
  const size_t bytes = sizeof(float) * (size_t)spec->nx * spec->ny * spec->nz * spec->ntypes;
  MMO_CK(cudaMemcpy(ctx->d_grid, values, bytes, cudaMemcpyHostToDevice), "grid upload");
  ctx->grid_ok = true;
  ++ctx->epoch;
  return grid_map(ctx);
}

int mmo_grid_values(mmo_ctx* ctx, float* values) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->grid_ok) return fail(ctx, MMO_ESTATE, "mmo_grid_values: no grids");
  if (!values) return fail(ctx, MMO_EINVAL, "mmo_grid_values: values is NULL");
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before grid download");
  const size_t bytes = sizeof(float) * (size_t)ctx->grid_n[0] * ctx->grid_n[1] * ctx->grid_n[2] *
                       ctx->grid_anum.size();
  MMO_CK(cudaMemcpy(values, ctx->d_grid, bytes, cudaMemcpyDeviceToHost), "grid download");
  return MMO_OK;
}

int mmo_grid_dims(const mmo_ctx* ctx, int* ntypes, int* nx, int* ny, int* nz) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->grid_ok) return MMO_ESTATE;
  if (ntypes) *ntypes = (int)ctx->grid_anum.size();
  if (nx) *nx = ctx->grid_n[0];
  if (ny) *ny = ctx->grid_n[1];
  if (nz) *nz = ctx->grid_n[2];
  return MMO_OK;
}

int mmo_grid_build_stats(const mmo_ctx* ctx, double* points, double* pairs_evaluated,
                         double* pairs_within_cutoff) {
  if (!ctx) return MMO_EINVAL;
  if (points) *points = ctx->grid_stats[0];
  if (pairs_evaluated) *pairs_evaluated = ctx->grid_stats[1];
  if (pairs_within_cutoff) *pairs_within_cutoff = ctx->grid_stats[2];
  return MMO_OK;
}

int mmo_grid_device(const mmo_ctx* ctx, const float** d_values) {
  if (!ctx || !d_values) return MMO_EINVAL;
  if (!ctx->grid_ok) return MMO_ESTATE;
  *d_values = ctx->d_grid;
  return MMO_OK;
}

int mmo_ene_inter_grid(mmo_ctx* ctx, int n, const double* xs, const double* ys, const double* zs,
                       const double* q, const int* anum, double* out, int* status) {
  if (!ctx) return MMO_EINVAL;
  if (n < 0 || n > kMaxLig || !out || (n > 0 && (!xs || !ys || !zs || !q || !anum)))
    return fail(ctx, MMO_EINVAL, "mmo_ene_inter_grid: bad arguments (n <= %d)", kMaxLig);
  if (!ctx->grid_ok) return fail(ctx, MMO_ESTATE, "mmo_ene_inter_grid: no grids");
  if (status) *status = 0;
  if (n == 0) {
    *out = 0.0;
    return MMO_OK;
  }
  // staging: X[n][2] float4 | type[n] int ; output: E | status
  size_t off = 0;
  const size_t oX = take(off, sizeof(float4) * 2 * n);
  const size_t ot = take(off, sizeof(int) * n);
  const size_t in_bytes = off;
  size_t ooff = 0;
  const size_t oE = take(ooff, sizeof(double));
  const size_t oS = take(ooff, sizeof(int));
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  int r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_bytes);
  if (r) return r;
  if ((r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, ooff))) return r;
  float4* hX = reinterpret_cast<float4*>(ctx->h_in + oX);
  int* ht = reinterpret_cast<int*>(ctx->h_in + ot);
  const int nt = (int)ctx->grid_anum.size();
  for (int i = 0; i < n; ++i) {
    int t = -1;
    for (int l = 0; l < nt && t < 0; ++l)
      if (ctx->grid_anum[l] == anum[i] && ctx->grid_q[l] == q[i]) t = l;
    if (t < 0)
      return fail(ctx, MMO_EINVAL, "mmo_ene_inter_grid: atom %d (element %d, charge %.9g) has no "
                  "grid type", i, anum[i], q[i]);
    split_store(&hX[2 * i], xs[i] - ctx->origin[0], ys[i] - ctx->origin[1],
                zs[i] - ctx->origin[2], 0.f);
    ht[i] = t;
  }
  int* dS = reinterpret_cast<int*>(ctx->d_out + oS);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, in_bytes, cudaMemcpyHostToDevice, ctx->stream),
         "H2D");
  MMO_CK(launch_grid_inter_one(grid_look(ctx), reinterpret_cast<const float4*>(ctx->d_in + oX), n,
                               reinterpret_cast<const int*>(ctx->d_in + ot), ctx->d_grid,
                               reinterpret_cast<double*>(ctx->d_out + oE), dS, ctx->stream),
         "grid lookup kernel");
  ctx->last_launches = 1;
  MMO_CK(cudaMemcpyAsync(ctx->h_out + oE, ctx->d_out + oE, ooff - oE, cudaMemcpyDeviceToHost,
                         ctx->stream),
         "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  memcpy(out, ctx->h_out + oE, sizeof(double));
  if (status) memcpy(status, ctx->h_out + oS, sizeof(int));
  return MMO_OK;
}

int mmo_grid_atom_types(mmo_ctx* ctx, int* out) {
  if (!ctx) return MMO_EINVAL;
  if (!out) return fail(ctx, MMO_EINVAL, "mmo_grid_atom_types: out is NULL");
  if (!ctx->grid_map_ok) return fail(ctx, MMO_EINVAL, "%s", ctx->grid_map_err.c_str());
  std::copy(ctx->grid_lt.begin(), ctx->grid_lt.end(), out);
  return MMO_OK;
}

// ---- protein masks, clash filters, docking, placement, desolvation ----------
namespace {

ClashArgs clash_args(const mmo_ctx* ctx, int tests) {
  ClashArgs ca{};
  ca.g = grid_look(ctx);
  ca.vdw = ctx->masks_ok ? ctx->d_vdw : nullptr;
  ca.tests = tests;
  for (int a = 0; a < kNTypes; ++a) {
    ca.heavy[a] = kUff[a].anum > 1;
    for (int b = 0; b < kNTypes; ++b) {
      // Ptable.vdW_clash_params2 (src/ptable.ml:62-80): (0.8 (r_i + r_j))^2
      const double x = 0.8 * (vdw_radius(kUff[a].anum) + vdw_radius(kUff[b].anum));
      ca.clash2[a * kNTypes + b] = (float)(x * x);
    }
  }
  return ca;
}

size_t lattice_points(const mmo_ctx* ctx) {
  return (size_t)ctx->grid_n[0] * ctx->grid_n[1] * ctx->grid_n[2];
}

// posed coordinates of B poses into the scratch (the rebuild kernel only)
int pose_only(mmo_ctx* ctx, int B, const float* d_dofs, int flags, int* d_status,
              cudaStream_t st) {
  int r;
  if ((r = ensure_scratch(ctx, B, ctx->lig.L, 1, false))) return r;
  PoseIO io{};
  io.dofs = d_dofs;
  io.status = d_status;
  io.err = ctx->d_err;
  io.zero_err = 0;
  io.B = B;
  io.ox = ctx->origin_f[0];
  io.oy = ctx->origin_f[1];
  io.oz = ctx->origin_f[2];
  MMO_CK(launch_rebuild(ctx->lig, io, ctx->scr, flags & kFlagRecenter, st), "rebuild kernel");
  return MMO_OK;
}

}  // namespace

int mmo_build_masks(mmo_ctx* ctx, const double* radius, double r_water) {
  if (!ctx) return MMO_EINVAL;
  if (ctx->prot.P <= 0 || !ctx->d_cull)
    return fail(ctx, MMO_ESTATE, "mmo_build_masks: no protein: call mmo_set_protein first");
  if (!ctx->grid_ok)
    return fail(ctx, MMO_ESTATE, "mmo_build_masks: no lattice: build or load the grids first");
  if (!radius || !(r_water >= 0) || !std::isfinite(r_water))
    return fail(ctx, MMO_EINVAL, "mmo_build_masks: bad arguments");
  const int P = ctx->prot.P;
  std::vector<float> rf(P);
  std::vector<double> rd(P);
  double rmax = 0.0;
  for (int k = 0; k < P; ++k) {
    const double v = radius[ctx->cull_perm[k]];
    if (!(v >= 0) || !std::isfinite(v))
      return fail(ctx, MMO_EINVAL, "mmo_build_masks: atom %d: bad radius", ctx->cull_perm[k]);
    rd[k] = v;
    rf[k] = (float)v;
    rmax = std::max(rmax, v);
  }
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before mask build");
  const size_t np = lattice_points(ctx);
  int r;
  if ((r = grow(ctx, (void**)&ctx->d_vdw, &ctx->cap_vdw, np, "vdW mask"))) return r;
  if ((r = grow(ctx, (void**)&ctx->d_shell, &ctx->cap_shell, np, "solvent shell mask"))) return r;
  if ((r = grow(ctx, (void**)&ctx->d_vcell, &ctx->cap_vcell, np, "vdW cell mask"))) return r;
  char* d_tab = nullptr;
  MMO_CK(cudaMalloc((void**)&d_tab, (sizeof(double) + sizeof(float)) * (size_t)P), "radii");
  cudaError_t e = cudaMemcpy(d_tab, rd.data(), sizeof(double) * P, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d_tab + sizeof(double) * P, rf.data(), sizeof(float) * P,
                   cudaMemcpyHostToDevice);
  MaskBuild mb{};
  mb.radius = reinterpret_cast<const float*>(d_tab + sizeof(double) * P);
  mb.nx = ctx->grid_n[0];
  mb.ny = ctx->grid_n[1];
  mb.nz = ctx->grid_n[2];
  for (int d = 0; d < 3; ++d) mb.o[d] = ctx->grid_origin[d] - ctx->origin[d];
  mb.step = ctx->grid_step;
  mb.r_w = (float)r_water;
  mb.r_max = (float)rmax;
  if (e == cudaSuccess)
    e = launch_masks(ctx->cull, mb, reinterpret_cast<const double*>(d_tab), ctx->d_vdw,
                     ctx->d_shell, ctx->stream);
  if (e == cudaSuccess) e = launch_cell_masks(grid_look(ctx), ctx->d_vdw, ctx->d_vcell, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_tab);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "mask build");
  ctx->masks_ok = true;
  ctx->desolv_ok = false;
  ++ctx->epoch;
  return MMO_OK;
}

int mmo_load_masks(mmo_ctx* ctx, const uint8_t* vdw, const uint8_t* shell) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->grid_ok)
    return fail(ctx, MMO_ESTATE, "mmo_load_masks: no lattice: build or load the grids first");
  if (!vdw || !shell) return fail(ctx, MMO_EINVAL, "mmo_load_masks: NULL mask");
  const size_t np = lattice_points(ctx);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before mask upload");
  int r;
  if ((r = grow(ctx, (void**)&ctx->d_vdw, &ctx->cap_vdw, np, "vdW mask"))) return r;
  if ((r = grow(ctx, (void**)&ctx->d_shell, &ctx->cap_shell, np, "solvent shell mask"))) return r;
  MMO_CK(cudaMemcpy(ctx->d_vdw, vdw, np, cudaMemcpyHostToDevice), "vdW mask upload");
  MMO_CK(cudaMemcpy(ctx->d_shell, shell, np, cudaMemcpyHostToDevice), "shell mask upload");
  if ((r = grow(ctx, (void**)&ctx->d_vcell, &ctx->cap_vcell, np, "vdW cell mask"))) return r;
  MMO_CK(launch_cell_masks(grid_look(ctx), ctx->d_vdw, ctx->d_vcell, ctx->stream), "cell masks");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync after mask upload");
  ctx->masks_ok = true;
  ctx->desolv_ok = false;
  ++ctx->epoch;
  return MMO_OK;
}

int mmo_mask_values(mmo_ctx* ctx, uint8_t* vdw, uint8_t* shell) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->masks_ok) return fail(ctx, MMO_ESTATE, "mmo_mask_values: no masks");
  const size_t np = lattice_points(ctx);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before mask download");
  if (vdw) MMO_CK(cudaMemcpy(vdw, ctx->d_vdw, np, cudaMemcpyDeviceToHost), "vdW mask download");
  if (shell)
    MMO_CK(cudaMemcpy(shell, ctx->d_shell, np, cudaMemcpyDeviceToHost), "shell mask download");
  return MMO_OK;
}

int mmo_clash_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags, int tests,
                           int* d_out, void* stream) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (B < 0 || (B > 0 && (!d_dofs || !d_out)) || (tests & ~7))
    return fail(ctx, MMO_EINVAL, "mmo_clash_poses: bad arguments");
  if ((tests & MMO_CLASH_HEAVY) && ctx->prot.P <= 0)
    return fail(ctx, MMO_ESTATE, "MMO_CLASH_HEAVY: no protein");
  if ((tests & MMO_CLASH_GRID) && !ctx->masks_ok)
    return fail(ctx, MMO_ESTATE, "MMO_CLASH_GRID: no masks: call mmo_build_masks first");
  if (B == 0) return MMO_OK;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int r;
  if ((r = pose_only(ctx, B, d_dofs, flags, d_out, st))) return r;
  MMO_CK(launch_clash(ctx->lig, ctx->scr.X, B, ctx->cull, clash_args(ctx, tests), d_out, st),
         "clash kernel");
  return MMO_OK;
}

int mmo_clash_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, int tests, int* out) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (B < 0 || (B > 0 && (!dofs || !out))) return fail(ctx, MMO_EINVAL, "mmo_clash_poses: bad arguments");
  if (B == 0) return MMO_OK;
  const size_t nd = 6 + ctx->lig.nrb;
  const size_t in_b = sizeof(float) * B * nd, out_b = sizeof(int) * B;
  int r;
  if ((r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_b))) return r;
  if ((r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, out_b))) return r;
  memcpy(ctx->h_in, dofs, in_b);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, in_b, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  if ((r = mmo_clash_poses_device(ctx, B, reinterpret_cast<const float*>(ctx->d_in), flags, tests,
                                  reinterpret_cast<int*>(ctx->d_out), ctx->stream)))
    return r;
  MMO_CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, out_b, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  memcpy(out, ctx->h_out, out_b);
  return MMO_OK;
}

int mmo_so3_rotations(int n, double* R) {
  if (n < 0 || (n > 0 && !R)) return MMO_EINVAL;
  // SO3.super_fibonacci (src/SO3.ml:18-32), then Quat.to_axis_angle and
  // Rot.of_axis_angle (src/quat.ml:32-36, src/rot.ml:121-146)
  const double kPiH = 4.0 * std::atan(1.0);
  const double phi = std::sqrt(2.0), psi = 1.533751168755204288118041;
  for (int i = 0; i < n; ++i) {
    const double s = (double)i + 0.5, t = s / (double)n, d = 2.0 * kPiH * s;
    const double cr = std::sqrt(t), cR = std::sqrt(1.0 - t), al = d / phi, be = d / psi;
    const double w = cr * std::sin(al), x = cr * std::cos(al), y = cR * std::sin(be),
                 z = cR * std::cos(be);
    const double mag = std::sqrt(x * x + y * y + z * z);
    const double ux = x / mag, uy = y / mag, uz = z / mag, th = 2.0 * std::atan2(mag, w);
    const double c = std::cos(th), sn = std::sin(th), o = 1.0 - c;
    double* M = R + 9 * (size_t)i;
    M[0] = c + ux * ux * o;
    M[1] = ux * uy * o - uz * sn;
    M[2] = ux * uz * o + uy * sn;
    M[3] = ux * uy * o + uz * sn;
    M[4] = c + uy * uy * o;
    M[5] = uy * uz * o - ux * sn;
    M[6] = ux * uz * o - uy * sn;
    M[7] = uy * uz * o + ux * sn;
    M[8] = c + uz * uz * o;
  }
  return MMO_OK;
}

int mmo_dock_exhaustive(mmo_ctx* ctx, const mmo_dock_spec* sp, double* top_scores,
                        long long* top_frames, mmo_dock_result* res) {
  if (!ctx) return MMO_EINVAL;
  if (!sp || !res) return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: bad arguments");
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (!ctx->grid_map_ok)
    return fail(ctx, MMO_ESTATE, "mmo_dock_exhaustive: %s", ctx->grid_map_err.c_str());
  if (!ctx->masks_ok)
    return fail(ctx, MMO_ESTATE, "mmo_dock_exhaustive: no masks: call mmo_build_masks first");
  if (!(sp->roi_radius > 0) || !std::isfinite(sp->roi_radius) || !(sp->trans_step > 0) ||
      !std::isfinite(sp->trans_step) || sp->n_rotations < 1 || sp->topk < 1 ||
      sp->topk > kDockMaxK || !std::isfinite(sp->const_intra))
    return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: bad spec");
  if ((sp->topk > 0 && !top_scores))
    return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: top_scores is NULL");
  const int L = ctx->lig.L, nrot = sp->n_rotations, k = sp->topk;
  // Mol.is_ligand_center_vdW_occuppied on the centred reference conformer
  double cen[3] = {0, 0, 0};
  for (int a = 0; a < L; ++a) {
    cen[0] += ctx->lx[a];
    cen[1] += ctx->ly[a];
    cen[2] += ctx->lz[a];
  }
  for (int d = 0; d < 3; ++d) cen[d] /= L;
  int center_occ = 0;
  for (int a = 0; a < L; ++a) {
    const double ra = sp->lig_radius ? sp->lig_radius[a] : vdw_radius(kUff[ctx->ltype[a]].anum);
    const double dx = cen[0] - ctx->lx[a], dy = cen[1] - ctx->ly[a], dz = cen[2] - ctx->lz[a];
    if (std::sqrt(dx * dx + dy * dy + dz * dz) < ra) center_occ = 1;
  }
  // the position lattice (Grid.from_box trans_step of the ROI's cube), kept inside the ROI
  const double r = sp->roi_radius, step = sp->trans_step;
  for (int d = 0; d < 3; ++d) {
    const double lo = (sp->roi_center[d] - r - ctx->grid_origin[d]) / ctx->grid_step;
    const double hi = (sp->roi_center[d] + r - ctx->grid_origin[d]) / ctx->grid_step;
    if (!(std::fabs(lo) < 1e6) || !(std::fabs(hi) < 1e6))
      return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: the ROI is far off the grids' lattice");
  }
  const long long pdim = (long long)std::ceil(2.0 * r / step) + 1;
  if (pdim * pdim * pdim > (long long)INT32_MAX)
    return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: too many positions");
  std::vector<int> pos;
  for (long long kk = 0; kk < pdim; ++kk)
    for (long long jj = 0; jj < pdim; ++jj)
      for (long long ii = 0; ii < pdim; ++ii) {
        const double x = sp->roi_center[0] - r + step * ii, y = sp->roi_center[1] - r + step * jj,
                     z = sp->roi_center[2] - r + step * kk;
        const double dx = x - sp->roi_center[0], dy = y - sp->roi_center[1],
                     dz = z - sp->roi_center[2];
        if (dx * dx + dy * dy + dz * dz < r * r)
          pos.push_back((int)(ii + jj * pdim + kk * pdim * pdim));
      }
  const long long total = (long long)pos.size() * nrot;
  // CTA tiles of rtile rotations x (kDockPerBlock / rtile) positions; the
  // tile's rotated atoms (24 B per atom) take at most 24 KB of shared memory
  int rtile = 1;
  while (rtile * 2 <= kDockPerBlock && rtile * 2 * L * 24 <= 24576 && rtile < nrot) rtile *= 2;
  const long long ptile = kDockPerBlock / rtile;
  const long long blocks = ((long long)pos.size() + ptile - 1) / ptile * ((nrot + rtile - 1) / rtile);
  if (blocks > (long long)INT32_MAX / kDockMaxK)
    return fail(ctx, MMO_EINVAL, "mmo_dock_exhaustive: too many poses");
  std::vector<double> rot(9 * (size_t)nrot);
  mmo_so3_rotations(nrot, rot.data());
  // device blob: rotations | positions | two candidate buffers | counters
  const size_t ncand = (size_t)std::max<long long>(blocks, 1) * k;
  size_t off = 0;
  const size_t o_rot = take(off, sizeof(double) * rot.size());
  const size_t o_pos = take(off, sizeof(int) * std::max<size_t>(pos.size(), 1));
  const size_t o_c0 = take(off, 2 * sizeof(unsigned long long) * ncand);
  const size_t o_c1 = take(off, 2 * sizeof(unsigned long long) * ncand);
  const size_t o_cnt = take(off, 2 * sizeof(unsigned long long));
  const size_t o_off = take(off, sizeof(float) * 6 * (size_t)nrot * L);
  const size_t o_pc = take(off, sizeof(float4) * 2 * std::max<size_t>(pos.size(), 1));
  const size_t o_pk = take(off, sizeof(int) * 2 * std::max<size_t>(pos.size(), 1));
  int rc;
  if ((rc = grow(ctx, &ctx->d_dock, &ctx->cap_dock, off, "docking buffers"))) return rc;
  char* base = static_cast<char*>(ctx->d_dock);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before docking");
  MMO_CK(cudaMemcpy(base + o_rot, rot.data(), sizeof(double) * rot.size(), cudaMemcpyHostToDevice),
         "rotations upload");
  if (!pos.empty())
    MMO_CK(cudaMemcpy(base + o_pos, pos.data(), sizeof(int) * pos.size(), cudaMemcpyHostToDevice),
           "positions upload");
  MMO_CK(cudaMemsetAsync(base + o_cnt, 0, 2 * sizeof(unsigned long long), ctx->stream), "counters");
  DockArgs a{};
  a.ref = ctx->lig.ref64;
  a.lig_type = ctx->d_grid_lt;
  a.grids = ctx->d_grid;
  a.g = grid_look(ctx);
  a.vcell = ctx->d_vcell;
  a.rot = reinterpret_cast<const double*>(base + o_rot);
  a.off = reinterpret_cast<float*>(base + o_off);
  a.pcell = reinterpret_cast<float4*>(base + o_pc);
  a.pcell_k = reinterpret_cast<int*>(base + o_pk);
  a.pos_idx = reinterpret_cast<const int*>(base + o_pos);
  a.L = L;
  a.npos = (int)pos.size();
  a.nrot = nrot;
  a.pdim = (int)pdim;
  a.rtile = rtile;
  for (int d = 0; d < 3; ++d) a.p0[d] = sp->roi_center[d] - r - ctx->origin[d];
  a.pstep = step;
  a.center_occ = center_occ;
  a.const_intra = sp->const_intra;
  a.k = k;
  a.cand = reinterpret_cast<unsigned long long*>(base + o_c0);
  a.counts = reinterpret_cast<unsigned long long*>(base + o_cnt);
  cudaEvent_t ev[2] = {nullptr, nullptr};
  MMO_CK(cudaEventCreate(&ev[0]), "event");
  MMO_CK(cudaEventCreate(&ev[1]), "event");
  cudaError_t e = cudaEventRecord(ev[0], ctx->stream);
  if (e == cudaSuccess) e = launch_dock(a, (int)blocks, ctx->stream);
  // merge the candidates k at a time until one group remains
  unsigned long long* cur = a.cand;
  unsigned long long* nxt = reinterpret_cast<unsigned long long*>(base + o_c1);
  long long n = blocks * k;
  while (e == cudaSuccess && n > k) {
    e = launch_topk_merge(cur, (int)n, k, nxt, ctx->stream);
    n = (n + kDockPerBlock - 1) / kDockPerBlock * k;
    std::swap(cur, nxt);
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev[1], ctx->stream);
  std::vector<unsigned long long> host(2 * (size_t)k + 2, ~0ull);
  if (e == cudaSuccess && blocks > 0)
    e = cudaMemcpyAsync(host.data(), cur, 2 * sizeof(unsigned long long) * k,
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host.data() + 2 * k, base + o_cnt, 2 * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "exhaustive docking");
  *res = mmo_dock_result{};
  res->best_score = HUGE_VAL;
  res->positions = (long long)pos.size();
  res->poses = total;
  res->scored = (long long)host[2 * k];
  res->clashed = (long long)host[2 * k + 1];
  res->ms = ms;
  int nt = 0;
  for (int t = 0; t < k && blocks > 0; ++t) {
    const unsigned long long key = host[2 * t], fr = host[2 * t + 1];
    if (key == ~0ull) break;
    const unsigned long long u = (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
    double sc;
    memcpy(&sc, &u, sizeof sc);
    top_scores[nt] = sc;
    if (top_frames) top_frames[nt] = (long long)fr;
    if (nt == 0) {
      res->best_score = sc;
      const long long pi = (long long)(fr / (unsigned long long)nrot);
      res->best_rot = (int)(fr % (unsigned long long)nrot);
      const long long ii = pi % pdim, jj = (pi / pdim) % pdim, kk = pi / (pdim * pdim);
      res->best_pos[0] = sp->roi_center[0] - r + step * ii;
      res->best_pos[1] = sp->roi_center[1] - r + step * jj;
      res->best_pos[2] = sp->roi_center[2] - r + step * kk;
    }
    ++nt;
  }
  res->n_top = nt;
  return MMO_OK;
}

int mmo_place_in_roi(mmo_ctx* ctx, const double center[3], double radius, int n,
                     unsigned long long seed, float* dofs, long long* trials) {
  if (!ctx) return MMO_EINVAL;
  if (!center || !(radius > 0) || !std::isfinite(radius) || n < 0 || (n > 0 && !dofs))
    return fail(ctx, MMO_EINVAL, "mmo_place_in_roi: bad arguments");
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (ctx->prot.P <= 0) return fail(ctx, MMO_ESTATE, "no protein: call mmo_set_protein first");
  if (n == 0) return MMO_OK;
  const int per = 64, nd = 6 + ctx->lig.nrb;
  size_t off = 0;
  const size_t o_out = take(off, sizeof(float) * 7 * (size_t)n * per);
  const size_t o_ids = take(off, sizeof(int) * (size_t)n);
  int rc;
  if ((rc = grow(ctx, &ctx->d_dock, &ctx->cap_dock, off, "placement buffers"))) return rc;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before placement");
  char* base = static_cast<char*>(ctx->d_dock);
  PlaceArgs a{};
  a.ref = ctx->lig.ref64;
  a.type = ctx->lig.type;
  a.L = ctx->lig.L;
  a.per_slot = per;
  for (int d = 0; d < 3; ++d) a.c[d] = center[d] - ctx->origin[d];
  a.r = radius;
  a.key0 = (uint32_t)(seed & 0xffffffffu);
  a.key1 = (uint32_t)(seed >> 32);
  a.out = reinterpret_cast<float*>(base + o_out);
  a.slot_id = reinterpret_cast<const int*>(base + o_ids);
  const ClashArgs ca = clash_args(ctx, MMO_CLASH_HEAVY);
  // open placements; candidate c of placement s uses Philox counter (s, c, draw, 1)
  std::vector<int> todo(n);
  std::iota(todo.begin(), todo.end(), 0);
  std::vector<float> host((size_t)7 * n * per);
  long long drawn = 0;
  for (int c0 = 0; !todo.empty(); c0 += per) {
    if (c0 >= 100000)
      return fail(ctx, MMO_ESTATE,
                  "mmo_place_in_roi: placement %d found no clash-free pose in 100000 candidates",
                  todo[0]);
    const int m = (int)todo.size();
    a.slots = m;
    a.c0 = c0;
    MMO_CK(cudaMemcpy(base + o_ids, todo.data(), sizeof(int) * m, cudaMemcpyHostToDevice),
           "placement ids upload");
    MMO_CK(launch_place(a, ctx->cull, ca, ctx->stream), "placement kernel");
    MMO_CK(cudaMemcpyAsync(host.data(), a.out, sizeof(float) * 7 * (size_t)m * per,
                           cudaMemcpyDeviceToHost, ctx->stream),
           "placement download");
    MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
    std::vector<int> still;
    for (int t = 0; t < m; ++t) {
      int hit = -1;
      for (int c = 0; c < per && hit < 0; ++c)
        if (host[(size_t)7 * (per * t + c) + 6] != 0.f) hit = c;
      if (hit < 0) {
        drawn += per;
        still.push_back(todo[t]);
        continue;
      }
      drawn += hit + 1;
      const float* o = &host[(size_t)7 * (per * t + hit)];
      float* d = dofs + (size_t)nd * todo[t];
      for (int q = 0; q < 3; ++q) d[q] = (float)((double)o[q] + ctx->origin[q]);
      for (int q = 3; q < 6; ++q) d[q] = o[q];
      for (int q = 6; q < nd; ++q) d[q] = 0.f;
    }
    todo.swap(still);
  }
  if (trials) *trials = drawn;
  return MMO_OK;
}

int mmo_set_ligand_radii(mmo_ctx* ctx, const double* radius) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (!radius) return fail(ctx, MMO_EINVAL, "mmo_set_ligand_radii: radius is NULL");
  const int L = ctx->lig.L;
  for (int a = 0; a < L; ++a)
    if (!(radius[a] >= 0) || !std::isfinite(radius[a]))
      return fail(ctx, MMO_EINVAL, "mmo_set_ligand_radii: atom %d: bad radius", a);
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before radii upload");
  int r;
  if ((r = grow(ctx, (void**)&ctx->d_lradius, &ctx->cap_lradius, sizeof(double) * L, "ligand radii")))
    return r;
  MMO_CK(cudaMemcpy(ctx->d_lradius, radius, sizeof(double) * L, cudaMemcpyHostToDevice),
         "ligand radii upload");
  ctx->lradius.assign(radius, radius + L);
  return MMO_OK;
}

int mmo_protein_desolv(mmo_ctx* ctx, const double center[3], double radius, double* out) {
  if (!ctx) return MMO_EINVAL;
  if (!center || !(radius > 0) || !std::isfinite(radius))
    return fail(ctx, MMO_EINVAL, "mmo_protein_desolv: bad arguments");
  if (!ctx->masks_ok)
    return fail(ctx, MMO_ESTATE, "mmo_protein_desolv: no masks: call mmo_build_masks first");
  if (ctx->prot.P <= 0 || !ctx->d_cull) return fail(ctx, MMO_ESTATE, "no protein");
  const int nx = ctx->grid_n[0], ny = ctx->grid_n[1], nz = ctx->grid_n[2];
  const size_t np = lattice_points(ctx);
  DesolvBuild db{};
  db.shell = ctx->d_shell;
  db.nx = nx;
  db.ny = ny;
  db.nz = nz;
  for (int d = 0; d < 3; ++d) {
    db.o[d] = ctx->grid_origin[d] - ctx->origin[d];
    db.c[d] = center[d] - ctx->origin[d];
  }
  db.step = ctx->grid_step;
  db.r2 = radius * radius;
  const double vol = db.step * db.step * db.step;
  db.scale = (1.0 / 4.0 - 1.0 / 78.5) / (8.0 * (4.0 * std::atan(1.0))) * vol / (kElec * kElec);
  std::vector<int3> tiles;
  for (int tz = 0; tz < (nz + 1) / 2; ++tz)
    for (int ty = 0; ty < (ny + 3) / 4; ++ty)
      for (int tx = 0; tx < (nx + 3) / 4; ++tx) {
        const int lo[3] = {4 * tx, 4 * ty, 2 * tz};
        const int hi[3] = {std::min(4 * tx + 3, nx - 1), std::min(4 * ty + 3, ny - 1),
                           std::min(2 * tz + 1, nz - 1)};
        double d2 = 0.0;
        for (int d = 0; d < 3; ++d) {
          const double a0 = db.o[d] + db.step * lo[d], a1 = db.o[d] + db.step * hi[d];
          const double g = db.c[d] < a0 ? a0 - db.c[d] : (db.c[d] > a1 ? db.c[d] - a1 : 0.0);
          d2 += g * g;
        }
        if (d2 < db.r2) tiles.push_back(make_int3(tx, ty, tz));
      }
  db.ntiles = (int)tiles.size();
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync before desolvation");
  int r;
  if ((r = grow(ctx, (void**)&ctx->d_desolv, &ctx->cap_desolv, sizeof(double) * np,
                "desolvation contributions")))
    return r;
  int3* d_tiles = nullptr;
  MMO_CK(cudaMalloc((void**)&d_tiles, sizeof(int3) * std::max<size_t>(tiles.size(), 1)), "tiles");
  cudaError_t e = cudaSuccess;
  if (!tiles.empty())
    e = cudaMemcpy(d_tiles, tiles.data(), sizeof(int3) * tiles.size(), cudaMemcpyHostToDevice);
  db.tiles = d_tiles;
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_desolv, 0, sizeof(double) * np, ctx->stream);
  if (e == cudaSuccess) e = launch_prot_desolv(ctx->cull, db, ctx->d_desolv, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_tiles);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "protein desolvation");
  if (out)
    MMO_CK(cudaMemcpy(out, ctx->d_desolv, sizeof(double) * np, cudaMemcpyDeviceToHost),
           "desolvation download");
  ctx->desolv_ok = true;
  return MMO_OK;
}

int mmo_desolvation_poses_device(mmo_ctx* ctx, int B, const float* d_dofs, int flags,
                                 double r_water, double* d_prot, double* d_lig, int* d_status,
                                 void* stream) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (!ctx->desolv_ok)
    return fail(ctx, MMO_ESTATE, "mmo_desolvation_poses: call mmo_protein_desolv first");
  if ((int)ctx->lradius.size() != ctx->lig.L)
    return fail(ctx, MMO_ESTATE, "mmo_desolvation_poses: call mmo_set_ligand_radii first");
  if (B < 0 || (B > 0 && (!d_dofs || !d_prot || !d_lig || !d_status)) || !(r_water >= 0) ||
      !std::isfinite(r_water))
    return fail(ctx, MMO_EINVAL, "mmo_desolvation_poses: bad arguments");
  if (B == 0) return MMO_OK;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int r;
  if ((r = pose_only(ctx, B, d_dofs, flags, d_status, st))) return r;
  MMO_CK(cudaMemsetAsync(d_status, 0, sizeof(int) * B, st), "status reset");
  DesolvPose d{};
  d.X = ctx->scr.X;
  d.q = ctx->lig.q;
  d.radius = ctx->d_lradius;
  d.shell = ctx->d_shell;
  d.contrib = ctx->d_desolv;
  d.g = grid_look(ctx);
  d.step = ctx->grid_step;
  d.r_w = (float)r_water;
  d.L = ctx->lig.L;
  d.B = B;
  d.cap = 262144;
  d.scale = (1.0 / 4.0 - 1.0 / 78.5) / (8.0 * (4.0 * std::atan(1.0))) * ctx->grid_step *
            ctx->grid_step * ctx->grid_step;
  d.prot = d_prot;
  d.lig = d_lig;
  d.status = d_status;
  MMO_CK(launch_desolv_pose(d, st), "desolvation kernel");
  return MMO_OK;
}

int mmo_desolvation_poses(mmo_ctx* ctx, int B, const float* dofs, int flags, double r_water,
                          double* prot, double* lig, int* status) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  if (B < 0 || (B > 0 && (!dofs || !prot || !lig || !status)))
    return fail(ctx, MMO_EINVAL, "mmo_desolvation_poses: bad arguments");
  if (B == 0) return MMO_OK;
  const size_t nd = 6 + ctx->lig.nrb;
  const size_t in_b = sizeof(float) * B * nd;
  const size_t o_lig = sizeof(double) * B, o_st = 2 * sizeof(double) * B;
  const size_t out_b = o_st + sizeof(int) * B;
  int r;
  if ((r = grow_host(ctx, &ctx->h_in, &ctx->d_in, &ctx->cap_in, in_b))) return r;
  if ((r = grow_host(ctx, &ctx->h_out, &ctx->d_out, &ctx->cap_out, out_b))) return r;
  memcpy(ctx->h_in, dofs, in_b);
  MMO_CK(cudaMemcpyAsync(ctx->d_in, ctx->h_in, in_b, cudaMemcpyHostToDevice, ctx->stream), "H2D");
  if ((r = mmo_desolvation_poses_device(
           ctx, B, reinterpret_cast<const float*>(ctx->d_in), flags, r_water,
           reinterpret_cast<double*>(ctx->d_out), reinterpret_cast<double*>(ctx->d_out + o_lig),
           reinterpret_cast<int*>(ctx->d_out + o_st), ctx->stream)))
    return r;
  MMO_CK(cudaMemcpyAsync(ctx->h_out, ctx->d_out, out_b, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  MMO_CK(cudaStreamSynchronize(ctx->stream), "sync");
  memcpy(prot, ctx->h_out, sizeof(double) * B);
  memcpy(lig, ctx->h_out + o_lig, sizeof(double) * B);
  memcpy(status, ctx->h_out + o_st, sizeof(int) * B);
  return MMO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batched scoring (mmo_score_poses_noalloc).
//
// The work buffers of a call (posed coordinates, per-chunk energy and
// gradient partials, intra-ligand energies) live in one file-scope device
// array of kNoAllocBytes instead of buffers that grow with cudaMalloc.  Every
// GPU that loads this library holds the array until the process exits.  In
// host code the name g_noalloc_scratch is only a host-side stand-in for the
// array, not a device address, so the kernels get the address that
// cudaGetSymbolAddress returns for the current device.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocBytes = size_t(32) << 20;  // 32 MiB per GPU
constexpr int kNoAllocDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocDevices] = {};

// Device address of the static scratch on `device`, looked up once per device
// with that device current.
int noalloc_scratch(mmo_ctx* ctx, int device, unsigned char** out) {
  if (device < 0 || device >= kNoAllocDevices)
    return fail(ctx, MMO_EINVAL, "mmo_score_poses_noalloc: device %d above %d", device,
                kNoAllocDevices - 1);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    MMO_CK(cudaSetDevice(device), "set device");
    MMO_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch), "static scratch address");
    g_noalloc_ptr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_ptr[device]);
  return MMO_OK;
}

}  // namespace

extern "C" int mmo_score_poses_noalloc(mmo_ctx* ctx, int B, const float* d_dofs, int flags,
                                       double* d_E, float* d_grad, int* d_status, void* stream) {
  if (!ctx) return MMO_EINVAL;
  if (!ctx->has_lig) return fail(ctx, MMO_ESTATE, "no ligand: call mmo_set_ligand first");
  const bool use_grid = (flags & MMO_F_INTER) && (flags & MMO_F_GRID);
  if (use_grid && !ctx->grid_map_ok)
    return fail(ctx, MMO_ESTATE, "MMO_F_GRID: %s", ctx->grid_map_err.c_str());
  if ((flags & MMO_F_INTER) && !use_grid && ctx->prot.P <= 0)
    return fail(ctx, MMO_ESTATE, "no protein: call mmo_set_protein first");
  if (B < 0 || (B > 0 && (!d_dofs || !d_E || !d_status)))
    return fail(ctx, MMO_EINVAL, "mmo_score_poses_noalloc: bad batch arguments");
  if ((flags & MMO_F_GRAD) && !d_grad)
    return fail(ctx, MMO_EINVAL, "mmo_score_poses_noalloc: MMO_F_GRAD needs grad_out");
  if (B == 0) return MMO_OK;
  const bool grad = flags & MMO_F_GRAD;
  const bool inter = use_grid || ((flags & MMO_F_INTER) && ctx->prot.P > 0);
  const int L = ctx->lig.L;
  // scratch layout: X[B][L][2] | (gradient: Y[B][L][2] | rec[B][nrb][3] | cen[B][2]) |
  // Epart[B][C][L] | (gradient: Gpart[B][C][L])
  const size_t nrb = std::max(1, ctx->lig.nrb);
  const size_t fixed = 256 * 6 + sizeof(float4) * 2 * (size_t)B * L +
                       (grad ? sizeof(float4) * (2 * (size_t)B * L + 3 * (size_t)B * nrb + 2 * B)
                             : 0);
  const size_t per_chunk = (sizeof(double) + (grad ? sizeof(float4) : 0)) * (size_t)B * L;
  const int nslices = inter && !use_grid ? (ctx->prot.P + kSliceAtoms - 1) / kSliceAtoms : 1;
  const long c_fit = fixed < kNoAllocBytes ? (long)((kNoAllocBytes - fixed) / per_chunk) : 0;
  if (c_fit < nslices) {
    const size_t need = fixed + per_chunk * nslices;
    return fail(ctx, MMO_EINVAL,
                "mmo_score_poses_noalloc: %d poses of %d atoms need %zu bytes of scratch, above "
                "the %zu-byte static scratch; score fewer poses per call",
                B, L, need, kNoAllocBytes);
  }
  unsigned char* base = nullptr;
  int r = noalloc_scratch(ctx, ctx->device, &base);
  if (r) return r;
  MMO_CK(cudaSetDevice(ctx->device), "set device");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  PairPlan plan{};
  int C = 1;
  if (inter && !use_grid) {
    plan = plan_for(ctx, B, grad);
    const int c_slice = std::max(1, std::min(plan.C / nslices, (int)(c_fit / nslices)));
    C = c_slice * nslices;
    const long npb = (B + 32L * plan.kp - 1) / (32L * plan.kp);
    const long need = (npb * L * c_slice + plan.threads / 32 - 1) / (plan.threads / 32);
    plan.C = C;
    plan.blocks = (int)std::max(1L, std::min((long)plan.blocks, need));
  }
  size_t off = 0;
  Scratch s{};
  s.X = reinterpret_cast<float4*>(base + take(off, sizeof(float4) * 2 * (size_t)B * L));
  off = (off + 255) & ~size_t(255);
  if (grad) {
    s.Y = reinterpret_cast<float4*>(base + take(off, sizeof(float4) * 2 * (size_t)B * L));
    off = (off + 255) & ~size_t(255);
    s.rec = reinterpret_cast<float4*>(base + take(off, sizeof(float4) * 3 * (size_t)B * nrb));
    off = (off + 255) & ~size_t(255);
    s.cen = reinterpret_cast<float4*>(base + take(off, sizeof(float4) * 2 * (size_t)B));
    off = (off + 255) & ~size_t(255);
  }
  s.Epart = reinterpret_cast<double*>(base + take(off, sizeof(double) * (size_t)B * C * L));
  off = (off + 255) & ~size_t(255);
  s.Gpart = grad ? reinterpret_cast<float4*>(base + take(off, sizeof(float4) * (size_t)B * C * L))
                 : nullptr;
  s.C = C;
  if (off > kNoAllocBytes) return fail(ctx, MMO_EINVAL, "mmo_score_poses_noalloc: layout overflow");
  PoseIO io{};
  io.dofs = d_dofs;
  io.E = d_E;
  io.grad = grad ? d_grad : nullptr;
  io.status = d_status;
  io.err = ctx->d_err;
  io.zero_err = 0;
  io.B = B;
  io.ox = ctx->origin_f[0];
  io.oy = ctx->origin_f[1];
  io.oz = ctx->origin_f[2];
  int fl = flags & (kFlagInter | kFlagIntra | kFlagGrad | kFlagRecenter);
  if (!inter) fl &= ~kFlagInter;
  // every region a kernel reads is written first in this call: X, Y, the
  // torsion records and the centroids by the rebuild, each (pose, chunk,
  // atom) partial by the pair sweep or the grid lookup
  MMO_CK(launch_rebuild(ctx->lig, io, s, fl, st), "rebuild kernel");
  if (use_grid)
    MMO_CK(launch_grid_inter(grid_look(ctx), s.X, B * L, L, ctx->d_grid_lt, ctx->d_grid, s.Epart,
                             grad ? s.Gpart : nullptr, d_status, grad, st),
           "grid lookup kernel");
  else if (inter)
    MMO_CK(launch_pairs_batched(ctx->prot, ctx->d_tab4, ctx->lig, s, B, fl, ctx->ph, plan,
                                ctx->d_err, st),
           "batched pair kernel");
  MMO_CK(launch_finish(ctx->lig, io, s, fl, ctx->ph, st), "finish kernel");
  return MMO_OK;
}

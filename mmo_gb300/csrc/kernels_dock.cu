// kernels_dock.cu -- the clients of the scorer around a binding site:
//
// * k_masks: the protein's vdW volume and first solvent shell on the grids'
//   lattice (Lds.vdW_volume, Lds.first_solvent_shell; UnixJunkie/MMO
//   src/lds.ml:149-196): a point is in the volume when it is within r_i of an
//   atom, in the shell when it is within r_i + r_w of an atom and in no volume;
// * k_clash: per pose, Mol.ligand_atoms_clash_fast (src/mol.ml:1077-1088),
//   Mol.heavy_atom_clash (src/mol.ml:1170-1190) and Mol.protein_ligand_clash
//   (src/mol.ml:1195-1207, G3D.vdW_clash_OR src/G3D.ml:159-185);
// * k_dock + k_topk_merge: Lds.exhaustive_rigid_ligand_docking
//   (src/lds.ml:1040-1114), every (position, rotation) pose of the ROI's
//   translation lattice scored by grid interpolation after the vdW clash test,
//   and the k lowest scores;
// * k_place: Lds.place_ligand_in_ROI (src/lds.ml:308-345), candidate random
//   placements tested for heavy-atom clashes in parallel;
// * k_prot_desolv, k_desolv_pose: Lds.protein_desolv and
//   Lds.desolvation_penalty (src/lds.ml:198-267).
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kList = 64;   // compacted atoms per warp
constexpr int kWarps = 8;   // warps per CTA of the lattice kernels
constexpr double kPiD = 3.14159265358979323846;
constexpr int kDockAtoms = 4;  // atoms of a pose in flight together

__device__ __forceinline__ float wmin(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ float wmax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// G3D's eight corners of the cell of lattice coordinate u (device frame,
// in steps): a corner off the lattice counts as not set.  Returns the OR and
// writes the AND of the corners' mask bytes.
__device__ __forceinline__ bool corners(const GridLook& g, const uint8_t* mask, double u, double v,
                                        double w, bool* all) {
  bool any = false, every = true;
  const bool ok = u > -1.0 && v > -1.0 && w > -1.0 && u < 2e9 && v < 2e9 && w < 2e9;
  const int i0 = ok ? (int)u : 0, j0 = ok ? (int)v : 0, k0 = ok ? (int)w : 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int i = i0 + (c & 1), j = j0 + ((c >> 1) & 1), k = k0 + (c >> 2);
    bool bit = false;
    if (ok && i < g.nx && j < g.ny && k < g.nz)
      bit = mask[i + (size_t)j * g.nx + (size_t)k * g.nx * g.ny] != 0;
    any = any || bit;
    every = every && bit;
  }
  *all = every;
  return any;
}

// ---- masks ------------------------------------------------------------------
// A warp per 4 x 4 x 2 tile of points; the protein atoms whose sphere of
// r_i + r_w meets the tile's box are staged in the warp's list.  A distance
// within 1e-4 (relative) of a sphere is decided again in FP64.
__global__ void __launch_bounds__(kWarps * 32) k_masks(DevCull cull, MaskBuild mb,
                                                       const double* radius64, uint8_t* vdw,
                                                       uint8_t* shell) {
  __shared__ float4 s_list[kWarps][kList][2];
  __shared__ int s_idx[kWarps][kList];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tx_n = (mb.nx + 3) / 4, ty_n = (mb.ny + 3) / 4, tz_n = (mb.nz + 1) / 2;
  const long long tile = (long long)blockIdx.x * kWarps + w;
  if (tile >= (long long)tx_n * ty_n * tz_n) return;
  const int tx = (int)(tile % tx_n), ty = (int)((tile / tx_n) % ty_n),
            tz = (int)(tile / ((long long)tx_n * ty_n));
  const int i = tx * 4 + (lane & 3), j = ty * 4 + ((lane >> 2) & 3), k = tz * 2 + (lane >> 4);
  const bool in = i < mb.nx && j < mb.ny && k < mb.nz;
  const double px = mb.o[0] + mb.step * i, py = mb.o[1] + mb.step * j, pz = mb.o[2] + mb.step * k;
  const float xh = (float)px, yh = (float)py, zh = (float)pz;
  const float xl = (float)(px - xh), yl = (float)(py - yh), zl = (float)(pz - zh);
  const float big = 1e30f;
  const float blx = wmin(in ? xh : big), bly = wmin(in ? yh : big), blz = wmin(in ? zh : big);
  const float bhx = wmax(in ? xh : -big), bhy = wmax(in ? yh : -big), bhz = wmax(in ? zh : -big);
  const float R = mb.r_max + mb.r_w + 1e-3f;
  bool in_vdw = false, in_out = false;
  float4(*wl)[2] = s_list[w];
  int* wi = s_idx[w];
  auto evaluate = [&](int n) {
    __syncwarp();
    for (int v = 0; v < n; ++v) {
      const float4 p = wl[v][0], pl = wl[v][1];
      const float dx = (xh - p.x) + (xl - pl.x);
      const float dy = (yh - p.y) + (yl - pl.y);
      const float dz = (zh - p.z) + (zl - pl.z);
      const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
      const float r = p.w, ro = p.w + mb.r_w;
      const float ri2 = r * r, ro2 = ro * ro;
      bool a = d2 < ri2, b = d2 < ro2;
      if (fabsf(d2 - ri2) < 1e-4f * ri2 || fabsf(d2 - ro2) < 1e-4f * ro2) {
        const double r64 = radius64[wi[v]];
        const double ex = px - ((double)p.x + (double)pl.x), ey = py - ((double)p.y + (double)pl.y),
                     ez = pz - ((double)p.z + (double)pl.z);
        const double e2 = ex * ex + ey * ey + ez * ez;
        a = e2 < r64 * r64;
        b = e2 < (r64 + (double)mb.r_w) * (r64 + (double)mb.r_w);
      }
      in_vdw = in_vdw || a;
      in_out = in_out || b;
    }
    __syncwarp();
  };
  for (int r = 0; r < cull.nrows; ++r) {
    const float4 rb = cull.row_box[r];
    const float ey = fmaxf(fmaxf(rb.x - bhy, bly - rb.y), 0.f);
    const float ez = fmaxf(fmaxf(rb.z - bhz, blz - rb.w), 0.f);
    if (fmaf(ey, ey, ez * ez) >= R * R) continue;
    const int a = cull.row_start[r], b = cull.row_start[r + 1];
    int cnt = 0;
    for (int i0 = a; i0 < b; i0 += 32) {
      const int ia = i0 + lane;
      bool take = false;
      float4 ph = make_float4(0.f, 0.f, 0.f, 0.f);
      float ra = 0.f;
      if (ia < b) {
        ph = cull.atoms[2 * (size_t)ia];
        ra = mb.radius[ia] + mb.r_w + 1e-3f;
        const float ex = fmaxf(fmaxf(blx - ph.x, ph.x - bhx), 0.f);
        const float fy = fmaxf(fmaxf(bly - ph.y, ph.y - bhy), 0.f);
        const float fz = fmaxf(fmaxf(blz - ph.z, ph.z - bhz), 0.f);
        take = fmaf(ex, ex, fmaf(fy, fy, fz * fz)) < ra * ra;
      }
      const unsigned m = __ballot_sync(kFull, take);
      if (take) {
        const int at = cnt + __popc(m & ((1u << lane) - 1u));
        wl[at][0] = make_float4(ph.x, ph.y, ph.z, mb.radius[ia]);
        wl[at][1] = cull.atoms[2 * (size_t)ia + 1];
        wi[at] = ia;
      }
      cnt += __popc(m);
      if (cnt >= 32) {
        evaluate(cnt);
        cnt = 0;
      }
    }
    evaluate(cnt);
  }
  if (!in) return;
  const size_t idx = (size_t)i + (size_t)j * mb.nx + (size_t)k * mb.nx * mb.ny;
  if (vdw) vdw[idx] = in_vdw ? 1 : 0;
  if (shell) shell[idx] = (in_out && !in_vdw) ? 1 : 0;
}

// Per cell (i, j, k) of the lattice: bit 0 = any of its eight corners in the
// mask (G3D.vdW_clash_OR), bit 1 = all of them (vdW_clash_AND); corners off the
// lattice count as not set.
__global__ void k_cell_masks(GridLook g, const uint8_t* __restrict__ mask, uint8_t* cell) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)g.nx * g.ny * g.nz;
  if (t >= n) return;
  const int i = (int)(t % g.nx), j = (int)((t / g.nx) % g.ny), k = (int)(t / ((long long)g.nx * g.ny));
  bool any = false, every = true;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int ii = i + (c & 1), jj = j + ((c >> 1) & 1), kk = k + (c >> 2);
    const bool bit = ii < g.nx && jj < g.ny && kk < g.nz &&
                     mask[ii + (size_t)jj * g.nx + (size_t)kk * g.nx * g.ny] != 0;
    any = any || bit;
    every = every && bit;
  }
  cell[t] = (any ? 1 : 0) | (every ? 2 : 0);
}

// ---- clash tests of posed ligands ------------------------------------------------
// Protein heavy atoms within kHeavyClashMax of (x, y, z) (device frame) that
// clash with a ligand atom of type lt: rows whose (y, z) box is that close,
// atoms of a row sorted by x.
__device__ bool heavy_clash_at(const DevCull& cull, const float* c2, const uint8_t* heavy,
                               float x, float xl, float y, float yl, float z, float zl, int lt) {
  const float R = kHeavyClashMax + 1e-3f;
  for (int r = 0; r < cull.nrows; ++r) {
    const float4 rb = cull.row_box[r];
    const float ey = fmaxf(fmaxf(rb.x - y, y - rb.y), 0.f);
    const float ez = fmaxf(fmaxf(rb.z - z, z - rb.w), 0.f);
    if (fmaf(ey, ey, ez * ez) >= R * R) continue;
    for (int ia = cull.row_start[r]; ia < cull.row_start[r + 1]; ++ia) {
      const float4 p = cull.atoms[2 * (size_t)ia];
      if (p.x < x - R) continue;
      if (p.x > x + R) break;
      const float4 pl = cull.atoms[2 * (size_t)ia + 1];
      const int pt = __float_as_int(pl.w) / (16 * kNTypes);
      if (!heavy[pt]) continue;
      const float dx = (x - p.x) + (xl - pl.x), dy = (y - p.y) + (yl - pl.y),
                  dz = (z - p.z) + (zl - pl.z);
      if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < c2[lt * kNTypes + pt]) return true;
    }
  }
  return false;
}

__global__ void __launch_bounds__(256) k_clash(DevLigand lig, const float4* X, int B, DevCull cull,
                                               ClashArgs ca, int* out) {
  __shared__ float s_c2[kNTypes * kNTypes];
  __shared__ uint8_t s_heavy[kNTypes];
  for (int t = threadIdx.x; t < kNTypes * kNTypes; t += blockDim.x) s_c2[t] = ca.clash2[t];
  if (threadIdx.x < kNTypes) s_heavy[threadIdx.x] = ca.heavy[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (b >= B) return;
  const int L = lig.L;
  const float4* Xb = X + (size_t)b * L * 2;
  bool intra = false, heavy = false, grid = false;
  if (ca.tests & kClashIntra) {
    for (int p = lane; p < lig.npairs; p += 32) {
      const int2 ij = lig.pair_ij[p];
      const float4 ah = Xb[2 * ij.x], al = Xb[2 * ij.x + 1], bh = Xb[2 * ij.y], bl = Xb[2 * ij.y + 1];
      const float dx = split_diff(ah.x, al.x, bh.x, bl.x), dy = split_diff(ah.y, al.y, bh.y, bl.y),
                  dz = split_diff(ah.z, al.z, bh.z, bl.z);
      if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) < s_c2[lig.type[ij.x] * kNTypes + lig.type[ij.y]])
        intra = true;
    }
  }
  for (int a = lane; a < L; a += 32) {
    const float4 h = Xb[2 * a], l = Xb[2 * a + 1];
    if ((ca.tests & kClashGrid) && ca.vdw) {
      bool all;
      const double u = ((double)h.x + (double)l.x - ca.g.o[0]) * ca.g.inv;
      const double v = ((double)h.y + (double)l.y - ca.g.o[1]) * ca.g.inv;
      const double w = ((double)h.z + (double)l.z - ca.g.o[2]) * ca.g.inv;
      grid = grid || corners(ca.g, ca.vdw, u, v, w, &all);
    }
    if ((ca.tests & kClashHeavy) && !heavy && s_heavy[lig.type[a]])
      heavy = heavy_clash_at(cull, s_c2, s_heavy, h.x, l.x, h.y, l.y, h.z, l.z, lig.type[a]);
  }
  const unsigned bi = __ballot_sync(kFull, intra), bh = __ballot_sync(kFull, heavy),
                 bg = __ballot_sync(kFull, grid);
  if (lane == 0)
    out[b] = (bi ? kClashIntra : 0) | (bh ? kClashHeavy : 0) | (bg ? kClashGrid : 0);
}

// ---- exhaustive docking ---------------------------------------------------------
// (score, frame) keys: a double as an unsigned integer in the same order
__device__ __forceinline__ unsigned long long sort_key(double s) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(s);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// ascending bitonic sort of n (a power of 2) (key, frame) pairs in shared memory
__device__ void block_sort(unsigned long long* sk, unsigned long long* sf, int n) {
  for (int size = 2; size <= n; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
        const int pos = 2 * stride * (t / stride) + (t % stride), par = pos + stride;
        const bool up = (pos & size) == 0;
        const unsigned long long ka = sk[pos], kb = sk[par], fa = sf[pos], fb = sf[par];
        const bool gt = ka > kb || (ka == kb && fa > fb);
        if (gt == up) {
          sk[pos] = kb;
          sk[par] = ka;
          sf[pos] = fb;
          sf[par] = fa;
        }
      }
    }
  __syncthreads();
}

// The rotated ligand in lattice units, once per (rotation, atom):
// off[r][a] = R_r x_a / step as float pairs (hi x, y, z, lo x, y, z); rotation
// and scaling in FP64.
__global__ void k_dock_offsets(DockArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < a.npos) {
    // the position's lattice coordinate: cell and float-pair fraction per axis
    const int pi = a.pos_idx[t];
    const int ii = pi % a.pdim, jj = (pi / a.pdim) % a.pdim, kk = pi / (a.pdim * a.pdim);
    const double up[3] = {(a.p0[0] + a.pstep * ii - a.g.o[0]) * a.g.inv,
                          (a.p0[1] + a.pstep * jj - a.g.o[1]) * a.g.inv,
                          (a.p0[2] + a.pstep * kk - a.g.o[2]) * a.g.inv};
    float4* P = a.pcell + 2 * (size_t)t;
    float v[6];
    int c[3];
    for (int d = 0; d < 3; ++d) {
      const double fu = floor(up[d]);
      c[d] = (int)fu;
      const double w = up[d] - fu;
      v[d] = (float)w;
      v[3 + d] = (float)(w - v[d]);
    }
    P[0] = make_float4(v[0], v[1], v[2], __int_as_float(c[0]));
    P[1] = make_float4(v[3], v[4], v[5], 0.f);
    a.pcell_k[2 * (size_t)t] = c[1];
    a.pcell_k[2 * (size_t)t + 1] = c[2];
  }
  if (t >= a.nrot * a.L) return;
  const int r = t / a.L, at = t % a.L;
  const double* M = a.rot + 9 * (size_t)r;
  const double rx = a.ref[3 * at], ry = a.ref[3 * at + 1], rz = a.ref[3 * at + 2];
  const double u[3] = {(M[0] * rx + M[1] * ry + M[2] * rz) * a.g.inv,
                       (M[3] * rx + M[4] * ry + M[5] * rz) * a.g.inv,
                       (M[6] * rx + M[7] * ry + M[8] * rz) * a.g.inv};
  float* o = a.off + 6 * (size_t)t;
  for (int d = 0; d < 3; ++d) {
    const float h = (float)u[d];
    o[d] = h;
    o[3 + d] = (float)(u[d] - h);
  }
}

// Cell of the lattice coordinate iu + (fh + fl) + (oh + ol): i = floor, w the
// fraction in [0, 1), from float pairs (TwoSum of the high parts, the low parts
// added); exact to about 1e-13 cells for |offsets| below 2^20.
__device__ __forceinline__ void cell_of(int iu, float fh, float fl, float oh, float ol, int& i,
                                        float& w) {
  const float s = __fadd_rn(fh, oh);
  const float bp = __fsub_rn(s, fh), ap = __fsub_rn(s, bp);
  const float e = __fadd_rn(__fsub_rn(fh, ap), __fsub_rn(oh, bp));
  const float lo = __fadd_rn(e, __fadd_rn(fl, ol));
  const float f = floorf(s);
  float frac = __fadd_rn(__fsub_rn(s, f), lo);
  int k = (int)f;
  if (frac < 0.f) {
    frac = __fadd_rn(frac, 1.f);
    --k;
  } else if (frac >= 1.f) {
    frac = __fsub_rn(frac, 1.f);
    ++k;
  }
  if (frac >= 1.f) frac = 0.99999994f;  // a rounding of (1 - tiny) + 1 back to 1
  i = iu + k;
  w = frac;
}

// G3D's eight corners of the cell (i, w) per axis (u = i + w), from the cell
// masks of k_cell_masks: the corner index truncates u toward zero
// (int_of_float), so u in (-1, 0) uses cell 0 and u <= -1 none; a cell off the
// lattice has no corner set.  Returns the mask bits (1: any, 2: all).
__device__ __forceinline__ int cell_bits(const GridLook& g, const uint8_t* __restrict__ cell,
                                         int i, float wi, int j, float wj, int k, float wk) {
  const bool ok = (i >= 0 || (i == -1 && wi > 0.f)) && (j >= 0 || (j == -1 && wj > 0.f)) &&
                  (k >= 0 || (k == -1 && wk > 0.f));
  const int i0 = max(i, 0), j0 = max(j, 0), k0 = max(k, 0);
  if (!ok || i0 >= g.nx || j0 >= g.ny || k0 >= g.nz) return 0;
  return cell[i0 + (size_t)j0 * g.nx + (size_t)k0 * g.nx * g.ny];
}

// A CTA per tile of rtile rotations x (kDockPerBlock / rtile) positions (the
// tile's rotated atoms staged in shared memory; a warp's poses share a
// position, so their lookups fall near each other).  One thread per pose: the
// position's lattice coordinate split (FP64, once per position) into a cell
// and a float-pair fraction, each atom's cell from the rotation's
// offsets (float pairs), the eight-corner vdW test of every atom (a clash ends
// the pose), then the trilinear interpolation of the atom's grid (FP32 weights
// and values, a compensated FP32 sum over the atoms).
__global__ void __launch_bounds__(kDockBlock) k_dock(DockArgs a) {
  extern __shared__ unsigned long long dsm[];
  unsigned long long* sk = dsm;
  unsigned long long* sf = dsm + kDockPerBlock;
  float* s_off = reinterpret_cast<float*>(dsm + 2 * kDockPerBlock);  // [rtile][L][6]
  __shared__ int s_t[kMaxLig];
  __shared__ unsigned s_cnt[2];
  // the block's tile: rotations [r0, r0 + rtile) x positions [p0, p0 + ptile)
  const int R = a.rtile, Pt = kDockPerBlock / a.rtile;
  const int npb = (a.npos + Pt - 1) / Pt;
  const int r0 = (blockIdx.x / npb) * R, p0 = (blockIdx.x % npb) * Pt;
  const int nr = min(R, a.nrot - r0);
  for (int t = threadIdx.x; t < a.L; t += blockDim.x) s_t[t] = a.lig_type[t];
  for (int t = threadIdx.x; t < nr * a.L * 6; t += blockDim.x)
    s_off[t] = a.off[6 * (size_t)r0 * a.L + t];
  if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t nxy = (size_t)a.g.nx * a.g.ny, per = nxy * a.g.nz;
  unsigned scored = 0, clashed = 0;
  for (int q = 0; q < kDockPerBlock / kDockBlock; ++q) {
    const int slot = q * kDockBlock + threadIdx.x;
    const int rl = slot % R, ps = p0 + slot / R, r = r0 + rl;
    unsigned long long key = ~0ull, fr = ~0ull;
    if (rl < nr && ps < a.npos) {
      const int pi = a.pos_idx[ps];
      fr = (unsigned long long)pi * (unsigned long long)a.nrot + (unsigned long long)r;
      const float4 P0 = a.pcell[2 * (size_t)ps], P1 = a.pcell[2 * (size_t)ps + 1];
      const int iu[3] = {__float_as_int(P0.w), a.pcell_k[2 * (size_t)ps],
                         a.pcell_k[2 * (size_t)ps + 1]};
      const float fh[3] = {P0.x, P0.y, P0.z}, fl[3] = {P1.x, P1.y, P1.z};
      bool skip = false;
      if (a.center_occ)
        skip = (cell_bits(a.g, a.vcell, iu[0], fh[0], iu[1], fh[1], iu[2], fh[2]) & 2) != 0;
      if (!skip) {
        const float* off = s_off + 6 * (size_t)rl * a.L;
        float eh = 0.f, el = 0.f;  // compensated sum over the atoms (Neumaier)
        bool clash = false;
        // kDockAtoms atoms at a time: their loads are independent and overlap
        for (int at = 0; at < a.L && !clash; at += kDockAtoms) {
          const int na = min(kDockAtoms, a.L - at);
          int ci[kDockAtoms][3];
          float cw[kDockAtoms][3];
          int bits[kDockAtoms];
          int anyb = 0;
#pragma unroll
          for (int u = 0; u < kDockAtoms; ++u) {
            bits[u] = 0;
            if (u < na) {
              const float* o = off + 6 * (at + u);
#pragma unroll
              for (int d = 0; d < 3; ++d)
                cell_of(iu[d], fh[d], fl[d], o[d], o[3 + d], ci[u][d], cw[u][d]);
              bits[u] = cell_bits(a.g, a.vcell, ci[u][0], cw[u][0], ci[u][1], cw[u][1], ci[u][2],
                                  cw[u][2]);
            }
            anyb |= bits[u];
          }
          if (anyb & 1) {
            clash = true;
            break;
          }
#pragma unroll
          for (int u = 0; u < kDockAtoms; ++u) {
            if (u < na && ci[u][0] >= 0 && ci[u][1] >= 0 && ci[u][2] >= 0 &&
                ci[u][0] <= a.g.nx - 2 && ci[u][1] <= a.g.ny - 2 && ci[u][2] <= a.g.nz - 2) {
              const float* gv = a.grids + per * s_t[at + u] + ci[u][0] + (size_t)ci[u][1] * a.g.nx +
                                ci[u][2] * nxy;
              const float wx = cw[u][0], wy = cw[u][1], wz = cw[u][2];
              const float hx = 1.f - wx, hy = 1.f - wy, hz = 1.f - wz;
              const float c00 = fmaf(gv[1], wx, gv[0] * hx);
              const float c10 = fmaf(gv[1 + a.g.nx], wx, gv[a.g.nx] * hx);
              const float c01 = fmaf(gv[1 + nxy], wx, gv[nxy] * hx);
              const float c11 = fmaf(gv[1 + a.g.nx + nxy], wx, gv[a.g.nx + nxy] * hx);
              const float c0 = fmaf(c10, wy, c00 * hy), c1 = fmaf(c11, wy, c01 * hy);
              const float t = fmaf(c1, wz, c0 * hz);
              const float sum = __fadd_rn(eh, t);
              el = __fadd_rn(el, fabsf(eh) >= fabsf(t) ? __fadd_rn(__fsub_rn(eh, sum), t)
                                                       : __fadd_rn(__fsub_rn(t, sum), eh));
              eh = sum;
            }
          }
        }
        if (clash) {
          ++clashed;
        } else {
          ++scored;
          key = sort_key(a.const_intra + ((double)eh + (double)el));
        }
      }
    }
    sk[slot] = key;
    sf[slot] = fr;
  }
  for (int o = 16; o > 0; o >>= 1) {
    scored += __shfl_xor_sync(kFull, scored, o);
    clashed += __shfl_xor_sync(kFull, clashed, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_cnt[0], scored);
    atomicAdd(&s_cnt[1], clashed);
  }
  block_sort(sk, sf, kDockPerBlock);
  for (int t = threadIdx.x; t < a.k; t += blockDim.x) {
    a.cand[2 * ((size_t)blockIdx.x * a.k + t)] = sk[t];
    a.cand[2 * ((size_t)blockIdx.x * a.k + t) + 1] = sf[t];
  }
  if (threadIdx.x == 0) {
    atomicAdd(a.counts, (unsigned long long)s_cnt[0]);
    atomicAdd(a.counts + 1, (unsigned long long)s_cnt[1]);
  }
}

// the k smallest of each group of kDockPerBlock candidates
__global__ void __launch_bounds__(kDockBlock) k_topk_merge(const unsigned long long* in, int n,
                                                           int k, unsigned long long* out) {
  extern __shared__ unsigned long long dsm[];
  unsigned long long* sk = dsm;
  unsigned long long* sf = dsm + kDockPerBlock;
  const size_t base = (size_t)blockIdx.x * kDockPerBlock;
  for (int t = threadIdx.x; t < kDockPerBlock; t += blockDim.x) {
    const size_t g = base + t;
    sk[t] = g < (size_t)n ? in[2 * g] : ~0ull;
    sf[t] = g < (size_t)n ? in[2 * g + 1] : ~0ull;
  }
  block_sort(sk, sf, kDockPerBlock);
  for (int t = threadIdx.x; t < k; t += blockDim.x) {
    out[2 * ((size_t)blockIdx.x * k + t)] = sk[t];
    out[2 * ((size_t)blockIdx.x * k + t) + 1] = sf[t];
  }
}

// ---- placement in the ROI ---------------------------------------------------------
// Rot.rx / ry / rz (src/rot.ml:22-46)
__device__ void axis_rot(int axis, double th, double R[9]) {
  double s, c;
  sincos(th, &s, &c);
  for (int m = 0; m < 9; ++m) R[m] = 0.0;
  if (axis == 0) {
    R[0] = 1.0; R[4] = c; R[5] = s; R[7] = -s; R[8] = c;
  } else if (axis == 1) {
    R[0] = c; R[2] = -s; R[4] = 1.0; R[6] = s; R[8] = c;
  } else {
    R[0] = c; R[1] = s; R[3] = -s; R[4] = c; R[8] = 1.0;
  }
}

__device__ void mat_mul(const double A[9], const double B[9], double C[9]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
}

// One thread per candidate (slot, c): a point uniform in the ROI's cube
// (Bbox.rand_point_inside) kept when inside the sphere, a rotation
// Move.rand_rot_full (three rotations by angles uniform in [-pi, pi] about
// Ox, Oy or Oz, src/move.ml:20-39), kept when no ligand heavy atom clashes
// with a protein heavy atom.  Random numbers: Philox4x32-10, counter
// (slot, c, draw, 1), key = the seed.
__global__ void __launch_bounds__(128) k_place(PlaceArgs a, DevCull cull, ClashArgs ca) {
  __shared__ float s_c2[kNTypes * kNTypes];
  __shared__ uint8_t s_heavy[kNTypes];
  for (int t = threadIdx.x; t < kNTypes * kNTypes; t += blockDim.x) s_c2[t] = ca.clash2[t];
  if (threadIdx.x < kNTypes) s_heavy[threadIdx.x] = ca.heavy[threadIdx.x];
  __syncthreads();
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)a.slots * a.per_slot) return;
  const int s = a.slot_id[tid / a.per_slot];
  const uint32_t c = (uint32_t)(a.c0 + tid % a.per_slot);
  uint4 r[4];
#pragma unroll
  for (int d = 0; d < 4; ++d) r[d] = philox(make_uint4((uint32_t)s, c, (uint32_t)d, 1u), a.key0, a.key1);
  const double px = a.c[0] - a.r + 2.0 * a.r * u01(r[0].x, r[0].y);
  const double py = a.c[1] - a.r + 2.0 * a.r * u01(r[0].z, r[0].w);
  const double pz = a.c[2] - a.r + 2.0 * a.r * u01(r[1].x, r[1].y);
  float* o = a.out + 7 * (size_t)tid;
  const double dx = px - a.c[0], dy = py - a.c[1], dz = pz - a.c[2];
  bool ok = dx * dx + dy * dy + dz * dz < a.r * a.r;
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, M[9], T[9];
  const double th[3] = {(2.0 * u01(r[1].z, r[1].w) - 1.0) * kPiD,
                        (2.0 * u01(r[2].x, r[2].y) - 1.0) * kPiD,
                        (2.0 * u01(r[2].z, r[2].w) - 1.0) * kPiD};
  const int ax[3] = {min(2, (int)(u01(r[3].x, r[3].y) * 3.0)),
                     min(2, (int)(u01(r[3].z, r[3].w) * 3.0)),
                     min(2, (int)(u01(r[3].y, r[3].x) * 3.0))};
  for (int m = 0; m < 3; ++m) {
    axis_rot(ax[m], th[m], M);
    mat_mul(M, R, T);  // rotations apply right to left
    for (int e = 0; e < 9; ++e) R[e] = T[e];
  }
  for (int at = 0; at < a.L && ok; ++at) {
    if (!s_heavy[a.type[at]]) continue;
    const double rx = a.ref[3 * at], ry = a.ref[3 * at + 1], rz = a.ref[3 * at + 2];
    const double x = R[0] * rx + R[1] * ry + R[2] * rz + px;
    const double y = R[3] * rx + R[4] * ry + R[5] * rz + py;
    const double z = R[6] * rx + R[7] * ry + R[8] * rz + pz;
    const float xh = (float)x, yh = (float)y, zh = (float)z;
    if (heavy_clash_at(cull, s_c2, s_heavy, xh, (float)(x - xh), yh, (float)(y - yh), zh,
                       (float)(z - zh), a.type[at]))
      ok = false;
  }
  // Rot.decompose (src/rot.ml:71-75)
  const double beta = atan2(-R[6], sqrt(R[0] * R[0] + R[3] * R[3]));
  const double icb = 1.0 / cos(beta);
  o[0] = (float)px;
  o[1] = (float)py;
  o[2] = (float)pz;
  o[3] = (float)atan2(R[7] * icb, R[8] * icb);
  o[4] = (float)beta;
  o[5] = (float)atan2(R[3] * icb, R[0] * icb);
  o[6] = ok ? 1.f : 0.f;
}

// ---- desolvation ------------------------------------------------------------------
// Per point of the protein's solvent shell inside the ROI: C vol sum_j
// (q_j / d^2)^2 over the protein atoms within 12 A (the atoms carry K q; the
// scale holds 1 / K^2).  A warp per 4 x 4 x 2 tile, atoms listed through the
// row index, per-row FP32 sums added in FP64.
__global__ void __launch_bounds__(kWarps * 32) k_prot_desolv(DevCull cull, DesolvBuild db,
                                                             double* out) {
  __shared__ float4 s_list[kWarps][kList][2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * kWarps + w;
  if (tile >= db.ntiles) return;
  const int3 t = db.tiles[tile];
  const int i = t.x * 4 + (lane & 3), j = t.y * 4 + ((lane >> 2) & 3), k = t.z * 2 + (lane >> 4);
  const bool in = i < db.nx && j < db.ny && k < db.nz;
  const size_t idx = (size_t)i + (size_t)j * db.nx + (size_t)k * db.nx * db.ny;
  const double px = db.o[0] + db.step * i, py = db.o[1] + db.step * j, pz = db.o[2] + db.step * k;
  const double mx = px - db.c[0], my = py - db.c[1], mz = pz - db.c[2];
  const bool act = in && db.shell[idx] && mx * mx + my * my + mz * mz < db.r2;
  if (!__any_sync(kFull, act)) return;
  const float xh = (float)px, yh = (float)py, zh = (float)pz;
  const float xl = (float)(px - xh), yl = (float)(py - yh), zl = (float)(pz - zh);
  const float big = 1e30f;
  const float blx = wmin(act ? xh : big), bly = wmin(act ? yh : big), blz = wmin(act ? zh : big);
  const float bhx = wmax(act ? xh : -big), bhy = wmax(act ? yh : -big), bhz = wmax(act ? zh : -big);
  double acc = 0.0;
  float4(*wl)[2] = s_list[w];
  for (int r = 0; r < cull.nrows; ++r) {
    const float4 rb = cull.row_box[r];
    const float ey = fmaxf(fmaxf(rb.x - bhy, bly - rb.y), 0.f);
    const float ez = fmaxf(fmaxf(rb.z - bhz, blz - rb.w), 0.f);
    if (fmaf(ey, ey, ez * ez) >= kCullR2) continue;
    const int a = cull.row_start[r], b = cull.row_start[r + 1];
    float racc = 0.f;
    int cnt = 0;
    for (int i0 = a; i0 < b; i0 += 32) {
      const int ia = i0 + lane;
      bool take = false;
      float4 ph = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ia < b) {
        ph = cull.atoms[2 * (size_t)ia];
        const float ex = fmaxf(fmaxf(blx - ph.x, ph.x - bhx), 0.f);
        const float fy = fmaxf(fmaxf(bly - ph.y, ph.y - bhy), 0.f);
        const float fz = fmaxf(fmaxf(blz - ph.z, ph.z - bhz), 0.f);
        take = fmaf(ex, ex, fmaf(fy, fy, fz * fz)) < kCullR2;
      }
      const unsigned m = __ballot_sync(kFull, take);
      if (take) {
        const int at = cnt + __popc(m & ((1u << lane) - 1u));
        wl[at][0] = ph;
        wl[at][1] = cull.atoms[2 * (size_t)ia + 1];
      }
      cnt += __popc(m);
      if (cnt >= 32 || i0 + 32 >= b) {
        __syncwarp();
        for (int v = 0; v < cnt; ++v) {
          const float4 p = wl[v][0], pl = wl[v][1];
          const float dx = (xh - p.x) + (xl - pl.x), dy = (yh - p.y) + (yl - pl.y),
                      dz = (zh - p.z) + (zl - pl.z);
          const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          const float x = p.w / d2;
          racc += d2 < kCut2 ? x * x : 0.f;
        }
        __syncwarp();
        cnt = 0;
      }
    }
    acc += (double)racc;
  }
  if (act) out[idx] = db.scale * acc;
}

// A block per pose: the pose's solvent shell (points within r_a + r_w of an
// atom and within r_b of none) on a box of the lattice about the pose, as two
// bit masks in shared memory filled from each atom's cube of cells (as
// Lds.atom_bitmask_set), then every point of both shells: the protein's
// contribution and C vol sum_a (q_a / d^2)^2 over the atoms within 12 A.
__global__ void __launch_bounds__(256) k_desolv_pose(DesolvPose d) {
  extern __shared__ unsigned bsm[];
  const int words = (d.cap + 31) / 32;
  unsigned* outer = bsm;
  unsigned* inner = bsm + words;
  __shared__ double s_x[kMaxLig], s_y[kMaxLig], s_z[kMaxLig], s_r[kMaxLig];
  __shared__ float s_q[kMaxLig];
  __shared__ int s_lo[3], s_n[3], s_ok;
  __shared__ double s_red[2][8];
  const int b = blockIdx.x, L = d.L;
  if (b >= d.B) return;
  for (int a = threadIdx.x; a < L; a += blockDim.x) {
    const float4 h = d.X[2 * ((size_t)b * L + a)], l = d.X[2 * ((size_t)b * L + a) + 1];
    s_x[a] = (double)h.x + (double)l.x;
    s_y[a] = (double)h.y + (double)l.y;
    s_z[a] = (double)h.z + (double)l.z;
    s_r[a] = d.radius[a];
    s_q[a] = d.q[a];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int a = 0; a < L; ++a) {
      const double p[3] = {s_x[a], s_y[a], s_z[a]}, rr = s_r[a] + d.r_w;
      for (int q = 0; q < 3; ++q) {
        lo[q] = fmin(lo[q], p[q] - rr);
        hi[q] = fmax(hi[q], p[q] + rr);
      }
    }
    const int nn[3] = {d.g.nx, d.g.ny, d.g.nz};
    long long tot = 1;
    for (int q = 0; q < 3; ++q) {
      const double a0 = floor((lo[q] - d.g.o[q]) * d.g.inv) - 1.0;
      const double a1 = ceil((hi[q] - d.g.o[q]) * d.g.inv) + 1.0;
      const int l0 = (int)fmax(0.0, fmin(a0, (double)nn[q] - 1));
      const int l1 = (int)fmax(0.0, fmin(a1, (double)nn[q] - 1));
      s_lo[q] = l0;
      s_n[q] = l1 - l0 + 1;
      tot *= s_n[q];
    }
    s_ok = tot <= d.cap;
    if (!s_ok) atomicOr(&d.status[b], 1);
  }
  __syncthreads();
  if (!s_ok) {
    if (threadIdx.x == 0) {
      d.prot[b] = 0.0;
      d.lig[b] = 0.0;
    }
    return;
  }
  const int bx = s_n[0], by = s_n[1], bz = s_n[2];
  const int npts = bx * by * bz;
  for (int t = threadIdx.x; t < 2 * words; t += blockDim.x) bsm[t] = 0u;
  __syncthreads();
  // cube of each atom: ceil((r_max + r_w) / step) cells about its cell
  double rmax = 0.0;
  for (int a = 0; a < L; ++a) rmax = fmax(rmax, s_r[a]);
  const int rs = (int)ceil((rmax + d.r_w) / d.step);
  const int side = 2 * rs + 1, cube = side * side * side;
  for (int pass = 0; pass < 2; ++pass) {
    unsigned* bits = pass == 0 ? outer : inner;
    for (long long t = threadIdx.x; t < (long long)L * cube; t += blockDim.x) {
      const int a = (int)(t / cube), c = (int)(t % cube);
      const int di = c % side - rs, dj = (c / side) % side - rs, dk = c / (side * side) - rs;
      const int i = (int)((s_x[a] - d.g.o[0]) * d.g.inv) + di - s_lo[0];
      const int j = (int)((s_y[a] - d.g.o[1]) * d.g.inv) + dj - s_lo[1];
      const int k = (int)((s_z[a] - d.g.o[2]) * d.g.inv) + dk - s_lo[2];
      if (i < 0 || j < 0 || k < 0 || i >= bx || j >= by || k >= bz) continue;
      const double ex = s_x[a] - (d.g.o[0] + d.step * (i + s_lo[0]));
      const double ey = s_y[a] - (d.g.o[1] + d.step * (j + s_lo[1]));
      const double ez = s_z[a] - (d.g.o[2] + d.step * (k + s_lo[2]));
      const double rr = pass == 0 ? s_r[a] + d.r_w : s_r[a];
      if (ex * ex + ey * ey + ez * ez < rr * rr) {
        const int p = i + j * bx + k * bx * by;
        atomicOr(&bits[p >> 5], 1u << (p & 31));
      }
    }
    __syncthreads();
  }
  double pd = 0.0, ld = 0.0;
  for (int p = threadIdx.x; p < npts; p += blockDim.x) {
    const unsigned bit = 1u << (p & 31);
    if (!(outer[p >> 5] & bit) || (inner[p >> 5] & bit)) continue;
    const int i = p % bx + s_lo[0], j = (p / bx) % by + s_lo[1], k = p / (bx * by) + s_lo[2];
    const size_t gidx = (size_t)i + (size_t)j * d.g.nx + (size_t)k * d.g.nx * d.g.ny;
    if (!d.shell[gidx]) continue;
    pd += d.contrib[gidx];
    const double x = d.g.o[0] + d.step * i, y = d.g.o[1] + d.step * j, z = d.g.o[2] + d.step * k;
    for (int a = 0; a < L; ++a) {
      const double ex = x - s_x[a], ey = y - s_y[a], ez = z - s_z[a];
      const double d2 = ex * ex + ey * ey + ez * ez;
      if (d2 < 144.0) {
        const double v = (double)s_q[a] / d2;
        ld += v * v;
      }
    }
  }
  pd = warp_sum(pd);
  ld = warp_sum(ld);
  if ((threadIdx.x & 31) == 0) {
    s_red[0][threadIdx.x >> 5] = pd;
    s_red[1][threadIdx.x >> 5] = ld;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0.0, a1 = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      a0 += s_red[0][q];
      a1 += s_red[1][q];
    }
    d.prot[b] = a0;
    d.lig[b] = d.scale * a1;
  }
}

}  // namespace

cudaError_t launch_masks(const DevCull& cull, const MaskBuild& mb, const double* radius64,
                         uint8_t* vdw, uint8_t* shell, cudaStream_t st) {
  const long long tiles = (long long)((mb.nx + 3) / 4) * ((mb.ny + 3) / 4) * ((mb.nz + 1) / 2);
  if (tiles <= 0) return cudaSuccess;
  const long long blocks = (tiles + kWarps - 1) / kWarps;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_masks<<<(unsigned)blocks, kWarps * 32, 0, st>>>(cull, mb, radius64, vdw, shell);
  return cudaGetLastError();
}

cudaError_t launch_cell_masks(const GridLook& g, const uint8_t* mask, uint8_t* cell,
                              cudaStream_t st) {
  const long long n = (long long)g.nx * g.ny * g.nz;
  if (n <= 0) return cudaSuccess;
  k_cell_masks<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, mask, cell);
  return cudaGetLastError();
}

cudaError_t launch_clash(const DevLigand& lig, const float4* X, int B, const DevCull& cull,
                         const ClashArgs& ca, int* out, cudaStream_t st) {
  if (B <= 0) return cudaSuccess;
  k_clash<<<(B + 7) / 8, 256, 0, st>>>(lig, X, B, cull, ca, out);
  return cudaGetLastError();
}

cudaError_t launch_dock(const DockArgs& a, int blocks, cudaStream_t st) {
  if (blocks <= 0) return cudaSuccess;
  const int no = max(a.nrot * a.L, a.npos);
  k_dock_offsets<<<(no + 255) / 256, 256, 0, st>>>(a);
  const int smem = 2 * kDockPerBlock * (int)sizeof(unsigned long long) +
                   a.rtile * a.L * 6 * (int)sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(k_dock, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_dock<<<blocks, kDockBlock, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_topk_merge(const unsigned long long* in, int n, int k, unsigned long long* out,
                              cudaStream_t st) {
  const int smem = 2 * kDockPerBlock * (int)sizeof(unsigned long long);
  cudaError_t e =
      cudaFuncSetAttribute(k_topk_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int blocks = (n + kDockPerBlock - 1) / kDockPerBlock;
  k_topk_merge<<<blocks, kDockBlock, smem, st>>>(in, n, k, out);
  return cudaGetLastError();
}

cudaError_t launch_place(const PlaceArgs& a, const DevCull& cull, const ClashArgs& ca,
                         cudaStream_t st) {
  const long long n = (long long)a.slots * a.per_slot;
  if (n <= 0) return cudaSuccess;
  k_place<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a, cull, ca);
  return cudaGetLastError();
}

cudaError_t launch_prot_desolv(const DevCull& cull, const DesolvBuild& db, double* out,
                               cudaStream_t st) {
  if (db.ntiles <= 0) return cudaSuccess;
  k_prot_desolv<<<(db.ntiles + kWarps - 1) / kWarps, kWarps * 32, 0, st>>>(cull, db, out);
  return cudaGetLastError();
}

cudaError_t launch_desolv_pose(const DesolvPose& d, cudaStream_t st) {
  if (d.B <= 0) return cudaSuccess;
  const int smem = 2 * ((d.cap + 31) / 32) * (int)sizeof(unsigned);
  cudaError_t e =
      cudaFuncSetAttribute(k_desolv_pose, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_desolv_pose<<<d.B, 256, smem, st>>>(d);
  return cudaGetLastError();
}

}  // namespace mmo

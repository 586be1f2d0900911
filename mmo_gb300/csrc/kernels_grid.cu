// kernels_grid.cu -- precomputed interaction grids and the energy they give.
//
// k_grid_build: the values of Lds.pre_calculate_FF_components_grid
// (UnixJunkie/MMO src/lds.ml:452-469, the point sum Mol.ene_inter_UFF_shifted_grid
// of src/mol.ml:964-989): for every lattice point within the mask sphere and
// every ligand atom type l = (element a_l, charge q_l),
//   E_l(p) = min(max_E, q_l phi(p) + V_{a_l}(p)),
//   phi(p) = K sum_i w q_i / r,  V_a(p) = sum_i w D_ia (p6^2 - 2 p6),
// over the protein atoms within 12 A (w the 12 A switch, r clamped at 0.01 A).
// A warp owns a 4 x 4 x 4 tile of lattice points (two per lane); the protein
// is read through its row index, culled against the tile's box and compacted
// per warp as in the cut-off sweep; pair terms in FP32, sums per row and
// per block of rows in FP32, over the blocks in compensated FP32.
//
// k_grid_inter: Mol.ene_inter_UFF_interp (src/mol.ml:1010-1020) with
// G3D.trilin (src/G3D.ml:97-157) for every (pose, ligand atom) entry, and the
// derivative of the trilinear form, into the same per-entry partials as the
// pair sweep (so the finishing pass adds the intra term and the adjoint).
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kGridList = 64;         // compacted atoms per warp (< 32 + 32)
constexpr int kGridFlushAtoms = 1024;  // protein atoms per FP32 block sum

__device__ __forceinline__ float gwmin(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
// acc + x as an unevaluated float pair (TwoSum: the rounding error of the
// high part's sum is exact and goes to the low part)
__device__ __forceinline__ float2 two_sum_add(float2 acc, float x) {
  const float s = __fadd_rn(acc.x, x);
  const float bp = __fsub_rn(s, acc.x);
  const float ap = __fsub_rn(s, bp);
  const float err = __fadd_rn(__fsub_rn(acc.x, ap), __fsub_rn(x, bp));
  return make_float2(s, __fadd_rn(acc.y, err));
}

__device__ __forceinline__ float gwmax(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// A warp owns a 4 x 4 x 2 KP tile of lattice points, KP per lane (lane
// (i, j, k0) holds k0, k0 + 2, ...).  The protein atoms that pass the box test
// are staged in the warp's shared list (both float4 halves), so the
// evaluation loop reads only shared memory (broadcast); the pair parameters of
// the atom's type for the NE grid elements follow as NE / 2 float4.  The block
// sums (compensated float pairs) live in shared memory: they change only at
// block ends.
constexpr int kGridWarps = 8;  // tiles per CTA

// NE = 0: the factorised form of geometric mixing, vdW sums A12, A6 shared by
// all elements; NE > 0: NE per-element vdW sums
template <int NE>
constexpr int grid_accs() {
  return NE == 0 ? 3 : NE + 1;
}
template <int NE>
constexpr int grid_el4() {
  return NE == 0 ? 1 : (NE + 1) / 2;
}
template <int NE, int KP>
constexpr int grid_smem_bytes() {
  return kNTypes * grid_el4<NE>() * 16 + kGridWarps * kGridList * 32 +
         kGridWarps * grid_accs<NE>() * KP * 32 * (int)sizeof(float2);
}

// The lattice points of one lane in a warp's tile: point c at (i, j, kk[c]),
// as float pairs in the device frame, whether it is on the lattice and in the
// mask sphere; and the box of the tile's masked points (warp-wide).
template <int KP>
struct TilePoints {
  int i, j, kk[KP];
  bool in_lattice[KP], masked[KP];
  float xh[KP], yh[KP], zh[KP], xl[KP], yl[KP], zl[KP];
  float blx, bly, blz, bhx, bhy, bhz;
};

template <int KP>
__device__ __forceinline__ TilePoints<KP> tile_points(const GridBuild& gb, int3 t, int lane) {
  static_assert(kGridTileX == 4 && kGridTileY == 4, "lane layout of the tile");
  TilePoints<KP> P;
  P.i = t.x * 4 + (lane & 3);
  P.j = t.y * 4 + ((lane >> 2) & 3);
  const float big = 1e30f;
  float lox = big, loy = big, loz = big, hix = -big, hiy = -big, hiz = -big;
#pragma unroll
  for (int c = 0; c < KP; ++c) {
    P.kk[c] = t.z * (2 * KP) + (lane >> 4) + 2 * c;
    P.in_lattice[c] = P.i < gb.nx && P.j < gb.ny && P.kk[c] < gb.nz;
    // lattice point in the device frame, as a float pair
    const double px = gb.o[0] + gb.step * P.i, py = gb.o[1] + gb.step * P.j,
                 pz = gb.o[2] + gb.step * P.kk[c];
    const double mx = px - gb.mc[0], my = py - gb.mc[1], mz = pz - gb.mc[2];
    P.masked[c] = P.in_lattice[c] && mx * mx + my * my + mz * mz < gb.mr2;
    P.xh[c] = (float)px;
    P.yh[c] = (float)py;
    P.zh[c] = (float)pz;
    P.xl[c] = (float)(px - P.xh[c]);
    P.yl[c] = (float)(py - P.yh[c]);
    P.zl[c] = (float)(pz - P.zh[c]);
    if (P.masked[c]) {
      lox = fminf(lox, P.xh[c]);
      loy = fminf(loy, P.yh[c]);
      loz = fminf(loz, P.zh[c]);
      hix = fmaxf(hix, P.xh[c]);
      hiy = fmaxf(hiy, P.yh[c]);
      hiz = fmaxf(hiz, P.zh[c]);
    }
  }
  P.blx = gwmin(lox);
  P.bly = gwmin(loy);
  P.blz = gwmin(loz);
  P.bhx = gwmax(hix);
  P.bhy = gwmax(hiy);
  P.bhz = gwmax(hiz);
  return P;
}

// The values of the lane's points for every grid type from the point's
// compensated sums ad[(e * KP + c) * 32] (e = ELEC: the electrostatic sum;
// FACT: e = 0, 1 the sums A12, A6; else e = the element's vdW sum), capped
// at max_E; 0 outside the mask sphere.
template <bool FACT, int KP, int ELEC>
__device__ __forceinline__ void grid_store(const GridBuild& gb, const TilePoints<KP>& P,
                                           const float2* ad, float* grids) {
  const size_t per = (size_t)gb.nx * gb.ny * gb.nz;
#pragma unroll
  for (int c = 0; c < KP; ++c) {
    if (!P.in_lattice[c]) continue;
    const size_t idx = (size_t)P.i + (size_t)P.j * gb.nx + (size_t)P.kk[c] * gb.nx * gb.ny;
    const float2 phi = ad[(ELEC * KP + c) * 32];
    float2 a12 = make_float2(0.f, 0.f), a6 = a12;
    if (FACT) {
      a12 = ad[(0 * KP + c) * 32];
      a6 = ad[(1 * KP + c) * 32];
    }
    for (int l = 0; l < gb.ntypes; ++l) {
      float v = 0.f;
      if (P.masked[c]) {
        float2 vdw;
        if (FACT) {
          // sqrt(D_e) (x_e^6 A12 - 2 x_e^3 A6) in float pairs
          const float4 f = gb.elf[gb.type_elem[l]];  // (sqrt(D_e), 2 x_e^3, x_e^6, 0)
          const float t1 = f.z * a12.x, t1l = fmaf(f.z, a12.x, -t1) + f.z * a12.y;
          const float t2 = f.y * a6.x, t2l = fmaf(f.y, a6.x, -t2) + f.y * a6.y;
          const float dh = __fsub_rn(t1, t2);
          const float bp = __fsub_rn(dh, t1), ap = __fsub_rn(dh, bp);
          const float dl = __fadd_rn(__fsub_rn(t1, ap), __fsub_rn(-t2, bp)) + (t1l - t2l);
          vdw = make_float2(f.x * dh, fmaf(f.x, dh, -(f.x * dh)) + f.x * dl);
        } else {
          vdw = ad[(gb.type_elem[l] * KP + c) * 32];
        }
        // q phi + V in float pairs: one rounding of the sum of the high parts,
        // the low parts added to it
        const float q = gb.type_qf[l];
        const float e = fmaf(q, phi.x, vdw.x) + fmaf(q, phi.y, vdw.y);
        v = e < gb.max_Ef ? e : gb.max_Ef;
      }
      grids[per * l + idx] = v;
    }
  }
}

// KP lattice points per lane (1 or 2): a warp tile of 4 x 4 x 2 KP points
template <int DIEL, int NE, int KP, bool COUNT>
__global__ void __launch_bounds__(kGridWarps * 32) k_grid_build(DevCull cull, GridBuild gb,
                                                                 float* grids) {
  constexpr int kGridPts = KP;
  constexpr bool FACT = NE == 0;
  constexpr int NACC = grid_accs<NE>(), ELEC = NACC - 1, NE2 = grid_el4<NE>();
  extern __shared__ __align__(16) float4 gsm[];
  // [ptype][NE2]: (X, 1/D) of 2 elements, or (c12, c6) of the protein type (NE = 0)
  float4* s_el = gsm;
  float4* s_list = s_el + kNTypes * NE2;               // [warp][kGridList][2] staged atoms
  float2* s_ad = reinterpret_cast<float2*>(s_list + kGridWarps * kGridList * 2);
  for (int k = threadIdx.x; k < kNTypes * NE2; k += blockDim.x) {
    const int pt = k / NE2, q = k % NE2;
    const float2 a = gb.el[pt * kGridElems + 2 * q];
    const float2 b = (!FACT && 2 * q + 1 < kGridElems) ? gb.el[pt * kGridElems + 2 * q + 1]
                                                       : make_float2(0.f, 0.f);
    s_el[k] = make_float4(a.x, a.y, b.x, b.y);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * kGridWarps + w;
  if (tile >= gb.ntiles) return;  // whole warps leave: no block-wide barrier follows
  const TilePoints<KP> P = tile_points<KP>(gb, gb.tiles[tile], lane);
  const float blx = P.blx, bly = P.bly, blz = P.blz, bhx = P.bhx, bhy = P.bhy, bhz = P.bhz;
  // Sums in three levels: the atoms of one row in FP32 (af), the rows of one
  // block of kGridFlushAtoms protein atoms in FP32 (bf), the blocks in
  // compensated FP32 (s_ad: hi + lo pairs updated by TwoSum, about twice the
  // FP32 precision, without the FP64 pipe).  Atoms the box test drops are beyond 12.04 A of every masked point
  // of the tile, where the switched terms are exactly 0, and a row or block
  // that is not visited adds exactly 0: each value is the same whatever the
  // tile's box (and so the mask) is.
  float2* ad = s_ad + (size_t)w * NACC * kGridPts * 32 + lane;  // [e][c] stride 32
  float af[kGridPts][NACC], bf[kGridPts][NACC];
#pragma unroll
  for (int c = 0; c < kGridPts; ++c)
#pragma unroll
    for (int e = 0; e < NACC; ++e) {
      af[c][e] = 0.f;
      bf[c][e] = 0.f;
      ad[(e * kGridPts + c) * 32] = make_float2(0.f, 0.f);
    }
  float4* wl = s_list + (size_t)w * kGridList * 2;
  unsigned n_eval[kGridPts] = {}, n_near[kGridPts] = {};
  auto evaluate = [&](int n) {
    __syncwarp();
    if (COUNT) {
#pragma unroll
      for (int c = 0; c < kGridPts; ++c) n_eval[c] += n;
    }
#pragma unroll 2
    for (int v = 0; v < n; ++v) {
      const float4 p = wl[2 * v], pl = wl[2 * v + 1];
      // pl.w holds the bits of type * kNTypes * 16 (the pair table's row offset)
      const float4* er = s_el + (__float_as_int(pl.w) / (16 * kNTypes)) * NE2;
      float4 prm[NE2];
#pragma unroll
      for (int q = 0; q < NE2; ++q) prm[q] = er[q];
#pragma unroll
      for (int c = 0; c < kGridPts; ++c) {
        const float dx = (P.xh[c] - p.x) + (P.xl[c] - pl.x);
        const float dy = (P.yh[c] - p.y) + (P.yl[c] - pl.y);
        const float dz = (P.zh[c] - p.z) + (P.zl[c] - pl.z);
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        if (COUNT) n_near[c] += r2 < kCut2;
        const float r2c = fmaxf(r2, kMinR2);
        const float ir = rsqrtf(r2c);
        const float ir2 = ir * ir;
        const float sw = fmaxf(fmaf(r2c, -1.0f / 144.0f, 1.0f), 0.0f);
        const float ws = sw * sw;
        af[c][ELEC] = fmaf(ws * p.w, DIEL == 0 ? ir : ir2, af[c][ELEC]);
        if (FACT) {
          // geometric mixing: D_ij (x_ij/r)^12 = c12_i c12_e / r^12 and
          // 2 D_ij (x_ij/r)^6 = 2 c6_i c6_e / r^6 with c12 = sqrt(D) x^6,
          // c6 = sqrt(D) x^3: two sums for every element
          const float ir6 = (ir2 * ir2) * ir2;
          af[c][0] = fmaf(ws * prm[0].x, ir6 * ir6, af[c][0]);
          af[c][1] = fmaf(ws * prm[0].y, ir6, af[c][1]);
        }
#pragma unroll
        for (int e = 0; e < NE; ++e) {
          // X = D^(1/3) x^2: q6 = (X / r^2)^3 = D (x/r)^6, and
          // D ((x/r)^12 - 2 (x/r)^6) = q6 (q6 / D - 2)
          const float X = (e & 1) ? prm[e / 2].z : prm[e / 2].x;
          const float iD = (e & 1) ? prm[e / 2].w : prm[e / 2].y;
          const float q2 = X * ir2;
          const float q6 = (q2 * q2) * q2;
          af[c][e] = fmaf(ws, q6 * fmaf(q6, iD, -2.0f), af[c][e]);
        }
      }
    }
    __syncwarp();
  };
  bool mine = false;
#pragma unroll
  for (int c = 0; c < kGridPts; ++c) mine = mine || P.masked[c];
  const bool any = __any_sync(kFull, mine);
  if (any) {
    bool dirty = false;
    for (int r = 0; r < cull.nrows; ++r) {
      const int a = cull.row_start[r], b = cull.row_start[r + 1];
      const float4 rb = cull.row_box[r];
      const float ey = fmaxf(fmaxf(rb.x - bhy, bly - rb.y), 0.f);
      const float ez = fmaxf(fmaxf(rb.z - bhz, blz - rb.w), 0.f);
      if (fmaf(ey, ey, ez * ez) < kCullR2) {
        int cnt = 0;
        for (int i0 = a; i0 < b; i0 += 32) {
          const int ia = i0 + lane;
          bool in = false;
          float4 ph = make_float4(0.f, 0.f, 0.f, 0.f);
          if (ia < b) {
            ph = cull.atoms[2 * (size_t)ia];
            const float ex = fmaxf(fmaxf(blx - ph.x, ph.x - bhx), 0.f);
            const float fy = fmaxf(fmaxf(bly - ph.y, ph.y - bhy), 0.f);
            const float fz = fmaxf(fmaxf(blz - ph.z, ph.z - bhz), 0.f);
            in = fmaf(ex, ex, fmaf(fy, fy, fz * fz)) < kCullR2;
          }
          const unsigned m = __ballot_sync(kFull, in);
          if (in) {
            const int at = cnt + __popc(m & ((1u << lane) - 1u));
            wl[2 * at] = ph;
            wl[2 * at + 1] = cull.atoms[2 * (size_t)ia + 1];
          }
          cnt += __popc(m);
          if (cnt >= 32) {
            evaluate(cnt);
            cnt = 0;
          }
        }
        evaluate(cnt);
#pragma unroll
        for (int c = 0; c < kGridPts; ++c)
#pragma unroll
          for (int e = 0; e < NACC; ++e) {
            bf[c][e] += af[c][e];
            af[c][e] = 0.f;
          }
        dirty = true;
      }
      // the block ends where the atom index crosses a multiple of kGridFlushAtoms
      if (dirty && (r + 1 == cull.nrows || (b - 1) / kGridFlushAtoms != b / kGridFlushAtoms)) {
#pragma unroll
        for (int c = 0; c < kGridPts; ++c)
#pragma unroll
          for (int e = 0; e < NACC; ++e) {
            float2& acc = ad[(e * kGridPts + c) * 32];
            acc = two_sum_add(acc, bf[c][e]);
            bf[c][e] = 0.f;
          }
        dirty = false;
      }
    }
  }
  if (COUNT) {
    unsigned long long ev = 0, cv = 0;
#pragma unroll
    for (int c = 0; c < kGridPts; ++c) {
      ev += P.masked[c] ? n_eval[c] : 0u;
      cv += P.masked[c] ? n_near[c] : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ev += __shfl_xor_sync(kFull, ev, o);
      cv += __shfl_xor_sync(kFull, cv, o);
    }
    if (lane == 0 && ev) {
      atomicAdd(gb.pairs, ev);
      atomicAdd(gb.pairs + 1, cv);
    }
  }
  grid_store<FACT, KP, ELEC>(gb, P, ad, grids);
}

// squared distance from (x, y, z) to the box [bl, bh]
__device__ __forceinline__ float gbox_d2(float x, float y, float z, const float* bl,
                                         const float* bh) {
  const float ex = fmaxf(fmaxf(bl[0] - x, x - bh[0]), 0.f);
  const float ey = fmaxf(fmaxf(bl[1] - y, y - bh[1]), 0.f);
  const float ez = fmaxf(fmaxf(bl[2] - z, z - bh[2]), 0.f);
  return fmaf(ex, ex, fmaf(ey, ey, ez * ez));
}

constexpr int kGridPairList = 64;  // compacted atom pairs per warp (< 32 + 32)
constexpr int kGridRec = 5;        // float4 per staged pair

template <int KP>
constexpr int grid_pk_smem_bytes() {
  return (kNTypes + 1) * 16 + kGridWarps * kGridPairList * kGridRec * 16 +
         kGridWarps * 3 * KP * 32 * (int)sizeof(float2);
}

// The factorised build (geometric mixing) on the packed FP32 instructions
// (add/mul/fma .f32x2) over pairs of protein atoms: the protein as the cut-off
// sweep's pairs (DevCull::pairs: the atoms of each row in pairs, negated
// coordinates, a null partner closing a row of odd length), the lane's
// lattice points in both halves of their registers.  A warp stages the pairs
// of a row that have an atom within 12.04 A of its tile's box, with the two
// atoms' (sqrt(D) x^6, sqrt(D) x^3), as five float4; every lane then sums
// them for its points, half a over the pairs' first atoms and half b over
// their partners (a split fixed by the layout), in the scalar kernel's
// arithmetic.  Atoms out of reach add exact zeros, so each value is the same
// bits whatever the tile's shape or the mask.
template <int DIEL, int KP, bool COUNT>
__global__ void __launch_bounds__(kGridWarps * 32) k_grid_build_pk(DevCull cull, GridBuild gb,
                                                                    float* grids) {
  constexpr int NACC = 3, ELEC = 2;
  extern __shared__ __align__(16) float4 gsm[];
  float4* s_cc = gsm;                           // [ptype] (c12, c6, 0, 0), the null type 0
  float4* s_list = s_cc + kNTypes + 1;          // [warp][kGridPairList][kGridRec]
  float2* s_ad = reinterpret_cast<float2*>(s_list + kGridWarps * kGridPairList * kGridRec);
  for (int k = threadIdx.x; k <= kNTypes; k += blockDim.x) {
    const float2 v = k < kNTypes ? gb.el[k * kGridElems] : make_float2(0.f, 0.f);
    s_cc[k] = make_float4(v.x, v.y, 0.f, 0.f);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * kGridWarps + w;
  if (tile >= gb.ntiles) return;  // whole warps leave: no block-wide barrier follows
  const TilePoints<KP> P = tile_points<KP>(gb, gb.tiles[tile], lane);
  const float bl[3] = {P.blx, P.bly, P.blz}, bh[3] = {P.bhx, P.bhy, P.bhz};
  float2 xh[KP], yh[KP], zh[KP], xl[KP], yl[KP], zl[KP];
#pragma unroll
  for (int c = 0; c < KP; ++c) {
    xh[c] = bc2(P.xh[c]);
    yh[c] = bc2(P.yh[c]);
    zh[c] = bc2(P.zh[c]);
    xl[c] = bc2(P.xl[c]);
    yl[c] = bc2(P.yl[c]);
    zl[c] = bc2(P.zl[c]);
  }
  // sums in three levels, as the scalar kernel: a row in FP32 (af), the rows of
  // a 1,024-atom block in FP32 (bf), the blocks as compensated float pairs
  float2* ad = s_ad + (size_t)w * NACC * KP * 32 + lane;  // [e][c] stride 32
  float2 af[KP][NACC], bf[KP][NACC];
#pragma unroll
  for (int c = 0; c < KP; ++c)
#pragma unroll
    for (int e = 0; e < NACC; ++e) {
      af[c][e] = bf[c][e] = bc2(0.f);
      ad[(e * KP + c) * 32] = make_float2(0.f, 0.f);
    }
  float4* wl = s_list + (size_t)w * kGridPairList * kGridRec;
  unsigned n_eval = 0, n_near[KP] = {};
  auto evaluate = [&](int n, int nnull) {
    __syncwarp();
    if (COUNT) n_eval += 2u * n - nnull;
#pragma unroll 2
    for (int v = 0; v < n; ++v) {
      const float4* rr = wl + kGridRec * v;
      const float4 r0 = rr[0], r1 = rr[1], r2 = rr[2], r3 = rr[3], r4 = rr[4];
#pragma unroll
      for (int c = 0; c < KP; ++c) {
        const float2 dx = __fadd2_rn(__fadd2_rn(xh[c], lo_pair(r0)), __fadd2_rn(xl[c], lo_pair(r2)));
        const float2 dy = __fadd2_rn(__fadd2_rn(yh[c], hi_pair(r0)), __fadd2_rn(yl[c], hi_pair(r2)));
        const float2 dz = __fadd2_rn(__fadd2_rn(zh[c], lo_pair(r1)), __fadd2_rn(zl[c], lo_pair(r3)));
        const float2 d2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
        if (COUNT)
          n_near[c] += (d2.x < kCut2) + (d2.y < kCut2 && __float_as_uint(r1.w) != 0x80000000u);
        const float2 r2c = make_float2(fmaxf(d2.x, kMinR2), fmaxf(d2.y, kMinR2));
        const float2 ir = make_float2(rsqrtf(r2c.x), rsqrtf(r2c.y));
        const float2 ir2 = __fmul2_rn(ir, ir);
        const float2 t = __ffma2_rn(r2c, bc2(-1.0f / 144.0f), bc2(1.0f));
        const float2 sw = make_float2(fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f));
        const float2 ws = __fmul2_rn(sw, sw);
        af[c][ELEC] = __ffma2_rn(__fmul2_rn(ws, hi_pair(r1)), DIEL == 0 ? ir : ir2, af[c][ELEC]);
        // D_ij (x_ij/r)^12 = c12_i c12_e / r^12, 2 D_ij (x_ij/r)^6 = 2 c6_i c6_e / r^6
        const float2 ir6 = __fmul2_rn(__fmul2_rn(ir2, ir2), ir2);
        af[c][0] = __ffma2_rn(__fmul2_rn(ws, lo_pair(r4)), __fmul2_rn(ir6, ir6), af[c][0]);
        af[c][1] = __ffma2_rn(__fmul2_rn(ws, hi_pair(r4)), ir6, af[c][1]);
      }
    }
    __syncwarp();
  };
  bool mine = false;
#pragma unroll
  for (int c = 0; c < KP; ++c) mine = mine || P.masked[c];
  if (__any_sync(kFull, mine)) {
    bool dirty = false;
    for (int r = 0; r < cull.nrows; ++r) {
      const int b = cull.row_start[r + 1];
      const float4 rb = cull.row_box[r];
      const float ey = fmaxf(fmaxf(rb.x - bh[1], bl[1] - rb.y), 0.f);
      const float ez = fmaxf(fmaxf(rb.z - bh[2], bl[2] - rb.w), 0.f);
      if (fmaf(ey, ey, ez * ez) < kCullR2) {
        const int pa = cull.pair_start[r], pb = cull.pair_start[r + 1];
        int cnt = 0, nnull = 0;
        for (int i0 = pa; i0 < pb; i0 += 32) {
          const int ip = i0 + lane;
          bool in = false, null_b = false;
          float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
          if (ip < pb) {
            q0 = cull.pairs[4 * (size_t)ip];
            q1 = cull.pairs[4 * (size_t)ip + 1];
            null_b = __float_as_uint(q1.w) == 0x80000000u;
            in = gbox_d2(-q0.x, -q0.z, -q1.x, bl, bh) < kCullR2 ||
                 (!null_b && gbox_d2(-q0.y, -q0.w, -q1.y, bl, bh) < kCullR2);
          }
          const unsigned m = __ballot_sync(kFull, in);
          if (in) {
            float4* dst = wl + kGridRec * (cnt + __popc(m & ((1u << lane) - 1u)));
            const float4 q2 = cull.pairs[4 * (size_t)ip + 2], q3 = cull.pairs[4 * (size_t)ip + 3];
            // q3.zw: the atoms' type row offsets of the pair table (type * kNTypes * 16)
            const float4 ca = s_cc[__float_as_int(q3.z) / (16 * kNTypes)];
            const float4 cb = s_cc[__float_as_int(q3.w) / (16 * kNTypes)];
            dst[0] = q0;
            dst[1] = q1;
            dst[2] = q2;
            dst[3] = q3;
            dst[4] = make_float4(ca.x, cb.x, ca.y, cb.y);
          }
          if (COUNT) nnull += __popc(__ballot_sync(kFull, in && null_b));
          cnt += __popc(m);
          if (cnt >= 32) {
            evaluate(cnt, nnull);
            cnt = 0;
            nnull = 0;
          }
        }
        evaluate(cnt, nnull);
#pragma unroll
        for (int c = 0; c < KP; ++c)
#pragma unroll
          for (int e = 0; e < NACC; ++e) {
            bf[c][e] = __fadd2_rn(bf[c][e], af[c][e]);
            af[c][e] = bc2(0.f);
          }
        dirty = true;
      }
      // the block ends where the atom index crosses a multiple of kGridFlushAtoms
      if (dirty && (r + 1 == cull.nrows || (b - 1) / kGridFlushAtoms != b / kGridFlushAtoms)) {
#pragma unroll
        for (int c = 0; c < KP; ++c)
#pragma unroll
          for (int e = 0; e < NACC; ++e) {
            float2& acc = ad[(e * KP + c) * 32];
            acc = two_sum_add(two_sum_add(acc, bf[c][e].x), bf[c][e].y);
            bf[c][e] = bc2(0.f);
          }
        dirty = false;
      }
    }
  }
  if (COUNT) {
    unsigned long long ev = 0, cv = 0;
#pragma unroll
    for (int c = 0; c < KP; ++c) {
      ev += P.masked[c] ? n_eval : 0u;
      cv += P.masked[c] ? n_near[c] : 0u;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ev += __shfl_xor_sync(kFull, ev, o);
      cv += __shfl_xor_sync(kFull, cv, o);
    }
    if (lane == 0 && ev) {
      atomicAdd(gb.pairs, ev);
      atomicAdd(gb.pairs + 1, cv);
    }
  }
  grid_store<true, KP, ELEC>(gb, P, ad, grids);
}

template <bool GRAD>
__global__ void k_grid_inter(GridLook g, const float4* __restrict__ X, int n, int L,
                             const int* __restrict__ atom_type, const float* __restrict__ grids,
                             double* Epart, float4* Gpart, int* status) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  float E, gx, gy, gz;
  if (!grid_entry<GRAD>(g, X[2 * (size_t)e], X[2 * (size_t)e + 1], atom_type[e % L], grids, E,
                        gx, gy, gz))
    atomicOr(&status[e / L], kStatusOffGrid);
  Epart[e] = (double)E;
  if (GRAD) Gpart[e] = make_float4(gx, gy, gz, 0.f);
}

// One ligand (the grid closure, mmo_ene_inter_grid) in one block of 128
// threads, an atom each: the energy summed in a fixed order into *Eout and the
// status (MMO_S_OFF_GRID when a corner is off the lattice) into *status.
__global__ void __launch_bounds__(kMaxLig) k_grid_inter_one(GridLook g, const float4* X, int n,
                                                          const int* atom_type,
                                                          const float* grids, double* Eout,
                                                          int* status) {
  __shared__ double ws[kMaxLig / 32];
  __shared__ int s_st;
  const int e = threadIdx.x, lane = e & 31;
  if (e == 0) s_st = 0;
  __syncthreads();
  double E = 0.0;
  if (e < n) {
    float ef, gx, gy, gz;
    if (!grid_entry<false>(g, X[2 * e], X[2 * e + 1], atom_type[e], grids, ef, gx, gy, gz))
      atomicOr(&s_st, kStatusOffGrid);
    E = (double)ef;
  }
  E = warp_sum(E);
  if (lane == 0) ws[e >> 5] = E;
  __syncthreads();
  if (e == 0) {
    double t = 0.0;
    for (int w = 0; w < kMaxLig / 32; ++w) t += ws[w];
    *Eout = t;
    *status = s_st;
  }
}

}  // namespace

namespace {
template <int DIEL, int NE, int KP, bool COUNT>
cudaError_t grid_build_as(const DevCull& cull, const GridBuild& gb, float* grids,
                          cudaStream_t st) {
  constexpr int smem = grid_smem_bytes<NE, KP>();
  // the opt-in above 48 KB (per device: set on every launch)
  const cudaError_t e = cudaFuncSetAttribute(k_grid_build<DIEL, NE, KP, COUNT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int blocks = (gb.ntiles + kGridWarps - 1) / kGridWarps;
  k_grid_build<DIEL, NE, KP, COUNT><<<blocks, kGridWarps * 32, smem, st>>>(cull, gb, grids);
  return cudaGetLastError();
}

// NE = the number of grid elements exactly, so that no element slot is
// evaluated in vain
template <int DIEL, int KP, bool COUNT>
cudaError_t grid_build_pk(const DevCull& cull, const GridBuild& gb, float* grids,
                          cudaStream_t st) {
  constexpr int smem = grid_pk_smem_bytes<KP>();
  const cudaError_t e = cudaFuncSetAttribute(k_grid_build_pk<DIEL, KP, COUNT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int blocks = (gb.ntiles + kGridWarps - 1) / kGridWarps;
  k_grid_build_pk<DIEL, KP, COUNT><<<blocks, kGridWarps * 32, smem, st>>>(cull, gb, grids);
  return cudaGetLastError();
}

template <int DIEL, int KP, bool COUNT>
cudaError_t grid_build_ne(const DevCull& cull, const GridBuild& gb, float* grids,
                          cudaStream_t st) {
  if (gb.fact) return grid_build_pk<DIEL, KP, COUNT>(cull, gb, grids, st);
  switch (gb.nelem) {
    case 1: return grid_build_as<DIEL, 1, KP, COUNT>(cull, gb, grids, st);
    case 2: return grid_build_as<DIEL, 2, KP, COUNT>(cull, gb, grids, st);
    case 3: return grid_build_as<DIEL, 3, KP, COUNT>(cull, gb, grids, st);
    case 4: return grid_build_as<DIEL, 4, KP, COUNT>(cull, gb, grids, st);
    case 5: return grid_build_as<DIEL, 5, KP, COUNT>(cull, gb, grids, st);
    case 6: return grid_build_as<DIEL, 6, KP, COUNT>(cull, gb, grids, st);
    case 7: return grid_build_as<DIEL, 7, KP, COUNT>(cull, gb, grids, st);
    case 8: return grid_build_as<DIEL, 8, KP, COUNT>(cull, gb, grids, st);
    case 9: return grid_build_as<DIEL, 9, KP, COUNT>(cull, gb, grids, st);
    case 10: return grid_build_as<DIEL, 10, KP, COUNT>(cull, gb, grids, st);
    case 11: return grid_build_as<DIEL, 11, KP, COUNT>(cull, gb, grids, st);
    default: return grid_build_as<DIEL, kGridElems, KP, COUNT>(cull, gb, grids, st);
  }
}

// the counting variant (pair statistics) exists for one point per lane only
template <int DIEL, bool COUNT>
cudaError_t grid_build_kp(const DevCull& cull, const GridBuild& gb, float* grids,
                          cudaStream_t st) {
  if (COUNT && gb.kp != 1) return cudaErrorInvalidValue;
  if (!COUNT && gb.kp == 4) {  // the packed (factorised) kernel only
    if (!gb.fact) return cudaErrorInvalidValue;
    return grid_build_pk<DIEL, 4, false>(cull, gb, grids, st);
  }
  if (!COUNT && gb.kp == 2) return grid_build_ne<DIEL, 2, false>(cull, gb, grids, st);
  return grid_build_ne<DIEL, 1, COUNT>(cull, gb, grids, st);
}
}  // namespace

cudaError_t launch_grid_build(const DevCull& cull, const GridBuild& gb, int dielectric,
                              float* grids, cudaStream_t st) {
  if (gb.ntiles <= 0) return cudaSuccess;
  if (gb.nelem < 1 || gb.nelem > kGridElems || (gb.kp != 1 && gb.kp != 2 && gb.kp != 4))
    return cudaErrorInvalidValue;
  const bool count = gb.pairs != nullptr;
  if (dielectric)
    return count ? grid_build_kp<1, true>(cull, gb, grids, st)
                 : grid_build_kp<1, false>(cull, gb, grids, st);
  return count ? grid_build_kp<0, true>(cull, gb, grids, st)
               : grid_build_kp<0, false>(cull, gb, grids, st);
}

cudaError_t launch_grid_inter_one(const GridLook& g, const float4* X, int n,
                                  const int* atom_type, const float* grids, double* Eout,
                                  int* status, cudaStream_t st) {
  if (n <= 0 || n > kMaxLig) return cudaErrorInvalidValue;
  k_grid_inter_one<<<1, kMaxLig, 0, st>>>(g, X, n, atom_type, grids, Eout, status);
  return cudaGetLastError();
}

cudaError_t launch_grid_inter(const GridLook& g, const float4* X, int n, int L,
                              const int* atom_type, const float* grids, double* Epart,
                              float4* Gpart, int* status, int grad, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (n + 255) / 256;
  if (grad) k_grid_inter<true><<<blocks, 256, 0, st>>>(g, X, n, L, atom_type, grids, Epart, Gpart, status);
  else k_grid_inter<false><<<blocks, 256, 0, st>>>(g, X, n, L, atom_type, grids, Epart, Gpart, status);
  return cudaGetLastError();
}

}  // namespace mmo

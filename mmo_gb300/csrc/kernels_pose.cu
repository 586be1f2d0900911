// kernels_pose.cu -- the per-pose kernels around the pair sweep.
//
// k_rebuild (a few threads per pose, double-float): the pose map of UnixJunkie/MMO --
// torsions applied in bond order, each rotating its group about the current
// (left, right) axis (src/optim.ml:68-71, src/mol.ml:610-631), the
// enclosing-radius check (src/mol.ml:576-591), then x = Rz(g) Ry(b) Rx(a) y + t
// (src/optim.ml:77-80, src/rot.ml:52-66), or with the centroid removed first
// for the Monte Carlo map (src/mol.ml:705-710).  All poses of a block share the
// ligand, so the threads of a warp walk the same atom indices in lockstep and
// keep their coordinates in shared memory laid out [atom][thread].
//
// k_finish (one warp per pose, lanes over atoms): the FP64 energy of the pose
// (inter partials + the intra-ligand term of src/mol.ml:881-903) and, with the
// gradient, the reverse pass through the rigid map and the torsion chain.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kRebuildThreads = 128;  // threads per rebuild block
constexpr int kWarpsPerBlock = 4;     // poses per finish block
constexpr int kFinishBlocksPerSM = 7;  // resident finish blocks: 4,096 poses in one wave on 152 SMs

// ---------------------------------------------------------------------------
// k_rebuild
// ---------------------------------------------------------------------------
// kStatusTooLong when 0.01 + sqrt(d2) > 12 A (mol.ml:576-591) for the largest
// squared distance d2 (double-float) from the centroid; the FP64 test runs only
// near the limit: with |lo| <= ulp(hi) / 2, hi < 143 gives a radius below
// 11.97 A and hi > 144.5 one above 12.02 A
__device__ __forceinline__ int too_long_of(float2 d2) {
  if (d2.x < 143.f) return 0;
  if (d2.x > 144.5f) return kStatusTooLong;
  return 0.01 + sqrt((double)d2.x + (double)d2.y) > 12.0 ? kStatusTooLong : 0;
}


__device__ __forceinline__ void store_pair(float4* X, float2 x, float2 y, float2 z) {
  X[0] = make_float4(x.x, y.x, z.x, 0.f);
  X[1] = make_float4(x.y, y.y, z.y, 0.f);
}

// TPP threads share one pose: each rotates its share of the atoms while the
// per-torsion axis and matrix are recomputed by all of them, and the sines and
// cosines of the pose's angles are computed once (FP64), split over the TPP
// threads.  Coordinates, axes, matrices and the rigid map are double-float.
// Small batches use many threads per pose (the one-pose path uses a whole
// warp), large batches few.
//
// rebuild_pose: one pose of the block's ligand; dof, Xo, Yo, reco, ceno and
// statuso point at the pose's own slots (dof readable even when !live).
// (not inlined: the one-system and the system-batch kernels share this code,
// so both round every operation the same way)
// entry k of the Rodrigues matrix of rot.ml:136-146 (c the cosine, o = 1 - c,
// u the axis, us = u sin)
__device__ __forceinline__ float2 rodrigues_entry(int k, float2 c, float2 ux, float2 uy, float2 uz,
                                                  float2 o, float2 xs, float2 ys, float2 zs) {
  switch (k) {
    case 0: return dadd(c, dmul(ux, dmul(ux, o)));
    case 1: return dsub(dmul(ux, dmul(uy, o)), zs);
    case 2: return dadd(dmul(ux, dmul(uz, o)), ys);
    case 3: return dadd(dmul(ux, dmul(uy, o)), zs);
    case 4: return dadd(c, dmul(uy, dmul(uy, o)));
    case 5: return dsub(dmul(uy, dmul(uz, o)), xs);
    case 6: return dsub(dmul(ux, dmul(uz, o)), ys);
    case 7: return dadd(dmul(uy, dmul(uz, o)), xs);
    default: return dadd(c, dmul(uz, dmul(uz, o)));
  }
}

// entry k of R = Rz(g) Ry(b) Rx(a) (rot.ml:52-66), k = 9..11 the translation
// (dof - origin), in double-float from the sines and cosines t[0..2] = (sin
// hi, sin lo, cos hi, cos lo) of a, b, g
__device__ __forceinline__ float2 rigid_entry_df(int k, const float4* t, const float* dof,
                                                 float orx, float ory, float orz) {
  const float2 sa = make_float2(t[0].x, t[0].y), ca = make_float2(t[0].z, t[0].w);
  const float2 sb = make_float2(t[1].x, t[1].y), cb = make_float2(t[1].z, t[1].w);
  const float2 sg = make_float2(t[2].x, t[2].y), cg = make_float2(t[2].z, t[2].w);
  switch (k) {
    case 0: return dmul(cb, cg);
    case 1: return dsub(dmul(dmul(cg, sa), sb), dmul(ca, sg));
    case 2: return dadd(dmul(sa, sg), dmul(dmul(ca, cg), sb));
    case 3: return dmul(cb, sg);
    case 4: return dadd(dmul(ca, cg), dmul(dmul(sa, sb), sg));
    case 5: return dsub(dmul(dmul(ca, sb), sg), dmul(cg, sa));
    case 6: return dneg(sb);
    case 7: return dmul(cb, sa);
    case 8: return dmul(ca, cb);
    case 9: return ts(dof[0], -orx);
    case 10: return ts(dof[1], -ory);
    default: return ts(dof[2], -orz);
  }
}

// the value v of lane `src` of this pose's group of TPP lanes
template <int TPP>
__device__ __forceinline__ float2 from_lane(float2 v, int src) {
  return make_float2(__shfl_sync(kFull, v.x, src, TPP), __shfl_sync(kFull, v.y, src, TPP));
}

// TPP threads share one pose: each rotates its share of the atoms; the
// torsion axis is recomputed by all of them, the entries of each matrix are
// split over them and exchanged by shuffles, and the sines and cosines of the
// pose's angles are computed once (FP64), split over the TPP threads.
// Coordinates, axes, matrices and the rigid map are double-float.  Small
// batches use many threads per pose (the one-pose path uses a whole warp),
// large batches fewer.
//
// rebuild_pose: one pose of the block's ligand; dof, Xo, Yo, reco, ceno and
// statuso point at the pose's own slots (dof readable even when !live).
// (not inlined: the one-system and the system-batch kernels share this code,
// so both round every operation the same way)
template <bool RECENTER, bool RECORD, int TPP>
__device__ __noinline__ void rebuild_pose(const DevLigand& lig, const float* dof, bool live,
                                             float orx, float ory, float orz, float4* Xo,
                                             float4* Yo, float4* reco, float4* ceno,
                                             int* statuso, const Scratch* sb, size_t e0) {
  constexpr int PPB = kRebuildThreads / TPP;  // poses per block
  constexpr int NANG = 3 + kMaxTors;
  // rebuild_smem's layout: [3][L][PPB] double-float coordinates, then
  // [PPB][NANG] double-float (sin, cos) of the angles, then (nested groups)
  // [PPB][nrb][12] the torsions' rotations about their reference axes
  extern __shared__ double sz[];
  const int tid = threadIdx.x, p = tid / TPP, sub = tid % TPP;
  const int L = lig.L, nrb = lig.nrb;
  float2* X = reinterpret_cast<float2*>(sz);
  float2* Yc = X + L * PPB;
  float2* Zc = X + 2 * L * PPB;
  float4* TSC = reinterpret_cast<float4*>(sz + 3 * L * PPB) + p * NANG;
  float2* ROT = reinterpret_cast<float2*>(reinterpret_cast<float4*>(sz + 3 * L * PPB) + PPB * NANG) +
                (size_t)p * nrb * 12;
#define AT(arr, a) arr[(a) * PPB + p]
  for (int a = sub; a < L; a += TPP) {
    AT(X, a) = lig.ref2[3 * a];
    AT(Yc, a) = lig.ref2[3 * a + 1];
    AT(Zc, a) = lig.ref2[3 * a + 2];
  }
  for (int k = sub; k < 3 + nrb; k += TPP) {
    float2 sn, cs;
    df_sincos(dof[3 + k], sn, cs);
    TSC[k] = make_float4(sn.x, sn.y, cs.x, cs.y);
  }
  __syncwarp();
  const float2 one = make_float2(1.f, 0.f);
  if (lig.nested) {
    // nested groups: each atom's rotations about the reference-frame axes,
    // innermost group first (equal to the bond-order application); the
    // rotations' entries split over the pose's lanes
    for (int e = sub; e < 12 * nrb; e += TPP) {
      const int t = e / 12, k = e - 12 * t;
      const float2* tx = lig.tax + 6 * t;
      if (k >= 9) {
        ROT[e] = tx[k - 6];
      } else {
        const float2 ux = tx[0], uy = tx[1], uz = tx[2];
        const float4 tsc = TSC[3 + t];
        const float2 sn = make_float2(tsc.x, tsc.y), cs = make_float2(tsc.z, tsc.w);
        ROT[e] = rodrigues_entry(k, cs, ux, uy, uz, dsub(one, cs), dmul(ux, sn), dmul(uy, sn),
                                 dmul(uz, sn));
      }
    }
    __syncwarp();
    for (int a = sub; a < L; a += TPP) {
      float2 x = AT(X, a), y = AT(Yc, a), z = AT(Zc, a);
      // the atom's own groups only, innermost first
      for (uint32_t mk = lig.ramask[a]; mk; mk &= mk - 1) {
        const float2* R = ROT + 12 * lig.tord[__ffs(mk) - 1];
        const float2 vx = dsub(x, R[9]), vy = dsub(y, R[10]), vz = dsub(z, R[11]);
        x = ddot3c(R[0], vx, R[1], vy, R[2], vz, R[9]);
        y = ddot3c(R[3], vx, R[4], vy, R[5], vz, R[10]);
        z = ddot3c(R[6], vx, R[7], vy, R[8], vz, R[11]);
      }
      AT(X, a) = x;
      AT(Yc, a) = y;
      AT(Zc, a) = z;
    }
    __syncwarp();
  }
  for (int t = 0; t < (lig.nested ? 0 : nrb); ++t) {
    const int2 bd = lig.bonds[t];
    const float2 cx = AT(X, bd.y), cy = AT(Yc, bd.y), cz = AT(Zc, bd.y);
    const float2 ax = dsub(cx, AT(X, bd.x)), ay = dsub(cy, AT(Yc, bd.x)),
                 az = dsub(cz, AT(Zc, bd.x));
    // 1 / |a|: the float estimate and one Newton step in double-float
    const float2 n2 = dadd(dadd(dmul(ax, ax), dmul(ay, ay)), dmul(az, az));
    const float r0 = rsqrtf(n2.x);
    const float2 err = dsub(one, dmul(n2, dmul(make_float2(r0, 0.f), make_float2(r0, 0.f))));
    const float2 inv = qts(r0, __fmul_rn(0.5f * r0, err.x));
    const float2 ux = dmul(ax, inv), uy = dmul(ay, inv), uz = dmul(az, inv);
    const float4 tsc = TSC[3 + t];
    const float2 sn = make_float2(tsc.x, tsc.y), cs = make_float2(tsc.z, tsc.w);
    const float2 o = dsub(one, cs);
    const float2 xs = dmul(ux, sn), ys = dmul(uy, sn), zs = dmul(uz, sn);
    // the nine entries, split over the pose's lanes
    float2 mine[(9 + TPP - 1) / TPP];
#pragma unroll
    for (int q = 0; q < (9 + TPP - 1) / TPP; ++q) {
      const int k = sub + q * TPP;
      mine[q] = k < 9 ? rodrigues_entry(k, cs, ux, uy, uz, o, xs, ys, zs) : one;
    }
    float2 R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = from_lane<TPP>(mine[k / TPP], k % TPP);
    __syncwarp();  // every thread of the pose has read the axis
    for (int k = lig.grp_off[t] + sub; k < lig.grp_off[t + 1]; k += TPP) {
      const int i = lig.grp_atoms[k];
      const float2 vx = dsub(AT(X, i), cx), vy = dsub(AT(Yc, i), cy), vz = dsub(AT(Zc, i), cz);
      AT(X, i) = ddot3c(R[0], vx, R[1], vy, R[2], vz, cx);
      AT(Yc, i) = ddot3c(R[3], vx, R[4], vy, R[5], vz, cy);
      AT(Zc, i) = ddot3c(R[6], vx, R[7], vy, R[8], vz, cz);
    }
    if (RECORD && !lig.nested && live && sub == 0) {
      float4* r = reco + (size_t)t * 3;
      r[0] = make_float4(cx.x, cy.x, cz.x, cs.x);
      r[1] = make_float4(ux.x, uy.x, uz.x, sn.x);
      r[2] = make_float4(inv.x, cx.y, cy.y, cz.y);  // 1 / |a| and the centre's lo part
    }
    __syncwarp();  // the rotated group is visible before the next axis is read
  }
  // centroid and enclosing radius, max_i (0.01 + |c - y_i|) > 12 (mol.ml:576-591)
  float2 mx = make_float2(0.f, 0.f), my = mx, mz = mx;
  for (int a = sub; a < L; a += TPP) {
    mx = dadd(mx, AT(X, a));
    my = dadd(my, AT(Yc, a));
    mz = dadd(mz, AT(Zc, a));
  }
#pragma unroll
  for (int o = TPP / 2; o > 0; o >>= 1) {
    mx = dadd(mx, dshfl_xor(mx, o));
    my = dadd(my, dshfl_xor(my, o));
    mz = dadd(mz, dshfl_xor(mz, o));
  }
  const float2 iL = make_float2(lig.ilh, lig.ill);  // df_of(1.0 / L)
  mx = dmul(mx, iL);
  my = dmul(my, iL);
  mz = dmul(mz, iL);
  float2 d2max = make_float2(0.f, 0.f);
  for (int a = sub; a < L; a += TPP) {
    const float2 dx = dsub(mx, AT(X, a)), dy = dsub(my, AT(Yc, a)), dz = dsub(mz, AT(Zc, a));
    const float2 d2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
    if (dgt(d2, d2max)) d2max = d2;
  }
#pragma unroll
  for (int o = TPP / 2; o > 0; o >>= 1) {
    const float2 other = dshfl_xor(d2max, o);
    if (dgt(other, d2max)) d2max = other;
  }
  const int status = too_long_of(d2max);
  // rigid map: twelve entries (rotation, translation) split over the pose's lanes
  float2 rm[(12 + TPP - 1) / TPP];
#pragma unroll
  for (int q = 0; q < (12 + TPP - 1) / TPP; ++q) {
    const int k = sub + q * TPP;
    rm[q] = k < 12 ? rigid_entry_df(k, TSC, dof, orx, ory, orz) : one;
  }
  float2 G[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) G[k] = from_lane<TPP>(rm[k / TPP], k % TPP);
  const float2 zero = make_float2(0.f, 0.f);
  const float2 ox = RECENTER ? mx : zero, oy = RECENTER ? my : zero, oz = RECENTER ? mz : zero;
  if (live) {
    for (int a = sub; a < L; a += TPP) {
      const float2 vx = dsub(AT(X, a), ox), vy = dsub(AT(Yc, a), oy), vz = dsub(AT(Zc, a), oz);
      const float2 px = ddot3c(G[0], vx, G[1], vy, G[2], vz, G[9]);
      const float2 py = ddot3c(G[3], vx, G[4], vy, G[5], vz, G[10]);
      const float2 pz = ddot3c(G[6], vx, G[7], vy, G[8], vz, G[11]);
      store_pair(Xo + (size_t)a * 2, px, py, pz);
      if (sb) {  // the cut-off sweep's entry binning (k_cull_bin's operations)
        const uint32_t cx = grid_cell(px.x, sb->glo[0], sb->ginv);
        const uint32_t cy = grid_cell(py.x, sb->glo[1], sb->ginv);
        const uint32_t cz = grid_cell(pz.x, sb->glo[2], sb->ginv);
        const int bn = sb->seg_of_atom[a] * kCullBins + (int)hilbert_cell(cx, cy, cz);
        sb->bin[e0 + a] = bn;
        sb->rank[e0 + a] = (int)atomicAdd(&sb->hist[bn], 1u);
      }
      if (RECORD && !lig.nested) {  // hi and lo parts: the reverse pass's lever arms
        Yo[2 * a] = make_float4(AT(X, a).x, AT(Yc, a).x, AT(Zc, a).x, 0.f);
        Yo[2 * a + 1] = make_float4(AT(X, a).y, AT(Yc, a).y, AT(Zc, a).y, 0.f);
      }
    }
    if (sub == 0) {
      if (RECORD && !lig.nested) {
        ceno[0] = make_float4(mx.x, my.x, mz.x, 0.f);
        ceno[1] = make_float4(mx.y, my.y, mz.y, 0.f);
      }
      *statuso = status;
    }
  }
#undef AT
}

template <bool RECENTER, bool RECORD, int TPP>
__global__ void __launch_bounds__(kRebuildThreads) k_rebuild(DevLigand lig, PoseIO io, Scratch scr) {
  constexpr int PPB = kRebuildThreads / TPP;
  const int b = blockIdx.x * PPB + (int)threadIdx.x / TPP;
  const bool live = b < io.B;
  const size_t bb = live ? b : 0;
  const int L = lig.L, nrb = lig.nrb, nd = 6 + nrb;
  rebuild_pose<RECENTER, RECORD, TPP>(
      lig, io.dofs + bb * nd, live, io.ox, io.oy, io.oz, scr.X + bb * L * 2,
      RECORD ? scr.Y + bb * L * 2 : nullptr, RECORD ? scr.rec + bb * nrb * 3 : nullptr,
      RECORD ? scr.cen + bb * 2 : nullptr, io.status + bb, scr.binning ? &scr : nullptr,
      bb * L);
  if (live && b == 0 && threadIdx.x % TPP == 0 && io.zero_err) *io.err = 0;
}

// ---------------------------------------------------------------------------
// k_finish
// ---------------------------------------------------------------------------
// Rodrigues matrix of rot.ml:136-146, row-major
__device__ __forceinline__ void axis_angle(float ux, float uy, float uz, float c, float s,
                                           float (&R)[9]) {
  const float o = 1.0f - c;
  R[0] = c + ux * ux * o;
  R[1] = ux * uy * o - uz * s;
  R[2] = ux * uz * o + uy * s;
  R[3] = ux * uy * o + uz * s;
  R[4] = c + uy * uy * o;
  R[5] = uy * uz * o - ux * s;
  R[6] = ux * uz * o - uy * s;
  R[7] = uy * uz * o + ux * s;
  R[8] = c + uz * uz * o;
}

template <int DIEL, int IFORM>
__device__ __forceinline__ float intra_pair_g(const float4* sh, const float4* sl, int i, int j,
                                              float4 par, float& e, float& dx, float& dy,
                                              float& dz, float4& ih, float4& jh, float4& il,
                                              float4& jl) {
  ih = sh[i];
  jh = sh[j];
  il = sl[i];
  jl = sl[j];
  dx = split_diff(ih.x, il.x, jh.x, jl.x);
  dy = split_diff(ih.y, il.y, jh.y, jl.y);
  dz = split_diff(ih.z, il.z, jh.z, jl.z);
  float g;
  uff_pair_eg<DIEL, IFORM>(dx, dy, dz, par.x, par.y, par.z, e, g);
  return g;
}

// shared memory of one finishing warp, in float4: coordinates hi and lo [L],
// torsion axes and centres [2 nrb], torsion records [3 nrb], then the per-lane
// torsion partials [nrb][33] as floats
__host__ __device__ constexpr int finish_warp_f4(int L, int nrb) {
  return 2 * L + 5 * nrb + (33 * nrb + 3) / 4;
}

// Final axis w_t and centre C_t of torsion t from the posed coordinates:
// saxis[t] = (w_t, index of the centre atom as int bits), saxis[nrb + t] = C_t
// (hi part).
__device__ __forceinline__ void torsion_frame(const DevLigand& lig, const float4* sxh,
                                              const float4* sxl, float4* saxis, int t) {
  const int nrb = lig.nrb;
  const int2 bd = lig.bonds[t];
  const float4 rh = sxh[bd.y], rl = sxl[bd.y];
  const float4 lh = sxh[bd.x], ll = sxl[bd.x];
  const float ax = split_diff(rh.x, rl.x, lh.x, ll.x), ay = split_diff(rh.y, rl.y, lh.y, ll.y),
              az = split_diff(rh.z, rl.z, lh.z, ll.z);
  const float inv = rsqrtf(ax * ax + ay * ay + az * az);
  saxis[t] = make_float4(ax * inv, ay * inv, az * inv, __int_as_float(bd.y));
  saxis[nrb + t] = rh;
}

// Interacting pair p (i < j): its energy into acc and, when crossing, the
// torsion terms (dE/dX_moving) . (w_t x (X_moving - C_t)) of every torsion
// whose group holds exactly one of the two atoms, into col[t * stride].
// (ij, par: the pair's atoms and parameters; amask: the atoms' group bits)
template <int DIEL, int IFORM>
__device__ __forceinline__ void intra_pair_terms_at(const float4* sxh, const float4* sxl,
                                                    const float4* saxis, int2 ij, float4 par,
                                                    const uint32_t* amask, bool crossing,
                                                    float& acc, float* col, int stride) {
  float ep, dx, dy, dz;
  float4 ih, jh, il, jl;
  const float g =
      intra_pair_g<DIEL, IFORM>(sxh, sxl, ij.x, ij.y, par, ep, dx, dy, dz, ih, jh, il, jl);
  acc += ep;
  uint32_t x = __float_as_uint(par.w);  // the torsions the pair straddles
  if (crossing && x) {
    const uint32_t mi = amask[ij.x];
    while (x) {
      const int t = __ffs(x) - 1;
      x &= x - 1;
      const bool in_i = (mi >> t) & 1u;
      // the lever X_moving - C_t from the hi/lo pairs: the hi parts alone
      // carry about 1e-6 A of rounding, which the cancelling terms amplify
      const float4 w = saxis[t];
      const int ci = __float_as_int(w.w);
      const float4 ch = sxh[ci], cl = sxl[ci];
      const float4 mh = in_i ? ih : jh, ml = in_i ? il : jl;
      const float lx = split_diff(mh.x, ml.x, ch.x, cl.x);
      const float ly = split_diff(mh.y, ml.y, ch.y, cl.y);
      const float lz = split_diff(mh.z, ml.z, ch.z, cl.z);
      const float v = dx * (w.y * lz - w.z * ly) + dy * (w.z * lx - w.x * lz) +
                      dz * (w.x * ly - w.y * lx);
      col[t * stride] = fmaf(in_i ? g : -g, v, col[t * stride]);
    }
  }
}

// the same for pair p of the ligand's list
template <int DIEL, int IFORM>
__device__ __forceinline__ void intra_pair_terms(const DevLigand& lig, const float4* sxh,
                                                 const float4* sxl, const float4* saxis, int p,
                                                 bool crossing, float& acc, float* col,
                                                 int stride) {
  intra_pair_terms_at<DIEL, IFORM>(sxh, sxl, saxis, lig.pair_ij[p], lig.pair_par[p], lig.amask,
                                   crossing, acc, col, stride);
}

// finish_pose: one warp, one pose.  ep / gp: the pose's inter partials
// [C][L]; Xb, Yb, recb, cenp, dof, grad, Eo, sto: the pose's own slots;
// Eio, when not null, gets the inter part of the energy;
// wsm: the warp's shared memory (finish_warp_f4 float4).  pre_dti non-null:
// the intra energy (pre_e) and the nested groups' torsion terms (pre_dti[t])
// were summed beforehand (k_finish_one), so the pair loop is skipped.
// (not inlined, as rebuild_pose)
template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__device__ __noinline__ void finish_pose(const DevLigand& lig, int C, const double* ep,
                                            const float4* gp, const float4* Xb, const float4* Yb,
                                            const float4* recb, const float4* cenp,
                                            const float* dof, float orx, float ory, float orz,
                                            float* grad, double* Eo, int* sto, double* Eio,
                                            int flags, float4* wsm, double pre_e = 0.0,
                                            const float* pre_dti = nullptr) {
  const bool pre = pre_dti != nullptr;
  const int lane = threadIdx.x & 31;
  const int L = lig.L, nrb = lig.nrb;
  float4* sxh = wsm;
  float4* sxl = sxh + L;
  float4* saxis = sxl + L;        // [nrb] final axes, then [nrb] centres
  float4* srec = saxis + 2 * nrb;  // [nrb][3] torsion records
  float* sdti = reinterpret_cast<float*>(srec + 3 * nrb);  // [nrb][33]
  if (GRAD && !lig.nested)  // the reverse pass reads them last: start the loads now
    for (int k = lane; k < 3 * nrb; k += 32) srec[k] = recb[k];
  const bool intra = flags & kFlagIntra, inter = flags & kFlagInter;
  double e = 0.0;
  if (inter)
    for (int k = lane; k < C * L; k += 32) e += ep[k];
  if (intra || (GRAD && lig.nested)) {  // (nested groups: the levers of the torsion sums)
    for (int a = lane; a < L; a += 32) {
      sxh[a] = Xb[(size_t)a * 2];
      sxl[a] = Xb[(size_t)a * 2 + 1];
    }
    __syncwarp();
  }
  const bool crossing = GRAD && intra && lig.nested && nrb > 0;
  if (crossing && !pre) {
    if (lane < nrb) torsion_frame(lig, sxh, sxl, saxis, lane);
    for (int t = 0; t < nrb; ++t) sdti[t * 33 + lane] = 0.f;
    __syncwarp();
  }
  if (intra && !pre) {
    // pairs lane, lane + 32, ... in that order, their records loaded four at a
    // time so that the loads' latencies overlap
    float acc = 0.f;
    for (int p0 = lane; p0 < lig.npairs; p0 += 4 * 32) {
      int2 ij[4];
      float4 par[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int p = p0 + 32 * u;
        ij[u] = p < lig.npairs ? lig.pair_ij[p] : make_int2(0, 0);
        par[u] = p < lig.npairs ? lig.pair_par[p] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (p0 + 32 * u < lig.npairs)
          intra_pair_terms_at<DIEL, IFORM>(sxh, sxl, saxis, ij[u], par[u], lig.amask, crossing,
                                           acc, sdti + lane, 33);
    }
    e += (double)acc;
  }
  if (intra && pre && lane == 0) e += pre_e;
  e = warp_sum(e);
  if (lane == 0) {
    *Eo = e;
    if (!isfinite(e)) *sto |= kStatusNonFinite;
  }
  if (Eio) {  // the inter partials alone, in the same order
    double ei = 0.0;
    if (inter)
      for (int k = lane; k < C * L; k += 32) ei += ep[k];
    ei = warp_sum(ei);
    if (lane == 0) *Eio = ei;
  }
  if (!GRAD) return;

  // dE/dX from the pair sweep (and the intra forces for general groups)
  float gx[kSlots], gy[kSlots], gz[kSlots];
#pragma unroll
  for (int s = 0; s < kSlots; ++s) gx[s] = gy[s] = gz[s] = 0.f;
  if (inter) {
    for (int c = 0; c < C; ++c) {
#pragma unroll
      for (int s = 0; s < kSlots; ++s) {
        const int a = lane + 32 * s;
        if (a < L) {
          const float4 g = gp[c * L + a];
          gx[s] += g.x;
          gy[s] += g.y;
          gz[s] += g.z;
        }
      }
    }
  }
  if (intra && !lig.nested) {
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      const int a = lane + 32 * s;
      if (a < L) {
        const float4 ah = sxh[a], al = sxl[a];
        float acc = 0.f;
        for (int k = lig.nb_off[a]; k < lig.nb_off[a + 1]; ++k) {
          const int j = lig.nb_idx[k];
          const float4 bh = sxh[j], bl = sxl[j];
          const float4 par = lig.nb_par[k];
          uff_pair<true, DIEL, IFORM>(split_diff(ah.x, al.x, bh.x, bl.x),
                                      split_diff(ah.y, al.y, bh.y, bl.y),
                                      split_diff(ah.z, al.z, bh.z, bl.z), par.x, par.y, par.z,
                                      acc, gx[s], gy[s], gz[s]);
        }
      }
    }
  }
  if (lig.nested) {
    // Nested groups: the gradient from the posed frame alone.  Rigid map:
    // dE/dt = F = sum G; dE/dR_kc = M_kc = sum_i G_ik Yc_ic with
    // Yc = R^T (X - t), so M = P R for P_rk = sum_i G_ir (X_i - t)_k.
    // Torsion t: w_t . sum_{i in G_t} (X_i - C_t) x (G_i - F / L) (F / L only
    // with the centroid removed) plus the straddling intra terms.
    __syncwarp();
    if (lane < nrb) torsion_frame(lig, sxh, sxl, saxis, lane);
    __syncwarp();
    float dti_mine = 0.f;
    if (crossing && pre) {
      if (lane < nrb) dti_mine = pre_dti[lane];
    } else if (crossing) {
      if (lane < nrb)
        for (int k = 0; k < 32; ++k) dti_mine += sdti[lane * 33 + k];
    }
    const float2 tx2 = ts(dof[0], -orx), ty2 = ts(dof[1], -ory), tz2 = ts(dof[2], -orz);
    float red[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) red[k] = 0.f;
    // the total force in double-float: the atoms' forces can cancel by orders
    // of magnitude in a clash
    float2 fsum[3] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      const int a = lane + 32 * s;
      if (a < L) {
        const float4 ph = sxh[a], pl = sxl[a];
        const float qx = split_diff(ph.x, pl.x, tx2.x, tx2.y);
        const float qy = split_diff(ph.y, pl.y, ty2.x, ty2.y);
        const float qz = split_diff(ph.z, pl.z, tz2.x, tz2.y);
        acc2(fsum[0], gx[s]);
        acc2(fsum[1], gy[s]);
        acc2(fsum[2], gz[s]);
        red[3] += gx[s] * qx; red[4] += gx[s] * qy; red[5] += gx[s] * qz;
        red[6] += gy[s] * qx; red[7] += gy[s] * qy; red[8] += gy[s] * qz;
        red[9] += gz[s] * qx; red[10] += gz[s] * qy; red[11] += gz[s] * qz;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) fsum[k] = dadd(fsum[k], dshfl_xor(fsum[k], o));
      red[k] = __fadd_rn(fsum[k].x, fsum[k].y);
    }
#pragma unroll
    for (int k = 3; k < 12; ++k) red[k] = warp_sum(red[k]);
    float sa, ca, sb, cb, sg, cg;
    sincosf(dof[3], &sa, &ca);
    sincosf(dof[4], &sb, &cb);
    sincosf(dof[5], &sg, &cg);
    if (lane == 0) {
      const float R[9] = {cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb,
                          cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa,
                          -sb,     cb * sa,                 ca * cb};
      float M[9];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          M[3 * r + c] = red[3 + 3 * r] * R[c] + red[4 + 3 * r] * R[3 + c] +
                         red[5 + 3 * r] * R[6 + c];
      // d R / d a, d b, d g of rot.ml:52-66, entry by entry
      const float dA[9] = {0.f, cg * ca * sb + sa * sg, ca * sg - sa * cg * sb,
                           0.f, -sa * cg + ca * sb * sg, -sa * sb * sg - cg * ca,
                           0.f, cb * ca, -sa * cb};
      const float dB[9] = {-sb * cg, cg * sa * cb, ca * cg * cb,
                           -sb * sg, sa * cb * sg, ca * cb * sg,
                           -cb, -sb * sa, -ca * sb};
      const float dG[9] = {-cb * sg, -sg * sa * sb - ca * cg, sa * cg - ca * sg * sb,
                           cb * cg, -ca * sg + sa * sb * cg, ca * sb * cg + sg * sa,
                           0.f, 0.f, 0.f};
      float ga = 0.f, gb = 0.f, gg = 0.f;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        ga += M[k] * dA[k];
        gb += M[k] * dB[k];
        gg += M[k] * dG[k];
      }
      grad[0] = red[0];
      grad[1] = red[1];
      grad[2] = red[2];
      grad[3] = ga;
      grad[4] = gb;
      grad[5] = gg;
    }
    const float iL = 1.0f / (float)L;
    const float fx = RECENTER ? red[0] * iL : 0.f, fy = RECENTER ? red[1] * iL : 0.f,
                fz = RECENTER ? red[2] * iL : 0.f;
    for (int t = 0; t < nrb; ++t) {
      const float4 w = saxis[t];
      const int ci = __float_as_int(w.w);
      const float4 ch = sxh[ci], cl = sxl[ci];
      float cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll
      for (int s = 0; s < kSlots; ++s) {
        if (32 * s >= L) break;  // uniform: no atoms in this slot
        if ((lig.gmask[t * kSlots + s] >> lane) & 1u) {
          const int a = lane + 32 * s;
          const float4 ah = sxh[a], al = sxl[a];
          const float lx = split_diff(ah.x, al.x, ch.x, cl.x);
          const float ly = split_diff(ah.y, al.y, ch.y, cl.y);
          const float lz = split_diff(ah.z, al.z, ch.z, cl.z);
          const float hx = gx[s] - fx, hy = gy[s] - fy, hz = gz[s] - fz;
          cx += ly * hz - lz * hy;
          cy += lz * hx - lx * hz;
          cz += lx * hy - ly * hx;
        }
      }
      const float v = warp_sum(w.x * cx + w.y * cy + w.z * cz);
      const float intra_t = __shfl_sync(kFull, dti_mine, t & 31);
      if (lane == 0) grad[6 + t] = v + intra_t;
    }
    return;
  }
  // coordinates after the torsions (recorded by k_rebuild): hi parts in
  // registers, lo parts in the warp's shared memory (the slot of the posed
  // coordinates' lo parts, which nothing reads from here on)
  float4* swl = sxl;
  __syncwarp();  // every lane is done with the posed coordinates
  float zx[kSlots], zy[kSlots], zz[kSlots];
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    const int a = lane + 32 * s;
    const float4 y = a < L ? Yb[2 * a] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (a < L) swl[a] = Yb[2 * a + 1];
    zx[s] = y.x;
    zy[s] = y.y;
    zz[s] = y.z;
  }
  const float4 cen = RECENTER ? cenp[0] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 cenl = RECENTER ? cenp[1] : make_float4(0.f, 0.f, 0.f, 0.f);
  float sa, ca, sb, cb, sg, cg;
  sincosf(dof[3], &sa, &ca);
  sincosf(dof[4], &sb, &cb);
  sincosf(dof[5], &sg, &cg);
  const float R[9] = {cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb,
                      cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa,
                      -sb,     cb * sa,                 ca * cb};
  // rigid map: dE/dt = sum G; dE/dR_kl = sum_i G_ik Yc_il
  float red[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) red[k] = 0.f;
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    if (lane + 32 * s < L) {
      const float4 w = swl[lane + 32 * s];
      const float yx = split_diff(zx[s], w.x, cen.x, cenl.x);
      const float yy = split_diff(zy[s], w.y, cen.y, cenl.y);
      const float yz = split_diff(zz[s], w.z, cen.z, cenl.z);
      red[0] += gx[s];
      red[1] += gy[s];
      red[2] += gz[s];
      red[3] += gx[s] * yx; red[4] += gx[s] * yy; red[5] += gx[s] * yz;
      red[6] += gy[s] * yx; red[7] += gy[s] * yy; red[8] += gy[s] * yz;
      red[9] += gz[s] * yx; red[10] += gz[s] * yy; red[11] += gz[s] * yz;
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) red[k] = warp_sum(red[k]);
  if (lane == 0) {
    const float* M = red + 3;
    // d R / d a, d b, d g of rot.ml:52-66, entry by entry
    const float dA[9] = {0.f, cg * ca * sb + sa * sg, ca * sg - sa * cg * sb,
                         0.f, -sa * cg + ca * sb * sg, -sa * sb * sg - cg * ca,
                         0.f, cb * ca, -sa * cb};
    const float dB[9] = {-sb * cg, cg * sa * cb, ca * cg * cb,
                         -sb * sg, sa * cb * sg, ca * cb * sg,
                         -cb, -sb * sa, -ca * sb};
    const float dG[9] = {-cb * sg, -sg * sa * sb - ca * cg, sa * cg - ca * sg * sb,
                         cb * cg, -ca * sg + sa * sb * cg, ca * sb * cg + sg * sa,
                         0.f, 0.f, 0.f};
    float ga = 0.f, gb = 0.f, gg = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      ga += M[k] * dA[k];
      gb += M[k] * dB[k];
      gg += M[k] * dG[k];
    }
    grad[0] = red[0];
    grad[1] = red[1];
    grad[2] = red[2];
    grad[3] = ga;
    grad[4] = gb;
    grad[5] = gg;
  }
  // adjoint of the pre-rigid coordinates: A = R^T G (minus its mean when the
  // centroid was removed)
  float ax[kSlots], ay[kSlots], az[kSlots];
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    ax[s] = R[0] * gx[s] + R[3] * gy[s] + R[6] * gz[s];
    ay[s] = R[1] * gx[s] + R[4] * gy[s] + R[7] * gz[s];
    az[s] = R[2] * gx[s] + R[5] * gy[s] + R[8] * gz[s];
  }
  if (RECENTER) {
    float mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
    for (int s = 0; s < kSlots; ++s)
      if (lane + 32 * s < L) {
        mx += ax[s];
        my += ay[s];
        mz += az[s];
      }
    const float inv = 1.0f / (float)L;
    mx = warp_sum(mx) * inv;
    my = warp_sum(my) * inv;
    mz = warp_sum(mz) * inv;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      ax[s] -= mx;
      ay[s] -= my;
      az[s] -= mz;
    }
  }
  // intra torsion terms of nested groups, each summed in lane order
  float dti_mine = 0.f;
  if (crossing && pre) {
    if (lane < nrb) dti_mine = pre_dti[lane];
  } else if (crossing) {
    __syncwarp();
    if (lane < nrb)
      for (int k = 0; k < 32; ++k) dti_mine += sdti[lane * 33 + k];
  }
  // reverse through the torsions, undoing each rotation on the way back
  __syncwarp();  // the prefetched torsion records
  for (int t = nrb - 1; t >= 0; --t) {
    const float4 r0 = srec[3 * t], r1 = srec[3 * t + 1], r2 = srec[3 * t + 2];
    const float ilen = r2.x;  // r2.yzw: the lo part of the centre r0.xyz
    float Rt[9];
    axis_angle(r1.x, r1.y, r1.z, r0.w, r1.w, Rt);
    float q[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) q[k] = 0.f;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      if (32 * s >= L) break;  // uniform: no atoms in this slot
      if ((lig.gmask[t * kSlots + s] >> lane) & 1u) {
        // v' = z - c from the hi/lo pairs (the hi parts alone carry the
        // rounding of coordinates far from the origin into the lever arms)
        const float4 w = swl[lane + 32 * s];
        const float px = split_diff(zx[s], w.x, r0.x, r2.y);
        const float py = split_diff(zy[s], w.y, r0.y, r2.z);
        const float pz = split_diff(zz[s], w.z, r0.z, r2.w);
        const float vx = Rt[0] * px + Rt[3] * py + Rt[6] * pz;                // v = R^T v'
        const float vy = Rt[1] * px + Rt[4] * py + Rt[7] * pz;
        const float vz = Rt[2] * px + Rt[5] * py + Rt[8] * pz;
        const float Ax = ax[s], Ay = ay[s], Az = az[s];
        // dtheta += A . (u x v')
        q[0] += Ax * (r1.y * pz - r1.z * py) + Ay * (r1.z * px - r1.x * pz) +
                Az * (r1.x * py - r1.y * px);
        // v x A
        q[1] += vy * Az - vz * Ay;
        q[2] += vz * Ax - vx * Az;
        q[3] += vx * Ay - vy * Ax;
        const float uv = r1.x * vx + r1.y * vy + r1.z * vz;
        const float Au = Ax * r1.x + Ay * r1.y + Az * r1.z;
        q[4] += uv * Ax + Au * vx;
        q[5] += uv * Ay + Au * vy;
        q[6] += uv * Az + Au * vz;
        q[7] += Ax;
        q[8] += Ay;
        q[9] += Az;
        ax[s] = Rt[0] * Ax + Rt[3] * Ay + Rt[6] * Az;
        ay[s] = Rt[1] * Ax + Rt[4] * Ay + Rt[7] * Az;
        az[s] = Rt[2] * Ax + Rt[5] * Ay + Rt[8] * Az;
        // z = c + v as a hi/lo pair
        float4 nw = make_float4(0.f, 0.f, 0.f, 0.f);
        dadd_into(r0.x, r2.y, vx, zx[s], nw.x);
        dadd_into(r0.y, r2.z, vy, zy[s], nw.y);
        dadd_into(r0.z, r2.w, vz, zz[s], nw.z);
        swl[lane + 32 * s] = nw;
      }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) q[k] = warp_sum(q[k]);
    // dE/du (Rodrigues form), projected on the sphere and moved to the axis atoms
    const float omc = 1.0f - r0.w;
    const float dUx = r1.w * q[1] + omc * q[4];
    const float dUy = r1.w * q[2] + omc * q[5];
    const float dUz = r1.w * q[3] + omc * q[6];
    const float uu = r1.x * dUx + r1.y * dUy + r1.z * dUz;
    const int2 bd = lig.bonds[t];
    const float dax = (dUx - r1.x * uu) * ilen;
    const float day = (dUy - r1.y * uu) * ilen;
    const float daz = (dUz - r1.z * uu) * ilen;
    // dE/dc = sum A - R^T sum A
    const float dCx = q[7] - (Rt[0] * q[7] + Rt[3] * q[8] + Rt[6] * q[9]);
    const float dCy = q[8] - (Rt[1] * q[7] + Rt[4] * q[8] + Rt[7] * q[9]);
    const float dCz = q[9] - (Rt[2] * q[7] + Rt[5] * q[8] + Rt[8] * q[9]);
    if (lane == (bd.y & 31)) {
#pragma unroll
      for (int s = 0; s < kSlots; ++s)
        if (s == (bd.y >> 5)) {
          ax[s] += dax + dCx;
          ay[s] += day + dCy;
          az[s] += daz + dCz;
        }
    }
    if (lane == (bd.x & 31)) {
#pragma unroll
      for (int s = 0; s < kSlots; ++s)
        if (s == (bd.x >> 5)) {
          ax[s] -= dax;
          ay[s] -= day;
          az[s] -= daz;
        }
    }
    const float intra_t = __shfl_sync(kFull, dti_mine, t & 31);
    if (lane == 0) grad[6 + t] = q[0] + intra_t;
  }
}

template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, kFinishBlocksPerSM)
    k_finish(DevLigand lig, PoseIO io, Scratch scr, int flags) {
  extern __shared__ __align__(16) float4 fsm[];
  const int wib = threadIdx.x >> 5;
  const int b = blockIdx.x * kWarpsPerBlock + wib;
  if (b >= io.B) return;
  const int L = lig.L, C = scr.C, nrb = lig.nrb, nd = 6 + nrb;
  const size_t ent = (size_t)b * L;
  finish_pose<GRAD, RECENTER, DIEL, IFORM>(
      lig, C, scr.Epart + ent * C, GRAD ? scr.Gpart + ent * C : nullptr, scr.X + ent * 2,
      GRAD ? scr.Y + ent * 2 : nullptr, GRAD ? scr.rec + (size_t)b * nrb * 3 : nullptr,
      GRAD ? scr.cen + b * 2 : nullptr, io.dofs + (size_t)b * nd, io.ox, io.oy, io.oz,
      GRAD ? io.grad + (size_t)b * nd : nullptr, io.E + b, io.status + b,
      io.E_inter ? io.E_inter + b : nullptr, flags, fsm + wib * finish_warp_f4(L, nrb));
}

// One pose (the one-pose path): the CTA's threads share the interacting pairs
// (the intra energy and the nested groups' torsion terms, each summed in a
// fixed order), then warp 0 runs the rest of finish_pose with those sums.
constexpr int kFinishOne = 256;

__host__ __device__ constexpr int finish_one_f4(int L, int nrb) {
  return 2 * L + 2 * nrb + kFinishOne / 64 + 1 + (nrb * (kFinishOne + 2) + 3) / 4 +
         finish_warp_f4(L, nrb);
}

// the body of k_finish_one, for a CTA of kFinishOne threads with fsm its
// finish_one_f4(L, nrb) float4 of shared memory
template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__device__ __forceinline__ void finish_one_cta(const DevLigand& lig, const PoseIO& io,
                                               const Scratch& scr, int flags, float4* fsm) {
  const int L = lig.L, nrb = lig.nrb, tid = threadIdx.x;
  float4* sxh = fsm;
  float4* sxl = sxh + L;
  float4* saxis = sxl + L;                                          // [2 nrb]
  double* sred = reinterpret_cast<double*>(saxis + 2 * nrb);        // [warps], then the total
  float* sdt = reinterpret_cast<float*>(saxis + 2 * nrb + kFinishOne / 64 + 1);
  float* stot = sdt + (size_t)nrb * (kFinishOne + 1);               // [nrb] torsion totals
  float4* wsm = saxis + 2 * nrb + kFinishOne / 64 + 1 + (nrb * (kFinishOne + 2) + 3) / 4;
  const bool intra = flags & kFlagIntra;
  const bool crossing = GRAD && intra && lig.nested && nrb > 0;
  if (intra)
    for (int a = tid; a < L; a += kFinishOne) {
      sxh[a] = scr.X[(size_t)a * 2];
      sxl[a] = scr.X[(size_t)a * 2 + 1];
    }
  if (crossing)
    for (int k = tid; k < nrb * (kFinishOne + 1); k += kFinishOne) sdt[k] = 0.f;
  __syncthreads();
  if (crossing && tid < nrb) torsion_frame(lig, sxh, sxl, saxis, tid);
  __syncthreads();
  if (intra) {
    float acc = 0.f;
    for (int p = tid; p < lig.npairs; p += kFinishOne)
      intra_pair_terms<DIEL, IFORM>(lig, sxh, sxl, saxis, p, crossing, acc, sdt + tid,
                                    kFinishOne + 1);
    const double w = warp_sum((double)acc);
    if ((tid & 31) == 0) sred[tid >> 5] = w;
  }
  __syncthreads();
  if (intra && tid == 0) {
    double e = 0.0;
    for (int k = 0; k < kFinishOne / 32; ++k) e += sred[k];
    sred[kFinishOne / 32] = e;
  }
  if (crossing && tid < nrb) {
    float t = 0.f;
    for (int k = 0; k < kFinishOne; ++k) t += sdt[tid * (kFinishOne + 1) + k];
    stot[tid] = t;
  }
  __syncthreads();
  if (tid >= 32) return;  // warp 0 alone from here: no block-wide barrier follows
  finish_pose<GRAD, RECENTER, DIEL, IFORM>(
      lig, scr.C, scr.Epart, GRAD ? scr.Gpart : nullptr, scr.X, GRAD ? scr.Y : nullptr,
      GRAD ? scr.rec : nullptr, GRAD ? scr.cen : nullptr, io.dofs, io.ox, io.oy, io.oz,
      GRAD ? io.grad : nullptr, io.E, io.status, io.E_inter, flags, wsm,
      intra ? sred[kFinishOne / 32] : 0.0, stot);
}

template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__global__ void __launch_bounds__(kFinishOne)
    k_finish_one(DevLigand lig, PoseIO io, Scratch scr, int flags) {
  extern __shared__ __align__(16) float4 fsm[];
  finish_one_cta<GRAD, RECENTER, DIEL, IFORM>(lig, io, scr, flags, fsm);
}

// ---------------------------------------------------------------------------
// k_one_pose: the one-pose path (the drop-in) in one launch.
//   1. every CTA rebuilds the pose.  For nested rotation groups
//      (DevLigand::nested: every two groups nested or disjoint, each axis
//      inside the groups that contain its group or on their axes) the
//      bond-order application of src/optim.ml:68-71 equals applying to each
//      atom the rotations of its groups about their axes in the reference
//      conformer, innermost group first: the rotations are built once (a
//      thread per matrix entry; axes, centres and the group order come from
//      the host) and every atom applies its own chain.  Other ligands take the
//      torsions in bond order (the operations of rebuild_pose), recording what
//      the reverse pass needs.  The angles' sines and cosines, the rigid map
//      and all sums are double-float on the FP32 pipe;
//   2. CTA 0, for nested groups with the intra term, sums the intra energy and
//      the terms of each torsion from the pairs that straddle its group; every
//      other CTA stages kOneChunk protein atoms in shared memory and sums their
//      pair terms against every ligand atom (kFinishOne / L threads per ligand
//      atom) into per-CTA partials;
//   3. the last CTA to arrive (an atomic count, nothing waits) adds the
//      partials in CTA order and finishes the pose.  For nested groups the
//      derivative of torsion t is a sum over its group in the posed frame,
//        dE/dtheta_t = w_t . sum_{i in G_t} (X_i - C_t) x (dE/dX_i - F / L)
//      (w_t the posed axis, C_t the posed centre atom, F the total force; F / L
//      only with the centroid removed), plus CTA 0's intra term, one warp per
//      torsion; the radius check runs on a spare warp meanwhile.  Other
//      ligands go through the work buffers and the one-pose finishing code
//      (finish_one_cta).
// ---------------------------------------------------------------------------
// shared-memory layout of k_one_pose, byte offsets (16-byte aligned)
struct OneLayout {
  int xh, xl, yr, rec, tsc, x, y, z, bonds, gmask, rig, cen, status, rot, ord, amask, uax;
  int sp, stype, pe, pg, qe, qg, sE, sG, saxis, sdt, sred, red, tT, tV, total;
};

__host__ __device__ inline int take16(int& off, int n) {
  const int p = off;
  off += (n + 15) / 16 * 16;
  return p;
}

__host__ __device__ inline OneLayout one_layout(int L, int nrb) {
  OneLayout o;
  int off = 0;
  o.xh = take16(off, 16 * L);
  o.xl = take16(off, 16 * L);
  o.yr = take16(off, 32 * L);
  o.rec = take16(off, 48 * nrb);
  o.tsc = take16(off, 16 * (3 + nrb));
  o.x = take16(off, 8 * L);
  o.y = take16(off, 8 * L);
  o.z = take16(off, 8 * L);
  o.bonds = take16(off, 8 * nrb);
  o.gmask = take16(off, 4 * nrb * kSlots);
  o.rig = take16(off, 8 * 12);
  o.cen = take16(off, 8 * 3);
  o.status = take16(off, 4);
  o.rot = take16(off, 8 * 12 * nrb);
  o.ord = take16(off, 4 * nrb);
  o.amask = take16(off, 4 * L);
  o.uax = take16(off, 8 * 3 * nrb);
  o.sp = take16(off, 32 * kOneChunk);
  o.stype = take16(off, 4 * kOneChunk);
  o.pe = take16(off, 4 * kFinishOne);
  o.pg = take16(off, 16 * kFinishOne);
  o.qe = take16(off, 8 * kFinishOne);
  o.qg = take16(off, 24 * kFinishOne);  // [3][kFinishOne] float2
  o.sE = take16(off, 8 * L);
  o.sG = take16(off, 16 * L);
  o.saxis = take16(off, 32 * nrb);
  o.sdt = take16(off, 4 * nrb * (kFinishOne + 1));
  o.sred = take16(off, 8 * (kFinishOne / 32 + 1));
  o.red = take16(off, 4 * 12);
  o.tT = take16(off, 16 * nrb);
  o.tV = take16(off, 16 * nrb);
  o.total = off;
  return o;
}

struct OneSmem {
  float4 *Xh, *Xl;     // [L] posed coordinates hi, lo
  float4* Y;           // [L][2] coordinates after the torsions hi, lo (bond-order path)
  float4* rec;         // [nrb][3] torsion records (bond-order path)
  float4* tsc;         // [3 + nrb] double-float (sin, cos) of the angles
  float2 *x, *y, *z;   // [L] double-float coordinates
  int2* bonds;         // [nrb]
  uint32_t* gmask;     // [nrb][kSlots]
  float2* G;           // [12] rigid map
  float2* cen;         // [3] centroid
  int* status;
  float2* rot;         // [nrb][12] reference-frame rotation of each torsion: matrix, centre
  int* ord;            // [nrb] torsions by group size, smallest first
  uint32_t* amask;     // [L] the groups of each atom (bit t: group t)
  float2* uax;         // [nrb][3] unit axis of each torsion in the reference conformer
  float4* sp;          // [kOneChunk][2] the CTA's protein atoms hi (q in w), lo
  int* stype;          // [kOneChunk] their types
  float* pe;           // [kFinishOne] per-thread pair sums
  float4* pg;
  float2* qe;          // [kFinishOne] per-thread sums of the partials (double-float)
  float2* qg;          // [3][kFinishOne]
  float2* sE;          // [L] inter energy per ligand atom (double-float)
  float4* sG;          // [L] dE/dX per ligand atom (inter terms)
  float4* saxis;       // [2 nrb] posed axes and centres (torsion_frame)
  float* sdt;          // [nrb][kFinishOne + 1] straddling intra terms per thread
  float2* sred;        // [warps] intra energy per warp (double-float)
  float* red;          // [12] total force and the rigid-map sums
  float4 *tT, *tV;     // [nrb] per torsion: sum of lever x force, sum of levers
};

__device__ __forceinline__ OneSmem one_smem(char* base, int L, int nrb) {
  const OneLayout o = one_layout(L, nrb);
  OneSmem m;
  m.Xh = reinterpret_cast<float4*>(base + o.xh);
  m.Xl = reinterpret_cast<float4*>(base + o.xl);
  m.Y = reinterpret_cast<float4*>(base + o.yr);
  m.rec = reinterpret_cast<float4*>(base + o.rec);
  m.tsc = reinterpret_cast<float4*>(base + o.tsc);
  m.x = reinterpret_cast<float2*>(base + o.x);
  m.y = reinterpret_cast<float2*>(base + o.y);
  m.z = reinterpret_cast<float2*>(base + o.z);
  m.bonds = reinterpret_cast<int2*>(base + o.bonds);
  m.gmask = reinterpret_cast<uint32_t*>(base + o.gmask);
  m.G = reinterpret_cast<float2*>(base + o.rig);
  m.cen = reinterpret_cast<float2*>(base + o.cen);
  m.status = reinterpret_cast<int*>(base + o.status);
  m.rot = reinterpret_cast<float2*>(base + o.rot);
  m.ord = reinterpret_cast<int*>(base + o.ord);
  m.amask = reinterpret_cast<uint32_t*>(base + o.amask);
  m.uax = reinterpret_cast<float2*>(base + o.uax);
  m.sp = reinterpret_cast<float4*>(base + o.sp);
  m.stype = reinterpret_cast<int*>(base + o.stype);
  m.pe = reinterpret_cast<float*>(base + o.pe);
  m.pg = reinterpret_cast<float4*>(base + o.pg);
  m.qe = reinterpret_cast<float2*>(base + o.qe);
  m.qg = reinterpret_cast<float2*>(base + o.qg);
  m.sE = reinterpret_cast<float2*>(base + o.sE);
  m.sG = reinterpret_cast<float4*>(base + o.sG);
  m.saxis = reinterpret_cast<float4*>(base + o.saxis);
  m.sdt = reinterpret_cast<float*>(base + o.sdt);
  m.sred = reinterpret_cast<float2*>(base + o.sred);
  m.red = reinterpret_cast<float*>(base + o.red);
  m.tT = reinterpret_cast<float4*>(base + o.tT);
  m.tV = reinterpret_cast<float4*>(base + o.tV);
  return m;
}

// unit vector (double-float) of the axis a = centre - left, with the inverse
// length; the operations of rebuild_pose
__device__ __forceinline__ void unit_axis(float2 ax, float2 ay, float2 az, float2& ux, float2& uy,
                                          float2& uz, float2& inv) {
  const float2 one = make_float2(1.f, 0.f);
  const float2 n2 = dadd(dadd(dmul(ax, ax), dmul(ay, ay)), dmul(az, az));
  const float r0 = rsqrtf(n2.x);
  const float2 err = dsub(one, dmul(n2, dmul(make_float2(r0, 0.f), make_float2(r0, 0.f))));
  inv = qts(r0, __fmul_rn(0.5f * r0, err.x));
  ux = dmul(ax, inv);
  uy = dmul(ay, inv);
  uz = dmul(az, inv);
}

// unit axis of the bond (left, centre) from the coordinates in shared memory
__device__ __forceinline__ void one_axis(const OneSmem& m, int2 bd, float2& ux, float2& uy,
                                         float2& uz, float2& inv) {
  unit_axis(dsub(m.x[bd.y], m.x[bd.x]), dsub(m.y[bd.y], m.y[bd.x]), dsub(m.z[bd.y], m.z[bd.x]),
            ux, uy, uz, inv);
}

// Reference conformer, the angles' sines and cosines (FP64, as rebuild_pose),
// the rigid map and the topology into shared memory.  For nested groups also
// the group sizes and, in warps 2-3 while warp 0 takes the FP64 sines and
// cosines, each torsion's unit axis and centre in the reference conformer.
__device__ __forceinline__ void one_load(const DevLigand& lig, const float* dof, float orx,
                                         float ory, float orz, const OneSmem& m) {
  const int tid = threadIdx.x, L = lig.L, nrb = lig.nrb;
  if (tid < 32) {
    for (int a = tid; a < 3 + nrb; a += 32) {
      float2 sn, cs;
      df_sincos(dof[3 + a], sn, cs);
      m.tsc[a] = make_float4(sn.x, sn.y, cs.x, cs.y);
    }
    __syncwarp();
    // rigid map: twelve entries (rotation, translation)
    if (tid < 12) m.G[tid] = rigid_entry_df(tid, m.tsc, dof, orx, ory, orz);
  } else if (lig.nested && tid >= 64 && tid < 64 + nrb) {
    // the torsion's unit axis and centre in the reference conformer, and the
    // group order (both from the host)
    const int t = tid - 64;
    const float2* tx = lig.tax + 6 * t;
    float2* r = m.rot + 12 * t;
    m.uax[3 * t] = tx[0];
    m.uax[3 * t + 1] = tx[1];
    m.uax[3 * t + 2] = tx[2];
    r[9] = tx[3];
    r[10] = tx[4];
    r[11] = tx[5];
    m.ord[t] = lig.tord[t];
  }
  if (tid < L) {
    m.x[tid] = lig.ref2[3 * tid];
    m.y[tid] = lig.ref2[3 * tid + 1];
    m.z[tid] = lig.ref2[3 * tid + 2];
    m.amask[tid] = lig.amask[tid];
  }
  for (int k = tid; k < nrb; k += blockDim.x) m.bonds[k] = lig.bonds[k];
  for (int k = tid; k < nrb * kSlots; k += blockDim.x) m.gmask[k] = lig.gmask[k];
}

// posed coordinates of atom a from its coordinates after the torsions
template <bool RECENTER>
__device__ __forceinline__ void one_posed(const OneSmem& m, int a, float2 x, float2 y, float2 z) {
  const float2 zero = make_float2(0.f, 0.f);
  const float2 vx = RECENTER ? dsub(x, m.cen[0]) : x, vy = RECENTER ? dsub(y, m.cen[1]) : y,
               vz = RECENTER ? dsub(z, m.cen[2]) : z;
  (void)zero;
  const float2 px = ddot3c(m.G[0], vx, m.G[1], vy, m.G[2], vz, m.G[9]);
  const float2 py = ddot3c(m.G[3], vx, m.G[4], vy, m.G[5], vz, m.G[10]);
  const float2 pz = ddot3c(m.G[6], vx, m.G[7], vy, m.G[8], vz, m.G[11]);
  m.Xh[a] = make_float4(px.x, py.x, pz.x, 0.f);
  m.Xl[a] = make_float4(px.y, py.y, pz.y, 0.f);
}

// warp 0: the centroid of the coordinates after the torsions (rebuild_pose's
// order for a pose of 32 lanes: atom a on lane a % 32, then the xor tree)
__device__ __forceinline__ void one_centroid(const DevLigand& lig, const OneSmem& m) {
  const int lane = threadIdx.x & 31, L = lig.L;
  float2 mx = make_float2(0.f, 0.f), my = mx, mz = mx;
  for (int a = lane; a < L; a += 32) {
    mx = dadd(mx, m.x[a]);
    my = dadd(my, m.y[a]);
    mz = dadd(mz, m.z[a]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = dadd(mx, dshfl_xor(mx, o));
    my = dadd(my, dshfl_xor(my, o));
    mz = dadd(mz, dshfl_xor(mz, o));
  }
  const float2 iL = make_float2(lig.ilh, lig.ill);  // df_of(1.0 / L)
  if (lane == 0) {
    m.cen[0] = dmul(mx, iL);
    m.cen[1] = dmul(my, iL);
    m.cen[2] = dmul(mz, iL);
  }
}

// warp 0, after one_centroid: the enclosing radius, max_i (0.01 + |c - y_i|)
// > 12 (mol.ml:576-591), into the status
__device__ __forceinline__ void one_radius(const DevLigand& lig, const OneSmem& m) {
  const int lane = threadIdx.x & 31, L = lig.L;
  __syncwarp();
  const float2 mx = m.cen[0], my = m.cen[1], mz = m.cen[2];
  float2 d2max = make_float2(0.f, 0.f);
  for (int a = lane; a < L; a += 32) {
    const float2 dx = dsub(mx, m.x[a]), dy = dsub(my, m.y[a]), dz = dsub(mz, m.z[a]);
    const float2 d2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
    if (dgt(d2, d2max)) d2max = d2;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float2 other = dshfl_xor(d2max, o);
    if (dgt(other, d2max)) d2max = other;
  }
  if (lane == 0) *m.status = too_long_of(d2max);
}

// Nested groups: the rotation of each torsion about its reference-frame axis
// (a thread per matrix entry), the group order, then each atom's chain of
// rotations, innermost group first, and (without the centroid) its posed
// coordinates.
template <bool RECENTER>
__device__ __forceinline__ void one_torsions_nested(const DevLigand& lig, const OneSmem& m) {
  const int tid = threadIdx.x, L = lig.L, nrb = lig.nrb;
  for (int e = tid; e < 9 * nrb; e += blockDim.x) {
    const int t = e / 9, k = e - 9 * t;
    const float2 ux = m.uax[3 * t], uy = m.uax[3 * t + 1], uz = m.uax[3 * t + 2];
    const float4 tsc = m.tsc[3 + t];
    const float2 sn = make_float2(tsc.x, tsc.y), cs = make_float2(tsc.z, tsc.w);
    const float2 o = dsub(make_float2(1.f, 0.f), cs);
    m.rot[12 * t + k] =
        rodrigues_entry(k, cs, ux, uy, uz, o, dmul(ux, sn), dmul(uy, sn), dmul(uz, sn));
  }
  __syncthreads();
  if (tid < L) {
    float2 x = m.x[tid], y = m.y[tid], z = m.z[tid];
    // the atom's own groups only, innermost first
    for (uint32_t mk = lig.ramask[tid]; mk; mk &= mk - 1) {
      const float2* R = m.rot + 12 * m.ord[__ffs(mk) - 1];
      const float2 vx = dsub(x, R[9]), vy = dsub(y, R[10]), vz = dsub(z, R[11]);
      x = ddot3c(R[0], vx, R[1], vy, R[2], vz, R[9]);
      y = ddot3c(R[3], vx, R[4], vy, R[5], vz, R[10]);
      z = ddot3c(R[6], vx, R[7], vy, R[8], vz, R[11]);
    }
    m.x[tid] = x;
    m.y[tid] = y;
    m.z[tid] = z;
    if (!RECENTER) one_posed<false>(m, tid, x, y, z);
  }
  __syncthreads();
  if (RECENTER) {
    if (tid < 32) one_centroid(lig, m);
    __syncthreads();
    if (tid < L) one_posed<true>(m, tid, m.x[tid], m.y[tid], m.z[tid]);
    __syncthreads();
  }
}

// Other ligands: the torsions in bond order, each rotating its group about
// the current axis (every thread recomputes the axis and its atom's matrix),
// with the records of the reverse pass when RECORD; then the centroid, the
// status and the posed coordinates.
template <bool RECENTER, bool RECORD>
__device__ __forceinline__ void one_torsions_seq(const DevLigand& lig, const OneSmem& m) {
  const int tid = threadIdx.x, L = lig.L, nrb = lig.nrb;
  for (int t = 0; t < nrb; ++t) {
    const int2 bd = m.bonds[t];
    const bool mine = tid < L && ((m.gmask[t * kSlots + (tid >> 5)] >> (tid & 31)) & 1u);
    if (mine || (RECORD && tid == 0)) {
      const float2 cx = m.x[bd.y], cy = m.y[bd.y], cz = m.z[bd.y];
      float2 ux, uy, uz, inv;
      one_axis(m, bd, ux, uy, uz, inv);
      const float4 tsc = m.tsc[3 + t];
      const float2 sn = make_float2(tsc.x, tsc.y), cs = make_float2(tsc.z, tsc.w);
      if (mine) {
        const float2 o = dsub(make_float2(1.f, 0.f), cs);
        const float2 xs = dmul(ux, sn), ys = dmul(uy, sn), zs = dmul(uz, sn);
        float2 R[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) R[k] = rodrigues_entry(k, cs, ux, uy, uz, o, xs, ys, zs);
        // the axis atoms are outside the group: no thread of the group reads a
        // coordinate another one writes
        const float2 vx = dsub(m.x[tid], cx), vy = dsub(m.y[tid], cy), vz = dsub(m.z[tid], cz);
        m.x[tid] = ddot3c(R[0], vx, R[1], vy, R[2], vz, cx);
        m.y[tid] = ddot3c(R[3], vx, R[4], vy, R[5], vz, cy);
        m.z[tid] = ddot3c(R[6], vx, R[7], vy, R[8], vz, cz);
      }
      if (RECORD && tid == 0) {
        m.rec[3 * t] = make_float4(cx.x, cy.x, cz.x, cs.x);
        m.rec[3 * t + 1] = make_float4(ux.x, uy.x, uz.x, sn.x);
        m.rec[3 * t + 2] = make_float4(inv.x, cx.y, cy.y, cz.y);
      }
    }
    __syncthreads();  // the rotated group is visible before the next axis is read
  }
  if (RECORD && tid < L) {
    m.Y[2 * tid] = make_float4(m.x[tid].x, m.y[tid].x, m.z[tid].x, 0.f);
    m.Y[2 * tid + 1] = make_float4(m.x[tid].y, m.y[tid].y, m.z[tid].y, 0.f);
  }
  if (tid < 32) {
    one_centroid(lig, m);
    one_radius(lig, m);
  }
  __syncthreads();
  if (tid < L) one_posed<RECENTER>(m, tid, m.x[tid], m.y[tid], m.z[tid]);
  __syncthreads();
}

// kPairBatch interacting pairs of one thread (pairs p0, p0 + kFinishOne, ...),
// loaded together so that their latencies overlap
constexpr int kPairBatch = 4;
struct PairBatch {
  int2 ij[kPairBatch];
  float4 par[kPairBatch];
};

__device__ __forceinline__ void load_pairs(const DevLigand& lig, int p0, PairBatch& b) {
#pragma unroll
  for (int u = 0; u < kPairBatch; ++u) {
    const int p = p0 + u * kFinishOne;
    b.ij[u] = p < lig.npairs ? lig.pair_ij[p] : make_int2(0, 0);
    b.par[u] = p < lig.npairs ? lig.pair_par[p] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// The intra CTA (nested groups): the intra energy and, with the gradient, the
// terms of each torsion from the pairs that straddle its group, from the
// posed coordinates alone; out[t] (t < nrb) the torsion terms, out[nrb],
// out[nrb + 1] the energy (double-float).
template <bool GRAD, int DIEL, int IFORM>
__device__ __forceinline__ void one_intra_terms(const DevLigand& lig, const OneSmem& m,
                                                float* out) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nrb = lig.nrb;
  constexpr int kWarps = kFinishOne / 32;
  const bool crossing = GRAD && nrb > 0;
  PairBatch pb;
  load_pairs(lig, tid, pb);
  if (crossing) {
    if (tid < nrb) torsion_frame(lig, m.Xh, m.Xl, m.saxis, tid);
    for (int k = tid; k < nrb * (kFinishOne + 1); k += kFinishOne) m.sdt[k] = 0.f;
  }
  __syncthreads();
  float acc = 0.f;
  for (int p0 = tid; p0 < lig.npairs; p0 += kPairBatch * kFinishOne) {
    if (p0 != tid) load_pairs(lig, p0, pb);
#pragma unroll
    for (int u = 0; u < kPairBatch; ++u)
      if (p0 + u * kFinishOne < lig.npairs)
        intra_pair_terms_at<DIEL, IFORM>(m.Xh, m.Xl, m.saxis, pb.ij[u], pb.par[u], m.amask,
                                         crossing, acc, m.sdt + tid, kFinishOne + 1);
  }
  float2 w = make_float2(acc, 0.f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) w = dadd(w, dshfl_xor(w, o));
  if (lane == 0) m.sred[warp] = w;
  __syncthreads();
  if (crossing)
    for (int t = warp; t < nrb; t += kWarps) {  // each torsion's column, in a fixed order
      float d = 0.f;
      for (int k = lane; k < kFinishOne; k += 32) d += m.sdt[t * (kFinishOne + 1) + k];
      d = warp_sum(d);
      if (lane == 0) out[t] = d;
    }
  if (tid == 0) {
    float2 e = m.sred[0];
    for (int k = 1; k < kWarps; ++k) e = dadd(e, m.sred[k]);
    out[nrb] = e.x;
    out[nrb + 1] = e.y;
  }
}

// The finish of a pose with nested groups in the last CTA, from shared memory
// (the inter partials summed, the torsion frames, the status) and the intra
// CTA's terms (intra_g; nullptr without the intra term): energy, status and
// with the gradient the rigid-map sums and the torsion derivatives
//   dE/dtheta_t = w_t . sum_{i in G_t} (X_i - C_t) x (dE/dX_i - F / L) + intra_t,
// one warp per item (energy on warp 0; twelve rigid sums and the torsions on
// warps 1, 2, ...).
template <bool GRAD, bool RECENTER>
__device__ __forceinline__ void finish_one_nested(const DevLigand& lig, const PoseIO& io,
                                                  const OneSmem& m, int flags,
                                                  const float* intra_g, int extra_status) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, L = lig.L, nrb = lig.nrb;
  constexpr int kWarps = kFinishOne / 32;
  if (warp == 0) {  // double-float sums; FP64 only for the outputs
    float2 ei = make_float2(0.f, 0.f);
    if (flags & kFlagInter)
      for (int a = lane; a < L; a += 32) ei = dadd(ei, m.sE[a]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ei = dadd(ei, dshfl_xor(ei, o));
    if (lane == 0) {
      float2 t = ei;
      if (intra_g) t = dadd(t, make_float2(__ldcg(intra_g + nrb), __ldcg(intra_g + nrb + 1)));
      const double e = (double)t.x + (double)t.y;
      io.E[0] = e;
      io.status[0] = *m.status | extra_status | (isfinite(e) ? 0 : kStatusNonFinite);
      if (io.E_inter) io.E_inter[0] = (double)ei.x + (double)ei.y;
    }
  }
  if (!GRAD) return;
  for (int it = (warp + kWarps - 1) % kWarps; it < 12 + nrb; it += kWarps) {
    if (it < 12) {
      // total force (q < 3) and M_rc = sum_i G_ir Yc_ic (q = 3 + 3 r + c), Yc
      // the coordinates after the torsions less the rotation origin
      const int q = it;
      float s = 0.f;
      if (q < 3) {  // the total force in double-float (clash forces cancel)
        float2 f = make_float2(0.f, 0.f);
        for (int a = lane; a < L; a += 32) {
          const float4 g = m.sG[a];
          acc2(f, q == 0 ? g.x : (q == 1 ? g.y : g.z));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) f = dadd(f, dshfl_xor(f, o));
        if (lane == 0) m.red[q] = __fadd_rn(f.x, f.y);
        continue;
      }
      for (int a = lane; a < L; a += 32) {
        const float4 g = m.sG[a];
        {
          const int r = (q - 3) / 3, c = q - 3 - 3 * r;
          const float gr = r == 0 ? g.x : (r == 1 ? g.y : g.z);
          const float2 yv = c == 0 ? m.x[a] : (c == 1 ? m.y[a] : m.z[a]);
          const float2 ce = RECENTER ? m.cen[c] : make_float2(0.f, 0.f);
          s += gr * split_diff(yv.x, yv.y, ce.x, ce.y);
        }
      }
      s = warp_sum(s);
      if (lane == 0) m.red[q] = s;
    } else {
      const int t = it - 12;
      const float4 w = m.saxis[t];
      const int ci = __float_as_int(w.w);
      const float4 ch = m.Xh[ci], cl = m.Xl[ci];
      float tx = 0.f, ty = 0.f, tz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
      for (int a = lane; a < L; a += 32) {
        if ((m.gmask[t * kSlots + (a >> 5)] >> (a & 31)) & 1u) {
          const float4 g = m.sG[a];
          const float4 ah = m.Xh[a], al = m.Xl[a];
          // the lever X_i - C_t from the hi/lo pairs
          const float lx = split_diff(ah.x, al.x, ch.x, cl.x);
          const float ly = split_diff(ah.y, al.y, ch.y, cl.y);
          const float lz = split_diff(ah.z, al.z, ch.z, cl.z);
          tx += ly * g.z - lz * g.y;
          ty += lz * g.x - lx * g.z;
          tz += lx * g.y - ly * g.x;
          if (RECENTER) {
            vx += lx;
            vy += ly;
            vz += lz;
          }
        }
      }
      tx = warp_sum(tx);
      ty = warp_sum(ty);
      tz = warp_sum(tz);
      if (RECENTER) {
        vx = warp_sum(vx);
        vy = warp_sum(vy);
        vz = warp_sum(vz);
        if (lane == 0) {
          m.tT[t] = make_float4(tx, ty, tz, 0.f);
          m.tV[t] = make_float4(vx, vy, vz, 0.f);
        }
      } else if (lane == 0) {
        io.grad[6 + t] = w.x * tx + w.y * ty + w.z * tz + (intra_g ? __ldcg(intra_g + t) : 0.f);
      }
    }
  }
  __syncthreads();
  if (RECENTER && tid < nrb) {
    // sum_i l_i x (G_i - F / L) = T - V x F / L
    const float iL = 1.0f / (float)L;
    const float fx = m.red[0] * iL, fy = m.red[1] * iL, fz = m.red[2] * iL;
    const float4 T = m.tT[tid], V = m.tV[tid], w = m.saxis[tid];
    const float cx = T.x - (V.y * fz - V.z * fy), cy = T.y - (V.z * fx - V.x * fz),
                cz = T.z - (V.x * fy - V.y * fx);
    io.grad[6 + tid] = w.x * cx + w.y * cy + w.z * cz + (intra_g ? __ldcg(intra_g + tid) : 0.f);
  }
  if (tid == kFinishOne - 32) {  // the rigid map: translation, then d R / d a, d b, d g of rot.ml:52-66
    const float* M = m.red + 3;
    float sa, ca, sb, cb, sg, cg;
    sincosf(io.dofs[3], &sa, &ca);
    sincosf(io.dofs[4], &sb, &cb);
    sincosf(io.dofs[5], &sg, &cg);
    const float dA[9] = {0.f, cg * ca * sb + sa * sg, ca * sg - sa * cg * sb,
                         0.f, -sa * cg + ca * sb * sg, -sa * sb * sg - cg * ca,
                         0.f, cb * ca, -sa * cb};
    const float dB[9] = {-sb * cg, cg * sa * cb, ca * cg * cb,
                         -sb * sg, sa * cb * sg, ca * cb * sg,
                         -cb, -sb * sa, -ca * sb};
    const float dG[9] = {-cb * sg, -sg * sa * sb - ca * cg, sa * cg - ca * sg * sb,
                         cb * cg, -ca * sg + sa * sb * cg, ca * sb * cg + sg * sa,
                         0.f, 0.f, 0.f};
    float ga = 0.f, gb = 0.f, gg = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      ga += M[k] * dA[k];
      gb += M[k] * dB[k];
      gg += M[k] * dG[k];
    }
    io.grad[0] = m.red[0];
    io.grad[1] = m.red[1];
    io.grad[2] = m.red[2];
    io.grad[3] = ga;
    io.grad[4] = gb;
    io.grad[5] = gg;
  }
}

// static shared memory of k_one_pose (type table and flags), rounded up
constexpr int kOneStatic = 2048;
static_assert(sizeof(float2) * kNTypes * kNTypes + 32 <= kOneStatic, "k_one_pose static smem");

template <bool GRAD, bool RECENTER, int DIEL, int FORM, int IFORM>
__global__ void __launch_bounds__(kFinishOne)
    k_one_pose(DevLigand lig, DevProtein prot, const float4* __restrict__ tab4, PoseIO io,
               Scratch scr, OneScratch os, int flags) {
  extern __shared__ __align__(16) float4 osm[];
  __shared__ float2 stab[kNTypes * kNTypes];
  __shared__ int s_last, s_offgrid;
  const int tid = threadIdx.x, L = lig.L, nrb = lig.nrb;
  const bool nested = lig.nested;
  const OneSmem m = one_smem(reinterpret_cast<char*>(osm), L, nrb);
  if (blockIdx.x == 0 && tid == 0 && io.zero_err) *io.err = 0;
  // CTA 0 takes the intra terms when os.with_intra (nested groups), the others
  // a chunk of protein atoms each; their loads overlap the rebuild
  const bool intra_cta = os.with_intra && blockIdx.x == 0;
  const int c = blockIdx.x - os.with_intra;  // the pair chunk
  const int c0 = c * kOneChunk, n = intra_cta || os.grid ? 0 : min(kOneChunk, prot.P - c0);
  if (tid < n) {
    m.sp[2 * tid] = prot.atoms[2 * (c0 + tid)];
    m.sp[2 * tid + 1] = prot.atoms[2 * (c0 + tid) + 1];
    m.stype[tid] = prot.type[c0 + tid];
  }
  for (int k = tid; k < kNTypes * kNTypes; k += blockDim.x) {
    const float4 v = tab4[k];  // (X, 1 / D, x^2, D)
    stab[k] = make_float2(v.z, v.w);
  }
  const int S = kFinishOne / L;  // threads per ligand atom in the pair sums
  const int j = tid % L, g = tid / L;
  const float qj = g < S ? lig.q[j] : 0.f;
  const int lt = g < S ? lig.type[j] : 0;
  one_load(lig, io.dofs, io.ox, io.oy, io.oz, m);
  __syncthreads();
  if (nested) {
    one_torsions_nested<RECENTER>(lig, m);  // the status waits for the last CTA
  } else {
    one_torsions_seq<RECENTER, GRAD>(lig, m);
  }
  if (intra_cta) {
    one_intra_terms<GRAD, DIEL, IFORM>(lig, m, os.intra);
  } else if (os.grid) {
    // MMO_F_GRID: the inter terms of every ligand atom from its type's grid
    // (k_grid_inter's lookup), a thread per atom
    if (tid == 0) s_offgrid = 0;
    __syncthreads();
    if (tid < L) {
      float e, gx, gy, gz;
      if (!grid_entry<GRAD>(os.gl, m.Xh[tid], m.Xl[tid], os.grid_lt[tid], os.grids, e, gx, gy,
                            gz))
        atomicOr(&s_offgrid, kStatusOffGrid);
      os.E[tid] = make_float2(e, 0.f);
      if (GRAD) os.G[tid] = make_float4(gx, gy, gz, 0.f);
    }
    __syncthreads();
    if (tid == 0) *os.gstat = s_offgrid;
  } else {
    // the pair terms of this CTA's protein atoms
    if (g < S) {
      const float4 xh = m.Xh[j], xl = m.Xl[j];
      float ae = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
      for (int i = g; i < n; i += S) {
        const float4 p = m.sp[2 * i], pl = m.sp[2 * i + 1];
        const float2 xd = stab[m.stype[i] * kNTypes + lt];
        uff_pair<GRAD, DIEL, FORM>(split_diff(xh.x, xl.x, p.x, pl.x),
                                   split_diff(xh.y, xl.y, p.y, pl.y),
                                   split_diff(xh.z, xl.z, p.z, pl.z), xd.x, xd.y, p.w * qj, ae,
                                   gx, gy, gz);
      }
      m.pe[tid] = ae;
      m.pg[tid] = make_float4(gx, gy, gz, 0.f);
    }
    __syncthreads();
    if (tid < L) {
      float2 e = make_float2(0.f, 0.f);
      float sx = 0.f, sy = 0.f, sz = 0.f;
      for (int k = 0; k < S; ++k) {
        acc2(e, m.pe[k * L + tid]);
        if (GRAD) {
          const float4 p = m.pg[k * L + tid];
          sx += p.x;
          sy += p.y;
          sz += p.z;
        }
      }
      os.E[(size_t)c * L + tid] = e;
      if (GRAD) os.G[(size_t)c * L + tid] = make_float4(sx, sy, sz, 0.f);
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(os.arrive, 1u) == (unsigned)gridDim.x - 1u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // the last CTA.  Nested groups with the gradient: the posed torsion frames
  if (GRAD && nested && tid < nrb) torsion_frame(lig, m.Xh, m.Xl, m.saxis, tid);
  // the partials of every pair CTA, thread (jq, gq) over chunks gq, gq + Sq, ...
  // (double-float sums on the FP32 pipe; loads in batches of kBatch)
  const int npair = gridDim.x - os.with_intra;
  constexpr int kBatch = 10;
  const float2 z2 = make_float2(0.f, 0.f);
  float2 e = z2, sx = z2, sy = z2, sz = z2;
  float2 ev[kBatch];
  float4 gv[kBatch];
  // the last warp is left free for the status
  const int Sq = (kFinishOne - 32) / L;
  const int jq = tid % L, gq = tid / L;
  const bool summing = gq < Sq;
  int k0 = gq;
  auto load_batch = [&]() {
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int k = k0 + u * Sq;
      ev[u] = k < npair ? __ldcg(os.E + (size_t)k * L + jq) : z2;
      if (GRAD)
        gv[u] = k < npair ? __ldcg(os.G + (size_t)k * L + jq) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  if (summing) load_batch();
  // nested groups: the last warp (whole) takes the status meanwhile
  if (nested && tid >= kFinishOne - 32) {
    if (!RECENTER) one_centroid(lig, m);
    one_radius(lig, m);
  }
  if (summing) {
    while (k0 < npair) {
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        e = dadd(e, ev[u]);
        if (GRAD) {
          acc2(sx, gv[u].x);
          acc2(sy, gv[u].y);
          acc2(sz, gv[u].z);
        }
      }
      k0 += kBatch * Sq;
      if (k0 < npair) load_batch();
    }
    m.qe[tid] = e;
    if (GRAD) {
      m.qg[tid] = sx;
      m.qg[kFinishOne + tid] = sy;
      m.qg[2 * kFinishOne + tid] = sz;
    }
  }
  __syncthreads();
  if (tid < L) {
    float2 e = z2, sx = z2, sy = z2, sz = z2;
    for (int k = 0; k < Sq; ++k) {
      e = dadd(e, m.qe[k * L + tid]);
      if (GRAD) {
        sx = dadd(sx, m.qg[k * L + tid]);
        sy = dadd(sy, m.qg[kFinishOne + k * L + tid]);
        sz = dadd(sz, m.qg[2 * kFinishOne + k * L + tid]);
      }
    }
    m.sE[tid] = e;
    if (GRAD)
      m.sG[tid] = make_float4(__fadd_rn(sx.x, sx.y), __fadd_rn(sy.x, sy.y),
                              __fadd_rn(sz.x, sz.y), 0.f);
  }
  if (tid == 0) *os.arrive = 0u;  // ready for the next launch
  const int gst = os.grid ? __ldcg(os.gstat) : 0;  // the lookup CTA's off-lattice bit
  __syncthreads();
  if (nested) {
    finish_one_nested<GRAD, RECENTER>(lig, io, m, flags, os.with_intra ? os.intra : nullptr,
                                      gst);
    return;
  }
  // other ligands: the work buffers of the one-pose finishing code
  for (int a = tid; a < L; a += blockDim.x) {
    scr.Epart[a] = (double)m.sE[a].x + (double)m.sE[a].y;
    if (GRAD) scr.Gpart[a] = m.sG[a];
    scr.X[2 * a] = m.Xh[a];
    scr.X[2 * a + 1] = m.Xl[a];
    if (GRAD) {
      scr.Y[2 * a] = m.Y[2 * a];
      scr.Y[2 * a + 1] = m.Y[2 * a + 1];
    }
  }
  if (GRAD) {
    for (int k = tid; k < 3 * nrb; k += blockDim.x) scr.rec[k] = m.rec[k];
    if (tid == 0) {
      scr.cen[0] = make_float4(m.cen[0].x, m.cen[1].x, m.cen[2].x, 0.f);
      scr.cen[1] = make_float4(m.cen[0].y, m.cen[1].y, m.cen[2].y, 0.f);
    }
  }
  if (tid == 0) io.status[0] = *m.status | gst;
  __syncthreads();  // the buffers above are written before the finish reads them
  finish_one_cta<GRAD, RECENTER, DIEL, IFORM>(lig, io, scr, flags, osm);
}


// one warp: intra-ligand energy of one set of hi/lo coordinates X[L][2]
// (mol.ml:881-903)
template <int DIEL, int IFORM>
__global__ void k_intra_plain(DevLigand lig, const float4* X, double* out) {
  float acc = 0.f, d0 = 0.f, d1 = 0.f, d2 = 0.f;
  for (int p = threadIdx.x; p < lig.npairs; p += 32) {
    const int2 ij = lig.pair_ij[p];
    const float4 par = lig.pair_par[p];
    const float4 ih = X[2 * ij.x], il = X[2 * ij.x + 1], jh = X[2 * ij.y], jl = X[2 * ij.y + 1];
    uff_pair<false, DIEL, IFORM>(split_diff(ih.x, il.x, jh.x, jl.x),
                                 split_diff(ih.y, il.y, jh.y, jl.y),
                                 split_diff(ih.z, il.z, jh.z, jl.z), par.x, par.y, par.z, acc,
                                 d0, d1, d2);
  }
  const double e = warp_sum((double)acc);
  if (threadIdx.x == 0) out[0] = e;
}

template <bool RC, bool REC, int TPP>
cudaError_t rebuild_t(const DevLigand& lig, const PoseIO& io, const Scratch& s, cudaStream_t st) {
  constexpr int PPB = kRebuildThreads / TPP;
  const int blocks = (io.B + PPB - 1) / PPB;
  const size_t smem = rebuild_smem(lig.L, lig.nrb, PPB);
  cudaError_t e = cudaFuncSetAttribute(k_rebuild<RC, REC, TPP>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_rebuild<RC, REC, TPP><<<blocks, kRebuildThreads, smem, st>>>(lig, io, s);
  return cudaGetLastError();
}

template <bool RC, bool REC>
cudaError_t rebuild_tpp(int tpp, const DevLigand& lig, const PoseIO& io, const Scratch& s,
                        cudaStream_t st) {
  switch (tpp) {
    case 1: return rebuild_t<RC, REC, 1>(lig, io, s, st);
    case 2: return rebuild_t<RC, REC, 2>(lig, io, s, st);
    case 4: return rebuild_t<RC, REC, 4>(lig, io, s, st);
    case 8: return rebuild_t<RC, REC, 8>(lig, io, s, st);
    case 16: return rebuild_t<RC, REC, 16>(lig, io, s, st);
    default: return rebuild_t<RC, REC, 32>(lig, io, s, st);
  }
}

template <bool G, bool RC, int DIEL, int IFORM>
cudaError_t finish_t(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                     cudaStream_t st) {
  if (io.B == 1) {  // one pose: a CTA shares its intra pairs
    const int smem = finish_one_f4(lig.L, lig.nrb) * (int)sizeof(float4);
    if (smem > 48 * 1024) {
      const cudaError_t e = cudaFuncSetAttribute(k_finish_one<G, RC, DIEL, IFORM>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
    }
    k_finish_one<G, RC, DIEL, IFORM><<<1, kFinishOne, smem, st>>>(lig, io, s, flags);
    return cudaGetLastError();
  }
  const int blocks = (io.B + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const int smem = kWarpsPerBlock * finish_warp_f4(lig.L, lig.nrb) * (int)sizeof(float4);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k_finish<G, RC, DIEL, IFORM>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  k_finish<G, RC, DIEL, IFORM><<<blocks, kWarpsPerBlock * 32, smem, st>>>(lig, io, s, flags);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ragged batch of systems: the same per-pose bodies, one system per block
// ---------------------------------------------------------------------------
template <bool RECENTER, bool RECORD, int TPP>
__global__ void __launch_bounds__(kRebuildThreads)
    k_sys_rebuild(DevSystems S, PoseIO io, Scratch scr) {
  __shared__ DevLigand slig;
  const SysBlk blk = S.rblk[blockIdx.x];
  if (threadIdx.x == 0) slig = S.lig[blk.sys];
  __syncthreads();
  const SysInfo& inf = S.info[blk.sys];
  const int p = (int)threadIdx.x / TPP;
  const bool live = p < blk.n;
  const int lp = blk.p0 + (live ? p : 0);
  const int L = slig.L, nrb = slig.nrb;
  const size_t b = (size_t)inf.pose0 + lp, ent = (size_t)inf.ent0 + (size_t)lp * L;
  const size_t rec = (size_t)inf.rec0 + (size_t)lp * nrb;
  rebuild_pose<RECENTER, RECORD, TPP>(
      slig, io.dofs + (size_t)inf.dof0 + (size_t)lp * (6 + nrb), live, inf.ox, inf.oy, inf.oz,
      scr.X + ent * 2, RECORD ? scr.Y + ent * 2 : nullptr, RECORD ? scr.rec + rec * 3 : nullptr,
      RECORD ? scr.cen + b * 2 : nullptr, io.status + b, nullptr, 0);
}

template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, kFinishBlocksPerSM)
    k_sys_finish(DevSystems S, PoseIO io, Scratch scr, int flags) {
  extern __shared__ __align__(16) float4 fsm[];
  __shared__ DevLigand slig;
  const SysBlk blk = S.fblk[blockIdx.x];
  if (threadIdx.x == 0) slig = S.lig[blk.sys];
  __syncthreads();
  const int wib = threadIdx.x >> 5;
  if (wib >= blk.n) return;
  const SysInfo& inf = S.info[blk.sys];
  const int lp = blk.p0 + wib;
  const int L = slig.L, nrb = slig.nrb;
  const size_t b = (size_t)inf.pose0 + lp, ent = (size_t)inf.ent0 + (size_t)lp * L;
  const size_t rec = (size_t)inf.rec0 + (size_t)lp * nrb, dof = (size_t)inf.dof0 + (size_t)lp * (6 + nrb);
  finish_pose<GRAD, RECENTER, DIEL, IFORM>(
      slig, 1, scr.Epart + ent, GRAD ? scr.Gpart + ent : nullptr, scr.X + ent * 2,
      GRAD ? scr.Y + ent * 2 : nullptr, GRAD ? scr.rec + rec * 3 : nullptr,
      GRAD ? scr.cen + b * 2 : nullptr, io.dofs + dof, inf.ox, inf.oy, inf.oz,
      GRAD ? io.grad + dof : nullptr, io.E + b, io.status + b, nullptr, flags,
      fsm + wib * finish_warp_f4(S.Lmax, S.nrbmax));
}

template <bool RC, bool REC>
cudaError_t sys_rebuild_tpp(int tpp, const DevSystems& S, int nblk, const PoseIO& io,
                            const Scratch& s, cudaStream_t st) {
  const int ppb = kRebuildThreads / tpp;
  const int smem = (int)rebuild_smem(S.Lmax, S.nrbmax, ppb);
#define MMO_SR(T)                                                                          \
  case T: {                                                                                \
    cudaError_t e = cudaFuncSetAttribute(k_sys_rebuild<RC, REC, T>,                        \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem); \
    if (e != cudaSuccess) return e;                                                        \
    k_sys_rebuild<RC, REC, T><<<nblk, kRebuildThreads, smem, st>>>(S, io, s);              \
    return cudaGetLastError();                                                             \
  }
  switch (tpp) {
    MMO_SR(1) MMO_SR(2) MMO_SR(4) MMO_SR(8) MMO_SR(16) MMO_SR(32)
  }
#undef MMO_SR
  return cudaErrorInvalidValue;
}

template <bool G, bool RC, int DIEL, int IFORM>
cudaError_t sys_finish_t(const DevSystems& S, int nblk, const PoseIO& io, const Scratch& s,
                         int flags, cudaStream_t st) {
  const int smem = kWarpsPerBlock * finish_warp_f4(S.Lmax, S.nrbmax) * (int)sizeof(float4);
  if (smem + (int)sizeof(DevLigand) > 48 * 1024) {  // the opt-in counts the static slig
    const cudaError_t e = cudaFuncSetAttribute(k_sys_finish<G, RC, DIEL, IFORM>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  k_sys_finish<G, RC, DIEL, IFORM><<<nblk, kWarpsPerBlock * 32, smem, st>>>(S, io, s, flags);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_rebuild(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                           cudaStream_t st) {
  if (io.B <= 0) return cudaSuccess;
  const bool rc = flags & kFlagRecenter;
  const bool rec = (flags & kFlagGrad) && io.grad;
  // threads per pose: up to a warp per pose while the batch keeps fewer than
  // about 160,000 threads in flight (half of GB300's 152 x 2,048), within 200 KB
  // of shared memory; more threads per pose shorten each pose's chain
  int tpp = 32;
  while (tpp > 1 && (long)io.B * (tpp / 2) >= kRebuildThreadsInFlight) tpp /= 2;
  while (tpp < 32 && rebuild_smem(lig.L, lig.nrb, kRebuildThreads / tpp) > 200 * 1024) tpp *= 2;
  if (rc) return rec ? rebuild_tpp<true, true>(tpp, lig, io, s, st)
                     : rebuild_tpp<true, false>(tpp, lig, io, s, st);
  return rec ? rebuild_tpp<false, true>(tpp, lig, io, s, st)
             : rebuild_tpp<false, false>(tpp, lig, io, s, st);
}

namespace {

template <bool G, bool RC, int D, int F, int IF>
cudaError_t one_t(const DevLigand& lig, const DevProtein& prot, const float4* tab4,
                  const PoseIO& io, const Scratch& s, const OneScratch& os, int flags, int smem,
                  cudaStream_t st, int* stage) {
  *stage = 1;
  // the opt-in counts the static type table too (kOneStatic bytes)
  if (smem + kOneStatic > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k_one_pose<G, RC, D, F, IF>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
  }
  *stage = 2;
  k_one_pose<G, RC, D, F, IF><<<os.npair + os.with_intra, kFinishOne, smem, st>>>(lig, prot, tab4, io, s, os, flags);
  return cudaGetLastError();
}

}  // namespace

int one_pose_smem(int L, int nrb) {
  return std::max(one_layout(L, nrb).total, finish_one_f4(L, nrb) * (int)sizeof(float4)) +
         kOneStatic;
}

cudaError_t launch_one_pose(const DevLigand& lig, const DevProtein& prot, const float4* tab4,
                            const PoseIO& io, const Scratch& s, const OneScratch& os, int flags,
                            const Physics& ph, cudaStream_t st, int* stage) {
  const bool g = (flags & kFlagGrad) && io.grad;
  const bool rc = flags & kFlagRecenter;
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0, i = ph.intra_form ? 0 : 1;
  const int smem = one_pose_smem(lig.L, lig.nrb) - kOneStatic;  // dynamic part
#define MMO_ONE(G, RC) \
  if (d == 0) { \
    if (f == 0) return i ? one_t<G, RC, 0, 0, 1>(lig, prot, tab4, io, s, os, flags, smem, st, stage) \
                         : one_t<G, RC, 0, 0, 0>(lig, prot, tab4, io, s, os, flags, smem, st, stage); \
    return i ? one_t<G, RC, 0, 1, 1>(lig, prot, tab4, io, s, os, flags, smem, st, stage) \
             : one_t<G, RC, 0, 1, 0>(lig, prot, tab4, io, s, os, flags, smem, st, stage); \
  } \
  if (f == 0) return i ? one_t<G, RC, 1, 0, 1>(lig, prot, tab4, io, s, os, flags, smem, st, stage) \
                       : one_t<G, RC, 1, 0, 0>(lig, prot, tab4, io, s, os, flags, smem, st, stage); \
  return i ? one_t<G, RC, 1, 1, 1>(lig, prot, tab4, io, s, os, flags, smem, st, stage) \
           : one_t<G, RC, 1, 1, 0>(lig, prot, tab4, io, s, os, flags, smem, st, stage);
  if (g) {
    if (rc) { MMO_ONE(true, true) }
    MMO_ONE(true, false)
  }
  if (rc) { MMO_ONE(false, true) }
  MMO_ONE(false, false)
#undef MMO_ONE
}

// intra_form: 0 plain (IFORM 1), 1 shifted (IFORM 0)
cudaError_t launch_finish(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                          const Physics& ph, cudaStream_t st) {
  if (io.B <= 0) return cudaSuccess;
  const bool g = (flags & kFlagGrad) && io.grad;
  const bool rc = flags & kFlagRecenter;
  const int d = ph.dielectric ? 1 : 0, f = ph.intra_form ? 0 : 1;
#define MMO_FN(G, RC, D, F) return finish_t<G, RC, D, F>(lig, io, s, flags, st)
#define MMO_FN_D(G, RC)                                                   \
  if (d == 0) { if (f) MMO_FN(G, RC, 0, 1); else MMO_FN(G, RC, 0, 0); } \
  else { if (f) MMO_FN(G, RC, 1, 1); else MMO_FN(G, RC, 1, 0); }
  if (!g) {
    MMO_FN_D(false, false)
  }
  if (rc) {
    MMO_FN_D(true, true)
  } else {
    MMO_FN_D(true, false)
  }
#undef MMO_FN_D
#undef MMO_FN
}


cudaError_t launch_intra_plain(const DevLigand& lig, const float4* X, int form, int dielectric,
                               double* out, cudaStream_t st) {
  const int f = form ? 0 : 1;
  if (dielectric) {
    if (f) k_intra_plain<1, 1><<<1, 32, 0, st>>>(lig, X, out);
    else k_intra_plain<1, 0><<<1, 32, 0, st>>>(lig, X, out);
  } else {
    if (f) k_intra_plain<0, 1><<<1, 32, 0, st>>>(lig, X, out);
    else k_intra_plain<0, 0><<<1, 32, 0, st>>>(lig, X, out);
  }
  return cudaGetLastError();
}


cudaError_t launch_sys_rebuild(const DevSystems& S, int nblk, int tpp, const PoseIO& io,
                               const Scratch& s, int flags, cudaStream_t st) {
  if (nblk <= 0) return cudaSuccess;
  const bool rc = flags & kFlagRecenter;
  const bool rec = (flags & kFlagGrad) && io.grad;
  if (rc) return rec ? sys_rebuild_tpp<true, true>(tpp, S, nblk, io, s, st)
                     : sys_rebuild_tpp<true, false>(tpp, S, nblk, io, s, st);
  return rec ? sys_rebuild_tpp<false, true>(tpp, S, nblk, io, s, st)
             : sys_rebuild_tpp<false, false>(tpp, S, nblk, io, s, st);
}

cudaError_t launch_sys_finish(const DevSystems& S, int nblk, const PoseIO& io, const Scratch& s,
                              int flags, const Physics& ph, cudaStream_t st) {
  if (nblk <= 0) return cudaSuccess;
  const bool g = (flags & kFlagGrad) && io.grad;
  const bool rc = flags & kFlagRecenter;
  const int d = ph.dielectric ? 1 : 0, f = ph.intra_form ? 0 : 1;
#define MMO_SF(G, RC, D, F) return sys_finish_t<G, RC, D, F>(S, nblk, io, s, flags, st)
#define MMO_SF_D(G, RC)                                                   \
  if (d == 0) { if (f) MMO_SF(G, RC, 0, 1); else MMO_SF(G, RC, 0, 0); } \
  else { if (f) MMO_SF(G, RC, 1, 1); else MMO_SF(G, RC, 1, 0); }
  if (!g) {
    MMO_SF_D(false, false)
  }
  if (rc) {
    MMO_SF_D(true, true)
  } else {
    MMO_SF_D(true, false)
  }
#undef MMO_SF_D
#undef MMO_SF
}

}  // namespace mmo

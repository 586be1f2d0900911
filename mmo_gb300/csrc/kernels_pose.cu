// kernels_pose.cu -- warp-per-pose kernels: pose rebuild (+ intra-ligand
// energy) before the pair sweep, and the finishing pass after it (energy
// reduction, intra-ligand gradient, reverse pass through the rigid map and
// the torsion chain).
//
// Pose map (UnixJunkie/MMO): torsions applied in bond order, each rotating its
// group about the current (left, right) axis (src/optim.ml:68-71,
// src/mol.ml:610-631); enclosing-radius check (src/mol.ml:576-591); then
// x = Rz(g) Ry(b) Rx(a) y + t (src/optim.ml:77-80, src/rot.ml:52-66), or with
// the centroid removed first for the Monte Carlo map (src/mol.ml:705-710).
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;

struct TorsRec {
  float cx, cy, cz, ux, uy, uz, ilen, ct, st;
};

__device__ __forceinline__ float pick(const float (&v)[kSlots], int slot) {
  float r = v[0];
#pragma unroll
  for (int s = 1; s < kSlots; ++s)
    if (slot == s) r = v[s];
  return r;
}

// coordinates of atom idx, read from the lane that owns it
__device__ __forceinline__ float3 fetch(const float (&x)[kSlots], const float (&y)[kSlots],
                                        const float (&z)[kSlots], int idx) {
  const int owner = idx & 31, slot = idx >> 5;
  return make_float3(__shfl_sync(kFull, pick(x, slot), owner),
                     __shfl_sync(kFull, pick(y, slot), owner),
                     __shfl_sync(kFull, pick(z, slot), owner));
}

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

// Rz(g) Ry(b) Rx(a) of rot.ml:52-66
__device__ __forceinline__ void rot_xyz(const float* dof, float (&R)[9], float (&cs)[6]) {
  float sa, ca, sb, cb, sg, cg;
  sincosf(dof[3], &sa, &ca);
  sincosf(dof[4], &sb, &cb);
  sincosf(dof[5], &sg, &cg);
  R[0] = cb * cg;
  R[1] = cg * sa * sb - ca * sg;
  R[2] = sa * sg + ca * cg * sb;
  R[3] = cb * sg;
  R[4] = ca * cg + sa * sb * sg;
  R[5] = ca * sb * sg - cg * sa;
  R[6] = -sb;
  R[7] = cb * sa;
  R[8] = ca * cb;
  cs[0] = ca; cs[1] = sa; cs[2] = cb; cs[3] = sb; cs[4] = cg; cs[5] = sg;
}

template <bool RECORD>
__device__ __forceinline__ void torsion_chain(const DevLigand& lig, const float* tau, int lane,
                                              float (&zx)[kSlots], float (&zy)[kSlots],
                                              float (&zz)[kSlots], TorsRec* rec) {
  for (int t = 0; t < lig.nrb; ++t) {
    const int2 bd = lig.bonds[t];
    const float3 pl = fetch(zx, zy, zz, bd.x);
    const float3 pr = fetch(zx, zy, zz, bd.y);
    const float ax = pr.x - pl.x, ay = pr.y - pl.y, az = pr.z - pl.z;
    const float len = sqrtf(ax * ax + ay * ay + az * az);
    const float ux = ax / len, uy = ay / len, uz = az / len;
    float sn, cs;
    sincosf(tau[t], &sn, &cs);
    float R[9];
    axis_angle(ux, uy, uz, cs, sn, R);
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      if ((lig.gmask[t * kSlots + s] >> lane) & 1u) {
        const float vx = zx[s] - pr.x, vy = zy[s] - pr.y, vz = zz[s] - pr.z;
        zx[s] = R[0] * vx + R[1] * vy + R[2] * vz + pr.x;
        zy[s] = R[3] * vx + R[4] * vy + R[5] * vz + pr.y;
        zz[s] = R[6] * vx + R[7] * vy + R[8] * vz + pr.z;
      }
    }
    if (RECORD && lane == 0) rec[t] = TorsRec{pr.x, pr.y, pr.z, ux, uy, uz, 1.0f / len, cs, sn};
  }
}

__device__ __forceinline__ void load_ref(const DevLigand& lig, int lane, float (&zx)[kSlots],
                                         float (&zy)[kSlots], float (&zz)[kSlots]) {
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    const int a = lane + 32 * s;
    float4 r = a < lig.L ? lig.ref[a] : make_float4(0.f, 0.f, 0.f, 0.f);
    zx[s] = r.x;
    zy[s] = r.y;
    zz[s] = r.z;
  }
}

__device__ __forceinline__ float3 centroid(const DevLigand& lig, int lane, const float (&zx)[kSlots],
                                           const float (&zy)[kSlots], const float (&zz)[kSlots]) {
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
  for (int s = 0; s < kSlots; ++s)
    if (lane + 32 * s < lig.L) {
      sx += zx[s];
      sy += zy[s];
      sz += zz[s];
    }
  const float inv = 1.0f / (float)lig.L;
  return make_float3(warp_sum(sx) * inv, warp_sum(sy) * inv, warp_sum(sz) * inv);
}

// ---- FP64 pose map (k_rebuild) --------------------------------------------
__device__ __forceinline__ double pickd(const double (&v)[kSlots], int slot) {
  double r = v[0];
#pragma unroll
  for (int s = 1; s < kSlots; ++s)
    if (slot == s) r = v[s];
  return r;
}

__device__ __forceinline__ double3 fetchd(const double (&x)[kSlots], const double (&y)[kSlots],
                                          const double (&z)[kSlots], int idx) {
  const int owner = idx & 31, slot = idx >> 5;
  return make_double3(__shfl_sync(kFull, pickd(x, slot), owner),
                      __shfl_sync(kFull, pickd(y, slot), owner),
                      __shfl_sync(kFull, pickd(z, slot), owner));
}

__device__ __forceinline__ double warp_maxd(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// sine and cosine of angle k of the pose ([a, b, g, tau_0 ...]), computed
// once by lane (k & 31) in round (k >> 5) and read back by every lane
struct AngleTable {
  double s0, c0, s1, c1;
  __device__ __forceinline__ void get(int k, double& s, double& c) const {
    const int owner = k & 31;
    const bool hi = k >= 32;
    s = __shfl_sync(kFull, hi ? s1 : s0, owner);
    c = __shfl_sync(kFull, hi ? c1 : c0, owner);
  }
};

__device__ __forceinline__ AngleTable angle_table(const float* dof, int nrb, int lane) {
  AngleTable t{0.0, 1.0, 0.0, 1.0};
  const int n = 3 + nrb;
  if (lane < n) sincos((double)dof[3 + lane], &t.s0, &t.c0);
  if (lane + 32 < n) sincos((double)dof[3 + lane + 32], &t.s1, &t.c1);
  return t;
}

__device__ __forceinline__ void store_split(float4* X, double x, double y, double z) {
  const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
  X[0] = make_float4(xh, yh, zh, 0.f);
  X[1] = make_float4(__double2float_rn(x - (double)xh), __double2float_rn(y - (double)yh),
                     __double2float_rn(z - (double)zh), 0.f);
}

// ---------------------------------------------------------------------------
// k_rebuild: posed coordinates X[b][a] (device frame, hi/lo floats) computed
// in FP64 and, optionally, the intra-ligand energy of mol.ml:881-903 (IFORM 1)
// or 853-877 (IFORM 0).
// ---------------------------------------------------------------------------
template <bool RECENTER, int DIEL, int IFORM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_rebuild(DevLigand lig, PoseIO io, Scratch scr, int with_intra) {
  __shared__ float4 sxh[kWarpsPerBlock][kMaxLig];
  __shared__ float4 sxl[kWarpsPerBlock][kMaxLig];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int b = blockIdx.x * kWarpsPerBlock + wib;
  if (b >= io.B) return;
  const int L = lig.L, nrb = lig.nrb, nd = 6 + nrb;
  const float* dof = io.dofs + (size_t)b * nd;
  const AngleTable ang = angle_table(dof, nrb, lane);
  double zx[kSlots], zy[kSlots], zz[kSlots];
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    const int a = lane + 32 * s;
    zx[s] = a < L ? lig.ref64[3 * a] : 0.0;
    zy[s] = a < L ? lig.ref64[3 * a + 1] : 0.0;
    zz[s] = a < L ? lig.ref64[3 * a + 2] : 0.0;
  }
  // torsions in bond order (optim.ml:68-71, mol.ml:610-631)
  for (int t = 0; t < nrb; ++t) {
    const int2 bd = lig.bonds[t];
    const double3 pl = fetchd(zx, zy, zz, bd.x);
    const double3 pr = fetchd(zx, zy, zz, bd.y);
    const double ax = pr.x - pl.x, ay = pr.y - pl.y, az = pr.z - pl.z;
    const double inv = rnorm3d(ax, ay, az);
    const double ux = ax * inv, uy = ay * inv, uz = az * inv;
    double sn, cs;
    ang.get(3 + t, sn, cs);
    const double o = 1.0 - cs;
    const double R0 = cs + ux * ux * o, R1 = ux * uy * o - uz * sn, R2 = ux * uz * o + uy * sn;
    const double R3 = ux * uy * o + uz * sn, R4 = cs + uy * uy * o, R5 = uy * uz * o - ux * sn;
    const double R6 = ux * uz * o - uy * sn, R7 = uy * uz * o + ux * sn, R8 = cs + uz * uz * o;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      if ((lig.gmask[t * kSlots + s] >> lane) & 1u) {
        const double vx = zx[s] - pr.x, vy = zy[s] - pr.y, vz = zz[s] - pr.z;
        zx[s] = R0 * vx + R1 * vy + R2 * vz + pr.x;
        zy[s] = R3 * vx + R4 * vy + R5 * vz + pr.y;
        zz[s] = R6 * vx + R7 * vy + R8 * vz + pr.z;
      }
    }
  }
  // centroid and enclosing radius (mol.ml:576-591)
  double cx = 0.0, cy = 0.0, cz = 0.0;
#pragma unroll
  for (int s = 0; s < kSlots; ++s)
    if (lane + 32 * s < L) {
      cx += zx[s];
      cy += zy[s];
      cz += zz[s];
    }
  cx = warp_sum(cx) / L;
  cy = warp_sum(cy) / L;
  cz = warp_sum(cz) / L;
  double rad = 0.0;
#pragma unroll
  for (int s = 0; s < kSlots; ++s)
    if (lane + 32 * s < L) {
      const double dx = cx - zx[s], dy = cy - zy[s], dz = cz - zz[s];
      rad = fmax(rad, 0.01 + sqrt(dx * dx + dy * dy + dz * dz));
    }
  const int status = warp_maxd(rad) > 12.0 ? kStatusTooLong : 0;
  // rigid map: Rz(g) Ry(b) Rx(a) (rot.ml:52-66), then + t
  double sa, ca, sb, cb, sg, cg;
  ang.get(0, sa, ca);
  ang.get(1, sb, cb);
  ang.get(2, sg, cg);
  const double R0 = cb * cg, R1 = cg * sa * sb - ca * sg, R2 = sa * sg + ca * cg * sb;
  const double R3 = cb * sg, R4 = ca * cg + sa * sb * sg, R5 = ca * sb * sg - cg * sa;
  const double R6 = -sb, R7 = cb * sa, R8 = ca * cb;
  const double tx = (double)dof[0] - (double)io.ox, ty = (double)dof[1] - (double)io.oy,
               tz = (double)dof[2] - (double)io.oz;
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    const int a = lane + 32 * s;
    if (a < L) {
      double vx = zx[s], vy = zy[s], vz = zz[s];
      if (RECENTER) {
        vx -= cx;
        vy -= cy;
        vz -= cz;
      }
      float4* out = scr.X + ((size_t)b * L + a) * 2;
      store_split(out, R0 * vx + R1 * vy + R2 * vz + tx, R3 * vx + R4 * vy + R5 * vz + ty,
                  R6 * vx + R7 * vy + R8 * vz + tz);
      sxh[wib][a] = out[0];
      sxl[wib][a] = out[1];
    }
  }
  double e_intra = 0.0;
  if (with_intra) {
    __syncwarp();
    float acc = 0.f, d0 = 0.f, d1 = 0.f, d2 = 0.f;
    for (int p = lane; p < lig.npairs; p += 32) {
      const int2 ij = lig.pair_ij[p];
      const float4 par = lig.pair_par[p];
      const float4 ih = sxh[wib][ij.x], il = sxl[wib][ij.x];
      const float4 jh = sxh[wib][ij.y], jl = sxl[wib][ij.y];
      uff_pair<false, DIEL, IFORM>(split_diff(ih.x, il.x, jh.x, jl.x),
                                   split_diff(ih.y, il.y, jh.y, jl.y),
                                   split_diff(ih.z, il.z, jh.z, jl.z), par.x, par.y, par.z, acc,
                                   d0, d1, d2);
    }
    e_intra = warp_sum((double)acc);
  }
  if (lane == 0) {
    io.status[b] = status;
    if (with_intra) scr.Eintra[b] = e_intra;
    if (b == 0 && io.zero_err) *io.err = 0;
  }
}

// ---------------------------------------------------------------------------
// k_finish: E[b] = sum of inter partials (FP64) + E_intra; with GRAD the
// intra-ligand gradient and the reverse pass to dE/d[x, y, z, a, b, g, tau].
// ---------------------------------------------------------------------------
template <bool GRAD, bool RECENTER, int DIEL, int IFORM>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_finish(DevLigand lig, PoseIO io, Scratch scr, int flags) {
  __shared__ float4 sxh[kWarpsPerBlock][kMaxLig];
  __shared__ float4 sxl[kWarpsPerBlock][kMaxLig];
  __shared__ TorsRec srec[kWarpsPerBlock][kMaxTors];
  __shared__ float4 saxis[kWarpsPerBlock][2 * kMaxTors];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int b = blockIdx.x * kWarpsPerBlock + wib;
  if (b >= io.B) return;
  const int L = lig.L, C = scr.C, nd = 6 + lig.nrb;
  double e = 0.0;
  if (flags & kFlagInter) {
    const double* ep = scr.Epart + (size_t)b * C * L;
    for (int k = lane; k < C * L; k += 32) e += ep[k];
    e = warp_sum(e);
  }
  if (flags & kFlagIntra) e += scr.Eintra[b];
  if (lane == 0) {
    io.E[b] = e;
    if (!isfinite(e)) io.status[b] |= kStatusNonFinite;
  }
  if (!GRAD) return;

  // dE/dX from the pair sweep
  float gx[kSlots], gy[kSlots], gz[kSlots];
#pragma unroll
  for (int s = 0; s < kSlots; ++s) gx[s] = gy[s] = gz[s] = 0.f;
  if (flags & kFlagInter) {
    const float4* gp = scr.Gpart + (size_t)b * C * L;
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
  // forward again, recording each torsion's axis
  const float* dof = io.dofs + (size_t)b * nd;
  float zx[kSlots], zy[kSlots], zz[kSlots];
  load_ref(lig, lane, zx, zy, zz);
  torsion_chain<true>(lig, dof + 6, lane, zx, zy, zz, srec[wib]);
  const float3 c = RECENTER ? centroid(lig, lane, zx, zy, zz) : make_float3(0.f, 0.f, 0.f);
  float R[9], cs[6];
  rot_xyz(dof, R, cs);
  const bool intra = flags & kFlagIntra;
  if (intra) {
    // intra-ligand gradient at the stored hi/lo posed coordinates
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      const int a = lane + 32 * s;
      if (a < L) {
        sxh[wib][a] = scr.X[((size_t)b * L + a) * 2];
        sxl[wib][a] = scr.X[((size_t)b * L + a) * 2 + 1];
      }
    }
    __syncwarp();
  }
  if (intra && !lig.nested) {
    // general groups: intra forces per atom, through the full reverse pass
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      const int a = lane + 32 * s;
      if (a < L) {
        const float4 ah = sxh[wib][a], al = sxl[wib][a];
        float acc = 0.f;
        for (int k = lig.nb_off[a]; k < lig.nb_off[a + 1]; ++k) {
          const int j = lig.nb_idx[k];
          const float4 bh = sxh[wib][j], bl = sxl[wib][j];
          const float4 par = lig.nb_par[k];
          uff_pair<true, DIEL, IFORM>(split_diff(ah.x, al.x, bh.x, bl.x),
                                      split_diff(ah.y, al.y, bh.y, bl.y),
                                      split_diff(ah.z, al.z, bh.z, bl.z), par.x, par.y, par.z,
                                      acc, gx[s], gy[s], gz[s]);
        }
      }
    }
  }
  // nested groups: dE_intra/dtau_t = sum over interacting pairs with exactly
  // one atom in group t of (dE/dX_moving) . (w_t x (X_moving - C_t)), w_t and
  // C_t the final axis of bond t; the term adds nothing to the rigid DOFs.
  // Keeping the large, cancelling intra forces out of the per-atom sums keeps
  // the FP32 reverse pass accurate.
  float dti[kMaxTors];
#pragma unroll
  for (int t = 0; t < kMaxTors; ++t) dti[t] = 0.f;
  if (intra && lig.nested && lig.nrb > 0) {
    if (lane < lig.nrb) {
      const int2 bd = lig.bonds[lane];
      const float4 rh = sxh[wib][bd.y], rl = sxl[wib][bd.y];
      const float4 lh = sxh[wib][bd.x], ll = sxl[wib][bd.x];
      const float ax = split_diff(rh.x, rl.x, lh.x, ll.x), ay = split_diff(rh.y, rl.y, lh.y, ll.y),
                  az = split_diff(rh.z, rl.z, lh.z, ll.z);
      const float inv = rsqrtf(ax * ax + ay * ay + az * az);
      saxis[wib][lane] = make_float4(ax * inv, ay * inv, az * inv, 0.f);
      saxis[wib][kMaxTors + lane] = rh;
    }
    __syncwarp();
    for (int p = lane; p < lig.npairs; p += 32) {
      const int2 ij = lig.pair_ij[p];
      const float4 par = lig.pair_par[p];
      const float4 ih = sxh[wib][ij.x], il = sxl[wib][ij.x];
      const float4 jh = sxh[wib][ij.y], jl = sxl[wib][ij.y];
      const float dx = split_diff(ih.x, il.x, jh.x, jl.x);
      const float dy = split_diff(ih.y, il.y, jh.y, jl.y);
      const float dz = split_diff(ih.z, il.z, jh.z, jl.z);
      const float g = uff_pair_g<DIEL, IFORM>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), par.x, par.y,
                                              par.z);
#pragma unroll
      for (int t = 0; t < kMaxTors; ++t) {
        if (t < lig.nrb) {
          const bool in_i = (lig.gmask[t * kSlots + (ij.x >> 5)] >> (ij.x & 31)) & 1u;
          const bool in_j = (lig.gmask[t * kSlots + (ij.y >> 5)] >> (ij.y & 31)) & 1u;
          if (in_i != in_j) {
            const float4 w = saxis[wib][t], cc = saxis[wib][kMaxTors + t];
            const float4 m = in_i ? ih : jh;
            const float lx = m.x - cc.x, ly = m.y - cc.y, lz = m.z - cc.z;
            // d . (w x l)
            const float v = dx * (w.y * lz - w.z * ly) + dy * (w.z * lx - w.x * lz) +
                            dz * (w.x * ly - w.y * lx);
            dti[t] = fmaf(in_i ? g : -g, v, dti[t]);
          }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < kMaxTors; ++t)
      if (t < lig.nrb) dti[t] = warp_sum(dti[t]);
  }
  // rigid map: dE/dt = sum G; dE/dR_kl = sum_i G_ik Yc_il
  float red[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) red[k] = 0.f;
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    if (lane + 32 * s < L) {
      const float yx = zx[s] - c.x, yy = zy[s] - c.y, yz = zz[s] - c.z;
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
  float* grad = io.grad + (size_t)b * nd;
  if (lane == 0) {
    const float ca = cs[0], sa = cs[1], cb = cs[2], sb = cs[3], cg = cs[4], sg = cs[5];
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
  __syncwarp();
  // reverse through the torsions, undoing each rotation on the way back
  for (int t = lig.nrb - 1; t >= 0; --t) {
    const TorsRec rc = srec[wib][t];
    float Rt[9];
    axis_angle(rc.ux, rc.uy, rc.uz, rc.ct, rc.st, Rt);
    float q[10];
#pragma unroll
    for (int k = 0; k < 10; ++k) q[k] = 0.f;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      if ((lig.gmask[t * kSlots + s] >> lane) & 1u) {
        const float px = zx[s] - rc.cx, py = zy[s] - rc.cy, pz = zz[s] - rc.cz;  // v'
        const float vx = Rt[0] * px + Rt[3] * py + Rt[6] * pz;                  // v = R^T v'
        const float vy = Rt[1] * px + Rt[4] * py + Rt[7] * pz;
        const float vz = Rt[2] * px + Rt[5] * py + Rt[8] * pz;
        const float Ax = ax[s], Ay = ay[s], Az = az[s];
        // dtheta += A . (u x v')
        q[0] += Ax * (rc.uy * pz - rc.uz * py) + Ay * (rc.uz * px - rc.ux * pz) +
                Az * (rc.ux * py - rc.uy * px);
        // v x A
        q[1] += vy * Az - vz * Ay;
        q[2] += vz * Ax - vx * Az;
        q[3] += vx * Ay - vy * Ax;
        const float uv = rc.ux * vx + rc.uy * vy + rc.uz * vz;
        const float Au = Ax * rc.ux + Ay * rc.uy + Az * rc.uz;
        q[4] += uv * Ax + Au * vx;
        q[5] += uv * Ay + Au * vy;
        q[6] += uv * Az + Au * vz;
        q[7] += Ax;
        q[8] += Ay;
        q[9] += Az;
        ax[s] = Rt[0] * Ax + Rt[3] * Ay + Rt[6] * Az;
        ay[s] = Rt[1] * Ax + Rt[4] * Ay + Rt[7] * Az;
        az[s] = Rt[2] * Ax + Rt[5] * Ay + Rt[8] * Az;
        zx[s] = vx + rc.cx;
        zy[s] = vy + rc.cy;
        zz[s] = vz + rc.cz;
      }
    }
#pragma unroll
    for (int k = 0; k < 10; ++k) q[k] = warp_sum(q[k]);
    const float omc = 1.0f - rc.ct;
    const float dUx = rc.st * q[1] + omc * q[4];
    const float dUy = rc.st * q[2] + omc * q[5];
    const float dUz = rc.st * q[3] + omc * q[6];
    const float uu = rc.ux * dUx + rc.uy * dUy + rc.uz * dUz;
    const float dax = (dUx - rc.ux * uu) * rc.ilen;
    const float day = (dUy - rc.uy * uu) * rc.ilen;
    const float daz = (dUz - rc.uz * uu) * rc.ilen;
    // dE/dc = sum A - R^T sum A
    const float dCx = q[7] - (Rt[0] * q[7] + Rt[3] * q[8] + Rt[6] * q[9]);
    const float dCy = q[8] - (Rt[1] * q[7] + Rt[4] * q[8] + Rt[7] * q[9]);
    const float dCz = q[9] - (Rt[2] * q[7] + Rt[5] * q[8] + Rt[8] * q[9]);
    const int2 bd = lig.bonds[t];
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
    if (lane == 0) {
      float intra_t = 0.f;
#pragma unroll
      for (int k = 0; k < kMaxTors; ++k)
        if (k == t) intra_t = dti[k];
      grad[6 + t] = q[0] + intra_t;
    }
  }
}

// one warp: sum of n FP64 partials
__global__ void k_reduce_plain(const double* Epart, int n, double* out) {
  double e = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) e += Epart[k];
  e = warp_sum(e);
  if (threadIdx.x == 0) out[0] = e;
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

template <bool RC, int DIEL, int IFORM>
cudaError_t rebuild_t(const DevLigand& lig, const PoseIO& io, const Scratch& s, int intra,
                      cudaStream_t st) {
  const int blocks = (io.B + kWarpsPerBlock - 1) / kWarpsPerBlock;
  k_rebuild<RC, DIEL, IFORM><<<blocks, kWarpsPerBlock * 32, 0, st>>>(lig, io, s, intra);
  return cudaGetLastError();
}

template <bool G, bool RC, int DIEL, int IFORM>
cudaError_t finish_t(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                     cudaStream_t st) {
  const int blocks = (io.B + kWarpsPerBlock - 1) / kWarpsPerBlock;
  k_finish<G, RC, DIEL, IFORM><<<blocks, kWarpsPerBlock * 32, 0, st>>>(lig, io, s, flags);
  return cudaGetLastError();
}

}  // namespace

// intra_form: 0 plain (IFORM 1), 1 shifted (IFORM 0)
cudaError_t launch_rebuild(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                           int intra_form, int dielectric, cudaStream_t st) {
  if (io.B <= 0) return cudaSuccess;
  const bool rc = flags & kFlagRecenter;
  const int intra = (flags & kFlagIntra) ? 1 : 0;
  const int d = dielectric ? 1 : 0, f = intra_form ? 0 : 1;
#define MMO_RB(RC, D, F) return rebuild_t<RC, D, F>(lig, io, s, intra, st)
  if (rc) {
    if (d == 0) { if (f) MMO_RB(true, 0, 1); else MMO_RB(true, 0, 0); }
    else { if (f) MMO_RB(true, 1, 1); else MMO_RB(true, 1, 0); }
  } else {
    if (d == 0) { if (f) MMO_RB(false, 0, 1); else MMO_RB(false, 0, 0); }
    else { if (f) MMO_RB(false, 1, 1); else MMO_RB(false, 1, 0); }
  }
#undef MMO_RB
}

cudaError_t launch_finish(const DevLigand& lig, const PoseIO& io, const Scratch& s, int flags,
                          const Physics& ph, cudaStream_t st) {
  if (io.B <= 0) return cudaSuccess;
  const bool g = (flags & kFlagGrad) && io.grad;
  const bool rc = flags & kFlagRecenter;
  const int d = ph.dielectric ? 1 : 0, f = ph.intra_form ? 0 : 1;
#define MMO_FN(G, RC, D, F) return finish_t<G, RC, D, F>(lig, io, s, flags, st)
#define MMO_FN_D(G, RC)                                              \
  if (d == 0) { if (f) MMO_FN(G, RC, 0, 1); else MMO_FN(G, RC, 0, 0); } \
  else { if (f) MMO_FN(G, RC, 1, 1); else MMO_FN(G, RC, 1, 0); }
  if (!g) {
    MMO_FN(false, false, 0, 1);  // reduction only: physics-independent
  }
  if (rc) {
    MMO_FN_D(true, true)
  } else {
    MMO_FN_D(true, false)
  }
#undef MMO_FN_D
#undef MMO_FN
}

cudaError_t launch_reduce_plain(const double* Epart, int n, double* out, cudaStream_t st) {
  k_reduce_plain<<<1, 32, 0, st>>>(Epart, n, out);
  return cudaGetLastError();
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

}  // namespace mmo

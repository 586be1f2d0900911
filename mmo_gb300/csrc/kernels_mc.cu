// kernels_mc.cu -- Monte Carlo chains in dihedral space around the batched
// scorer: the moves and Metropolis step of Lds.simulate_lig (UnixJunkie/MMO
// src/lds.ml:882-995; moves src/move.ml:14-54, src/mol.ml:635-647; step-size
// adaptation src/lds.ml:586-621) and a gradient-descent minimiser over the
// hand-written adjoint.  One thread per chain; the scoring between the
// propose and accept kernels is the batched pipeline of the other files, so a
// step is a fixed launch sequence that a CUDA graph can hold.
//
// State lives in the optimiser layout (src/optim.ml:19-22): [x, y, z, a, b, g,
// tau_0 ...] with the pose x = R(a, b, g) (Y - centroid(Y)) + t of
// Mol.center_rotate_translate_copy (src/mol.ml:705-710), Y the conformer after
// the torsions.  A rigid move left-multiplies R by a small rotation and
// decomposes it back into (a, b, g) (src/rot.ml:52-75); a conformer move
// changes one torsion angle.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr double kPi = 3.14159265358979323846;

// standard normal pair from two uniforms (Box-Muller)
__device__ __forceinline__ void normal2(double u1, double u2, double& n0, double& n1) {
  const double r = sqrt(-2.0 * log(1.0 - u1));  // 1 - u1 in (0, 1]
  double s, c;
  sincos(2.0 * kPi * u2, &s, &c);
  n0 = r * c;
  n1 = r * s;
}

__device__ __forceinline__ double wrap_pi(double a) {
  a = fmod(a + kPi, 2.0 * kPi);
  if (a < 0.0) a += 2.0 * kPi;
  return a - kPi;
}

__device__ __forceinline__ int* chain_counts(const MCDev& s, int nrb, int b) {
  return s.cnt + (size_t)b * (kMcCounts + 2 * nrb);
}

__global__ void k_mc_init(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  float* st = s.steps + (size_t)b * (2 + p.nrb);
  st[0] = p.rot;
  st[1] = p.trans;
  for (int i = 0; i < p.nrb; ++i) st[2 + i] = p.tors;
  int* c = chain_counts(s, p.nrb, b);
  for (int i = 0; i < kMcCounts + 2 * p.nrb; ++i) c[i] = 0;
  s.accepted[b] = 0;
  s.status_or[b] = 0;
}

// after the first scoring of the start poses: best = start
__global__ void k_mc_start(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  s.E_best[b] = s.E_cur[b];
  s.status_or[b] |= s.st_trial[b];
  for (int k = 0; k < p.nd; ++k) s.best[(size_t)b * p.nd + k] = s.cur[(size_t)b * p.nd + k];
}

__global__ void k_mc_propose(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  const int nd = p.nd, nrb = p.nrb;
  const float* cur = s.cur + (size_t)b * nd;
  float* tr = s.trial + (size_t)b * nd;
  for (int k = 0; k < nd; ++k) tr[k] = cur[k];
  int* c = chain_counts(s, nrb, b);
  const int step = c[0];
  const float* st = s.steps + (size_t)b * (2 + nrb);
  const uint4 r0 = philox(make_uint4((uint32_t)b, (uint32_t)step, 0u, 0u), p.key0, p.key1);
  const uint4 r1 = philox(make_uint4((uint32_t)b, (uint32_t)step, 1u, 0u), p.key0, p.key1);
  const bool rigid = nrb == 0 || (step & 1) == 0;  // lds.ml:659-660, 883
  if (rigid) {
    double ax = 0.0, ay = 0.0, az = 0.0, th, dt[3];
    if (p.law == kMcGaussian) {
      double n[8];
      normal2(u01(r0.x, r0.y), u01(r0.z, r0.w), n[0], n[1]);
      normal2(u01(r1.x, r1.y), u01(r1.z, r1.w), n[2], n[3]);
      const uint4 r2 = philox(make_uint4((uint32_t)b, (uint32_t)step, 2u, 0u), p.key0, p.key1);
      normal2(u01(r2.x, r2.y), u01(r2.z, r2.w), n[4], n[5]);
      const double il = rsqrt(fmax(n[0] * n[0] + n[1] * n[1] + n[2] * n[2], 1e-300));
      ax = n[0] * il;  // uniform direction
      ay = n[1] * il;
      az = n[2] * il;
      th = (double)st[0] * n[3];
      dt[0] = (double)st[1] * n[4];
      dt[1] = (double)st[1] * n[5];
      const uint4 r3 = philox(make_uint4((uint32_t)b, (uint32_t)step, 3u, 0u), p.key0, p.key1);
      double n6, n7;
      normal2(u01(r3.x, r3.y), u01(r3.z, r3.w), n6, n7);
      dt[2] = (double)st[1] * n6;
    } else {
      // Move.rand_rot: theta in [-dr, dr] about one of Ox, Oy, Oz; Move.rand_trans:
      // a direction in [-1, 1]^3 times dt
      th = (2.0 * u01(r0.x, r0.y) - 1.0) * (double)st[0];
      const int axis = min(2, (int)(u01(r0.z, r0.w) * 3.0));
      ax = axis == 0;
      ay = axis == 1;
      az = axis == 2;
      dt[0] = (2.0 * u01(r1.x, r1.y) - 1.0) * (double)st[1];
      dt[1] = (2.0 * u01(r1.z, r1.w) - 1.0) * (double)st[1];
      const uint4 r2 = philox(make_uint4((uint32_t)b, (uint32_t)step, 2u, 0u), p.key0, p.key1);
      dt[2] = (2.0 * u01(r2.x, r2.y) - 1.0) * (double)st[1];
    }
    // R' = Rm R, Rm = rotation by th about (ax, ay, az) (rot.ml:121-146),
    // R = r_xyz(a, b, g) (rot.ml:52-66)
    double sa, ca, sb, cb, sg, cg, sn, cs;
    sincos((double)cur[3], &sa, &ca);
    sincos((double)cur[4], &sb, &cb);
    sincos((double)cur[5], &sg, &cg);
    const double R[9] = {cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb,
                         cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa,
                         -sb,     cb * sa,                 ca * cb};
    sincos(th, &sn, &cs);
    const double o = 1.0 - cs;
    const double M[9] = {cs + ax * ax * o,      ax * ay * o - az * sn, ax * az * o + ay * sn,
                         ax * ay * o + az * sn, cs + ay * ay * o,      ay * az * o - ax * sn,
                         ax * az * o - ay * sn, ay * az * o + ax * sn, cs + az * az * o};
    double Q[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        Q[3 * i + j] = M[3 * i] * R[j] + M[3 * i + 1] * R[3 + j] + M[3 * i + 2] * R[6 + j];
    // Rot.decompose (rot.ml:71-75)
    const double beta = atan2(-Q[6], sqrt(Q[0] * Q[0] + Q[3] * Q[3]));
    const double icb = 1.0 / cos(beta);
    tr[3] = (float)atan2(Q[7] * icb, Q[8] * icb);
    tr[4] = (float)beta;
    tr[5] = (float)atan2(Q[3] * icb, Q[0] * icb);
    for (int k = 0; k < 3; ++k) tr[k] = (float)((double)cur[k] + dt[k]);
    s.moved[b] = -1;
  } else {
    // Mol.tweak_rbond: one bond, an angle in [-dr_i, dr_i] (or a Gaussian
    // step), every flip_every-th conformer move Mol.flip_rbond in [-pi, pi]
    const int i = min(nrb - 1, (int)(u01(r0.x, r0.y) * nrb));
    double d;
    if (p.law == kMcGaussian) {
      double n0, n1;
      normal2(u01(r0.z, r0.w), u01(r1.x, r1.y), n0, n1);
      d = (double)st[2 + i] * n0;
    } else {
      const int confs = c[3];
      const bool flip = p.flip_every > 0 && confs > 0 && confs % p.flip_every == 0;
      d = (2.0 * u01(r0.z, r0.w) - 1.0) * (flip ? kPi : (double)st[2 + i]);
    }
    tr[6 + i] = (float)wrap_pi((double)cur[6 + i] + d);
    s.moved[b] = i;
  }
}

// Metropolis: accept when E' <= E or U < exp(-(E' - E) / kT), compared in
// FP64 (lds.ml:931-934); a trial pose whose status is not clean is rejected.
__global__ void k_mc_accept(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  const int nd = p.nd, nrb = p.nrb;
  int* c = chain_counts(s, nrb, b);
  const int step = c[0];
  const double Et = s.E_trial[b], E0 = s.E_cur[b];
  const int stt = s.st_trial[b];
  s.status_or[b] |= stt;
  const bool ok = stt == 0 && isfinite(Et);
  bool acc = false;
  if (ok) {
    if (Et <= E0) {
      acc = true;
    } else {
      const uint4 r = philox(make_uint4((uint32_t)b, (uint32_t)step, 7u, 0u), p.key0, p.key1);
      acc = u01(r.x, r.y) < exp(-(Et - E0) / p.kT);
    }
  }
  if (acc) {
    for (int k = 0; k < nd; ++k) s.cur[(size_t)b * nd + k] = s.trial[(size_t)b * nd + k];
    s.E_cur[b] = Et;
    s.accepted[b] += 1;
  }
  if (ok && Et < s.E_best[b]) {
    s.E_best[b] = Et;
    for (int k = 0; k < nd; ++k) s.best[(size_t)b * nd + k] = s.trial[(size_t)b * nd + k];
  }
  // step-size adaptation per block of 100 moves (lds.ml:586-621, params.ml:29):
  // acceptance <= 0.45 scales the step by 0.95, >= 0.55 by 1.05 (angles capped at pi)
  float* st = s.steps + (size_t)b * (2 + nrb);
  const int mv = s.moved[b];
  if (mv < 0) {
    c[1] += acc;
    c[2] += 1;
    if (p.adapt && c[2] % kMcBlock == 0) {
      const float ratio = (float)c[1] / (float)kMcBlock;
      if (ratio <= 0.45f) {
        st[0] *= 0.95f;
        st[1] *= 0.95f;
      } else if (ratio >= 0.55f) {
        st[0] = fminf((float)kPi, st[0] * 1.05f);
        st[1] *= 1.05f;
      }
      c[1] = 0;
    }
  } else {
    int* bc = c + kMcCounts;
    bc[2 * mv] += acc;
    bc[2 * mv + 1] += 1;
    c[3] += 1;
    if (p.adapt && c[3] % (kMcBlock * nrb) == 0) {
      for (int i = 0; i < nrb; ++i) {
        if (bc[2 * i + 1] > 0) {
          const float ratio = (float)bc[2 * i] / (float)bc[2 * i + 1];
          if (ratio <= 0.45f) st[2 + i] *= 0.95f;
          else if (ratio >= 0.55f) st[2 + i] = fminf((float)kPi, st[2 + i] * 1.05f);
        }
        bc[2 * i] = bc[2 * i + 1] = 0;
      }
    }
  }
  c[0] = step + 1;
}

// gradient descent: a step of length eta along -g in the max norm
__global__ void k_gd_begin(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  s.eta[b] = p.gd_step;
}

__global__ void k_gd_propose(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  const int nd = p.nd;
  const float* g = s.G_cur + (size_t)b * nd;
  const float* cur = s.cur + (size_t)b * nd;
  float* tr = s.trial + (size_t)b * nd;
  float gm = 0.f;
  for (int k = 0; k < nd; ++k) gm = fmaxf(gm, fabsf(g[k]));
  const float f = gm > 0.f && isfinite(gm) ? s.eta[b] / gm : 0.f;
  for (int k = 0; k < nd; ++k) tr[k] = cur[k] - f * g[k];
  for (int k = 6; k < nd; ++k) tr[k] = (float)wrap_pi((double)tr[k]);
}

// keep the step when the energy went down (then lengthen the next), else halve
__global__ void k_gd_accept(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  const int nd = p.nd;
  const double Et = s.E_trial[b];
  const int stt = s.st_trial[b];
  s.status_or[b] |= stt;
  if (stt == 0 && isfinite(Et) && Et < s.E_cur[b]) {
    for (int k = 0; k < nd; ++k) {
      s.cur[(size_t)b * nd + k] = s.trial[(size_t)b * nd + k];
      s.G_cur[(size_t)b * nd + k] = s.G_trial[(size_t)b * nd + k];
    }
    s.E_cur[b] = Et;
    s.eta[b] *= 1.2f;
    if (Et < s.E_best[b]) {
      s.E_best[b] = Et;
      for (int k = 0; k < nd; ++k) s.best[(size_t)b * nd + k] = s.trial[(size_t)b * nd + k];
    }
  } else {
    s.eta[b] *= 0.5f;
  }
}

// the first gradient of a minimisation belongs to the current pose
__global__ void k_gd_take(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  for (int k = 0; k < p.nd; ++k) s.G_cur[(size_t)b * p.nd + k] = s.G_trial[(size_t)b * p.nd + k];
}

__global__ void k_philox(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, int n, uint4* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = philox(make_uint4((uint32_t)i, c1, c2, 0u), k0, k1);
}

inline int nblk(int B) { return (B + 127) / 128; }

}  // namespace

#define MMO_MC_LAUNCH(K)                                      \
  cudaError_t launch_##K(const MCDev& s, const MCParams& p, cudaStream_t st) { \
    if (p.B <= 0) return cudaSuccess;                         \
    K<<<nblk(p.B), 128, 0, st>>>(s, p);                       \
    return cudaGetLastError();                                \
  }
MMO_MC_LAUNCH(k_mc_init)
MMO_MC_LAUNCH(k_mc_start)
MMO_MC_LAUNCH(k_mc_propose)
MMO_MC_LAUNCH(k_mc_accept)
MMO_MC_LAUNCH(k_gd_begin)
MMO_MC_LAUNCH(k_gd_propose)
MMO_MC_LAUNCH(k_gd_accept)
MMO_MC_LAUNCH(k_gd_take)
#undef MMO_MC_LAUNCH

cudaError_t launch_philox(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, int n, uint4* out,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_philox<<<(n + 255) / 256, 256, 0, st>>>(k0, k1, c1, c2, n, out);
  return cudaGetLastError();
}

}  // namespace mmo

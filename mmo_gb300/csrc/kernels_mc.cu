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

__device__ __forceinline__ int* chain_counts(const MCDev& s, int b) {
  return s.cnt + (size_t)b * kMcCounts;
}

// Sliding window of the last kMcBlock accept / reject events (SW.ml:7-37):
// w[0..3] event bits (a ring), w[4] next slot, w[5] events held, w[6] accepts
__device__ __forceinline__ int* chain_window(const MCDev& s, int nrb, int b, int k) {
  return s.win + ((size_t)b * (1 + nrb) + k) * kMcWin;
}

__device__ __forceinline__ void sw_reset(int* w) {
  for (int i = 0; i < kMcWin; ++i) w[i] = 0;
}

// SW.process: the event enters; beyond the window's length the oldest leaves
__device__ __forceinline__ void sw_process(int* w, bool evt) {
  const int head = w[4];
  uint32_t* bits = reinterpret_cast<uint32_t*>(w);
  const uint32_t m = 1u << (head & 31);
  if (w[5] == kMcBlock) {  // full: the slot being written holds the oldest event
    if (bits[head >> 5] & m) w[6] -= 1;
  } else {
    w[5] += 1;
  }
  bits[head >> 5] = evt ? (bits[head >> 5] | m) : (bits[head >> 5] & ~m);
  w[6] += evt ? 1 : 0;
  w[4] = head + 1 == kMcBlock ? 0 : head + 1;
}

// SW.get_ratio: accepts / events (NaN before the first event)
__device__ __forceinline__ double sw_ratio(const int* w) { return (double)w[6] / (double)w[5]; }

__global__ void k_mc_init(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  double* st = s.steps + (size_t)b * (2 + p.nrb);
  st[0] = p.rot;
  st[1] = p.trans;
  for (int i = 0; i < p.nrb; ++i) st[2 + i] = p.tors;
  int* c = chain_counts(s, b);
  for (int i = 0; i < kMcCounts; ++i) c[i] = 0;
  for (int k = 0; k <= p.nrb; ++k) sw_reset(chain_window(s, p.nrb, b, k));
  for (int k = 0; k < 6; ++k) s.start[(size_t)b * 6 + k] = s.cur[(size_t)b * p.nd + k];
  s.accepted[b] = 0;
  s.resets[b] = 0;
  s.stopped[b] = 0;
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

// A quad of lanes per chain: the rigid move's random draws (Box-Muller) and the
// sines and cosines of the current angles run on separate lanes, and each lane
// then forms the same products; every FP64 operation is the one-thread
// sequence's, on the same inputs, so the proposal keeps its bits.
constexpr int kQuad = 4;

// the quad's own lanes (quads leave the kernel independently)
__device__ __forceinline__ unsigned quad_mask() { return 0xfu << (threadIdx.x & 28); }
__device__ __forceinline__ double quad_get(double v, int src) {
  return __shfl_sync(quad_mask(), v, src, kQuad);
}

__global__ void k_mc_propose(MCDev s, MCParams p) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = gt / kQuad, q = gt % kQuad;
  // the whole quad leaves together (B kQuad threads run, a multiple of the quad)
  if (b >= p.B) return;
  const int nd = p.nd, nrb = p.nrb;
  const float* cur = s.cur + (size_t)b * nd;
  float* tr = s.trial + (size_t)b * nd;
  for (int k = q; k < nd; k += kQuad) tr[k] = cur[k];
  const int* c = chain_counts(s, b);
  const int step = c[0];
  const double* st = s.steps + (size_t)b * (2 + nrb);
  const bool rigid = (step & 1) == 0;  // lds.ml:659-660, 883
  if (s.stopped[b] || (!rigid && nrb == 0)) {
    // an ended chain stays; a ligand without rotatable bonds makes no
    // conformer move (its odd frames re-score the same pose, lds.ml:797-798)
    if (q == 0) s.moved[b] = -2;
    return;
  }
  if (rigid) {
    // lane q: Philox draw q (its two uniforms, or the normal pair from them)
    // and, for q < 3, the sine and cosine of the current angle 3 + q
    const uint4 rq = philox(make_uint4((uint32_t)b, (uint32_t)step, (uint32_t)q, 0u), p.key0,
                            p.key1);
    double nq0, nq1;
    if (p.law == kMcGaussian) {
      normal2(u01(rq.x, rq.y), u01(rq.z, rq.w), nq0, nq1);
    } else {
      nq0 = u01(rq.x, rq.y);
      nq1 = u01(rq.z, rq.w);
    }
    double sq = 0.0, cq = 1.0;
    if (q < 3) sincos((double)cur[3 + q], &sq, &cq);
    __syncwarp(quad_mask());
    double n[8];
#pragma unroll
    for (int k = 0; k < kQuad; ++k) {
      n[2 * k] = quad_get(nq0, k);
      n[2 * k + 1] = quad_get(nq1, k);
    }
    const double sa = quad_get(sq, 0), ca = quad_get(cq, 0);
    const double sb = quad_get(sq, 1), cb = quad_get(cq, 1);
    const double sg = quad_get(sq, 2), cg = quad_get(cq, 2);
    double ax = 0.0, ay = 0.0, az = 0.0, th, dt[3];
    if (p.law == kMcGaussian) {
      const double il = 1.0 / sqrt(fmax(n[0] * n[0] + n[1] * n[1] + n[2] * n[2], 1e-300));
      ax = n[0] * il;  // uniform direction
      ay = n[1] * il;
      az = n[2] * il;
      th = st[0] * n[3];
      dt[0] = st[1] * n[4];
      dt[1] = st[1] * n[5];
      dt[2] = st[1] * n[6];
    } else {
      // Move.rand_rot: theta in [-dr, dr] about one of Ox, Oy, Oz; Move.rand_trans:
      // a direction in [-1, 1]^3 times dt (n[k]: the uniforms of draws 0, 1, 2)
      th = (2.0 * n[0] - 1.0) * st[0];
      const int axis = min(2, (int)(n[1] * 3.0));
      ax = axis == 0;
      ay = axis == 1;
      az = axis == 2;
      dt[0] = (2.0 * n[2] - 1.0) * st[1];
      dt[1] = (2.0 * n[3] - 1.0) * st[1];
      dt[2] = (2.0 * n[4] - 1.0) * st[1];
    }
    // R' = Rm R, Rm = rotation by th about (ax, ay, az) (rot.ml:121-146),
    // R = r_xyz(a, b, g) (rot.ml:52-66)
    double sn, cs;
    sincos(th, &sn, &cs);
    const double R[9] = {cb * cg, cg * sa * sb - ca * sg, sa * sg + ca * cg * sb,
                         cb * sg, ca * cg + sa * sb * sg, ca * sb * sg - cg * sa,
                         -sb,     cb * sa,                 ca * cb};
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
    // Rot.decompose (rot.ml:71-75): lane 0 the first angle, lane 1 the third
    const double beta = atan2(-Q[6], sqrt(Q[0] * Q[0] + Q[3] * Q[3]));
    const double icb = 1.0 / cos(beta);
    if (q == 0) tr[3] = (float)atan2(Q[7] * icb, Q[8] * icb);
    if (q == 1) tr[5] = (float)atan2(Q[3] * icb, Q[0] * icb);
    if (q == 2) {
      tr[4] = (float)beta;
      for (int k = 0; k < 3; ++k) tr[k] = (float)((double)cur[k] + dt[k]);
    }
    if (q == 3) s.moved[b] = -1;
  } else if (q == 0) {
    const uint4 r0 = philox(make_uint4((uint32_t)b, (uint32_t)step, 0u, 0u), p.key0, p.key1);
    const uint4 r1 = philox(make_uint4((uint32_t)b, (uint32_t)step, 1u, 0u), p.key0, p.key1);
    // Mol.tweak_rbond: one bond, an angle in [-dr_i, dr_i] (or a Gaussian
    // step); Mol.flip_rbond in [-pi, pi] on conformer frames whose count of
    // earlier conformer frames is a positive multiple of flip_every
    // (lds.ml:783-793)
    const int i = min(nrb - 1, (int)(u01(r0.x, r0.y) * nrb));
    double d;
    if (p.law == kMcGaussian) {
      double n0, n1;
      normal2(u01(r0.z, r0.w), u01(r1.x, r1.y), n0, n1);
      d = st[2 + i] * n0;
    } else {
      const int confs = c[2];
      const bool flip = p.flip_every > 0 && confs > 0 && confs % p.flip_every == 0;
      d = (2.0 * u01(r0.z, r0.w) - 1.0) * (flip ? kPi : st[2 + i]);
    }
    tr[6 + i] = (float)wrap_pi((double)cur[6 + i] + d);
    s.moved[b] = i;
  }
}

// One frame of Lds.simulate_lig after the trial's scoring (lds.ml:906-988):
//  * hard ROI (roi_r > 0): a trial whose ligand centre (the translation of the
//    MC pose map) lies farther than roi_r from roi_c resets the chain;
//  * otherwise, with reset_zero, a trial whose inter energy is exactly 0 (the
//    ligand left the pocket) resets the chain;
//  * otherwise Metropolis: accept when E' <= E or U < exp(-(E' - E) / kT),
//    compared in FP64 (lds.ml:931-934); the event enters the rigid window or
//    the moved bond's window (SW.ml); a new lowest energy becomes the best
//    pose; on rigid frames after each 100 rigid frames the rigid steps adapt
//    to the rigid window's ratio (x0.95 at <= 0.45, x1.05 at >= 0.55, the
//    angle capped at pi, lds.ml:586-603), on conformer frames after each
//    100 nrb conformer frames every bond's step adapts to its own window
//    (lds.ml:606-621) -- kept only when the frame's move was accepted, since
//    the reference adapts the trial conformer (lds.ml:971-976).
// A reset (reset_run_params, lds.ml:652-671) puts the rigid part back to the
// start pose and the rigid steps to their initial values, clears the rigid
// window and sets the current and best energies to +inf (the next clean
// trial is accepted); the conformer, the bond steps and the bond windows stay.
// A trial that is not clean is rejected; an over-long trial conformer
// (Mol.Too_long, mol.ml:576-591) is rejected, or ends the chain with
// too_long_ends (the reference's exception leaves the frame loop,
// lds.ml:989-991).  Rigid trials ignore the over-long bit (the reference
// checks it on conformer moves only).
__global__ void k_mc_accept(MCDev s, MCParams p) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= p.B) return;
  const int nd = p.nd, nrb = p.nrb;
  int* c = chain_counts(s, b);
  const int step = c[0];
  const int mv = s.moved[b];
  const bool rigid = (step & 1) == 0;
  const double Et = s.E_trial[b], E0 = s.E_cur[b];
  const int stt = s.st_trial[b];
  float* cur = s.cur + (size_t)b * nd;
  const float* tr = s.trial + (size_t)b * nd;
  double* st = s.steps + (size_t)b * (2 + nrb);
  int event = 0;
  if (s.stopped[b]) {
    event = kMcStopped;
  } else {
    s.status_or[b] |= stt;
    bool reset = false;
    if (p.roi_r > 0.0) {
      const double dx = (double)tr[0] - p.roi_c[0], dy = (double)tr[1] - p.roi_c[1],
                   dz = (double)tr[2] - p.roi_c[2];
      reset = sqrt(dx * dx + dy * dy + dz * dz) > p.roi_r;
    }
    if (!reset && p.reset_zero && s.Ei_trial[b] == 0.0) reset = true;
    if (reset) {
      for (int k = 0; k < 6; ++k) cur[k] = s.start[(size_t)b * 6 + k];
      s.E_cur[b] = __longlong_as_double(0x7ff0000000000000ll);  // +inf
      s.E_best[b] = __longlong_as_double(0x7ff0000000000000ll);
      for (int k = 0; k < nd; ++k) s.best[(size_t)b * nd + k] = cur[k];
      st[0] = p.rot;
      st[1] = p.trans;
      sw_reset(chain_window(s, nrb, b, 0));
      s.resets[b] += 1;
      event = kMcReset;
    } else {
      const bool too_long = mv >= 0 && (stt & kStatusTooLong);
      const bool blocked = !isfinite(Et) || too_long || (stt & ~kStatusTooLong);
      if (too_long && p.too_long_ends) {
        s.stopped[b] = 1;
        event = kMcStopped;
      } else {
        bool acc = false;
        if (!blocked) {
          if (Et <= E0) {
            acc = true;
          } else {
            const uint4 r =
                philox(make_uint4((uint32_t)b, (uint32_t)step, 7u, 0u), p.key0, p.key1);
            acc = u01(r.x, r.y) < exp(-(Et - E0) / p.kT);
          }
        }
        if (mv == -1) sw_process(chain_window(s, nrb, b, 0), acc);
        else if (mv >= 0) sw_process(chain_window(s, nrb, b, 1 + mv), acc);
        if (acc) {
          for (int k = 0; k < nd; ++k) cur[k] = tr[k];
          s.E_cur[b] = Et;
          s.accepted[b] += 1;
        }
        if (!blocked && Et < s.E_best[b]) {
          s.E_best[b] = Et;
          for (int k = 0; k < nd; ++k) s.best[(size_t)b * nd + k] = tr[k];
        }
        if (p.adapt && rigid && c[1] > 0 && c[1] % kMcBlock == 0) {
          const double ratio = sw_ratio(chain_window(s, nrb, b, 0));
          if (ratio <= 0.45) {
            st[1] = 0.95 * st[1];
            st[0] = 0.95 * st[0];
          } else if (ratio >= 0.55) {
            st[1] = 1.05 * st[1];
            st[0] = fmin(kPi, 1.05 * st[0]);
          }
        }
        if (p.adapt && acc && mv >= 0 && c[2] > 0 && c[2] % (kMcBlock * nrb) == 0) {
          for (int i = 0; i < nrb; ++i) {
            const double ratio = sw_ratio(chain_window(s, nrb, b, 1 + i));
            if (ratio <= 0.45) st[2 + i] = 0.95 * st[2 + i];
            else if (ratio >= 0.55) st[2 + i] = fmin(kPi, 1.05 * st[2 + i]);
          }
        }
        event = (acc ? kMcAccepted : 0) | (blocked ? kMcBlocked : 0);
      }
    }
  }
  if (step < p.trace_steps) {
    const size_t o = (size_t)step * p.B + b;
    if (p.trace_dofs)
      for (int k = 0; k < nd; ++k) p.trace_dofs[o * nd + k] = tr[k];
    if (p.trace_E) p.trace_E[o] = Et;
    if (p.trace_event) p.trace_event[o] = event;
  }
  if (rigid) c[1] += 1;
  else c[2] += 1;
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
MMO_MC_LAUNCH(k_mc_accept)
MMO_MC_LAUNCH(k_gd_begin)
MMO_MC_LAUNCH(k_gd_propose)
MMO_MC_LAUNCH(k_gd_accept)
MMO_MC_LAUNCH(k_gd_take)
#undef MMO_MC_LAUNCH

// a quad of lanes per chain
cudaError_t launch_k_mc_propose(const MCDev& s, const MCParams& p, cudaStream_t st) {
  if (p.B <= 0) return cudaSuccess;
  k_mc_propose<<<nblk(p.B * kQuad), 128, 0, st>>>(s, p);
  return cudaGetLastError();
}

cudaError_t launch_philox(uint32_t k0, uint32_t k1, uint32_t c1, uint32_t c2, int n, uint4* out,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_philox<<<(n + 255) / 256, 256, 0, st>>>(k0, k1, c1, c2, n, out);
  return cudaGetLastError();
}

}  // namespace mmo

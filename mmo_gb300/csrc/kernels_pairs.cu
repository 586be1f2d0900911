// kernels_pairs.cu -- the ligand x protein pair sweep of
// Mol.ene_inter_UFF_shifted_brute / _shifted_bst / _global_brute
// (UnixJunkie/MMO src/mol.ml:796-849, 928-960), FP32 pair terms with an FP64
// accumulation across protein tiles, plus the hand-written adjoint dE/dX.
//
// Batched kernel (k_pairs): persistent CTAs; the protein slice sorted by UFF
// type is staged once per CTA into shared memory by the TMA bulk engine; a
// warp owns one ligand atom j (so the ligand type is warp-uniform) for 32 * KP
// poses (KP poses per lane in registers, as KP/2 pose pairs) and one protein
// chunk.  Each pose pair goes through Blackwell's packed FP32x2 FADD/FMUL/FFMA,
// so one instruction evaluates a term for two poses; each protein atom is
// stored in shared memory with every value doubled ({v, v}) and negated, so
// it feeds the packed operations directly.  Over a type run the pair
// parameters are warp-uniform.
//
// Plain kernel (k_pairs_plain): one pose; a warp owns (ligand atom, protein
// chunk) and its lanes stride over the chunk's protein atoms.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr int kFlush = 256;  // protein atoms per FP32 partial before the FP64 add
constexpr uint32_t kWaitPolls = 1u << 22;

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// One packed step: protein atom (q0..q3, negated and doubled) against a pose
// pair.  With Dp6 = (X / r^2)^3 = D p6 (X = D^(1/3) x^2) and p6 = Dp6 / D:
//   lj = Dp6 (Dp6 / D - 2),  e = lj + el,
//   -(2 dE/dr2 unswitched) r2 = e - Dp6 (10 - 11 p6)            (eps = 4)
//   -(2 dE/dr2 unswitched) r2 / 2 = e - Dp6 (4 - 5 p6)          (eps = 4 r)
// so nt below is -t (eps 4) or -t/2 (eps 4r), and g accumulates -dE/dd or
// -dE/dd / 2; the caller rescales.  mn tracks the smallest r2 for the
// 0.01 A clamp check.  (c1, c0) = (11/D, -10) or (5/D, -4).
template <bool GRAD, int DIEL, int FORM>
__device__ __forceinline__ void pair_step2(float2 xh, float2 yh, float2 zh, float2 xl, float2 yl,
                                           float2 zl, float4 q0, float4 q1, float4 q2,
                                           float4 q3, float2 qq, float2 X, float2 invD,
                                           float2 c1, float2 c0, float2& acc, float2& gx,
                                           float2& gy, float2& gz, float& mn) {
  const float2 dx = add2(add2(xh, make_float2(q0.x, q0.y)), add2(xl, make_float2(q2.x, q2.y)));
  const float2 dy = add2(add2(yh, make_float2(q0.z, q0.w)), add2(yl, make_float2(q2.z, q2.w)));
  const float2 dz = add2(add2(zh, make_float2(q1.x, q1.y)), add2(zl, make_float2(q3.x, q3.y)));
  const float2 r2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
  const float2 r2c = make_float2(fmaxf(r2.x, kMinR2), fmaxf(r2.y, kMinR2));
  const float2 ir = make_float2(rsqrtf(r2c.x), rsqrtf(r2c.y));
  const float2 ir2 = mul2(ir, ir);
  const float2 P = mul2(X, ir2);
  const float2 Dp6 = mul2(mul2(P, P), P);
  const float2 lj = mul2(Dp6, fma2(Dp6, invD, f2(-2.0f)));
  const float2 e = fma2(qq, DIEL == 0 ? ir : ir2, lj);
  float2 s = f2(1.0f);
  if (FORM == 0) {
    s = fma2(r2c, f2(-1.0f / 144.0f), f2(1.0f));
    s = make_float2(fmaxf(s.x, 0.0f), fmaxf(s.y, 0.0f));
    acc = fma2(mul2(s, s), e, acc);
  } else {
    acc = add2(acc, e);
  }
  if (GRAD) {
    const float2 nt = fma2(Dp6, fma2(Dp6, c1, c0), e);
    const float2 na = mul2(nt, ir2);
    float2 g = na;
    if (FORM == 0)
      g = mul2(s, fma2(s, na, mul2(e, f2(DIEL == 0 ? 1.0f / 36.0f : 1.0f / 72.0f))));
    mn = fminf(mn, fminf(r2.x, r2.y));
    gx = fma2(g, dx, gx);
    gy = fma2(g, dy, gy);
    gz = fma2(g, dz, gz);
  }
}

template <int KP, bool GRAD, int DIEL, int FORM>
__global__ void __launch_bounds__(KP >= 8 ? 256 : 512)
    k_pairs(DevProtein prot, PairTable4 tab, DevLigand lig, Scratch scr, int B, int slice0,
            int slice1, int chunk0, int C_slice, int chunk_len, int* err) {
  static_assert(KP % 2 == 0, "poses go in pairs");
  constexpr int NP = KP / 2;
  extern __shared__ __align__(16) float4 sp[];  // [slice][4]
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_runs[2 * kNTypes + 1];
  const int slice_len = slice1 - slice0;
  if (threadIdx.x < 2 * prot.nruns + 1) s_runs[threadIdx.x] = prot.runs[threadIdx.x];
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    const uint32_t bytes = (uint32_t)slice_len * 64u;
    mbar_expect_tx(&bar, bytes);
    constexpr uint32_t kPiece = 32768u;
    for (uint32_t off = 0; off < bytes; off += kPiece) {
      const uint32_t n = bytes - off < kPiece ? bytes - off : kPiece;
      bulk_g2s(reinterpret_cast<char*>(sp) + off,
               reinterpret_cast<const char*>(prot.atoms4 + 4 * (size_t)slice0) + off, n, &bar);
    }
  }
  __syncthreads();
  if (!mbar_wait(&bar, 0, kWaitPolls)) {
    // the copy did not land: flag it, give the copy one more bounded wait so
    // that it is not left writing into a finished CTA, and stop
    if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
    mbar_wait(&bar, 0, kWaitPolls);
    return;
  }

  const int L = lig.L;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int npb = (B + 32 * KP - 1) / (32 * KP);
  const int nitems = npb * C_slice * L;
  for (int item = blockIdx.x * wpb + (threadIdx.x >> 5); item < nitems;
       item += gridDim.x * wpb) {
    const int j = item % L;
    const int rest = item / L;
    const int cl = rest % C_slice;
    const int pb = rest / C_slice;
    const int c0 = slice0 + cl * chunk_len;
    const int c1 = min(c0 + chunk_len, slice1);
    const int ltype = lig.type[j];
    const float2 qj = f2(lig.q[j]);

    float2 xh[NP], yh[NP], zh[NP], xl[NP], yl[NP], zl[NP], acc[NP], gx[NP], gy[NP], gz[NP];
    double ad[KP];
    float mn = 1e30f;
#pragma unroll
    for (int m = 0; m < NP; ++m) {
      float4 h[2], l[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int b = pb * 32 * KP + (2 * m + u) * 32 + lane;
        h[u] = make_float4(1e4f, 1e4f, 1e4f, 0.f);
        l[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (b < B) {
          h[u] = scr.X[((size_t)b * L + j) * 2];
          l[u] = scr.X[((size_t)b * L + j) * 2 + 1];
        }
      }
      xh[m] = make_float2(h[0].x, h[1].x);
      yh[m] = make_float2(h[0].y, h[1].y);
      zh[m] = make_float2(h[0].z, h[1].z);
      xl[m] = make_float2(l[0].x, l[1].x);
      yl[m] = make_float2(l[0].y, l[1].y);
      zl[m] = make_float2(l[0].z, l[1].z);
      acc[m] = gx[m] = gy[m] = gz[m] = f2(0.f);
      ad[2 * m] = ad[2 * m + 1] = 0.0;
    }
    for (int r = 0; r < prot.nruns; ++r) {
      const int lo = max(c0, s_runs[r]);
      const int hi = min(c1, s_runs[r + 1]);
      if (lo >= hi) continue;
      const float4 pv = tab.v[s_runs[prot.nruns + 1 + r] * kNTypes + ltype];
      const float2 X = f2(pv.x), invD = f2(pv.y);
      const float2 k1 = f2(DIEL == 0 ? 11.0f * pv.y : 5.0f * pv.y);
      const float2 k0 = f2(DIEL == 0 ? -10.0f : -4.0f);
      for (int i0 = lo; i0 < hi; i0 += kFlush) {
        const int i1 = min(i0 + kFlush, hi);
#pragma unroll 2
        for (int i = i0 - slice0; i < i1 - slice0; ++i) {
          const float4 q0 = sp[4 * i], q1 = sp[4 * i + 1], q2 = sp[4 * i + 2], q3 = sp[4 * i + 3];
          const float2 qq = mul2(make_float2(q1.z, q1.w), qj);
#pragma unroll
          for (int m = 0; m < NP; ++m)
            pair_step2<GRAD, DIEL, FORM>(xh[m], yh[m], zh[m], xl[m], yl[m], zl[m], q0, q1, q2, q3,
                                         qq, X, invD, k1, k0, acc[m], gx[m], gy[m], gz[m], mn);
        }
#pragma unroll
        for (int m = 0; m < NP; ++m) {
          ad[2 * m] += (double)acc[m].x;
          ad[2 * m + 1] += (double)acc[m].y;
          acc[m] = f2(0.f);
        }
      }
    }
    float gs = DIEL == 0 ? -1.0f : -2.0f;
    if (GRAD && __any_sync(0xffffffffu, mn < kMinR2)) {
      // a pair closer than 0.01 A, where the clamped distance makes the
      // derivative 0: redo this item's gradient with the per-pair test
      gs = 1.0f;
#pragma unroll
      for (int m = 0; m < NP; ++m) {
        float sx0 = 0.f, sy0 = 0.f, sz0 = 0.f, sx1 = 0.f, sy1 = 0.f, sz1 = 0.f, e0 = 0.f, e1 = 0.f;
        for (int r = 0; r < prot.nruns; ++r) {
          const int lo = max(c0, s_runs[r]);
          const int hi = min(c1, s_runs[r + 1]);
          if (lo >= hi) continue;
          const float4 pv = tab.v[s_runs[prot.nruns + 1 + r] * kNTypes + ltype];
          for (int i = lo - slice0; i < hi - slice0; ++i) {
            const float4 q0 = sp[4 * i], q1 = sp[4 * i + 1], q2 = sp[4 * i + 2], q3 = sp[4 * i + 3];
            const float qq = q1.z * qj.x;
            uff_pair<true, DIEL, FORM>((xh[m].x + q0.x) + (xl[m].x + q2.x),
                                       (yh[m].x + q0.z) + (yl[m].x + q2.z),
                                       (zh[m].x + q1.x) + (zl[m].x + q3.x), pv.z, pv.w, qq, e0,
                                       sx0, sy0, sz0);
            uff_pair<true, DIEL, FORM>((xh[m].y + q0.x) + (xl[m].y + q2.x),
                                       (yh[m].y + q0.z) + (yl[m].y + q2.z),
                                       (zh[m].y + q1.x) + (zl[m].y + q3.x), pv.z, pv.w, qq, e1,
                                       sx1, sy1, sz1);
          }
        }
        gx[m] = make_float2(sx0, sx1);
        gy[m] = make_float2(sy0, sy1);
        gz[m] = make_float2(sz0, sz1);
      }
    }
    const int cg = chunk0 + cl;
#pragma unroll
    for (int m = 0; m < NP; ++m) {
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int b = pb * 32 * KP + (2 * m + u) * 32 + lane;
        if (b < B) {
          const size_t o = ((size_t)b * scr.C + cg) * L + j;
          scr.Epart[o] = ad[2 * m + u];
          if (GRAD)
            scr.Gpart[o] = make_float4(gs * (u ? gx[m].y : gx[m].x), gs * (u ? gy[m].y : gy[m].x),
                                       gs * (u ? gz[m].y : gz[m].x), 0.f);
        }
      }
    }
  }
}

template <bool GRAD, int DIEL, int FORM>
__global__ void __launch_bounds__(256)
    k_pairs_plain(DevProtein prot, PairTable tab, const float4* X, const float* lig_q,
                  const int* lig_type, int L, int C, int chunk_len, double* Epart,
                  float4* Gpart) {
  __shared__ float2 stab[kNTypes * kNTypes];
  for (int k = threadIdx.x; k < kNTypes * kNTypes; k += blockDim.x) stab[k] = tab.xd[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (item >= C * L) return;
  const int j = item % L, c = item / L;
  const int c0 = c * chunk_len, c1 = min(c0 + chunk_len, prot.P);
  const float4 xh = X[2 * j], xl = X[2 * j + 1];
  const float qj = lig_q[j];
  const int lt = lig_type[j];
  float ae = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int i = c0 + lane; i < c1; i += 32) {
    const float4 p = prot.atoms[2 * i], pl = prot.atoms[2 * i + 1];
    const float2 xd = stab[prot.type[i] * kNTypes + lt];
    uff_pair<GRAD, DIEL, FORM>(split_diff(xh.x, xl.x, p.x, pl.x), split_diff(xh.y, xl.y, p.y, pl.y),
                               split_diff(xh.z, xl.z, p.z, pl.z), xd.x, xd.y, p.w * qj, ae, gx,
                               gy, gz);
  }
  const double e = warp_sum((double)ae);
  if (GRAD) {
    gx = warp_sum(gx);
    gy = warp_sum(gy);
    gz = warp_sum(gz);
  }
  if (lane == 0) {
    Epart[c * L + j] = e;
    if (GRAD) Gpart[c * L + j] = make_float4(gx, gy, gz, 0.f);
  }
}

using PairsFn = void (*)(DevProtein, PairTable4, DevLigand, Scratch, int, int, int, int, int, int,
                         int*);

template <int KP>
PairsFn pick_batched(bool grad, int diel, int form) {
  if (grad) {
    if (diel) return form ? k_pairs<KP, true, 1, 1> : k_pairs<KP, true, 1, 0>;
    return form ? k_pairs<KP, true, 0, 1> : k_pairs<KP, true, 0, 0>;
  }
  if (diel) return form ? k_pairs<KP, false, 1, 1> : k_pairs<KP, false, 1, 0>;
  return form ? k_pairs<KP, false, 0, 1> : k_pairs<KP, false, 0, 0>;
}

PairsFn pick(int kp, bool grad, const Physics& ph) {
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0;
  switch (kp) {
    case 2: return pick_batched<2>(grad, d, f);
    case 8: return pick_batched<8>(grad, d, f);
    default: return pick_batched<4>(grad, d, f);
  }
}

}  // namespace

int pairs_batched_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem_bytes) {
  PairsFn fn = pick(kp, grad != 0, ph);
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem_bytes) != cudaSuccess)
    return 0;
  return nb;
}

cudaError_t launch_pairs_batched(const DevProtein& prot, const PairTable4& tab,
                                 const DevLigand& lig, const Scratch& s, int B, int flags,
                                 const Physics& ph, const PairPlan& plan, int* d_err,
                                 cudaStream_t st) {
  if (B <= 0 || prot.P <= 0 || lig.L <= 0) return cudaSuccess;
  const bool grad = flags & kFlagGrad;
  PairsFn fn = pick(plan.kp, grad, ph);
  const int nslices = (prot.P + kSliceAtoms - 1) / kSliceAtoms;
  const int C_slice = s.C / nslices;
  const int slice_len = (prot.P + nslices - 1) / nslices;
  for (int sl = 0; sl < nslices; ++sl) {
    const int s0 = sl * slice_len, s1 = min(s0 + slice_len, prot.P);
    if (s0 >= s1) break;
    const int chunk_len = (s1 - s0 + C_slice - 1) / C_slice;
    const int smem = (s1 - s0) * 64;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    fn<<<plan.blocks, plan.threads, smem, st>>>(prot, tab, lig, s, B, s0, s1, sl * C_slice,
                                                 C_slice, chunk_len, d_err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_pairs_plain(const DevProtein& prot, const PairTable& tab, const float4* X,
                               const float* lig_q, const int* lig_type, int L, int C,
                               double* Epart, float4* Gpart, int grad, const Physics& ph,
                               cudaStream_t st) {
  if (L <= 0 || C <= 0) return cudaSuccess;
  const int chunk_len = (prot.P + C - 1) / C;
  const int blocks = (C * L + 7) / 8;
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0;
#define MMO_PL(G, D, F) \
  k_pairs_plain<G, D, F><<<blocks, 256, 0, st>>>(prot, tab, X, lig_q, lig_type, L, C, chunk_len, Epart, Gpart)
  if (grad) {
    if (d) { if (f) MMO_PL(true, 1, 1); else MMO_PL(true, 1, 0); }
    else { if (f) MMO_PL(true, 0, 1); else MMO_PL(true, 0, 0); }
  } else {
    if (d) { if (f) MMO_PL(false, 1, 1); else MMO_PL(false, 1, 0); }
    else { if (f) MMO_PL(false, 0, 1); else MMO_PL(false, 0, 0); }
  }
#undef MMO_PL
  return cudaGetLastError();
}

}  // namespace mmo

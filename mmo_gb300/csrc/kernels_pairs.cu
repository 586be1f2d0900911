// kernels_pairs.cu -- the ligand x protein pair sweep of
// Mol.ene_inter_UFF_shifted_brute / _shifted_bst / _global_brute
// (UnixJunkie/MMO src/mol.ml:796-849, 928-960), FP32 pair terms with an FP64
// accumulation across protein tiles, plus the hand-written adjoint dE/dX.
//
// Batched kernel (k_pairs): persistent CTAs; the protein slice sorted by UFF
// type is staged once per CTA into shared memory by the TMA bulk engine; a
// warp owns one ligand atom j (so the ligand type is warp-uniform) for 32 * KP
// poses (KP poses per lane in registers) and one protein chunk; over a type
// run the pair parameters are warp-uniform, so a pair costs one broadcast
// shared-memory load per KP poses and about 35 FP32 instructions.  (Packed
// FP32x2 arithmetic, measured on GB300, ran this loop slower: the FMA pipe,
// not instruction issue, then bounds it.)
//
// Plain kernel (k_pairs_plain): one pose; a warp owns (ligand atom, protein
// chunk) and its lanes stride over the chunk's protein atoms.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr int kFlush = 256;  // protein atoms per FP32 partial before the FP64 add
constexpr uint32_t kWaitPolls = kWaitPollsDefault;

// dE/dX of one pose for the protein atoms [c0, c1) with the per-pair test
// of the 0.01 A clamp (rarely needed, so kept out of the main loop's registers)
template <int DIEL, int FORM>
__device__ __noinline__ float3 exact_grad(const float4* sp, int slice0, int c0, int c1,
                                          const int* s_runs, int nruns, const float4* tabv,
                                          int ltype, float qj, float xh, float yh, float zh,
                                          float xl, float yl, float zl) {
  float e = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int r = 0; r < nruns; ++r) {
    const int lo = max(c0, s_runs[r]);
    const int hi = min(c1, s_runs[r + 1]);
    if (lo >= hi) continue;
    const float4 pv = tabv[s_runs[nruns + 1 + r] * kNTypes + ltype];
    for (int i = lo - slice0; i < hi - slice0; ++i) {
      const float4 p = sp[2 * i], pl = sp[2 * i + 1];
      uff_pair<true, DIEL, FORM>((xh - p.x) + (xl - pl.x), (yh - p.y) + (yl - pl.y),
                                 (zh - p.z) + (zl - pl.z), pv.z, pv.w, p.w * qj, e, gx, gy, gz);
    }
  }
  return make_float3(gx, gy, gz);
}

template <int KP, bool GRAD, int DIEL, int FORM>
__global__ void __launch_bounds__(512)
    k_pairs(DevProtein prot, const float4* __restrict__ tabv, DevLigand lig, Scratch scr, int B,
            int slice0, int slice1, int chunk0, int C_slice, int chunk_len, int* err) {
  extern __shared__ __align__(16) float4 sp[];  // [slice][2]
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_runs[2 * kNTypes + 1];
  const int slice_len = slice1 - slice0;
  if (threadIdx.x < 2 * prot.nruns + 1) s_runs[threadIdx.x] = prot.runs[threadIdx.x];
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    const uint32_t bytes = (uint32_t)slice_len * 32u;
    mbar_expect_tx(&bar, bytes);
    constexpr uint32_t kPiece = 32768u;
    for (uint32_t off = 0; off < bytes; off += kPiece) {
      const uint32_t n = bytes - off < kPiece ? bytes - off : kPiece;
      bulk_g2s(reinterpret_cast<char*>(sp) + off,
               reinterpret_cast<const char*>(prot.atoms + 2 * (size_t)slice0) + off, n, &bar);
    }
  }
  __syncthreads();
  if (!mbar_wait(&bar, 0, scr.first_wait_polls)) {
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
    const float qj = lig.q[j];

    float xh[KP], yh[KP], zh[KP], xl[KP], yl[KP], zl[KP], acc[KP], gx[KP], gy[KP], gz[KP];
    double ad[KP];
    float mn = 1e30f;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int b = pb * 32 * KP + k * 32 + lane;
      float4 h = make_float4(1e4f, 1e4f, 1e4f, 0.f), l = make_float4(0.f, 0.f, 0.f, 0.f);
      if (b < B) {
        h = scr.X[((size_t)b * L + j) * 2];
        l = scr.X[((size_t)b * L + j) * 2 + 1];
      }
      xh[k] = h.x;
      yh[k] = h.y;
      zh[k] = h.z;
      xl[k] = l.x;
      yl[k] = l.y;
      zl[k] = l.z;
      acc[k] = gx[k] = gy[k] = gz[k] = 0.f;
      ad[k] = 0.0;
    }
    for (int r = 0; r < prot.nruns; ++r) {
      const int lo = max(c0, s_runs[r]);
      const int hi = min(c1, s_runs[r + 1]);
      if (lo >= hi) continue;
      const float4 pv = tabv[s_runs[prot.nruns + 1 + r] * kNTypes + ltype];
      const float c1v = (DIEL == 0 ? 11.0f : 5.0f) * pv.y;
      const float c0v = DIEL == 0 ? -10.0f : -4.0f;
      for (int i0 = lo; i0 < hi; i0 += kFlush) {
        const int i1 = min(i0 + kFlush, hi);
#pragma unroll 4
        for (int i = i0 - slice0; i < i1 - slice0; ++i) {
          const float4 p = sp[2 * i], pl = sp[2 * i + 1];
          const float qq = p.w * qj;
#pragma unroll
          for (int k = 0; k < KP; ++k)
            pair_step<GRAD, DIEL, FORM>(xh[k], yh[k], zh[k], xl[k], yl[k], zl[k], p, pl, qq, pv.x,
                                        pv.y, c1v, c0v, acc[k], gx[k], gy[k], gz[k], mn);
        }
#pragma unroll
        for (int k = 0; k < KP; ++k) {
          ad[k] += (double)acc[k];
          acc[k] = 0.f;
        }
      }
    }
    float gs = DIEL == 0 ? -1.0f : -2.0f;
    if (GRAD && __any_sync(0xffffffffu, mn < kMinR2)) {
      // a pair closer than 0.01 A, where the clamped distance makes the
      // derivative 0: redo this item's gradient with the per-pair test
      gs = 1.0f;
#pragma unroll
      for (int k = 0; k < KP; ++k) {
        const float3 g = exact_grad<DIEL, FORM>(sp, slice0, c0, c1, s_runs, prot.nruns, tabv, ltype,
                                                qj, xh[k], yh[k], zh[k], xl[k], yl[k], zl[k]);
        gx[k] = g.x;
        gy[k] = g.y;
        gz[k] = g.z;
      }
    }
    const int cg = chunk0 + cl;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int b = pb * 32 * KP + k * 32 + lane;
      if (b < B) {
        const size_t o = ((size_t)b * scr.C + cg) * L + j;
        scr.Epart[o] = ad[k];
        if (GRAD) scr.Gpart[o] = make_float4(gs * gx[k], gs * gy[k], gs * gz[k], 0.f);
      }
    }
  }
}

template <bool GRAD, int DIEL, int FORM>
__global__ void __launch_bounds__(256)
    k_pairs_plain(DevProtein prot, PairTable tab, const float4* X, const float* lig_q,
                  const int* lig_type, int L, int C, int chunk_len, double* Epart,
                  float4* Gpart, double* Eout, unsigned* arrive) {
  __shared__ float2 stab[kNTypes * kNTypes];
  __shared__ double wsum[8];
  __shared__ int s_last;
  for (int k = threadIdx.x; k < kNTypes * kNTypes; k += blockDim.x) stab[k] = tab.xd[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (item < C * L) {
    const int j = item % L, c = item / L;
    const int c0 = c * chunk_len, c1 = min(c0 + chunk_len, prot.P);
    const float4 xh = X[2 * j], xl = X[2 * j + 1];
    const float qj = lig_q[j];
    const int lt = lig_type[j];
    float ae = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
    for (int i = c0 + lane; i < c1; i += 32) {
      const float4 p = prot.atoms[2 * i], pl = prot.atoms[2 * i + 1];
      const float2 xd = stab[prot.type[i] * kNTypes + lt];
      uff_pair<GRAD, DIEL, FORM>(split_diff(xh.x, xl.x, p.x, pl.x),
                                 split_diff(xh.y, xl.y, p.y, pl.y),
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
  if (!Eout) return;
  // Eout: the last block to arrive adds every partial in a fixed order, so
  // that one launch gives the total (an atomic count, nothing waits)
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(arrive, 1u) == gridDim.x - 1u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double s = 0.0;
  for (int k = threadIdx.x; k < C * L; k += blockDim.x) s += __ldcg(Epart + k);
  s = warp_sum(s);
  if (lane == 0) wsum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    *Eout = t;
    *arrive = 0u;  // ready for the next launch
  }
}

// The two parts of the inter energy for one ligand (mmo_ene_inter_parts): as
// k_pairs_plain, with the electrostatic partials in Epart[0, C L) and the van
// der Waals ones in Epart[C L, 2 C L); the last block to arrive adds each set
// in a fixed order into Eout[0], Eout[1].
template <int DIEL, int FORM>
__global__ void __launch_bounds__(256)
    k_pairs_parts(DevProtein prot, PairTable tab, const float4* X, const float* lig_q,
                  const int* lig_type, int L, int C, int chunk_len, double* Epart, double* Eout,
                  unsigned* arrive) {
  __shared__ float2 stab[kNTypes * kNTypes];
  __shared__ double wsum[2][8];
  __shared__ int s_last;
  for (int k = threadIdx.x; k < kNTypes * kNTypes; k += blockDim.x) stab[k] = tab.xd[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int item = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (item < C * L) {
    const int j = item % L, c = item / L;
    const int c0 = c * chunk_len, c1 = min(c0 + chunk_len, prot.P);
    const float4 xh = X[2 * j], xl = X[2 * j + 1];
    const float qj = lig_q[j];
    const int lt = lig_type[j];
    float ael = 0.f, alj = 0.f;
    for (int i = c0 + lane; i < c1; i += 32) {
      const float4 p = prot.atoms[2 * i], pl = prot.atoms[2 * i + 1];
      const float2 xd = stab[prot.type[i] * kNTypes + lt];
      uff_pair_parts<DIEL, FORM>(split_diff(xh.x, xl.x, p.x, pl.x),
                                 split_diff(xh.y, xl.y, p.y, pl.y),
                                 split_diff(xh.z, xl.z, p.z, pl.z), xd.x, xd.y, p.w * qj, ael,
                                 alj);
    }
    const double el = warp_sum((double)ael), lj = warp_sum((double)alj);
    if (lane == 0) {
      Epart[c * L + j] = el;
      Epart[C * L + c * L + j] = lj;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(arrive, 1u) == gridDim.x - 1u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int part = 0; part < 2; ++part) {
    double s = 0.0;
    for (int k = threadIdx.x; k < C * L; k += blockDim.x) s += __ldcg(Epart + part * C * L + k);
    s = warp_sum(s);
    if (lane == 0) wsum[part][threadIdx.x >> 5] = s;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[threadIdx.x][w];
    Eout[threadIdx.x] = t;
  }
  if (threadIdx.x == 0) *arrive = 0u;  // ready for the next launch
}

using PairsFn = void (*)(DevProtein, const float4*, DevLigand, Scratch, int, int, int, int, int,
                         int, int*);

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
    case 1: return pick_batched<1>(grad, d, f);
    case 2: return pick_batched<2>(grad, d, f);
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

cudaError_t launch_pairs_batched(const DevProtein& prot, const float4* tab,
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
    const int smem = (s1 - s0) * 32;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    fn<<<plan.blocks, plan.threads, smem, st>>>(prot, tab, lig, s, B, s0, s1, sl * C_slice,
                                                 C_slice, chunk_len, d_err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_pairs_parts(const DevProtein& prot, const PairTable& tab, const float4* X,
                               const float* lig_q, const int* lig_type, int L, int C,
                               double* Epart, const Physics& ph, cudaStream_t st, double* Eout,
                               unsigned* arrive) {
  if (L <= 0 || C <= 0) return cudaSuccess;
  const int chunk_len = (prot.P + C - 1) / C;
  const int blocks = (C * L + 7) / 8;
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0;
#define MMO_PP(D, F) \
  k_pairs_parts<D, F><<<blocks, 256, 0, st>>>(prot, tab, X, lig_q, lig_type, L, C, chunk_len, Epart, Eout, arrive)
  if (d) { if (f) MMO_PP(1, 1); else MMO_PP(1, 0); }
  else { if (f) MMO_PP(0, 1); else MMO_PP(0, 0); }
#undef MMO_PP
  return cudaGetLastError();
}

cudaError_t launch_pairs_plain(const DevProtein& prot, const PairTable& tab, const float4* X,
                               const float* lig_q, const int* lig_type, int L, int C,
                               double* Epart, float4* Gpart, int grad, const Physics& ph,
                               cudaStream_t st, double* Eout, unsigned* arrive) {
  if (L <= 0 || C <= 0) return cudaSuccess;
  const int chunk_len = (prot.P + C - 1) / C;
  const int blocks = (C * L + 7) / 8;
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0;
#define MMO_PL(G, D, F) \
  k_pairs_plain<G, D, F><<<blocks, 256, 0, st>>>(prot, tab, X, lig_q, lig_type, L, C, chunk_len, Epart, Gpart, Eout, arrive)
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

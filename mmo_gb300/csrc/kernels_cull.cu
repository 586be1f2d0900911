// kernels_cull.cu -- the cut-off sweep of the shifted form
// (Mol.ene_inter_UFF_shifted_bst, UnixJunkie/MMO src/mol.ml:928-962: the
// reference visits, for each ligand atom, only the protein atoms that its
// bisector-tree neighbour query returns within 12 A).  Here the query is made for a
// group of 32 * KP (pose, ligand atom) entries at once:
//
//   (the pose rebuild bins the entries: ligand type segment, Hilbert cell of
//   each entry's position, count and rank)
//   k_cull_scan     bin counts -> first slot of each bin (one CTA per segment)
//   k_cull_scatter  entries copied into slot order
//   k_cull_items    broad phase: the (group, protein piece) items within 12 A
//   k_pairs_cull    persistent CTAs, protein staged in shared memory (TMA bulk
//                   copy) or read from global memory; a warp takes (group,
//                   piece) items from a work counter, bounds its group by a box
//                   and sweeps the rows of the piece that come within 12 A of
//                   the box, and the last piece of a group to finish sums the
//                   group's pieces in piece order
//
// Slot order only decides which entries share a warp.  Skipped pairs add
// exact zeros and the FP32 partials are flushed at fixed rows, so the result
// of an entry is the same whichever entries share its group.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr uint32_t kWaitPolls = kWaitPollsDefault;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kListCap = 64;  // a warp's list: under 32 left over plus one window of 32
constexpr int kTabRows = kNullTypeRow + 1;  // protein types of the shared pair table

// the pair table in shared memory: [ptype][ltype] (X, 1/D, c1, 0) with
// c1 = 11/D (eps = 4) or 5/D (eps = 4r), and the null type row of zeros
template <int DIEL>
__device__ __forceinline__ void stage_pair_table(const float4* __restrict__ tabv, float4* s_tab) {
  for (int k = threadIdx.x; k < kTabRows * kNTypes; k += blockDim.x) {
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (k < kNTypes * kNTypes) {
      v = tabv[k];
      v = make_float4(v.x, v.y, (DIEL == 0 ? 11.0f : 5.0f) * v.y, 0.f);
    }
    s_tab[k] = v;
  }
}


constexpr int kScanThreads = 1024;
constexpr int kScanPer = kCullBins / kScanThreads;  // 32 consecutive bins per thread
constexpr int kScanSmem = kScanThreads * (kScanPer + 1) * 4;  // padded rows: no bank conflicts

// Exclusive scan of one segment's bin counts into first slots: coalesced
// loads into shared memory, a serial scan of 32 consecutive bins per thread
// and one block scan of the thread sums.  Also clears the work counter, the
// pair counter and the groups' arrival counters of the sweep.
__global__ void __launch_bounds__(kScanThreads) k_cull_scan(unsigned* hist, CullSegs seg,
                                                             unsigned* queue, int* arrive,
                                                             int narrive) {
  extern __shared__ unsigned sh[];  // [kScanThreads][kScanPer + 1]
  __shared__ unsigned wsum[kScanThreads / 32];
  unsigned* h = hist + (size_t)blockIdx.x * kCullBins;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll 8
  for (int k = 0; k < kScanPer; ++k) {
    const int i = k * kScanThreads + t;
    sh[(i / kScanPer) * (kScanPer + 1) + i % kScanPer] = h[i];
  }
  __syncthreads();
  unsigned* row = sh + t * (kScanPer + 1);
  unsigned s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) s += row[k];
  unsigned inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    unsigned v = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned u = __shfl_up_sync(kFull, v, o);
      if (lane >= o) v += u;
    }
    wsum[lane] = v;  // inclusive over warps
  }
  __syncthreads();
  unsigned run = (unsigned)seg.off[blockIdx.x] + (w ? wsum[w - 1] : 0u) + inc - s;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const unsigned c = row[k];
    row[k] = run;
    run += c;
  }
  __syncthreads();
#pragma unroll 8
  for (int k = 0; k < kScanPer; ++k) {
    const int i = k * kScanThreads + t;
    h[i] = sh[(i / kScanPer) * (kScanPer + 1) + i % kScanPer];
  }
  for (int k = blockIdx.x * blockDim.x + t; k < narrive; k += gridDim.x * blockDim.x) arrive[k] = 0;
  if (blockIdx.x == 0 && t == 0) {
    queue[0] = 0u;  // the sweep's work counter
    queue[1] = 0u;  // its items, counted by the broad phase
    *reinterpret_cast<unsigned long long*>(queue + 2) = 0ull;
  }
}

__global__ void k_cull_scatter(const float4* __restrict__ X, int n, int L,
                               const float* __restrict__ lig_q, const unsigned* __restrict__ hist,
                               const int* __restrict__ bin, const int* __restrict__ rank,
                               float4* Xs, int* order) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int slot = (int)hist[bin[e]] + rank[e];
  const float4 h = X[2 * (size_t)e], l = X[2 * (size_t)e + 1];
  Xs[2 * (size_t)slot] = make_float4(h.x, h.y, h.z, lig_q[e % L]);
  Xs[2 * (size_t)slot + 1] = make_float4(l.x, l.y, l.z, 0.f);
  order[slot] = e;
}

// (X, 1/D, c1) of the protein atoms a and b of a pair against the warp's
// ligand type (trow): their rows of the pair table, at the byte offsets a3.zw
__device__ __forceinline__ void pair_params(const float4* trow, float4 a3, float2& X, float2& iD,
                                            float2& c1) {
  const float* ta =
      reinterpret_cast<const float*>(reinterpret_cast<const char*>(trow) + __float_as_int(a3.z));
  const float* tb =
      reinterpret_cast<const float*>(reinterpret_cast<const char*>(trow) + __float_as_int(a3.w));
  X = make_float2(ta[0], tb[0]);
  iD = make_float2(ta[1], tb[1]);
  c1 = make_float2(ta[2], tb[2]);
}

// Protein records: read from shared memory (the staged copy) or, with GLOB,
// from global memory through the read-only path (L1 / L2)
template <bool GLOB>
__device__ __forceinline__ float4 ldp(const float4* p) {
  if constexpr (GLOB) return __ldg(p);
  else return *p;
}
template <bool GLOB>
__device__ __forceinline__ int ldi(const int* p) {
  if constexpr (GLOB) return __ldg(p);
  else return *p;
}

// dE/dX of one entry over the protein pairs [a0, a1) with the per-pair test
// of the 0.01 A clamp; the same arithmetic in the same order as the sweep, so
// entries without a clamped pair get the sweep's value bit for bit.
template <int DIEL, int FORM, bool GLOB>
__device__ __noinline__ float3 cull_exact_grad(const float4* sp, const float4* trow, int a0, int a1,
                                               float q, float xh, float yh, float zh, float xl,
                                               float yl, float zl) {
  constexpr float c0 = DIEL == 0 ? -10.0f : -4.0f;
  float2 acc = bc2(0.f), gx = bc2(0.f), gy = bc2(0.f), gz = bc2(0.f);
  float mn = 1e30f;
  for (int i = a0; i < a1; ++i) {
    const float4* pp = sp + 4 * i;
    const float4 p0 = ldp<GLOB>(pp), p1 = ldp<GLOB>(pp + 1), p2 = ldp<GLOB>(pp + 2),
                 p3 = ldp<GLOB>(pp + 3);
    float2 X, iD, c1;
    pair_params(trow, p3, X, iD, c1);
    pair_step_ab<true, DIEL, FORM, true>(bc2(xh), bc2(yh), bc2(zh), bc2(xl), bc2(yl), bc2(zl),
                                         bc2(q), p0, p1, p2, p3, X, iD, c1, c0, acc, gx, gy, gz,
                                         mn);
  }
  return make_float3(gx.x + gx.y, gy.x + gy.y, gz.x + gz.y);
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// squared distance from (x, y, z) to the box [bl, bh]
__device__ __forceinline__ float box_d2(float x, float y, float z, float blx, float bly, float blz,
                                        float bhx, float bhy, float bhz) {
  const float ex = fmaxf(fmaxf(blx - x, x - bhx), 0.f);
  const float ey = fmaxf(fmaxf(bly - y, y - bhy), 0.f);
  const float ez = fmaxf(fmaxf(blz - z, z - bhz), 0.f);
  return fmaf(ex, ex, fmaf(ey, ey, ez * ez));
}

// One warp's work for one (group, protein piece) item: the group's entries
// [slot0, s_end) (32 * KP slots, padding repeats the last entry) against the
// piece's rows [r0, r1) (sp: pairs of atoms, s_rbox, s_rs: first pair of each
// row, s_flush; in shared memory, or in global memory with GLOB), then the
// piece's partials at P0 + kpc * PS (+ slot - slot0).  The last of the
// group's npieces items to arrive sums them in piece order: with LISTED the
// pieces of plist[0 .. npieces) (the broad phase's list, every one written),
// otherwise pieces 0 .. npieces - 1 whose flag at V0 + q says visited.  CULL
// false visits every atom (the global form).
template <int KP, bool GRAD, int DIEL, int FORM, bool CULL, bool LISTED = false, bool GLOB = false>
__device__ __forceinline__ void sweep_item(const float4* sp, const float4* s_rbox, const int* s_rs,
                                           const int* s_flush, int r0, int r1,
                                           const float4* trow, int slot0, int s_end, int* wl,
                                           const CullScratch& cs, long long P0, long long PS,
                                           int kpc, long long V0, int npieces, int* arrive,
                                           const int* plist = nullptr) {
  constexpr float c0v = DIEL == 0 ? -10.0f : -4.0f;
  constexpr int G = 32 * KP;
  const int lane = threadIdx.x & 31;
  // the lane's entries, each value in both halves (one per atom of a pair);
  // half x sums the even atoms of each row, half y the odd ones
  float2 xh[KP], yh[KP], zh[KP], xl[KP], yl[KP], zl[KP], q[KP];
  float2 acc[KP], gx[KP], gy[KP], gz[KP];
  double ad[KP];
  float blx = 1e30f, bly = 1e30f, blz = 1e30f, bhx = -1e30f, bhy = -1e30f, bhz = -1e30f;
#pragma unroll
  for (int k = 0; k < KP; ++k) {
    const int s = min(slot0 + k * 32 + lane, s_end - 1);
    const float4 h = cs.Xs[2 * (size_t)s], l = cs.Xs[2 * (size_t)s + 1];
    xh[k] = bc2(h.x);
    yh[k] = bc2(h.y);
    zh[k] = bc2(h.z);
    q[k] = bc2(h.w);
    xl[k] = bc2(l.x);
    yl[k] = bc2(l.y);
    zl[k] = bc2(l.z);
    acc[k] = gx[k] = gy[k] = gz[k] = bc2(0.f);
    ad[k] = 0.0;
    blx = fminf(blx, h.x);
    bly = fminf(bly, h.y);
    blz = fminf(blz, h.z);
    bhx = fmaxf(bhx, h.x);
    bhy = fmaxf(bhy, h.y);
    bhz = fmaxf(bhz, h.z);
  }
  blx = warp_min(blx);
  bly = warp_min(bly);
  blz = warp_min(blz);
  bhx = warp_maxf(bhx);
  bhy = warp_maxf(bhy);
  bhz = warp_maxf(bhz);

  float mn = 1e30f;
  int visited = 0;       // pairs swept
  unsigned natoms = 0;   // atoms of them within reach of the box (the pair counter)
  // the pairs of the warp's candidate rows with an atom within 12 A of the
  // box, compacted in ascending order into the warp's list wl and swept 32 or
  // more at a time
  int cnt = 0;
  auto sweep = [&](int n) {
    __syncwarp();
#pragma unroll 2
    for (int v = 0; v < n; ++v) {
      const float4* pp = sp + 4 * wl[v];
      const float4 p0 = ldp<GLOB>(pp), p1 = ldp<GLOB>(pp + 1), p2 = ldp<GLOB>(pp + 2),
                   p3 = ldp<GLOB>(pp + 3);
      float2 X, iD, c1;
      pair_params(trow, p3, X, iD, c1);
#pragma unroll
      for (int k = 0; k < KP; ++k)
        pair_step_ab<GRAD, DIEL, FORM>(xh[k], yh[k], zh[k], xl[k], yl[k], zl[k], q[k], p0, p1, p2,
                                       p3, X, iD, c1, c0v, acc[k], gx[k], gy[k], gz[k], mn);
    }
    __syncwarp();
  };
  // rows in flush blocks: the FP32 partials go into the FP64 sums once per
  // block (fixed rows of the protein) and at the end of the piece
  for (int r = r0; r < r1;) {
    const int rend = min(r1, ldi<GLOB>(s_flush + r));
    for (; r < rend; ++r) {
      const float4 rb = ldp<GLOB>(s_rbox + r);
      const float dy = fmaxf(fmaxf(rb.x - bhy, bly - rb.y), 0.f);
      const float dz = fmaxf(fmaxf(rb.z - bhz, blz - rb.w), 0.f);
      if (CULL && fmaf(dy, dy, dz * dz) >= kCullR2) continue;
      const int a = ldi<GLOB>(s_rs + r), b = ldi<GLOB>(s_rs + r + 1);
      for (int i0 = a; i0 < b; i0 += 32) {
        const int i = i0 + lane;
        bool in_a = false, in_b = false;
        if (i < b) {
          const float4 p0 = ldp<GLOB>(sp + 4 * i), p1 = ldp<GLOB>(sp + 4 * i + 1);
          const bool null_b = __float_as_uint(p1.w) == 0x80000000u;
          in_a = !CULL || box_d2(-p0.x, -p0.z, -p1.x, blx, bly, blz, bhx, bhy, bhz) < kCullR2;
          in_b = !null_b &&
                 (!CULL || box_d2(-p0.y, -p0.w, -p1.y, blx, bly, blz, bhx, bhy, bhz) < kCullR2);
        }
        const bool in = in_a || in_b;
        const unsigned m = __ballot_sync(kFull, in);
        if (in) wl[cnt + __popc(m & ((1u << lane) - 1u))] = i;
        cnt += __popc(m);
        // the atoms that pass the test (a partner that does not is swept anyway)
        natoms += __popc(__ballot_sync(kFull, in_a)) + __popc(__ballot_sync(kFull, in_b));
        if (cnt >= 32) {
          sweep(cnt);
          visited += cnt;
          cnt = 0;
        }
      }
    }
    sweep(cnt);
    visited += cnt;
    cnt = 0;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      ad[k] += (double)acc[k].x;
      ad[k] += (double)acc[k].y;
      acc[k] = bc2(0.f);
    }
  }
  float3 gsum[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k)
    gsum[k] = make_float3(gx[k].x + gx[k].y, gy[k].x + gy[k].y, gz[k].x + gz[k].y);
  if (GRAD && __any_sync(kFull, mn < kMinR2)) {
    // a pair closer than 0.01 A, where the clamped distance makes the
    // derivative 0: redo the gradient over the piece with the per-pair test
    const int a0 = ldi<GLOB>(s_rs + r0), a1 = ldi<GLOB>(s_rs + r1);
#pragma unroll
    for (int k = 0; k < KP; ++k)
      gsum[k] = cull_exact_grad<DIEL, FORM, GLOB>(sp, trow, a0, a1, q[k].x, xh[k].x, yh[k].x,
                                                  zh[k].x, xl[k].x, yl[k].x, zl[k].x);
  }
  if (lane == 0 && natoms) atomicAdd(cs.pairs, (unsigned long long)natoms * G);
  constexpr float gs = DIEL == 0 ? -1.0f : -2.0f;
  if (LISTED || visited) {  // an unlisted or unvisited piece adds nothing
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int s = slot0 + k * 32 + lane;
      if (s < s_end) {
        const size_t o = (size_t)(P0 + (long long)kpc * PS) + (size_t)(s - slot0);
        cs.Ep[o] = ad[k];
        if (GRAD) cs.Gp[o] = make_float4(gs * gsum[k].x, gs * gsum[k].y, gs * gsum[k].z, 0.f);
      }
    }
  }
  // the last piece of the group to finish sums the group's pieces in piece
  // order (the arrival order does not matter)
  if (!LISTED && lane == 0) cs.vis[(size_t)V0 + kpc] = visited ? 1 : 0;
  __threadfence();  // every lane's partials before the arrival
  __syncwarp();
  int last = 0;
  if (lane == 0) last = atomicAdd(arrive, 1) == npieces - 1;
  last = __shfl_sync(kFull, last, 0);
  if (last) {
    __threadfence();
    const uint8_t* vg = cs.vis + (size_t)V0;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
      const int s = slot0 + k * 32 + lane;
      if (s >= s_end) continue;
      double E = 0.0;
      double sx = 0.0, sy = 0.0, sz = 0.0;
      for (int j = 0; j < npieces; ++j) {
        int q2 = j;
        if (LISTED) q2 = __ldcg(plist + j);
        else if (!__ldcg(vg + j)) continue;
        const size_t o = (size_t)(P0 + (long long)q2 * PS) + (size_t)(s - slot0);
        E += __ldcg(cs.Ep + o);
        if (GRAD) {
          const float4 g4 = __ldcg(cs.Gp + o);
          sx += g4.x;
          sy += g4.y;
          sz += g4.z;
        }
      }
      // an entry at a non-finite position can fall in a group far from the protein
      if (!isfinite(xh[k].x) || !isfinite(yh[k].x) || !isfinite(zh[k].x))
        E = __longlong_as_double(0x7ff8000000000000ll);
      const int e = cs.order[s];
      cs.Eout[e] = E;
      if (GRAD) cs.Gout[e] = make_float4((float)sx, (float)sy, (float)sz, 0.f);
    }
    if (LISTED) {
      // the group's piece partials are dead from here on: drop their L2 lines
      // without a write-back to DRAM (128-byte lines: G doubles of energy and
      // G float4 of gradient per piece, both aligned to G * 8 bytes)
      constexpr int kEl = 32 * KP * 8 / 128, kGl = GRAD ? 32 * KP * 16 / 128 : 0;
      for (int w = lane; w < npieces * (kEl + kGl); w += 32) {
        const int j = w / (kEl + kGl), l = w - j * (kEl + kGl);
        const int q2 = __ldcg(plist + j);
        const size_t o = (size_t)(P0 + (long long)q2 * PS);
        const char* a = l < kEl ? reinterpret_cast<const char*>(cs.Ep + o) + 128 * l
                                : reinterpret_cast<const char*>(cs.Gp + o) + 128 * (l - kEl);
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(a) : "memory");
      }
    }
  }
}

// The broad phase: one warp per entry group bounds the group's entries by a
// box and lists, in ascending order, the protein pieces whose box comes
// within sqrt(145) A of it (any other piece's pairs are all beyond the
// cut-off, so they would add exact zeros); it reserves one work item per
// listed piece in the flat item list (queue[1] counts them) and clears the
// group's arrival counter.
__global__ void k_cull_items(CullSegs seg, CullScratch cs, int ngroups) {
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (g >= ngroups) return;
  const int lane = threadIdx.x & 31, G = seg.G;
  const int slot0 = g * G;
  int t = 0;
  while (t + 1 < seg.nseg && slot0 >= seg.off[t + 1]) ++t;
  const int s_end = seg.off[t] + seg.n[t];
  float blx = 1e30f, bly = 1e30f, blz = 1e30f, bhx = -1e30f, bhy = -1e30f, bhz = -1e30f;
  for (int k = lane; k < G; k += 32) {
    const int s = min(slot0 + k, s_end - 1);
    const float4 h = cs.Xs[2 * (size_t)s];
    blx = fminf(blx, h.x);
    bly = fminf(bly, h.y);
    blz = fminf(blz, h.z);
    bhx = fmaxf(bhx, h.x);
    bhy = fmaxf(bhy, h.y);
    bhz = fmaxf(bhz, h.z);
  }
  blx = warp_min(blx);
  bly = warp_min(bly);
  blz = warp_min(blz);
  bhx = warp_maxf(bhx);
  bhy = warp_maxf(bhy);
  bhz = warp_maxf(bhz);
  // fminf / fmaxf skip NaN, so a group with a non-finite position can have a
  // box that excludes it: such a group keeps every piece (its energy is set
  // to NaN by the sweep's last arrival anyway)
  bool bad = false;
  for (int k = lane; k < G; k += 32) {
    const float4 h = cs.Xs[2 * (size_t)min(slot0 + k, s_end - 1)];
    bad = bad || !isfinite(h.x) || !isfinite(h.y) || !isfinite(h.z);
  }
  bad = __any_sync(kFull, bad);
  int* gl = cs.glist + (size_t)g * cs.npieces;
  int cnt = 0;
  for (int q0 = 0; q0 < cs.npieces; q0 += 32) {
    const int q = q0 + lane;
    bool in = false;
    if (q < cs.npieces) {
      const float4 lo = cs.pbox[2 * q], hi = cs.pbox[2 * q + 1];
      const float ex = fmaxf(fmaxf(lo.x - bhx, blx - hi.x), 0.f);
      const float ey = fmaxf(fmaxf(lo.y - bhy, bly - hi.y), 0.f);
      const float ez = fmaxf(fmaxf(lo.z - bhz, blz - hi.z), 0.f);
      in = bad || fmaf(ex, ex, fmaf(ey, ey, ez * ez)) < kCullR2;
    }
    const unsigned m = __ballot_sync(kFull, in);
    if (in) gl[cnt + __popc(m & ((1u << lane) - 1u))] = q;
    cnt += __popc(m);
  }
  int base = 0;
  if (lane == 0) {
    cs.gcount[g] = cnt;
    cs.arrive[g] = 0;
    base = cnt ? (int)atomicAdd(cs.queue + 1, (unsigned)cnt) : 0;
  }
  base = __shfl_sync(kFull, base, 0);
  __syncwarp();
  for (int k = lane; k < cnt; k += 32) cs.items[base + k] = make_int2(g, gl[k]);
  if (cnt == 0)  // no piece within reach: the group's inter terms are exact zeros
    for (int s = slot0 + lane; s < min(slot0 + G, s_end); s += 32) {
      const int e = cs.order[s];
      cs.Eout[e] = 0.0;
      if (cs.Gout) cs.Gout[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// The cut-off sweep: persistent CTAs; a warp takes (group, piece) items of
// the broad phase's list from a work counter.  The protein's pairs of atoms
// and row tables are either staged once per CTA in shared memory with the TMA
// bulk engine (GLOB false, proteins up to about 6,500 atoms) or read from
// global memory through the read-only path (GLOB true, any size).
template <int KP, bool GRAD, int DIEL, bool GLOB>
__global__ void __launch_bounds__(cull_max_threads(KP))
    k_pairs_cull(DevCull cull, const float4* __restrict__ tabv, CullSegs seg, CullScratch cs,
                 int* err) {
  extern __shared__ __align__(16) float4 sp[];  // staged: [npairs][4], then the tables below
  __shared__ __align__(8) uint64_t bar;
  const int NP = GLOB ? 0 : cull.npairs, nrows = GLOB ? 0 : cull.nrows;
  float4* s_rbox = sp + 4 * NP;
  float4* s_tab = s_rbox + nrows;                       // [ptype][ltype] (X, 1/D, c1, 0)
  int* s_rs = reinterpret_cast<int*>(s_tab + kTabRows * kNTypes);  // first pair of each row
  int* s_flush = s_rs + nrows + 1;                      // end of the row's flush block
  int* s_list = s_flush + nrows;                        // [warps][kListCap] atoms to sweep
  if (!GLOB) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      const uint32_t bytes = (uint32_t)NP * 64u;
      mbar_expect_tx(&bar, bytes);
      constexpr uint32_t kPiece = 32768u;
      for (uint32_t off = 0; off < bytes; off += kPiece) {
        const uint32_t n = bytes - off < kPiece ? bytes - off : kPiece;
        bulk_g2s(reinterpret_cast<char*>(sp) + off,
                 reinterpret_cast<const char*>(cull.pairs) + off, n, &bar);
      }
    }
    for (int k = threadIdx.x; k < nrows; k += blockDim.x) {
      s_rbox[k] = cull.row_box[k];
      s_flush[k] = cull.row_flush[k];
    }
    for (int k = threadIdx.x; k <= nrows; k += blockDim.x) s_rs[k] = cull.pair_start[k];
  }
  stage_pair_table<DIEL>(tabv, s_tab);
  __syncthreads();
  if (!GLOB && !mbar_wait(&bar, 0, cs.first_wait_polls)) {
    // the copy did not land in time: flag it, wait once more (bounded) for the
    // copy in flight so that it does not write into a finished CTA, and stop
    if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
    mbar_wait(&bar, 0, kWaitPolls);
    return;
  }
  const float4* pr = GLOB ? cull.pairs : sp;
  const float4* rbox = GLOB ? cull.row_box : s_rbox;
  const int* rs = GLOB ? cull.pair_start : s_rs;
  const int* fl = GLOB ? cull.row_flush : s_flush;

  constexpr int G = 32 * KP;
  const int lane = threadIdx.x & 31;
  const int nitems = (int)__ldcg(cs.queue + 1);
  for (;;) {
    int item = 0;
    if (lane == 0) item = (int)atomicAdd(cs.queue, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= nitems) break;
    const int2 it = __ldcg(cs.items + item);
    const int g = it.x, pc = it.y;
    const int slot0 = g * G;
    int t = 0;
    while (t + 1 < seg.nseg && slot0 >= seg.off[t + 1]) ++t;
    const int s_end = seg.off[t] + seg.n[t];
    const float4* trow = s_tab + seg.type[t];  // + the byte offset of the protein type's row
    const int r0 = __ldg(cs.piece_row + pc), r1 = __ldg(cs.piece_row + pc + 1);
    sweep_item<KP, GRAD, DIEL, 0, true, true, GLOB>(
        pr, rbox, rs, fl, r0, r1, trow, slot0, s_end, s_list + (threadIdx.x >> 5) * kListCap, cs,
        slot0, cs.slots, pc, 0, __ldcg(cs.gcount + g), &cs.arrive[g],
        cs.glist + (size_t)g * cs.npieces);
  }
}

// ---------------------------------------------------------------------------
// ragged batch of systems
// ---------------------------------------------------------------------------
constexpr int kSysSortThreads = 512;

// One CTA per system: its entries into slot order by (ligand type segment,
// Hilbert cell of an 8^3 grid over the system's protein), counted in shared
// memory; also clears the arrival counters of the system's groups.
__global__ void __launch_bounds__(kSysSortThreads)
    k_sys_sort(DevSystems S, const float4* __restrict__ X, CullScratch cs) {
  extern __shared__ unsigned ssm[];  // [nseg * kSysCells] counts, then [n] bin | rank << 16
  const int sys = blockIdx.x;
  const SysInfo inf = S.info[sys];
  const DevLigand& lig = S.lig[sys];
  const int L = inf.L, n = inf.poses * L, nb = inf.nseg * kSysCells;
  unsigned* hist = ssm;
  unsigned* br = ssm + nb;
  const int* seg_of_atom = lig.seg_of_atom;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) hist[k] = 0u;
  for (int k = threadIdx.x; k < inf.ngroups; k += blockDim.x) cs.arrive[inf.group0 + k] = 0;
  __syncthreads();
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const float4 h = X[2 * ((size_t)inf.ent0 + e)];
    const uint32_t cx = min(max(__float2int_rd((h.x - inf.glo[0]) * inf.ginv), 0), kSysGrid - 1);
    const uint32_t cy = min(max(__float2int_rd((h.y - inf.glo[1]) * inf.ginv), 0), kSysGrid - 1);
    const uint32_t cz = min(max(__float2int_rd((h.z - inf.glo[2]) * inf.ginv), 0), kSysGrid - 1);
    const unsigned bin = (unsigned)seg_of_atom[e % L] * kSysCells + hilbert_cell<3>(cx, cy, cz);
    const unsigned rank = atomicAdd(&hist[bin], 1u);
    br[e] = bin | (rank << 16);
  }
  __syncthreads();
  // per segment: exclusive scan of its cells into slots (a warp per segment)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = w; t < inf.nseg; t += blockDim.x >> 5) {
    unsigned* hs = hist + t * kSysCells;
    constexpr int per = kSysCells / 32;
    unsigned loc[per], sum = 0;
#pragma unroll
    for (int k = 0; k < per; ++k) {
      loc[k] = hs[lane * per + k];
      sum += loc[k];
    }
    unsigned inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned v = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += v;
    }
    unsigned run = (unsigned)S.seg_slot[inf.seg0 + t] + inc - sum;
#pragma unroll
    for (int k = 0; k < per; ++k) {
      hs[lane * per + k] = run;
      run += loc[k];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const unsigned v = br[e];
    const int slot = (int)(hist[v & 0xffffu] + (v >> 16));
    const size_t ge = (size_t)inf.ent0 + e;
    const float4 h = X[2 * ge], l = X[2 * ge + 1];
    cs.Xs[2 * (size_t)slot] = make_float4(h.x, h.y, h.z, lig.q[e % L]);
    cs.Xs[2 * (size_t)slot + 1] = make_float4(l.x, l.y, l.z, 0.f);
    cs.order[slot] = (int)ge;
  }
}

// Persistent CTAs over (system, protein piece) items: the piece's atoms are
// staged into shared memory by the TMA bulk engine, then the CTA's warps sweep
// every entry group of the system against it.
template <int KP, bool GRAD, int DIEL, int FORM>
__global__ void __launch_bounds__(cull_max_threads(KP), 1)
    k_sys_pairs(DevSystems S, const float4* __restrict__ tabv, CullScratch cs, int* err) {
  extern __shared__ __align__(16) float4 sp[];  // [piece pairs][4], then the row tables
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_item, s_fail;
  const int amax = S.piece_pairs_max, rmax = S.piece_rows_max;
  float4* s_rbox = sp + 4 * amax;
  float4* s_tab = s_rbox + rmax;
  int* s_rs = reinterpret_cast<int*>(s_tab + kTabRows * kNTypes);
  int* s_flush = s_rs + rmax + 1;
  int* s_list = s_flush + rmax;
  stage_pair_table<DIEL>(tabv, s_tab);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    s_fail = 0;
  }
  __syncthreads();
  constexpr int G = 32 * KP;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (uint32_t phase = 0;; phase ^= 1u) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(cs.queue, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= S.nitems) break;
    const int2 ip = S.item[item];
    const SysInfo& inf = S.info[ip.x];
    const int4 pc = S.piece[ip.y];  // pair0, pair1, row0, row1
    const int na = pc.y - pc.x, nr = pc.w - pc.z;
    if (threadIdx.x == 0) {
      const uint32_t bytes = (uint32_t)na * 64u;
      mbar_expect_tx(&bar, bytes);
      constexpr uint32_t kPiece = 32768u;
      for (uint32_t off = 0; off < bytes; off += kPiece) {
        const uint32_t m = bytes - off < kPiece ? bytes - off : kPiece;
        bulk_g2s(reinterpret_cast<char*>(sp) + off,
                 reinterpret_cast<const char*>(S.pairs + 4 * (size_t)pc.x) + off, m, &bar);
      }
    }
    for (int k = threadIdx.x; k < nr; k += blockDim.x) {
      s_rbox[k] = S.row_box[pc.z + k];
      s_rs[k] = S.row_start[pc.z + k] - pc.x;
      s_flush[k] = S.flush_end[pc.z + k] - pc.z;
    }
    if (threadIdx.x == 0) s_rs[nr] = na;
    if (threadIdx.x == 0 && !mbar_wait(&bar, phase, cs.first_wait_polls)) {
      atomicOr(err, kErrTimeout);
      mbar_wait(&bar, phase, kWaitPolls);
      s_fail = 1;
    }
    __syncthreads();
    if (s_fail) return;
    const int kpc = ip.y - inf.piece0;
    for (int g = inf.group0 + warp; g < inf.group0 + inf.ngroups; g += nwarps) {
      const SysGroup gr = S.group[g];
      const long long gl = g - inf.group0;
      sweep_item<KP, GRAD, DIEL, FORM, FORM == 0>(
          sp, s_rbox, s_rs, s_flush, 0, nr, s_tab + gr.ltype, gr.slot0, gr.s_end,
          s_list + warp * kListCap, cs, inf.part0 + gl * inf.npieces * G, G, kpc,
          inf.vis0 + gl * inf.npieces, inf.npieces, &cs.arrive[g]);
    }
    __syncthreads();  // the piece stays until every warp is done with it
  }
}

using SysFn = void (*)(DevSystems, const float4*, CullScratch, int*);

template <int KP>
SysFn pick_sys_kp(bool grad, int diel, int form) {
  if (grad) {
    if (diel) return form ? k_sys_pairs<KP, true, 1, 1> : k_sys_pairs<KP, true, 1, 0>;
    return form ? k_sys_pairs<KP, true, 0, 1> : k_sys_pairs<KP, true, 0, 0>;
  }
  if (diel) return form ? k_sys_pairs<KP, false, 1, 1> : k_sys_pairs<KP, false, 1, 0>;
  return form ? k_sys_pairs<KP, false, 0, 1> : k_sys_pairs<KP, false, 0, 0>;
}

SysFn pick_sys(int kp, bool grad, const Physics& ph) {
  const int d = ph.dielectric ? 1 : 0, f = ph.inter_form ? 1 : 0;
  switch (kp) {
    case 1: return pick_sys_kp<1>(grad, d, f);
    case 2: return pick_sys_kp<2>(grad, d, f);
    default: return pick_sys_kp<4>(grad, d, f);
  }
}

using CullFn = void (*)(DevCull, const float4*, CullSegs, CullScratch, int*);

template <int KP, bool GLOB>
CullFn pick_kp(bool grad, int diel) {
  if (grad) return diel ? k_pairs_cull<KP, true, 1, GLOB> : k_pairs_cull<KP, true, 0, GLOB>;
  return diel ? k_pairs_cull<KP, false, 1, GLOB> : k_pairs_cull<KP, false, 0, GLOB>;
}

CullFn pick_cull(int kp, bool grad, const Physics& ph, bool glob) {
  const int d = ph.dielectric ? 1 : 0;
  switch (kp) {
    case 1: return glob ? pick_kp<1, true>(grad, d) : pick_kp<1, false>(grad, d);
    case 2: return glob ? pick_kp<2, true>(grad, d) : pick_kp<2, false>(grad, d);
    default: return glob ? pick_kp<4, true>(grad, d) : pick_kp<4, false>(grad, d);
  }
}

}  // namespace

// dynamic shared memory of the cut-off sweep: staged, the protein's pairs and
// row tables, then the pair table and the warps' lists; global, the last two
int cull_smem_bytes(int npairs, int nrows, int threads, bool glob, int kp) {
  (void)kp;
  if (glob) npairs = nrows = 0;
  const long b = 64L * npairs + 16L * nrows + 16L * kTabRows * kNTypes + 4L * (nrows + 1) +
                 4L * nrows + 4L * kListCap * (threads / 32);
  return (int)((b + 15) / 16 * 16);
}

int cull_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem_bytes,
                    bool glob) {
  CullFn fn = pick_cull(kp, grad != 0, ph, glob);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) !=
      cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem_bytes) != cudaSuccess)
    return 0;
  return nb;
}

// (the entries were binned by the rebuild, rebuild_pose)
cudaError_t launch_cull_sort(const Scratch& s, const float* lig_q, int B, int L,
                             const CullSegs& seg, const CullScratch& cs, cudaStream_t st) {
  const int n = B * L;
  if (n <= 0) return cudaSuccess;
  const int tb = 256, nb = (n + tb - 1) / tb;
  cudaError_t e = cudaFuncSetAttribute(k_cull_scan, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kScanSmem);
  if (e != cudaSuccess) return e;
  k_cull_scan<<<seg.nseg, kScanThreads, kScanSmem, st>>>(cs.hist, seg, cs.queue, cs.arrive,
                                                         seg.off[seg.nseg] / seg.G);
  k_cull_scatter<<<nb, tb, 0, st>>>(s.X, n, L, lig_q, cs.hist, cs.bin, cs.rank, cs.Xs, cs.order);
  const int ngroups = seg.off[seg.nseg] / seg.G;
  k_cull_items<<<(ngroups + 7) / 8, 256, 0, st>>>(seg, cs, ngroups);
  return cudaGetLastError();
}

cudaError_t launch_pairs_cull(const DevCull& cull, const float4* tab, const CullSegs& seg,
                              const CullScratch& cs, int flags, const Physics& ph,
                              const CullPlan& plan, int* d_err, cudaStream_t st) {
  CullFn fn = pick_cull(plan.kp, (flags & kFlagGrad) != 0, ph, plan.global != 0);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, plan.smem);
  if (e != cudaSuccess) return e;
  fn<<<plan.blocks, plan.threads, plan.smem, st>>>(cull, tab, seg, cs, d_err);
  return cudaGetLastError();
}


int sys_pairs_smem(int piece_pairs_max, int piece_rows_max, int threads) {
  const long b = 64L * piece_pairs_max + 16L * piece_rows_max + 16L * kTabRows * kNTypes +
                 4L * (piece_rows_max + 1) + 4L * piece_rows_max + 4L * kListCap * (threads / 32);
  return (int)((b + 15) / 16 * 16);
}

int sys_pairs_max_blocks(int kp, int threads, int grad, const Physics& ph, int smem) {
  SysFn fn = pick_sys(kp, grad != 0, ph);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_sys_sort(const DevSystems& S, const Scratch& s, const CullScratch& cs,
                            int smem, cudaStream_t st) {
  if (S.nsys <= 0) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_sys_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_sys_sort<<<S.nsys, kSysSortThreads, smem, st>>>(S, s.X, cs);
  return cudaGetLastError();
}

cudaError_t launch_sys_pairs(const DevSystems& S, const float4* tab, const CullScratch& cs,
                             int kp, int threads, int blocks, int smem, int flags,
                             const Physics& ph, int* d_err, cudaStream_t st) {
  if (S.nitems <= 0) return cudaSuccess;
  SysFn fn = pick_sys(kp, (flags & kFlagGrad) != 0, ph);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  fn<<<blocks, threads, smem, st>>>(S, tab, cs, d_err);
  return cudaGetLastError();
}

}  // namespace mmo

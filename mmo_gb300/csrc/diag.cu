// diag.cu -- FP32 FMA throughput probe (the denominator of the pair kernel's
// roofline fraction): independent FMA chains, no memory traffic; and the
// double-float sine and cosine (df_sincos) over an array, for its accuracy
// check; and a count of the (entry, protein atom) pairs within a distance.
#include "mmo_internal.cuh"

namespace mmo {
namespace {

constexpr int kChains = 8;
constexpr int kUnroll = 16;

__global__ void __launch_bounds__(256) k_fma_peak(float* out, int iters, float seed) {
  float a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + (float)(threadIdx.x + c);
  const float m = 0.99999f, k = 1e-6f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int c = 0; c < kChains; ++c) a[c] = fmaf(a[c], m, k);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  if (s == -1.0f) out[0] = s;  // never true; keeps the chains live
}

// out[4 i .. 4 i + 3] = sin(x_i) hi, lo, cos(x_i) hi, lo from df_sincos
__global__ void k_df_sincos(const float* x, int n, float4* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 s, c;
  df_sincos(x[i], s, c);
  out[i] = make_float4(s.x, s.y, c.x, c.y);
}

// Entries (posed ligand atoms, hi/lo) against protein atoms closer than
// sqrt(r2cut): one entry per thread, the protein through shared memory in
// tiles of 1,024 atoms; the count into *out (one atomic add per warp).
__global__ void __launch_bounds__(256) k_count_within(const float4* __restrict__ X, int n,
                                                      const float4* __restrict__ atoms, int P,
                                                      float r2cut, unsigned long long* out) {
  __shared__ float4 tile[2 * 1024];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = e < n;
  const float4 xh = live ? X[2 * (size_t)e] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 xl = live ? X[2 * (size_t)e + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
  unsigned c = 0;
  for (int t0 = 0; t0 < P; t0 += 1024) {
    const int nt = min(1024, P - t0);
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * nt; k += blockDim.x) tile[k] = atoms[2 * (size_t)t0 + k];
    __syncthreads();
    if (live)
      for (int i = 0; i < nt; ++i) {
        const float4 ph = tile[2 * i], pl = tile[2 * i + 1];
        const float dx = split_diff(xh.x, xl.x, ph.x, pl.x);
        const float dy = split_diff(xh.y, xl.y, ph.y, pl.y);
        const float dz = split_diff(xh.z, xl.z, ph.z, pl.z);
        c += fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < r2cut ? 1u : 0u;
      }
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

}  // namespace

cudaError_t launch_count_within(const float4* X, int n, const float4* atoms, int P, float r2cut,
                                unsigned long long* out, cudaStream_t st) {
  if (n <= 0 || P <= 0) return cudaSuccess;
  k_count_within<<<(n + 255) / 256, 256, 0, st>>>(X, n, atoms, P, r2cut, out);
  return cudaGetLastError();
}

cudaError_t launch_df_sincos(const float* x, int n, float4* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_df_sincos<<<(n + 255) / 256, 256, 0, st>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t launch_fma_peak(int sms, int iters, float* out, cudaStream_t st, double* flops) {
  const int blocks = sms * 8, threads = 256;
  *flops = 2.0 * kChains * kUnroll * (double)iters * blocks * threads;
  k_fma_peak<<<blocks, threads, 0, st>>>(out, iters, 1.0f);
  return cudaGetLastError();
}

}  // namespace mmo

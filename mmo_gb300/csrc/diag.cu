// diag.cu -- FP32 FMA throughput probe (the denominator of the pair kernel's
// roofline fraction): independent FMA chains, no memory traffic; and the
// double-float sine and cosine (df_sincos) over an array, for its accuracy
// check.
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

}  // namespace

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

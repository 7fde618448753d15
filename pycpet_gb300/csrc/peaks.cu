// peaks.cu -- throughput microbenchmarks for the roofline denominators.
//
// The all-pairs Coulomb sums are bound by the FP32 pipe (FP32C form), the
// FP64 pipe (FP64 form) or the MUFU reciprocal square root.  Each kernel
// below runs kChains independent dependency chains per thread on every SM so
// the pipe, not latency, limits it; the result is operations per second:
//   kind 0  FFMA (fma.rn.f32), counted as 2 flops each
//   kind 1  DFMA (fma.rn.f64), 2 flops each
//   kind 2  MUFU rsqrt (rsqrt.approx.ftz.f32), 1 op each
//   kind 3  packed FFMA2 (fma.rn.f32x2), 4 flops each
#include "common.cuh"
#include "cpetgb.h"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void ffma_kernel(float* out, float a, float b) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3f + c;
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = __fmaf_rn(v[c], a, b);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 1234.5f) out[0] = s;  // keeps the chains alive
}

__global__ void dfma_kernel(double* out, double a, double b) {
  double v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < kIters / 16; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = __fma_rn(v[c], a, b);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 1234.5) out[0] = s;
}

__global__ void mufu_kernel(float* out) {
  float v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = 1.0f + threadIdx.x * 1e-3f + c;
  for (int i = 0; i < kIters / 4; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = rsqrt_mufu(v[c]);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  if (s == 1234.5f) out[0] = s;
}

__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
  unsigned long long d;
  asm volatile("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__global__ void ffma2_kernel(float* out, float a, float b) {
  unsigned long long v[kChains];
  unsigned long long aa, bb;
  asm("mov.b64 %0, {%1, %2};" : "=l"(aa) : "f"(a), "f"(a));
  asm("mov.b64 %0, {%1, %2};" : "=l"(bb) : "f"(b), "f"(b));
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    const float x = threadIdx.x * 1e-3f + c;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v[c]) : "f"(x), "f"(x + 0.5f));
  }
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = fma2(v[c], aa, bb);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v[c]));
    s += lo + hi;
  }
  if (s == 1234.5f) out[0] = s;
}

}  // namespace
}  // namespace cpetgb

extern "C" int cpetgb_measure_peak(int kind, double* ops_per_s) {
  using namespace cpetgb;
  if (!ops_per_s || kind < 0 || kind > 3) return CPETGB_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CPETGB_ENODEV;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CPETGB_ENODEV;
  const int threads = 512, blocks = sms * 4;
  void* out = nullptr;
  if (cudaMalloc(&out, 64) != cudaSuccess) return CPETGB_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&]() {
    switch (kind) {
      case 0: ffma_kernel<<<blocks, threads>>>(static_cast<float*>(out), 0.999f, 1e-3f); break;
      case 1: dfma_kernel<<<blocks, threads>>>(static_cast<double*>(out), 0.999, 1e-3); break;
      case 2: mufu_kernel<<<blocks, threads>>>(static_cast<float*>(out)); break;
      default: ffma2_kernel<<<blocks, threads>>>(static_cast<float*>(out), 0.999f, 1e-3f); break;
    }
  };
  launch();  // warm-up
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return CPETGB_ECUDA;
  const double threads_total = double(blocks) * threads;
  double ops;
  switch (kind) {
    case 0: ops = threads_total * kIters * kChains * 2.0; break;
    case 1: ops = threads_total * (kIters / 16) * kChains * 2.0; break;
    case 2: ops = threads_total * (kIters / 4) * kChains; break;
    default: ops = threads_total * kIters * kChains * 4.0; break;
  }
  *ops_per_s = ops * reps / (ms * 1e-3);
  return CPETGB_OK;
}

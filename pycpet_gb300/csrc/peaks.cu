// peaks.cu -- throughput microbenchmarks for the roofline denominators, and
// the check of the bounded device-side waits (wait_limit_kernel).
//
// The all-pairs Coulomb sums are bound by the FP32 pipe (FP32C form), the
// FP64 pipe (FP64 form) or the MUFU reciprocal square root.  Each kernel
// below runs kChains independent dependency chains per thread on every SM so
// the pipe, not latency, limits it; the result is operations per second:
//   kind 0  FFMA (fma.rn.f32), counted as 2 flops each
//   kind 1  DFMA (fma.rn.f64), 2 flops each
//   kind 2  MUFU rsqrt (rsqrt.approx.ftz.f32), 1 op each
//   kind 3  packed FFMA2 (fma.rn.f32x2), 4 flops each
//   kind 4  the streamline sweep's inner loop alone: pair evaluations per
//           second with 8,000 charges resident in shared memory, 4 line slots
//           per warp, packed f32x2 pair terms with the MUFU rsqrt and a Kahan
//           step every 32 charge pairs (the instruction mix of topo.cu's
//           sweep, without line bookkeeping): the rate that mix can reach
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

constexpr int kSweepSlots = 4, kSweepRun = 32, kSweepPairs = 4000, kSweepThreads = 512;

__global__ void __launch_bounds__(kSweepThreads, 1) sweep_loop_kernel(const float4* __restrict__ g,
                                                                      int reps, float* out) {
  extern __shared__ ulonglong2 sweep_sm[];
  for (int i = threadIdx.x; i < 2 * kSweepPairs; i += blockDim.x)
    sweep_sm[i] = reinterpret_cast<const ulonglong2*>(g)[i];
  __syncthreads();
  const ulonglong2* A = sweep_sm;
  const ulonglong2* B = sweep_sm + kSweepPairs;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t ex2[kSweepSlots][3];
  float acc[kSweepSlots][3], cmp[kSweepSlots][3];
#pragma unroll
  for (int e = 0; e < kSweepSlots; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = 0.1f * (e + 1) + 0.01f * c + 1e-3f * warp;
      ex2[e][c] = pk2(v, v);
      acc[e][c] = cmp[e][c] = 0.f;
    }
  for (int r = 0; r < reps; ++r) {
    for (int base = 0; base < kSweepPairs; base += 32 * kSweepRun) {
      uint64_t part[kSweepSlots][3];
#pragma unroll
      for (int e = 0; e < kSweepSlots; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) part[e][c] = 0ull;
      const int cnt = min(kSweepRun, (kSweepPairs - base) >> 5);
#pragma unroll 2
      for (int i = 0; i < cnt; ++i) {
        const ulonglong2 a = A[base + lane + 32 * i], b = B[base + lane + 32 * i];
#pragma unroll
        for (int e = 0; e < kSweepSlots; ++e) {
          const uint64_t dx = sub2(ex2[e][0], a.x), dy = sub2(ex2[e][1], a.y), dz = sub2(ex2[e][2], b.x);
          const uint64_t r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
          const uint64_t ri = rsqrt2(r2);
          const uint64_t w = mul2(mul2(b.y, ri), mul2(ri, ri));
          part[e][0] = fma2(w, dx, part[e][0]);
          part[e][1] = fma2(w, dy, part[e][1]);
          part[e][2] = fma2(w, dz, part[e][2]);
        }
      }
#pragma unroll
      for (int e = 0; e < kSweepSlots; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float lo, hi;
          upk2(part[e][c], lo, hi);
          kahan_add(acc[e][c], cmp[e][c], __fadd_rn(lo, hi));
        }
    }
  }
  float s = 0.f;
#pragma unroll
  for (int e = 0; e < kSweepSlots; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) s += acc[e][c] - cmp[e][c];
  if (s == 1234.5f) out[0] = s;
}

// A bounded wait that nothing completes: the mbarrier expects one arrival
// that never comes and no copy is issued, so each thread's wait runs out
// after limit_ns, records kDevWaitTimeout and returns (the path every
// kernel's waits take when a bulk copy does not complete).
__global__ void wait_limit_kernel(int* status, unsigned long long limit_ns) {
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  mbar_wait(&bar, 0, status, limit_ns);
}

}  // namespace

cudaError_t launch_wait_limit_check(int* status, unsigned long long limit_ns, cudaStream_t s) {
  wait_limit_kernel<<<1, 32, 0, s>>>(status, limit_ns);
  return cudaGetLastError();
}

}  // namespace cpetgb

namespace {

// kind 4: pair evaluations per second of sweep_loop_kernel on every SM.
int measure_sweep_loop(int sms, double* ops_per_s) {
  using namespace cpetgb;
  const size_t bytes = size_t(2) * kSweepPairs * sizeof(float4);
  const int smem = static_cast<int>(bytes), reps = 200;
  float4* g = nullptr;
  float* out = nullptr;
  if (cudaMalloc(&g, bytes) != cudaSuccess) return CPETGB_ENOMEM;
  if (cudaMalloc(&out, 64) != cudaSuccess) {
    cudaFree(g);
    return CPETGB_ENOMEM;
  }
  // charges 3-11 A from the slots' positions, charges +-0.3: finite terms
  float4* h = new float4[2 * kSweepPairs];
  for (int i = 0; i < 2 * kSweepPairs; ++i)
    h[i] = make_float4(3.f + (i % 7), 4.f + (i % 5), 5.f + (i % 3), (i % 2) ? 0.3f : -0.2f);
  cudaError_t err = cudaMemcpy(g, h, bytes, cudaMemcpyHostToDevice);
  delete[] h;
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(sweep_loop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  float ms = 0.f;
  if (err == cudaSuccess) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    sweep_loop_kernel<<<sms, kSweepThreads, smem>>>(g, 2, out);  // warm-up
    cudaEventRecord(e0);
    sweep_loop_kernel<<<sms, kSweepThreads, smem>>>(g, reps, out);
    cudaEventRecord(e1);
    err = cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  cudaFree(g);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return CPETGB_ECUDA;
  const double warps = double(sms) * (kSweepThreads / 32);
  *ops_per_s = warps * kSweepSlots * 2.0 * kSweepPairs * reps / (ms * 1e-3);
  return CPETGB_OK;
}

}  // namespace

extern "C" int cpetgb_measure_peak(int kind, double* ops_per_s) {
  using namespace cpetgb;
  if (!ops_per_s || kind < 0 || kind > 4) return CPETGB_EINVAL;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CPETGB_ENODEV;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return CPETGB_ENODEV;
  if (kind == 4) return measure_sweep_loop(sms, ops_per_s);
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

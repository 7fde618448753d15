// common.cuh -- device helpers shared by the Coulomb kernels (sm_103a).
//
//  * 1-D bulk async copies global->shared (cp.async.bulk, the TMA's untiled
//    form) completed through an mbarrier transaction count;
//  * bounded mbarrier waits: every wait gives up after a wall-clock limit read
//    from %globaltimer, records an error code in the caller-visible status word
//    and returns false, so no kernel of this library can spin forever;
//  * MUFU reciprocal square root and error-free FP32 sums (Kahan / TwoSum).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace cpetgb {

constexpr double kCoulomb = 14.3996451;  // V*A/e (CPET/utils/math_module.c:412)

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on phase `parity`.  On timeout (limit_ns of %globaltimer)
// records kDevWaitTimeout in *status (first error wins) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status,
                                          unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 0 && globaltimer_ns() - t0 > limit_ns) {
      if (status) atomicCAS(status, kDevOk, kDevWaitTimeout);
      return false;
    }
  }
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses
// 16-byte aligned) that completes on `bar`'s transaction count.
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// MUFU reciprocal square root (approximate, flush-to-zero).
__device__ __forceinline__ float rsqrt_mufu(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Packed FP32x2 arithmetic (two IEEE binary32 lanes in one 64-bit register
// pair; sm_100+).  One instruction issues two FP32 operations, which halves the
// issue slots of the pair loops; the FP32 pipe throughput itself is unchanged.
__device__ __forceinline__ uint64_t pk2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
// MUFU rsqrt of both lanes.
__device__ __forceinline__ uint64_t rsqrt2(uint64_t v) {
  float a, b;
  upk2(v, a, b);
  return pk2(rsqrt_mufu(a), rsqrt_mufu(b));
}

// Kahan (1965) compensated accumulation of t into (s, c); the true sum is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float t) {
  const float y = __fsub_rn(t, c);
  const float u = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(u, s), y);
  s = u;
}

// Knuth's TwoSum: a + b = s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Sum of two unevaluated float pairs (hi + lo), renormalised.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float bhi, float blo) {
  float s, e;
  two_sum(hi, bhi, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, blo));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

}  // namespace cpetgb

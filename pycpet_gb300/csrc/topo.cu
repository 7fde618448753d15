// topo.cu -- persistent streamline kernel (K3).
//
// Replaces thread_operation (CPET/utils/math_module.c:523-591), run by the
// reference once per streamline in a multiprocessing.Pool
// (CPET/source/calculator.py:675-712), and the windowed PyTorch pipeline of
// compute_topo_GPU_batch_filter (CPET/source/calculator.py:793-978,
// CPET/utils/gpu.py:24-399).  Semantics kept from thread_operation:
//   * Euler step x <- x + h * E/|E| with the unsoftened Coulomb field
//     (propagate_topo, math_module.c:489-503; calc_field_base 296-333);
//   * at most n_iter steps; the loop stops at the first position strictly
//     outside the box (math_module.c:539-554) and keeps that position;
//   * two extra steps from the start point and two from the end point, the
//     curvature |v' x v''| / |v'|^3 at both ends (curve, math_module.c:108-121)
//     with v' = x1 - x0, v'' = x2 - 2 x1 + x0, averaged; distance |x_end - x0|
//     (euclidean_dist, math_module.c:99-105).
// Results are written at the line's start-order index.
//
// Organisation (one persistent grid, all SMs):
//   * a warp owns S line slots; slot s lives in lane s (FP64 position, step
//     count, cap, phase) plus a small record in shared memory (start point and
//     the points needed for the curvature);
//   * every step the 32 lanes split the frame's charges (lane-strided) and
//     evaluate the field at all active slots' positions; the per-lane partial
//     sums are reduced across the warp;
//   * a slot whose line is finished writes its result and takes the next line
//     index from a global atomic counter: lines are retired and refilled
//     without any block-wide synchronisation, so short and long lines mix.
//
// Precision forms:
//   FP32C  charges are float4 (x,y,z,q) held resident in shared memory (one
//          bulk async copy per CTA); pair terms in FP32 with the MUFU rsqrt,
//          per-lane Kahan accumulation across charge tiles and an error-free
//          (TwoSum) warp reduction; the step vector is formed in FP32 and added
//          to an FP64 position; box test, curvature and distance in FP64.
//   FP64   every operation in IEEE double; charges read from global memory
//          (L2-resident) as (x,y,z,q) doubles.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kTopoThreads = 512;
constexpr int kTopoWarps = kTopoThreads / 32;
constexpr int kLaneTile = 8;                   // charges per lane between Kahan steps
constexpr int kChargePad = 32 * kLaneTile;     // resident charge array padding
constexpr int kSlots = 4;                      // line slots per warp

enum Phase : int { kMain = 0, kStart1 = 1, kStart2 = 2, kEnd1 = 3, kEnd2 = 4 };

struct SlotRec {      // per-slot record in shared memory (owner lane only)
  double x0[3], xip[3], xipp[3], xend[3], xe1[3];
};

__device__ __forceinline__ bool outside(const double p[3], const double h[3]) {
  return p[0] < -h[0] || p[0] > h[0] || p[1] < -h[1] || p[1] > h[1] || p[2] < -h[2] ||
         p[2] > h[2];
}

__device__ __forceinline__ double curve_f64(const double a[3], const double b[3]) {
  const double c0 = a[1] * b[2] - a[2] * b[1];
  const double c1 = a[2] * b[0] - a[0] * b[2];
  const double c2 = a[0] * b[1] - a[1] * b[0];
  const double nc = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  const double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  return nc / (na * na * na);
}

// Per-lane slot state (meaningful in lanes 0..S-1 only).
struct Slot {
  int line;     // -1 = idle
  int phase;
  int steps;
  int cap;
  double pos[3];  // where the next field evaluation happens
};

__device__ void slot_load(Slot& sl, SlotRec& rec, int line, const TopoParams& p) {
  sl.line = line;
  if (line < 0) return;
  const double* s = p.starts + 3 * static_cast<int64_t>(line);
  for (int k = 0; k < 3; ++k) {
    rec.x0[k] = s[k];
    sl.pos[k] = s[k];
  }
  sl.cap = max(p.n_iter[line], 0);
  if (sl.cap > kMaxLineCap) {  // refuse rather than run for hours
    atomicCAS(p.status, kDevOk, kDevBadCap);
    sl.cap = 0;
  }
  sl.steps = 0;
  if (sl.cap > 0) {
    sl.phase = kMain;
  } else {  // no loop step: the end point is the start point
    sl.phase = kStart1;
    for (int k = 0; k < 3; ++k) rec.xend[k] = s[k];
  }
}

// Advance one slot given the new position `nx` (= pos + step vector).
// Returns true when the line has finished (result written).
__device__ bool slot_advance(Slot& sl, SlotRec& rec, const double nx[3], const TopoParams& p) {
  switch (sl.phase) {
    case kMain: {
      sl.steps += 1;
      if (sl.steps == 1)
        for (int k = 0; k < 3; ++k) rec.xip[k] = nx[k];
      if (sl.steps == 2)
        for (int k = 0; k < 3; ++k) rec.xipp[k] = nx[k];
      if (outside(nx, p.half) || sl.steps >= sl.cap) {
        for (int k = 0; k < 3; ++k) rec.xend[k] = nx[k];
        if (sl.steps >= 2) {
          sl.phase = kEnd1;
          for (int k = 0; k < 3; ++k) sl.pos[k] = rec.xend[k];
        } else {
          sl.phase = kStart2;
          for (int k = 0; k < 3; ++k) sl.pos[k] = rec.xip[k];
        }
      } else {
        for (int k = 0; k < 3; ++k) sl.pos[k] = nx[k];
      }
      return false;
    }
    case kStart1:
      for (int k = 0; k < 3; ++k) rec.xip[k] = sl.pos[k] = nx[k];
      sl.phase = kStart2;
      return false;
    case kStart2:
      for (int k = 0; k < 3; ++k) {
        rec.xipp[k] = nx[k];
        sl.pos[k] = rec.xend[k];
      }
      sl.phase = kEnd1;
      return false;
    case kEnd1:
      for (int k = 0; k < 3; ++k) rec.xe1[k] = sl.pos[k] = nx[k];
      sl.phase = kEnd2;
      return false;
    default: {  // kEnd2: nx is the second step after the end point
      double v1[3], v2[3], w1[3], w2[3], dd = 0.0;
      for (int k = 0; k < 3; ++k) {
        v1[k] = rec.xip[k] - rec.x0[k];
        v2[k] = rec.xipp[k] - 2.0 * rec.xip[k] + rec.x0[k];
        w1[k] = rec.xe1[k] - rec.xend[k];
        w2[k] = nx[k] - 2.0 * rec.xe1[k] + rec.xend[k];
        const double d = rec.x0[k] - rec.xend[k];
        dd += d * d;
      }
      const int64_t li = sl.line;
      p.result[2 * li + 0] = sqrt(dd);
      p.result[2 * li + 1] = 0.5 * (curve_f64(v1, v2) + curve_f64(w1, w2));
      if (p.ends)
        for (int k = 0; k < 3; ++k) p.ends[3 * li + k] = rec.xend[k];
      if (p.steps) p.steps[li] = sl.steps;
      return true;
    }
  }
}

// ---------------------------------------------------------------------------
// Field sweep over the charges for NA active slots.
// ---------------------------------------------------------------------------

// FP32C, charges resident in shared memory (padded to kChargePad).
template <int NA>
__device__ __forceinline__ void sweep_f32(const float4* __restrict__ sm, int n_pad, int lane,
                                          const float (&ex)[kSlots][3], float (&hi)[kSlots][3],
                                          float (&lo)[kSlots][3]) {
  float acc[NA][3], cmp[NA][3];
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[e][c] = cmp[e][c] = 0.f;

  for (int base = lane; base < n_pad; base += 32 * kLaneTile) {
    float part[NA][3];
#pragma unroll
    for (int e = 0; e < NA; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) part[e][c] = 0.f;
#pragma unroll
    for (int i = 0; i < kLaneTile; ++i) {
      const float4 ch = sm[base + 32 * i];
#pragma unroll
      for (int e = 0; e < NA; ++e) {
        // explicit roundings: a line's result does not depend on which
        // other slots share its warp
        const float dx = __fsub_rn(ex[e][0], ch.x);
        const float dy = __fsub_rn(ex[e][1], ch.y);
        const float dz = __fsub_rn(ex[e][2], ch.z);
        const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
        const float ri = rsqrt_mufu(r2);
        const float w = __fmul_rn(__fmul_rn(ch.w, ri), __fmul_rn(ri, ri));
        part[e][0] = __fmaf_rn(w, dx, part[e][0]);
        part[e][1] = __fmaf_rn(w, dy, part[e][1]);
        part[e][2] = __fmaf_rn(w, dz, part[e][2]);
      }
    }
#pragma unroll
    for (int e = 0; e < NA; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) kahan_add(acc[e][c], cmp[e][c], part[e][c]);
  }
  // Lane partial = acc - cmp as an unevaluated pair; error-free butterfly.
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float h = acc[e][c], l = -cmp[e][c];
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, off);
        const float ol = __shfl_xor_sync(0xffffffffu, l, off);
        pair_add(h, l, oh, ol);
      }
      hi[e][c] = h;
      lo[e][c] = l;
    }
}

// FP64: charges from global memory (padded with zero charges far away).
template <int NA>
__device__ __forceinline__ void sweep_f64(const Charge64* __restrict__ g, int n_pad, int lane,
                                          const double (&ex)[kSlots][3], double (&E)[kSlots][3]) {
  double acc[NA][3];
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[e][c] = 0.0;
#pragma unroll 2
  for (int j = lane; j < n_pad; j += 32) {
    const Charge64 ch = g[j];
#pragma unroll
    for (int e = 0; e < NA; ++e) {
      const double dx = __dsub_rn(ex[e][0], ch.x);
      const double dy = __dsub_rn(ex[e][1], ch.y);
      const double dz = __dsub_rn(ex[e][2], ch.z);
      const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, __dmul_rn(dz, dz)));
      const double r = sqrt(r2);
      const double w = __ddiv_rn(ch.q, __dmul_rn(r2, r));
      acc[e][0] = __fma_rn(w, dx, acc[e][0]);
      acc[e][1] = __fma_rn(w, dy, acc[e][1]);
      acc[e][2] = __fma_rn(w, dz, acc[e][2]);
    }
  }
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double v = acc[e][c];
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      E[e][c] = v;
    }
}

// ---------------------------------------------------------------------------
// Persistent kernel.
// ---------------------------------------------------------------------------
template <int PREC, bool RESIDENT>
__global__ void __launch_bounds__(kTopoThreads, 1) topo_kernel(TopoParams p, int n_pad) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  SlotRec* recs = reinterpret_cast<SlotRec*>(smem_raw);  // [kTopoWarps][kSlots]
  const size_t rec_bytes = sizeof(SlotRec) * kTopoWarps * kSlots;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + rec_bytes);
  float4* sm_ch = reinterpret_cast<float4*>(smem_raw + rec_bytes + 128);
  const float4* ch32 = RESIDENT ? sm_ch : static_cast<const float4*>(p.packed);

  if constexpr (PREC == kFP32C && RESIDENT) {
    // Resident charges: bulk async copy of the packed frame, pad by stores.
    const int n = p.n_charges;
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t total = static_cast<uint32_t>(n) * 16u;
      mbar_arrive_expect_tx(bar, total);
      const char* src = static_cast<const char*>(p.packed);
      constexpr uint32_t kChunk = 32768;
      for (uint32_t off = 0; off < total; off += kChunk)
        bulk_g2s(reinterpret_cast<char*>(sm_ch) + off, src + off, min(kChunk, total - off), bar);
    }
    for (int j = n + threadIdx.x; j < n_pad; j += blockDim.x)
      sm_ch[j] = make_float4(1.0e4f, 1.0e4f, 1.0e4f, 0.f);
    const bool mine = mbar_wait(bar, 0, p.status);
    if (!__syncthreads_and(mine)) return;
  }

  SlotRec* my_rec = recs + warp * kSlots + (lane < kSlots ? lane : 0);
  Slot sl;
  sl.line = -1;
  sl.phase = kMain;
  sl.steps = sl.cap = 0;
  sl.pos[0] = sl.pos[1] = sl.pos[2] = 0.0;
  if (lane < kSlots) {
    const int li = atomicAdd(p.queue, 1);
    slot_load(sl, *my_rec, li < p.n_lines ? li : -1, p);
  }

  for (;;) {
    const unsigned active = __ballot_sync(0xffffffffu, lane < kSlots && sl.line >= 0);
    const int na = __popc(active);
    if (na == 0) break;
    // Evaluation positions of the active slots, broadcast to all lanes.
    using Real = typename std::conditional<PREC == kFP32C, float, double>::type;
    Real ex[kSlots][3];
    int my_rank = -1;
    {
      unsigned m = active;
#pragma unroll
      for (int e = 0; e < kSlots; ++e) {
        const int src = m ? (__ffs(m) - 1) : 0;
        if (m) m &= m - 1;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ex[e][c] = static_cast<Real>(__shfl_sync(0xffffffffu, sl.pos[c], src));
        if (src == lane && e < na) my_rank = e;
      }
    }

    double E[3] = {0.0, 0.0, 0.0};
    float Ef[3] = {0.f, 0.f, 0.f};
    if constexpr (PREC == kFP32C) {
      float hi[kSlots][3], lo[kSlots][3];
      switch (na) {
        case 1: sweep_f32<1>(ch32, n_pad, lane, ex, hi, lo); break;
        case 2: sweep_f32<2>(ch32, n_pad, lane, ex, hi, lo); break;
        case 3: sweep_f32<3>(ch32, n_pad, lane, ex, hi, lo); break;
        default: sweep_f32<4>(ch32, n_pad, lane, ex, hi, lo); break;
      }
#pragma unroll
      for (int e = 0; e < kSlots; ++e)
        if (e == my_rank)
#pragma unroll
          for (int c = 0; c < 3; ++c) Ef[c] = hi[e][c];
    } else {
      double Es[kSlots][3];
      const Charge64* g = static_cast<const Charge64*>(p.packed);
      switch (na) {
        case 1: sweep_f64<1>(g, n_pad, lane, ex, Es); break;
        case 2: sweep_f64<2>(g, n_pad, lane, ex, Es); break;
        case 3: sweep_f64<3>(g, n_pad, lane, ex, Es); break;
        default: sweep_f64<4>(g, n_pad, lane, ex, Es); break;
      }
#pragma unroll
      for (int e = 0; e < kSlots; ++e)
        if (e == my_rank)
#pragma unroll
          for (int c = 0; c < 3; ++c) E[c] = Es[e][c];
    }

    if (my_rank >= 0) {
      double nx[3];
      if constexpr (PREC == kFP32C) {
        // step vector in FP32 (E scaled by k does not change the direction)
        const float n2 = Ef[0] * Ef[0] + Ef[1] * Ef[1] + Ef[2] * Ef[2];
        const float s = __fdiv_rn(static_cast<float>(p.step), __fsqrt_rn(n2));
#pragma unroll
        for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + static_cast<double>(Ef[c] * s);
      } else {
        const double n = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
#pragma unroll
        for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + p.step * E[c] / n;
      }
      if (slot_advance(sl, *my_rec, nx, p)) {
        const int li = atomicAdd(p.queue, 1);
        slot_load(sl, *my_rec, li < p.n_lines ? li : -1, p);
      }
    }
    __syncwarp();
  }
}

size_t topo_smem_bytes(bool resident, int n_pad) {
  size_t b = sizeof(SlotRec) * kTopoWarps * kSlots + 128;
  if (resident) b += static_cast<size_t>(n_pad) * 16;
  return b;
}

template <int PREC, bool RESIDENT>
cudaError_t launch_topo_t(const TopoParams& p, int n_pad, int num_sms, cudaStream_t s) {
  const size_t smem = topo_smem_bytes(RESIDENT, n_pad);
  cudaError_t err = cudaFuncSetAttribute(topo_kernel<PREC, RESIDENT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
  if (err != cudaSuccess) return err;
  int per_sm = 1;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, topo_kernel<PREC, RESIDENT>,
                                                      kTopoThreads, smem);
  if (err != cudaSuccess) return err;
  per_sm = std::max(per_sm, 1);
  const int max_useful = (p.n_lines + kTopoWarps * kSlots - 1) / (kTopoWarps * kSlots);
  const int grid = std::max(1, std::min(num_sms * per_sm, max_useful));
  topo_kernel<PREC, RESIDENT><<<grid, kTopoThreads, smem, s>>>(p, n_pad);
  return cudaGetLastError();
}

}  // namespace

int topo_charge_pad() { return kChargePad; }

size_t topo_resident_limit(int prec) {
  if (prec != kFP32C) return 0;  // FP64 charges are read from global memory (L2)
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t fixed = topo_smem_bytes(false, 0);
  if (optin <= static_cast<int>(fixed)) return 0;
  size_t n = (static_cast<size_t>(optin) - fixed) / 16;
  return (n / kChargePad) * kChargePad;
}

// p.packed must hold round_up(n_charges, kChargePad) packed charges, the tail
// being zero charges placed far from the box (written by the pack kernel).
cudaError_t launch_topo(int prec, const TopoParams& p, int num_sms, cudaStream_t s) {
  if (p.n_lines <= 0) return cudaSuccess;
  const int n_pad = ((p.n_charges + kChargePad - 1) / kChargePad) * kChargePad;
  if (prec == kFP64) return launch_topo_t<kFP64, false>(p, n_pad, num_sms, s);
  if (static_cast<size_t>(n_pad) <= topo_resident_limit(kFP32C))
    return launch_topo_t<kFP32C, true>(p, n_pad, num_sms, s);
  return launch_topo_t<kFP32C, false>(p, n_pad, num_sms, s);
}

}  // namespace cpetgb

// grid.cu -- all-pairs Coulomb sums on point sets (K1 field, K2 potential).
//
// Replaces compute_looped_field (CPET/utils/math_module.c:405-451, field with
// r^2 clamped at 1e-6), calc_field (math_module.c:255-293, unclamped field at
// a point) and calc_esp_base (math_module.c:453-486, potential), which the
// reference evaluates one point at a time on one CPU core.
//
// Work decomposition: a CTA owns one GridItem = a tile of kGridSlotPts points
// of one frame (PPT points per thread, kept in registers) and a contiguous
// range of that frame's charges.  The charges stream through a ring of shared
// memory stages filled by 1-D bulk async copies (cp.async.bulk) that complete
// on mbarriers; every thread reads each staged charge as a broadcast and
// applies it to its PPT points.
//
// Precision forms:
//   FP32C  pair terms in FP32 with the MUFU rsqrt; each stage's contribution is
//          summed plainly in FP32 and then Kahan-added (compensated) into a
//          running (sum, compensation) pair per component; the result leaves
//          the CTA as a double.
//   FP64   every operation in IEEE double (plain sums), the drop-in form.
// A frame whose charges are split over several items writes per-split partial
// sums (doubles) that grid_final_kernel adds in split order: deterministic.
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kStages = 4;

template <int PREC>
struct GridCfg;
// FP32C charge record with every component duplicated, {x,x,y,y} {z,z,q,q}:
// one broadcast 16-byte shared load yields two ready f32x2 operands, and a
// packed instruction then evaluates the pair term for two grid points.
struct alignas(32) ChargeDup {
  ulonglong2 xy;
  ulonglong2 zq;
};
template <>
struct GridCfg<kFP32C> {
  using ChargeT = ChargeDup;
  using Real = float;
  static constexpr int kTile = 256;  // charges per stage (8 KiB)
};
template <>
struct GridCfg<kFP64> {
  using ChargeT = Charge64;
  using Real = double;
  static constexpr int kTile = 256;  // charges per stage (8 KiB)
};

__device__ __forceinline__ double rsqrt_f64(double x) { return rsqrt(x); }
__device__ __forceinline__ double charge_q(const Charge64& c) { return c.q; }
// {v, v} as one packed 64-bit value.
__device__ __forceinline__ uint64_t dup2(float v) {
  const uint64_t b = __float_as_uint(v);
  return b | (b << 32);
}

__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// Kahan accumulation on both lanes of packed pairs.
__device__ __forceinline__ void kahan_add2(uint64_t& s, uint64_t& c, uint64_t t) {
  const uint64_t y = sub2(t, c);
  const uint64_t u = add2(s, y);
  c = sub2(sub2(u, s), y);
  s = u;
}

constexpr int kKahanRun = 32;  // FP32C: charges summed plainly between Kahan steps

// FP32C body: this thread's points as G packed pairs (points k = 2g, 2g+1).
template <int KIND, bool CLAMP, int G>
__device__ __forceinline__ void grid_tile_f32x2(const ChargeDup* __restrict__ tl, int cnt,
                                                const uint64_t (&px)[G], const uint64_t (&py)[G],
                                                const uint64_t (&pz)[G], uint64_t (&acc)[3][G],
                                                uint64_t (&cmp)[3][G]) {
  constexpr int NC = (KIND == kField) ? 3 : 1;
  for (int j0 = 0; j0 < cnt; j0 += kKahanRun) {
    const int j1 = min(cnt, j0 + kKahanRun);
    uint64_t part[NC][G];
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int g = 0; g < G; ++g) part[c][g] = 0ull;
#pragma unroll 4
    for (int j = j0; j < j1; ++j) {
      const ulonglong2 xy = tl[j].xy;
      const ulonglong2 zq = tl[j].zq;
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const uint64_t dx = sub2(px[g], xy.x);
        const uint64_t dy = sub2(py[g], xy.y);
        const uint64_t dz = sub2(pz[g], zq.x);
        uint64_t r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
        if constexpr (CLAMP) {  // compute_looped_field's fmaxf(r^2, 1e-6f)
          float a, b;
          upk2(r2, a, b);
          r2 = pk2(fmaxf(a, 1e-6f), fmaxf(b, 1e-6f));
        }
        const uint64_t ri = rsqrt2(r2);
        if constexpr (KIND == kField) {
          const uint64_t w = mul2(mul2(zq.y, ri), mul2(ri, ri));
          part[0][g] = fma2(w, dx, part[0][g]);
          part[1][g] = fma2(w, dy, part[1][g]);
          part[2][g] = fma2(w, dz, part[2][g]);
        } else {
          part[0][g] = fma2(zq.y, ri, part[0][g]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int g = 0; g < G; ++g) kahan_add2(acc[c][g], cmp[c][g], part[c][g]);
  }
}

template <int PREC, int KIND, bool CLAMP, int PPT>
__global__ void __launch_bounds__(kGridThreads)
    grid_kernel(const GridItem* __restrict__ items, const void* __restrict__ packed,
                const double* __restrict__ points, double* __restrict__ out,
                double* __restrict__ partial, int* __restrict__ status) {
  using Cfg = GridCfg<PREC>;
  using ChargeT = typename Cfg::ChargeT;
  using Real = typename Cfg::Real;
  constexpr int TC = Cfg::kTile;
  constexpr int NC = (KIND == kField) ? 3 : 1;

  __shared__ alignas(128) ChargeT tile[kStages][TC];
  __shared__ alignas(8) uint64_t full[kStages];

  const GridItem it = items[blockIdx.x];
  const ChargeT* src = reinterpret_cast<const ChargeT*>(packed) + it.charge_off + it.n_begin;
  const int n = it.n_count;
  const int n_tiles = (n + TC - 1) / TC;
  const int tid = threadIdx.x;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&full[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](int t) {
    const int s = t % kStages;
    const int cnt = min(TC, n - t * TC);
    const uint32_t bytes = static_cast<uint32_t>(cnt * sizeof(ChargeT));
    mbar_arrive_expect_tx(&full[s], bytes);
    bulk_g2s(&tile[s][0], src + static_cast<int64_t>(t) * TC, bytes, &full[s]);
  };
  if (tid == 0) {
    for (int t = 0; t < min(kStages, n_tiles); ++t) issue(t);
  }

  // This thread's points, in registers (FP32C: packed in pairs).
  Real px[PPT], py[PPT], pz[PPT];
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int pl = tid + k * kGridThreads;
    if (pl < it.p_count) {
      const double* pp = points + 3 * (it.point_off + it.p_begin + pl);
      px[k] = static_cast<Real>(pp[0]);
      py[k] = static_cast<Real>(pp[1]);
      pz[k] = static_cast<Real>(pp[2]);
    } else {
      px[k] = py[k] = pz[k] = static_cast<Real>(1.0e4);  // far away, never written
    }
  }
  constexpr int G = PPT / 2;
  [[maybe_unused]] uint64_t px2[G], py2[G], pz2[G], acc2[3][G], cmp2[3][G];
  if constexpr (PREC == kFP32C) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
      px2[g] = pk2(px[2 * g], px[2 * g + 1]);
      py2[g] = pk2(py[2 * g], py[2 * g + 1]);
      pz2[g] = pk2(pz[2 * g], pz[2 * g + 1]);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc2[c][g] = cmp2[c][g] = 0ull;
    }
  }

  // FP64 running sums.
  Real acc[NC][PPT];
#pragma unroll
  for (int c = 0; c < NC; ++c)
#pragma unroll
    for (int k = 0; k < PPT; ++k) acc[c][k] = Real(0);

  bool ok = true;
  for (int t = 0; t < n_tiles; ++t) {
    const int s = t % kStages;
    const bool mine = mbar_wait(&full[s], static_cast<uint32_t>((t / kStages) & 1), status);
    ok = __syncthreads_and(mine) != 0;  // also: every thread is done with tile t-1
    if (!ok) break;
    if (tid == 0 && t >= 1 && (t - 1) + kStages < n_tiles) issue((t - 1) + kStages);

    const int cnt = min(TC, n - t * TC);
    const ChargeT* tl = &tile[s][0];
    if constexpr (PREC == kFP32C) {
      grid_tile_f32x2<KIND, CLAMP, G>(tl, cnt, px2, py2, pz2, acc2, cmp2);
    } else {
      Real part[NC][PPT];
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int k = 0; k < PPT; ++k) part[c][k] = Real(0);
#pragma unroll 4
      for (int j = 0; j < cnt; ++j) {
        const ChargeT ch = tl[j];
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          const Real dx = px[k] - ch.x;
          const Real dy = py[k] - ch.y;
          const Real dz = pz[k] - ch.z;
          Real r2 = dx * dx + dy * dy + dz * dz;
          if constexpr (CLAMP) r2 = fmax(r2, Real(1e-6));  // compute_looped_field's fmaxf
          const Real ri = rsqrt_f64(r2);
          if constexpr (KIND == kField) {
            const Real w = (charge_q(ch) * ri) * (ri * ri);
            part[0][k] += w * dx;
            part[1][k] += w * dy;
            part[2][k] += w * dz;
          } else {
            part[0][k] += charge_q(ch) * ri;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int k = 0; k < PPT; ++k) acc[c][k] += part[c][k];
    }
  }
  if (!ok) return;

#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int pl = tid + k * kGridThreads;
    if (pl >= it.p_count) continue;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double v;
      if constexpr (PREC == kFP32C) {
        float sl, sh, cl, ch;
        upk2(acc2[c][k / 2], sl, sh);
        upk2(cmp2[c][k / 2], cl, ch);
        const float sv = (k & 1) ? sh : sl, cv = (k & 1) ? ch : cl;
        v = (static_cast<double>(sv) - static_cast<double>(cv)) * kCoulomb;
      } else {
        v = static_cast<double>(acc[c][k]) * kCoulomb;
      }
      if (it.slot < 0) {
        out[NC * (it.point_off + it.p_begin + pl) + c] = v;
      } else {
        partial[(static_cast<int64_t>(it.slot) * kGridSlotPts + pl) * 3 + c] = v;
      }
    }
  }
}

template <int KIND>
__global__ void grid_final_kernel(const GridFinal* __restrict__ fin,
                                  const double* __restrict__ partial, double* __restrict__ out) {
  constexpr int NC = (KIND == kField) ? 3 : 1;
  const GridFinal f = fin[blockIdx.x];
  for (int i = threadIdx.x; i < f.p_count * NC; i += blockDim.x) {
    const int pl = i / NC, c = i % NC;
    double v = 0.0;
    for (int s = 0; s < f.n_split; ++s)
      v += partial[(static_cast<int64_t>(f.slot_base + s) * kGridSlotPts + pl) * 3 + c];
    out[NC * (f.out_row + pl) + c] = v;
  }
}

__global__ void pack_dup_f32_kernel(int64_t n, int64_t n_pad, const double* __restrict__ x,
                                    const double* __restrict__ q, ChargeDup* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v[4] = {1.0e4f, 1.0e4f, 1.0e4f, 0.f};  // zero charge far outside any box
    if (i < n) {
      v[0] = static_cast<float>(x[3 * i]);
      v[1] = static_cast<float>(x[3 * i + 1]);
      v[2] = static_cast<float>(x[3 * i + 2]);
      v[3] = static_cast<float>(q[i]);
    }
    ChargeDup c;
    c.xy = make_ulonglong2(dup2(v[0]), dup2(v[1]));
    c.zq = make_ulonglong2(dup2(v[2]), dup2(v[3]));
    out[i] = c;
  }
}

__global__ void pack_f64_kernel(int64_t n, int64_t n_pad, const double* __restrict__ x,
                                const double* __restrict__ q, Charge64* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    Charge64 c;
    if (i < n) {
      c.x = x[3 * i];
      c.y = x[3 * i + 1];
      c.z = x[3 * i + 2];
      c.q = q[i];
    } else {
      c.x = c.y = c.z = 1.0e4;
      c.q = 0.0;
    }
    out[i] = c;
  }
}

template <int PREC, int KIND, int PPT>
cudaError_t launch_grid_t(int clamp, int n_items, const GridItem* items, const void* packed,
                          const double* points, double* out, double* partial, int* status,
                          cudaStream_t s) {
  // same carveout as the streamline engine, so both fit on one SM
  cudaFuncSetAttribute(grid_kernel<PREC, KIND, true, PPT>,
                       cudaFuncAttributePreferredSharedMemoryCarveout,
                       cudaSharedmemCarveoutMaxShared);
  cudaFuncSetAttribute(grid_kernel<PREC, KIND, false, PPT>,
                       cudaFuncAttributePreferredSharedMemoryCarveout,
                       cudaSharedmemCarveoutMaxShared);
  if (clamp)
    grid_kernel<PREC, KIND, true, PPT>
        <<<n_items, kGridThreads, 0, s>>>(items, packed, points, out, partial, status);
  else
    grid_kernel<PREC, KIND, false, PPT>
        <<<n_items, kGridThreads, 0, s>>>(items, packed, points, out, partial, status);
  return cudaGetLastError();
}

template <int PREC, int KIND>
cudaError_t launch_grid_p(int clamp, int ppt, int n_items, const GridItem* items,
                          const void* packed, const double* points, double* out, double* partial,
                          int* status, cudaStream_t s) {
  return ppt == 8 ? launch_grid_t<PREC, KIND, 8>(clamp, n_items, items, packed, points, out,
                                                 partial, status, s)
                  : launch_grid_t<PREC, KIND, 4>(clamp, n_items, items, packed, points, out,
                                                 partial, status, s);
}

template <int PREC, int KIND, int PPT>
cudaError_t preload_t(int clamp) {
  cudaFuncAttributes a;
  return clamp ? cudaFuncGetAttributes(&a, grid_kernel<PREC, KIND, true, PPT>)
               : cudaFuncGetAttributes(&a, grid_kernel<PREC, KIND, false, PPT>);
}

}  // namespace

cudaError_t launch_pack_charges(int prec, int64_t n, int64_t n_pad, const double* x,
                                const double* q, void* packed, cudaStream_t s) {
  if (n_pad <= 0) return cudaSuccess;
  const int blocks = static_cast<int>(std::min<int64_t>((n_pad + 255) / 256, 4096));
  if (prec == kFP32C)
    pack_dup_f32_kernel<<<blocks, 256, 0, s>>>(n, n_pad, x, q, static_cast<ChargeDup*>(packed));
  else
    pack_f64_kernel<<<blocks, 256, 0, s>>>(n, n_pad, x, q, static_cast<Charge64*>(packed));
  return cudaGetLastError();
}

cudaError_t launch_grid(int prec, int kind, int clamp, int ppt, int n_items, const GridItem* items,
                        const void* packed, const double* points, double* out, double* partial,
                        int* status, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  if (prec == kFP32C) {
    return kind == kField ? launch_grid_p<kFP32C, kField>(clamp, ppt, n_items, items, packed, points,
                                                         out, partial, status, s)
                          : launch_grid_p<kFP32C, kEsp>(0, ppt, n_items, items, packed, points, out,
                                                       partial, status, s);
  }
  return kind == kField ? launch_grid_p<kFP64, kField>(clamp, ppt, n_items, items, packed, points,
                                                      out, partial, status, s)
                        : launch_grid_p<kFP64, kEsp>(0, ppt, n_items, items, packed, points, out,
                                                    partial, status, s);
}

cudaError_t preload_grid_kernels(int prec, int kind, int clamp, int ppt) {
  cudaError_t e;
  if (prec == kFP32C) {
    if (kind == kField)
      e = ppt == 8 ? preload_t<kFP32C, kField, 8>(clamp) : preload_t<kFP32C, kField, 4>(clamp);
    else
      e = ppt == 8 ? preload_t<kFP32C, kEsp, 8>(0) : preload_t<kFP32C, kEsp, 4>(0);
  } else {
    if (kind == kField)
      e = ppt == 8 ? preload_t<kFP64, kField, 8>(clamp) : preload_t<kFP64, kField, 4>(clamp);
    else
      e = ppt == 8 ? preload_t<kFP64, kEsp, 8>(0) : preload_t<kFP64, kEsp, 4>(0);
  }
  if (e != cudaSuccess) return e;
  cudaFuncAttributes a;
  e = kind == kField ? cudaFuncGetAttributes(&a, grid_final_kernel<kField>)
                     : cudaFuncGetAttributes(&a, grid_final_kernel<kEsp>);
  if (e != cudaSuccess) return e;
  return prec == kFP32C ? cudaFuncGetAttributes(&a, pack_dup_f32_kernel)
                        : cudaFuncGetAttributes(&a, pack_f64_kernel);
}

cudaError_t launch_grid_final(int kind, int n_final, const GridFinal* fin, const double* partial,
                              double* out, cudaStream_t s) {
  if (n_final <= 0) return cudaSuccess;
  if (kind == kField)
    grid_final_kernel<kField><<<n_final, 256, 0, s>>>(fin, partial, out);
  else
    grid_final_kernel<kEsp><<<n_final, 256, 0, s>>>(fin, partial, out);
  return cudaGetLastError();
}

}  // namespace cpetgb

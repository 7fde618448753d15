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
//
// The r^2 >= 1e-6 clamp of compute_looped_field only changes a pair term when
// a point lies within 1e-3 A of a charge.  A CTA takes the bounding box of its
// points once, tests each staged tile of charges against it (distance below
// kNearA) and runs the clamped loop only for tiles that hold such a charge;
// every other tile runs the unclamped loop, which gives the same values there.
//
// FP32C field refinement: where the field nearly cancels, FP32 rounding of the
// pair terms (about 1e-7 of each term) is a large fraction of |E|.  After the
// FP32C pass, grid_mag_hist_kernel and grid_flag_kernel find, per frame, the
// points whose |E| is below tau times the frame's median |E| (taken from a
// histogram of |E|^2) and grid_refine_kernel recomputes those
// points over all of the frame's charges in double-float arithmetic (pairs of
// floats, about 48 significant bits, on the FP32 pipe: GB300's FP64 pipe is
// 1/64 of its FP32 pipe).
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

// A staged charge closer than kNearA to the CTA's point box sends its tile
// through the clamped loop.  The clamp acts below 1e-3 A; the margin covers the
// FP32 rounding of coordinates up to 1e4 A.
constexpr float kNearA = 0.01f;

__device__ __forceinline__ void charge_xyz(const ChargeDup& c, float& x, float& y, float& z) {
  x = __uint_as_float(static_cast<uint32_t>(c.xy.x));
  y = __uint_as_float(static_cast<uint32_t>(c.xy.y));
  z = __uint_as_float(static_cast<uint32_t>(c.zq.x));
}
__device__ __forceinline__ void charge_xyz(const Charge64& c, float& x, float& y, float& z) {
  x = static_cast<float>(c.x);
  y = static_cast<float>(c.y);
  z = static_cast<float>(c.z);
}
// Squared distance from (x, y, z) to the box [lo, hi] (0 inside).
__device__ __forceinline__ float box_dist2(const float (&lo)[3], const float (&hi)[3], float x,
                                           float y, float z) {
  const float dx = fmaxf(fmaxf(lo[0] - x, x - hi[0]), 0.f);
  const float dy = fmaxf(fmaxf(lo[1] - y, y - hi[1]), 0.f);
  const float dz = fmaxf(fmaxf(lo[2] - z, z - hi[2]), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// One charge against this thread's G packed point pairs, added to part[].
template <int KIND, bool CLAMP, int G>
__device__ __forceinline__ void pair_terms_f32x2(const ChargeDup& ch, const uint64_t (&px)[G],
                                                 const uint64_t (&py)[G], const uint64_t (&pz)[G],
                                                 uint64_t (&part)[(KIND == kField) ? 3 : 1][G]) {
  const ulonglong2 xy = ch.xy;
  const ulonglong2 zq = ch.zq;
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

// FP32C body: this thread's points as G packed pairs (points k = 2g, 2g+1).
// CLAMP = true is the rare path (a staged charge next to the point box): the
// same arithmetic with the clamp, in a loop that is not unrolled, so it adds
// few registers to the kernel.
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
    if constexpr (CLAMP) {
#pragma unroll 1
      for (int j = j0; j < j1; ++j) pair_terms_f32x2<KIND, true, G>(tl[j], px, py, pz, part);
    } else {
#pragma unroll 4
      for (int j = j0; j < j1; ++j) pair_terms_f32x2<KIND, false, G>(tl[j], px, py, pz, part);
    }
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int g = 0; g < G; ++g) kahan_add2(acc[c][g], cmp[c][g], part[c][g]);
  }
}

// FP32C with 4 points per thread: at most 80 registers, so six CTAs (24
// warps) share an SM.
template <int PREC, int KIND, bool CLAMP, int PPT>
__global__ void __launch_bounds__(kGridThreads, PREC == kFP32C && PPT == 4 ? 6 : 0)
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

  // Bounding box of this CTA's points (clamped kernels only), kept in shared
  // memory so it holds no registers during the pair loops.
  __shared__ float box_s[6];
  if constexpr (CLAMP) {
    __shared__ float box_part[kGridThreads / 32][6];
    float v[6] = {3.0e38f, 3.0e38f, 3.0e38f, -3.0e38f, -3.0e38f, -3.0e38f};
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
      if (tid + k * kGridThreads < it.p_count) {
        const float c3[3] = {static_cast<float>(px[k]), static_cast<float>(py[k]),
                             static_cast<float>(pz[k])};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          v[a] = fminf(v[a], c3[a]);
          v[3 + a] = fmaxf(v[3 + a], c3[a]);
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        v[a] = fminf(v[a], __shfl_xor_sync(0xffffffffu, v[a], o));
        v[3 + a] = fmaxf(v[3 + a], __shfl_xor_sync(0xffffffffu, v[3 + a], o));
      }
    if ((tid & 31) == 0)
#pragma unroll
      for (int a = 0; a < 6; ++a) box_part[tid >> 5][a] = v[a];
    __syncthreads();
    if (tid < 6) {
      float b = box_part[0][tid];
#pragma unroll
      for (int w = 1; w < kGridThreads / 32; ++w)
        b = tid < 3 ? fminf(b, box_part[w][tid]) : fmaxf(b, box_part[w][tid]);
      box_s[tid] = b;
    }
    __syncthreads();
  }

  bool ok = true;
  for (int t = 0; t < n_tiles; ++t) {
    const int s = t % kStages;
    const bool mine = mbar_wait(&full[s], static_cast<uint32_t>((t / kStages) & 1), status);
    const int cnt = min(TC, n - t * TC);
    const ChargeT* tl = &tile[s][0];
    bool clamp_tile = false;
    if constexpr (CLAMP) {
      // Does this tile hold a charge next to the point box?  One barrier both
      // answers that and confirms every thread's wait (the common case).
      bool near = false;
      if (mine) {
        const float blo[3] = {box_s[0], box_s[1], box_s[2]};
        const float bhi[3] = {box_s[3], box_s[4], box_s[5]};
        for (int j = tid; j < cnt; j += kGridThreads) {
          float cx, cy, cz;
          charge_xyz(tl[j], cx, cy, cz);
          near |= box_dist2(blo, bhi, cx, cy, cz) < kNearA * kNearA;
        }
      }
      const int clean = __syncthreads_count(mine && !near);  // also: tile t-1 is done
      if (clean != kGridThreads) {
        ok = __syncthreads_and(mine) != 0;
        clamp_tile = true;
      }
    } else {
      ok = __syncthreads_and(mine) != 0;  // also: every thread is done with tile t-1
    }
    if (!ok) break;
    if (tid == 0 && t >= 1 && (t - 1) + kStages < n_tiles) issue((t - 1) + kStages);

    if constexpr (PREC == kFP32C) {
      if (CLAMP && clamp_tile)
        grid_tile_f32x2<KIND, true, G>(tl, cnt, px2, py2, pz2, acc2, cmp2);
      else
        grid_tile_f32x2<KIND, false, G>(tl, cnt, px2, py2, pz2, acc2, cmp2);
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
          if (CLAMP && clamp_tile) r2 = fmax(r2, Real(1e-6));  // compute_looped_field's fmaxf
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

// ---------------------------------------------------------------------------
// FP32C field refinement (see the header comment).
// ---------------------------------------------------------------------------
constexpr int kFlagThreads = 512;
constexpr int kFlagChunk = kFlagThreads * 8;  // points of a frame per flagging CTA
constexpr int kMagBins = 4096;  // bits 30..19 of the float |E|^2: exponent + 4 mantissa bits
constexpr int kBinsPerThread = kMagBins / kFlagThreads;
// 256 threads: the refinement CTAs must fit beside a serving engine launch
// that holds half of every SM's registers (engine.cu), as the grid CTAs do.
constexpr int kRefineThreads = 256;

// Integer-only reads of doubles.  GB300's FP64 pipe is 1/64 of its FP32 pipe
// and conversions from double run on it, so the refinement's helpers take a
// double apart with integer operations.
//   dbl_hi_float: sign, exponent and the leading 24 significand bits (the rest
//                 truncated); beyond the float range +-inf, below its normal
//                 range +-0; NaN stays NaN.
//   dbl_lo_float: the remaining 29 significand bits, v - dbl_hi_float(v),
//                 rounded to a float (|error| <= 2^-48 |v|); 0 where the high
//                 part is not a normal float, and flushed to 0 where it would
//                 be subnormal (|v| below about 1e-30: an absolute error
//                 under 1e-37).
__device__ __forceinline__ float dbl_hi_float(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const uint32_t sign = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  const int ex = static_cast<int>((b >> 52) & 0x7ff);
  const uint32_t mant = static_cast<uint32_t>((b >> 29) & 0x7fffffu);
  if (ex == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (mant ? 0x400000u : 0u));
  const int e = ex - 1023 + 127;
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  if (e <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | (static_cast<uint32_t>(e) << 23) | mant);
}
__device__ __forceinline__ float dbl_lo_float(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const uint32_t sign = static_cast<uint32_t>(b >> 32) & 0x80000000u;
  const int ex = static_cast<int>((b >> 52) & 0x7ff);
  const uint32_t r = static_cast<uint32_t>(b & 0x1fffffffull);  // 29 bits, weight 2^(ex - 1075)
  const int e_hi = ex - 1023 + 127;
  if (r == 0 || e_hi <= 0 || e_hi >= 255) return 0.f;
  const int t = 31 - __clz(static_cast<int>(r));  // top set bit, 0..28
  uint32_t m;
  int fe = ex - 1075 + t + 127;                   // float exponent of r's top bit
  if (t > 23) {                                   // round the low t - 23 bits, half up
    const int sh = t - 23;
    m = (r >> sh) + ((r >> (sh - 1)) & 1u);
    if (m == (1u << 24)) {
      m >>= 1;
      ++fe;
    }
  } else {
    m = r << (23 - t);
  }
  if (fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | (static_cast<uint32_t>(fe) << 23) | (m & 0x7fffffu));
}

// |E|^2 of one output row in FP32 from the truncated components (integer
// conversion, three FP32 operations): the key of the magnitude histogram.
__device__ __forceinline__ float field_norm2(const double* e) {
  const float x = dbl_hi_float(e[0]), y = dbl_hi_float(e[1]), z = dbl_hi_float(e[2]);
  return __fmaf_rn(x, x, __fmaf_rn(y, y, __fmul_rn(z, z)));
}

// Histogram of |E|^2 over the frames' points in 1/16-octave bins (of |E|^2;
// 1/32 octave of |E|): grid (frame, chunk of kFlagChunk points); each CTA
// counts its chunk in shared memory and adds its non-empty bins to the frame's
// row of hist[n_frames][kMagBins] (zeroed by the caller).
__global__ void __launch_bounds__(kFlagThreads)
    grid_mag_hist_kernel(const int64_t* __restrict__ desc, const double* __restrict__ out,
                         int* __restrict__ hist) {
  __shared__ int h[kMagBins];
  const int64_t po = desc[4 * blockIdx.x + 2], P = desc[4 * blockIdx.x + 3];
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * kFlagChunk;
  if (i0 >= P) return;
  const int64_t i1 = min(P, i0 + kFlagChunk);
  for (int b = threadIdx.x; b < kMagBins; b += kFlagThreads) h[b] = 0;
  __syncthreads();
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kFlagThreads) {
    const float m2 = field_norm2(out + 3 * (po + i));
    if (m2 <= 3.0e38f)  // finite (NaN compares false)
      atomicAdd(&h[__float_as_uint(m2) >> 19], 1);
  }
  __syncthreads();
  int* row = hist + static_cast<int64_t>(blockIdx.x) * kMagBins;
  for (int b = threadIdx.x; b < kMagBins; b += kFlagThreads)
    if (h[b]) atomicAdd(&row[b], h[b]);
}

// Grid (frame, chunk) as grid_mag_hist_kernel.  Every CTA finds its frame's
// scale -- the lower edge of the histogram bin holding the lower median of
// |E|^2 -- and appends each point of its chunk with |E|^2 below tau^2 times
// that scale to list[] as {output row, frame}.  The counts are exact
// integers, so the threshold and the set of points are deterministic.
__global__ void __launch_bounds__(kFlagThreads)
    grid_flag_kernel(const int64_t* __restrict__ desc, const double* __restrict__ out,
                     const int* __restrict__ hist, float tau2, int64_t* __restrict__ list,
                     int* __restrict__ count) {
  __shared__ int hs[kMagBins];
  __shared__ int part[kFlagThreads];
  __shared__ float scale_s;
  const int64_t po = desc[4 * blockIdx.x + 2], P = desc[4 * blockIdx.x + 3];
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * kFlagChunk;
  if (i0 >= P) return;
  const int64_t i1 = min(P, i0 + kFlagChunk);
  const int* row = hist + static_cast<int64_t>(blockIdx.x) * kMagBins;
  int own = 0;
#pragma unroll
  for (int k = 0; k < kBinsPerThread; ++k) {
    const int v = row[threadIdx.x * kBinsPerThread + k];
    hs[threadIdx.x * kBinsPerThread + k] = v;
    own += v;
  }
  part[threadIdx.x] = own;
  __syncthreads();
  if (threadIdx.x < 32) {
    constexpr int kPerLane = kFlagThreads / 32;
    const int lane = threadIdx.x;
    int mine = 0;
#pragma unroll
    for (int k = 0; k < kPerLane; ++k) mine += part[lane * kPerLane + k];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) {
      if (lane == 0) scale_s = 0.f;  // no finite value: nothing to refine
    } else {
      const int rank = (total - 1) / 2;
      const unsigned passed = __ballot_sync(0xffffffffu, incl > rank);
      if (lane == __ffs(passed) - 1) {
        int cum = incl - mine, t = lane * kPerLane;
        while (cum + part[t] <= rank) cum += part[t++];
        int b = t * kBinsPerThread;
        while (cum + hs[b] <= rank) cum += hs[b++];
        scale_s = __uint_as_float(static_cast<uint32_t>(b) << 19);
      }
    }
  }
  __syncthreads();
  // This CTA's points below the threshold, in thread order (point i0 + t +
  // kFlagThreads * k belongs to thread t), appended as one contiguous block.
  const float thr = __fmul_rn(tau2, scale_s);
  constexpr int kPer = kFlagChunk / kFlagThreads;
  unsigned mask = 0;
  int mine = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const int64_t i = i0 + threadIdx.x + int64_t(k) * kFlagThreads;
    if (i < i1 && field_norm2(out + 3 * (po + i)) < thr) {
      mask |= 1u << k;
      ++mine;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) part[warp] = incl;  // part[] is free again: the scale is known
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int w = 0; w < kFlagThreads / 32; ++w) {
      const int c = part[w];
      part[w] = run;
      run += c;
    }
    part[kFlagThreads / 32] = run ? atomicAdd(count, run) : 0;
  }
  __syncthreads();
  int k_out = part[kFlagThreads / 32] + part[warp] + incl - mine;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    if (mask & (1u << k)) {
      list[2 * k_out] = po + i0 + threadIdx.x + int64_t(k) * kFlagThreads;
      list[2 * k_out + 1] = blockIdx.x;
      ++k_out;
    }
  }
}

// Double-float ("float-float") arithmetic: a value is an unevaluated sum
// h + l of two floats with |l| <= ulp(h)/2, about 48 significant bits, built
// from the error-free transformations TwoSum (Knuth) and TwoProduct by FMA
// (Dekker / Kahan; see Muller et al., Handbook of Floating-Point Arithmetic,
// ch. 4 and 14).  Every operation below is written with explicit roundings
// (__fadd_rn, __fmul_rn, __fmaf_rn) so the compiler cannot contract or
// reorder the error terms.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// 1e-6 as a double-float pair: the float nearest to it and the float nearest
// to the rest (1e-6 - 9.99999997e-7 = 2.5e-15).
constexpr float kClampH = 1e-6f;
constexpr float kClampL = static_cast<float>(1e-6 - static_cast<double>(1e-6f));

// The field term of one charge at one point in double-float, added to
// (sh[k], sl[k]).  Point (ph, pl), charge coordinates (ch, cl) and charge
// (qh, ql) as float pairs.  Relative error of the term about 1e-13.
template <bool CLAMP>
__device__ __forceinline__ void df_field_term(const float (&ph)[3], const float (&pl)[3],
                                              const float4& chq, const float4& clq,
                                              float (&sh)[3], float (&sl)[3]) {
  const float ch[3] = {chq.x, chq.y, chq.z}, cl[3] = {clq.x, clq.y, clq.z};
  float dh[3], dl[3], sq[3], sqe[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float e;
    two_sum(ph[k], -ch[k], dh[k], e);                      // dh + e = ph - ch exactly
    dl[k] = __fadd_rn(e, __fsub_rn(pl[k], cl[k]));
    {  // renormalise: ph - ch may be exact (e = 0) while pl - cl is not small against it
      const float h = __fadd_rn(dh[k], dl[k]);
      dl[k] = __fsub_rn(dl[k], __fsub_rn(h, dh[k]));
      dh[k] = h;
    }
    two_prod(dh[k], dh[k], sq[k], sqe[k]);                 // dh^2 exactly
    sqe[k] = __fmaf_rn(__fadd_rn(dh[k], dh[k]), dl[k], sqe[k]);  // + 2 dh dl
  }
  float t1, e1, r2h, e2;
  two_sum(sq[0], sq[1], t1, e1);
  two_sum(t1, sq[2], r2h, e2);
  float r2l = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fadd_rn(sqe[0], sqe[1]), sqe[2]));
  {  // renormalise (|r2h| >= |r2l|)
    const float h = __fadd_rn(r2h, r2l);
    r2l = __fsub_rn(r2l, __fsub_rn(h, r2h));
    r2h = h;
  }
  // compute_looped_field's r^2 >= 1e-6, compared as double-float values
  // (lexicographically: both pairs are normalised), FP32 operations only.
  if (CLAMP && (r2h < kClampH || (r2h == kClampH && r2l < kClampL))) {
    r2h = kClampH;
    r2l = kClampL;
  }
  // r^-1: MUFU seed refined by one Newton step with the residual in double-float
  const float y0 = rsqrt_mufu(r2h);
  float a, ae, b, be;
  two_prod(y0, y0, a, ae);                                  // a + ae = y0^2
  two_prod(r2h, a, b, be);                                  // b + be = r2h a
  const float t = __fadd_rn(__fsub_rn(b, 1.0f), __fmaf_rn(r2h, ae, __fmaf_rn(r2l, a, be)));
  const float yl = __fmul_rn(__fmul_rn(-0.5f, y0), t);     // y = y0 + yl
  // y^3 = (a + (ae + 2 y0 yl)) (y0 + yl)
  const float y2l = __fmaf_rn(__fadd_rn(y0, y0), yl, ae);
  float y3h, e3;
  two_prod(a, y0, y3h, e3);
  const float y3l = __fmaf_rn(a, yl, __fmaf_rn(y2l, y0, e3));
  // w = q y^3
  float wh, e4;
  two_prod(chq.w, y3h, wh, e4);
  const float wl = __fmaf_rn(chq.w, y3l, __fmaf_rn(clq.w, y3h, e4));
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float p, pe, s, se;
    two_prod(wh, dh[k], p, pe);
    const float plo = __fmaf_rn(wh, dl[k], __fmaf_rn(wl, dh[k], pe));
    two_sum(sh[k], p, s, se);
    sh[k] = s;
    sl[k] = __fadd_rn(sl[k], __fadd_rn(se, plo));
  }
}

// Sum of two double-float values (h, l), renormalised.
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  float s, e;
  two_sum(h, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(l, bl));
  h = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(h, s));
}

// Recomputes the listed points in double-float arithmetic: one CTA per point
// at a time, the frame's charges (double-float records, pack_df_kernel) split
// over the threads.  Each thread keeps two independent sums (its even and odd
// charges), so two dependent double-float chains are in flight; the two are
// added at the end and the threads' sums combined by a fixed tree.
template <bool CLAMP>
__global__ void __launch_bounds__(kRefineThreads)
    grid_refine_kernel(const int64_t* __restrict__ desc, const int64_t* __restrict__ list,
                       const int* __restrict__ count, const double* __restrict__ points,
                       const float4* __restrict__ dfq, double* __restrict__ out) {
  __shared__ float red[kRefineThreads / 32][6];
  const int n_list = *count;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int e = blockIdx.x; e < n_list; e += gridDim.x) {
    const int64_t row = list[2 * e];
    const int64_t f = list[2 * e + 1];
    const int64_t co = desc[4 * f], n = desc[4 * f + 1];
    float ph[3], pl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      ph[k] = dbl_hi_float(points[3 * row + k]);
      pl[k] = dbl_lo_float(points[3 * row + k]);
    }
    float sh[3] = {0.f, 0.f, 0.f}, sl[3] = {0.f, 0.f, 0.f};
    float th[3] = {0.f, 0.f, 0.f}, tl[3] = {0.f, 0.f, 0.f};
    int64_t j = threadIdx.x;
    for (; j + kRefineThreads < n; j += 2 * kRefineThreads) {
      const float4 hi0 = dfq[2 * (co + j)], lo0 = dfq[2 * (co + j) + 1];
      const float4 hi1 = dfq[2 * (co + j + kRefineThreads)], lo1 = dfq[2 * (co + j + kRefineThreads) + 1];
      df_field_term<CLAMP>(ph, pl, hi0, lo0, sh, sl);
      df_field_term<CLAMP>(ph, pl, hi1, lo1, th, tl);
    }
    if (j < n) {
      const float4 hi0 = dfq[2 * (co + j)], lo0 = dfq[2 * (co + j) + 1];
      df_field_term<CLAMP>(ph, pl, hi0, lo0, sh, sl);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) df_add(sh[k], sl[k], th[k], tl[k]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float bh = __shfl_xor_sync(0xffffffffu, sh[k], o);
        const float bl = __shfl_xor_sync(0xffffffffu, sl[k], o);
        df_add(sh[k], sl[k], bh, bl);
      }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        red[warp][2 * k] = sh[k];
        red[warp][2 * k + 1] = sl[k];
      }
    __syncthreads();
    if (threadIdx.x < 3) {
      const int k = threadIdx.x;
      float h = red[0][2 * k], l = red[0][2 * k + 1];
#pragma unroll
      for (int w = 1; w < kRefineThreads / 32; ++w) df_add(h, l, red[w][2 * k], red[w][2 * k + 1]);
      out[3 * row + k] = (static_cast<double>(h) + static_cast<double>(l)) * kCoulomb;
    }
    __syncthreads();
  }
}

// Charges as double-float records {xh, yh, zh, qh} {xl, yl, zl, ql}.
__global__ void pack_df_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ q,
                               float4* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v[4] = {x[3 * i], x[3 * i + 1], x[3 * i + 2], q[i]};
    out[2 * i] = make_float4(dbl_hi_float(v[0]), dbl_hi_float(v[1]), dbl_hi_float(v[2]),
                             dbl_hi_float(v[3]));
    out[2 * i + 1] = make_float4(dbl_lo_float(v[0]), dbl_lo_float(v[1]), dbl_lo_float(v[2]),
                                 dbl_lo_float(v[3]));
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

cudaError_t launch_grid_refine(int n_frames, int64_t n_charges, int64_t max_points,
                               const int64_t* desc, const double* points, const double* x,
                               const double* q, double* out, int clamp, double tau, int64_t* list,
                               int* count, int* hist, void* df_charges, int num_sms, cudaStream_t s) {
  if (n_frames <= 0 || n_charges <= 0 || max_points <= 0 || !(tau > 0.0)) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, size_t(n_frames) * kMagBins * sizeof(int), s);
  if (e != cudaSuccess) return e;
  float4* dfq = static_cast<float4*>(df_charges);
  const int pack_blocks = static_cast<int>(std::min<int64_t>((n_charges + 255) / 256, 4096));
  pack_df_kernel<<<pack_blocks, 256, 0, s>>>(n_charges, x, q, dfq);
  const dim3 fgrid(n_frames, static_cast<unsigned>((max_points + kFlagChunk - 1) / kFlagChunk));
  grid_mag_hist_kernel<<<fgrid, kFlagThreads, 0, s>>>(desc, out, hist);
  const float tau2 = static_cast<float>(tau * tau);
  grid_flag_kernel<<<fgrid, kFlagThreads, 0, s>>>(desc, out, hist, tau2, list, count);
  const int ctas = std::max(num_sms, 1) * 8;
  if (clamp)
    grid_refine_kernel<true><<<ctas, kRefineThreads, 0, s>>>(desc, list, count, points, dfq, out);
  else
    grid_refine_kernel<false><<<ctas, kRefineThreads, 0, s>>>(desc, list, count, points, dfq, out);
  return cudaGetLastError();
}

int64_t grid_refine_hist_ints(int n_frames) { return int64_t(std::max(n_frames, 1)) * kMagBins; }

cudaError_t preload_grid_refine() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, grid_flag_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, grid_mag_hist_kernel);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, grid_refine_kernel<true>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, grid_refine_kernel<false>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, pack_df_kernel);
  return e;
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

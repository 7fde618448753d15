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
//   FP32C  charges in pairs of float4 records held in shared memory (bulk
//          async copies per CTA; a frame larger than shared memory keeps a
//          prefix there and streams the rest from L2); pair terms in FP32 with
//          the MUFU rsqrt,
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
constexpr int kLanePairs = 32;                  // charge pairs per lane between Kahan steps
constexpr int kChargePad32 = 64;                // FP32C frames: one charge pair per lane
constexpr int kChargePad64 = 256;               // FP64 frames
// Line slots per warp S (template parameter): 4 (default) or 2.

enum Phase : int { kMain = 0, kStart1 = 1, kStart2 = 2, kEnd1 = 3, kEnd2 = 4 };

struct SlotRec {      // per-slot record in shared memory (owner lane only)
  double x0[3], xip[3], xipp[3], xend[3], xe1[3];
};

__device__ __forceinline__ bool outside(const double p[3], const double h[3]) {
  return p[0] < -h[0] || p[0] > h[0] || p[1] < -h[1] || p[1] > h[1] || p[2] < -h[2] ||
         p[2] > h[2];
}

// Exact strict box test from the FP32 image pf = RN(p) of an FP64 position:
// RN is monotonic, so |pf| > RN(h) implies |p| > h and |pf| < RN(h) implies
// |p| < h; only a tie needs the FP64 comparison.
__device__ __forceinline__ bool outside_fast(const double p[3], const float pf[3],
                                             const double h[3], const float hf[3]) {
  bool out = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float a = fabsf(pf[k]);
    if (a > hf[k] || (a == hf[k] && fabs(p[k]) > h[k])) out = true;
  }
  return out;
}

__device__ __forceinline__ double curve_f64(const double a[3], const double b[3]) {
  const double c0 = a[1] * b[2] - a[2] * b[1];
  const double c1 = a[2] * b[0] - a[0] * b[2];
  const double c2 = a[0] * b[1] - a[1] * b[0];
  const double nc = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  const double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  return nc / (na * na * na);
}

// The frame a CTA is working on (uniform across the CTA).
struct FrameCtx {
  int64_t line_off;
  int n_lines;
  double step;
  double half[3];
  float hf[3];  // RN(half): the FP32 side of the exact box test
};

// Per-lane slot state (meaningful in lanes 0..S-1 only).
struct Slot {
  int line;     // -1 = idle
  int phase;
  int steps;
  int cap;
  double pos[3];  // where the next field evaluation happens
  float posf[3];  // its FP32 image (FP32C pair terms)
};

__device__ __forceinline__ void set_pos(Slot& sl, const double v[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    sl.pos[k] = v[k];
    sl.posf[k] = static_cast<float>(v[k]);
  }
}

__device__ void slot_load(Slot& sl, SlotRec& rec, int line, const TopoParams& p) {
  sl.line = line;
  if (line < 0) return;
  const double* s = p.starts + 3 * static_cast<int64_t>(line);
  double st[3];
  for (int k = 0; k < 3; ++k) rec.x0[k] = st[k] = s[k];
  set_pos(sl, st);
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
template <bool FAST_BOX>
__device__ bool slot_advance(Slot& sl, SlotRec& rec, const double nx[3], const TopoParams& p,
                             const FrameCtx& fc) {
  switch (sl.phase) {
    case kMain: {
      sl.steps += 1;
      if (sl.steps == 1)
        for (int k = 0; k < 3; ++k) rec.xip[k] = nx[k];
      if (sl.steps == 2)
        for (int k = 0; k < 3; ++k) rec.xipp[k] = nx[k];
      set_pos(sl, nx);
      const bool out =
          FAST_BOX ? outside_fast(sl.pos, sl.posf, fc.half, fc.hf) : outside(nx, fc.half);
      if (out || sl.steps >= sl.cap) {
        for (int k = 0; k < 3; ++k) rec.xend[k] = nx[k];
        if (sl.steps >= 2) {
          sl.phase = kEnd1;  // next evaluation at the end point (= nx)
        } else {
          sl.phase = kStart2;  // steps == 1: the end point is also x_init_plus
        }
      }
      return false;
    }
    case kStart1:
      for (int k = 0; k < 3; ++k) rec.xip[k] = nx[k];
      set_pos(sl, nx);
      sl.phase = kStart2;
      return false;
    case kStart2:
      for (int k = 0; k < 3; ++k) rec.xipp[k] = nx[k];
      set_pos(sl, rec.xend);
      sl.phase = kEnd1;
      return false;
    case kEnd1:
      for (int k = 0; k < 3; ++k) rec.xe1[k] = nx[k];
      set_pos(sl, nx);
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

// FP32C.  Charges in "pair" layout: A[p] = {x_2p, x_2p+1, y_2p, y_2p+1},
// B[p] = {z_2p, z_2p+1, q_2p, q_2p+1}, so each 64-bit half of a 16-byte load is
// a ready operand of the packed f32x2 instructions: one instruction evaluates
// a pair term for two charges.  Lanes take pairs lane-strided; every
// kLanePairs pairs (fewer in a frame's last run: frames are padded to one pair
// per lane only) the two packed streams are added and Kahan-accumulated.
template <int NA, int S, int UNROLL>
__device__ __forceinline__ void pair_run(const ulonglong2* __restrict__ A,
                                         const ulonglong2* __restrict__ B, int base, int cnt,
                                         const uint64_t (&ex2)[S][3], uint64_t (&part)[NA][3]) {
#pragma unroll UNROLL
  for (int i = 0; i < cnt; ++i) {
    const ulonglong2 a = A[base + 32 * i];  // {x pair, y pair}
    const ulonglong2 b = B[base + 32 * i];  // {z pair, q pair}
#pragma unroll
    for (int e = 0; e < NA; ++e) {
      const uint64_t dx = sub2(ex2[e][0], a.x);
      const uint64_t dy = sub2(ex2[e][1], a.y);
      const uint64_t dz = sub2(ex2[e][2], b.x);
      const uint64_t r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
      const uint64_t ri = rsqrt2(r2);
      const uint64_t w = mul2(mul2(b.y, ri), mul2(ri, ri));
      part[e][0] = fma2(w, dx, part[e][0]);
      part[e][1] = fma2(w, dy, part[e][1]);
      part[e][2] = fma2(w, dz, part[e][2]);
    }
  }
}

// Dipole pairs: A[p] = {x pair, y pair}, B[p] = {z pair, 3 mu_x pair},
// C[p] = {mu_y pair, mu_z pair}.  Per dipole the term of
// calc_field_base_dipole (CPET/utils/math_module.c:335-371) without the
// constant factor (the step only uses the field's direction):
//   r^-5 ((3 mu_x R_x + mu_y R_y + mu_z R_z) R_c - mu_c r^2)
//   = w R_c - r^-3 mu_c,  w = (3 mu_x R_x + mu_y R_y + mu_z R_z) r^-5,
// the x component taking mu_x as (3 mu_x) * (-1/3) r^-3.
template <int NA, int S, int UNROLL>
__device__ __forceinline__ void dipole_run(const ulonglong2* __restrict__ A,
                                           const ulonglong2* __restrict__ B,
                                           const ulonglong2* __restrict__ C, int base, int cnt,
                                           const uint64_t (&ex2)[S][3], uint64_t (&part)[NA][3]) {
  const uint64_t m_third = pk2(-1.f / 3.f, -1.f / 3.f), m_one = pk2(-1.f, -1.f);
#pragma unroll UNROLL
  for (int i = 0; i < cnt; ++i) {
    const ulonglong2 a = A[base + 32 * i];  // {x pair, y pair}
    const ulonglong2 b = B[base + 32 * i];  // {z pair, 3 mu_x pair}
    const ulonglong2 c = C[base + 32 * i];  // {mu_y pair, mu_z pair}
#pragma unroll
    for (int e = 0; e < NA; ++e) {
      const uint64_t dx = sub2(ex2[e][0], a.x);
      const uint64_t dy = sub2(ex2[e][1], a.y);
      const uint64_t dz = sub2(ex2[e][2], b.x);
      const uint64_t r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
      const uint64_t ri = rsqrt2(r2);
      const uint64_t ri2 = mul2(ri, ri);
      const uint64_t ri3 = mul2(ri2, ri);
      const uint64_t w = mul2(fma2(b.y, dx, fma2(c.x, dy, mul2(c.y, dz))), mul2(ri3, ri2));
      const uint64_t t3 = mul2(ri3, m_third), tn = mul2(ri3, m_one);
      part[e][0] = fma2(t3, b.y, fma2(w, dx, part[e][0]));
      part[e][1] = fma2(tn, c.x, fma2(w, dy, part[e][1]));
      part[e][2] = fma2(tn, c.y, fma2(w, dz, part[e][2]));
    }
  }
}

// Sources of a sweep.  kSrcOne: every pair from (A, B, C) -- a frame held
// entirely in shared memory, or one read entirely from global memory.
// kSrcSplit: pairs [0, res_pairs) from (sA, sB, sC), the shared-memory copy of
// a frame's first pairs, the rest from (A, B, C) in global memory (L2);
// res_pairs is a multiple of the 32 x kLanePairs pairs of one Kahan run, so
// every run reads one source and the sums are the same whichever part is
// resident.  The single-source loop is compiled on its own: with both sources
// in one loop the all-resident sweep ran 12% slower.
constexpr int kSrcOne = 0;
constexpr int kSrcSplit = 1;

// DIP: point dipoles (dipole_run, C used); otherwise point charges (pair_run).
template <int NA, int S, bool DIP = false, int SRC = kSrcOne>
__device__ __forceinline__ void sweep_f32x2(const ulonglong2* __restrict__ sA,
                                            const ulonglong2* __restrict__ sB,
                                            const ulonglong2* __restrict__ sC, int res_pairs,
                                            const ulonglong2* __restrict__ A,
                                            const ulonglong2* __restrict__ B,
                                            const ulonglong2* __restrict__ C, int n_pairs,
                                            int lane, const uint64_t (&ex2)[S][3], float& total) {
  float acc[NA][3], cmp[NA][3];
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[e][c] = cmp[e][c] = 0.f;

  // n_pairs is a multiple of 32: every lane runs the same number of pairs
  for (int base = 0; base < n_pairs; base += 32 * kLanePairs) {
    uint64_t part[NA][3];
#pragma unroll
    for (int e = 0; e < NA; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) part[e][c] = 0ull;
    const int left = (n_pairs - base) >> 5;
    // about eight independent pair chains in flight per lane: unroll 8 / NA
    constexpr int kUnroll = NA >= 3 ? 2 : (NA == 2 ? 4 : 8);
    const int cnt = left >= kLanePairs ? kLanePairs : left;
    if (SRC == kSrcSplit && base < res_pairs) {  // shared-memory copy
      if constexpr (DIP) {
        if (cnt == kLanePairs)
          dipole_run<NA, S, kUnroll>(sA, sB, sC, base + lane, kLanePairs, ex2, part);
        else
          dipole_run<NA, S, 1>(sA, sB, sC, base + lane, cnt, ex2, part);
      } else {
        if (cnt == kLanePairs)
          pair_run<NA, S, kUnroll>(sA, sB, base + lane, kLanePairs, ex2, part);
        else
          pair_run<NA, S, 1>(sA, sB, base + lane, cnt, ex2, part);
      }
    } else {  // global memory (kSrcSplit), or the one source
      if constexpr (DIP) {
        if (cnt == kLanePairs)
          dipole_run<NA, S, kUnroll>(A, B, C, base + lane, kLanePairs, ex2, part);
        else
          dipole_run<NA, S, 1>(A, B, C, base + lane, cnt, ex2, part);
      } else {
        if (cnt == kLanePairs)
          pair_run<NA, S, kUnroll>(A, B, base + lane, kLanePairs, ex2, part);
        else
          pair_run<NA, S, 1>(A, B, base + lane, cnt, ex2, part);
      }
    }
#pragma unroll
    for (int e = 0; e < NA; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float lo, hi2;
        upk2(part[e][c], lo, hi2);
        kahan_add(acc[e][c], cmp[e][c], __fadd_rn(lo, hi2));
      }
  }
  // Lane partials (acc - cmp, unevaluated pairs) as NV = 4S values v = 3e + c,
  // reduced across the warp by a reduce-scatter of error-free pair additions:
  // each of the LV levels halves the values a lane keeps, a butterfly finishes;
  // afterwards the lanes with (lane >> (5 - LV)) == v hold the total of value v.
  constexpr int NV = 4 * S;
  constexpr int LV = (S == 4) ? 4 : 3;
  float h[NV], l[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const int e = v / 3, c = v % 3;
    h[v] = (e < NA) ? acc[e < NA ? e : 0][c] : 0.f;
    l[v] = (e < NA) ? -cmp[e < NA ? e : 0][c] : 0.f;
  }
#pragma unroll
  for (int lvl = 0, half = NV / 2; lvl < LV; ++lvl, half >>= 1) {
    const int off = 16 >> lvl;
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int j = 0; j < half; ++j) {
      const float sh = upper ? h[j] : h[j + half];
      const float sl = upper ? l[j] : l[j + half];
      const float kh = upper ? h[j + half] : h[j];
      const float kl = upper ? l[j + half] : l[j];
      const float rh = __shfl_xor_sync(0xffffffffu, sh, off);
      const float rl = __shfl_xor_sync(0xffffffffu, sl, off);
      h[j] = kh;
      l[j] = kl;
      pair_add(h[j], l[j], rh, rl);
    }
  }
#pragma unroll
  for (int off = 16 >> LV; off >= 1; off >>= 1) {
    const float rh = __shfl_xor_sync(0xffffffffu, h[0], off);
    const float rl = __shfl_xor_sync(0xffffffffu, l[0], off);
    pair_add(h[0], l[0], rh, rl);
  }
  total = h[0];
}

// FP64: charges from global memory (padded with zero charges far away).  Every
// operation in double precision; r^-1 from the double rsqrt (1 ulp), whose few
// FP64-pipe operations replace a correctly rounded sqrt and division (GB300's
// FP64 pipe is 1/64 of its FP32 pipe).
template <int NA, int S>
__device__ __forceinline__ void sweep_f64(const Charge64* __restrict__ g, int n_pad, int lane,
                                          const double (&ex)[S][3], double (&E)[S][3]) {
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
      const double ri = rsqrt(r2);  // double-precision reciprocal square root (1 ulp)
      const double w = __dmul_rn(ch.q, __dmul_rn(ri, __dmul_rn(ri, ri)));
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

// FP64 dipoles: Dipole64 records read from global memory (L2), padded with
// zero moments far away.  Same term as dipole_run, in double precision (r^-1
// from the double rsqrt, as sweep_f64).
template <int NA, int S>
__device__ __forceinline__ void sweep_dipole_f64(const Dipole64* __restrict__ g, int n_pad, int lane,
                                                 const double (&ex)[S][3], double (&E)[S][3]) {
  double acc[NA][3];
#pragma unroll
  for (int e = 0; e < NA; ++e)
#pragma unroll
    for (int c = 0; c < 3; ++c) acc[e][c] = 0.0;
#pragma unroll 2
  for (int j = lane; j < n_pad; j += 32) {
    const Dipole64 d = g[j];
#pragma unroll
    for (int e = 0; e < NA; ++e) {
      const double dx = __dsub_rn(ex[e][0], d.x);
      const double dy = __dsub_rn(ex[e][1], d.y);
      const double dz = __dsub_rn(ex[e][2], d.z);
      const double r2 = __fma_rn(dx, dx, __fma_rn(dy, dy, __dmul_rn(dz, dz)));
      const double ri = rsqrt(r2);  // double-precision reciprocal square root (1 ulp)
      const double ri2 = __dmul_rn(ri, ri);
      const double r5 = __dmul_rn(__dmul_rn(ri2, ri2), ri);
      const double dot = __fma_rn(3.0 * d.mx, dx, __fma_rn(d.my, dy, __dmul_rn(d.mz, dz)));
      acc[e][0] = __fma_rn(r5, __fma_rn(dot, dx, -__dmul_rn(d.mx, r2)), acc[e][0]);
      acc[e][1] = __fma_rn(r5, __fma_rn(dot, dy, -__dmul_rn(d.my, r2)), acc[e][1]);
      acc[e][2] = __fma_rn(r5, __fma_rn(dot, dz, -__dmul_rn(d.mz, r2)), acc[e][2]);
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

// Residency of a launch's frames (kernel template RES): kResNone -- every
// frame read from global memory (L2); kResWhole -- each frame entirely in
// shared memory or read from L2; kResAny -- also frames of which only a prefix
// is resident (frames above the shared-memory limit).  The prefix sweeps are
// compiled only into kResAny kernels: with them in the kernel of whole-frame
// launches its instruction cache missed (no-instruction stalls 0.31 per issue
// instead of 0.05) and the 8,000-charge workload ran 6% slower.
constexpr int kResNone = 0;
constexpr int kResWhole = 1;
constexpr int kResAny = 2;

// The sweep of one frame of a kResAny launch: res_pairs of its n_pairs pairs
// are in shared memory.
template <int NA, int S, bool DIP>
__device__ __forceinline__ void sweep_frame_any(const ulonglong2* smA, const ulonglong2* smB,
                                                const ulonglong2* smC, int res_pairs,
                                                const ulonglong2* chA, const ulonglong2* chB,
                                                const ulonglong2* chC, int n_pairs, int lane,
                                                const uint64_t (&ex2)[S][3], float& total) {
  if (res_pairs >= n_pairs)
    sweep_f32x2<NA, S, DIP, kSrcOne>(nullptr, nullptr, nullptr, 0, smA, smB, smC, n_pairs, lane, ex2,
                                     total);
  else if (res_pairs > 0)
    sweep_f32x2<NA, S, DIP, kSrcSplit>(smA, smB, smC, res_pairs, chA, chB, chC, n_pairs, lane, ex2,
                                       total);
  else
    sweep_f32x2<NA, S, DIP, kSrcOne>(nullptr, nullptr, nullptr, 0, chA, chB, chC, n_pairs, lane, ex2,
                                     total);
}

// One line slot set per warp; processes the lines of frame `fc` (charge
// arrays chA/chB in the FP32C pair layout, or g in Charge64) until the frame's
// queue is exhausted and the warp's slots are drained.
// resident: the whole frame is in shared memory (kResWhole launches);
// res_pairs: pairs in shared memory (kResAny launches).
template <int PREC, int S, bool DIP, int RES>
__device__ __forceinline__ void run_frame(const TopoParams& p, const FrameCtx& fc, int* queue,
                                          const ulonglong2* chA, const ulonglong2* chB,
                                          const ulonglong2* chC, const ulonglong2* smA,
                                          const ulonglong2* smB, const ulonglong2* smC,
                                          bool resident, int res_pairs, int n_pad, SlotRec* my_rec,
                                          int lane) {
  Slot sl;
  sl.line = -1;
  sl.phase = kMain;
  sl.steps = sl.cap = 0;
  sl.pos[0] = sl.pos[1] = sl.pos[2] = 0.0;
  sl.posf[0] = sl.posf[1] = sl.posf[2] = 0.f;
  if (lane < S) {
    const int li = atomicAdd(queue, 1);
    slot_load(sl, *my_rec, li < fc.n_lines ? static_cast<int>(fc.line_off + li) : -1, p);
  }
  for (;;) {
    const unsigned active = __ballot_sync(0xffffffffu, lane < S && sl.line >= 0);
    const int na = __popc(active);
    if (na == 0) break;
    // owner lane of each active slot, in order; this lane's rank among them
    int src_of[S];
    int my_rank = -1;
    {
      unsigned m = active;
#pragma unroll
      for (int e = 0; e < S; ++e) {
        src_of[e] = m ? (__ffs(m) - 1) : 0;
        if (m) m &= m - 1;
        if (src_of[e] == lane && e < na) my_rank = e;
      }
    }

    double nx[3];
    if constexpr (PREC == kFP32C) {
      uint64_t ex2[S][3];
#pragma unroll
      for (int e = 0; e < S; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float v = __shfl_sync(0xffffffffu, sl.posf[c], src_of[e]);
          ex2[e][c] = pk2(v, v);
        }
      float total;
      const int n_pairs = n_pad / 2;
      if constexpr (RES == kResAny) {
        switch (na) {
          case 1:
            sweep_frame_any<1, S, DIP>(smA, smB, smC, res_pairs, chA, chB, chC, n_pairs, lane, ex2, total);
            break;
          case 2:
            sweep_frame_any<2, S, DIP>(smA, smB, smC, res_pairs, chA, chB, chC, n_pairs, lane, ex2, total);
            break;
          case 3:
            sweep_frame_any<(S > 2 ? 3 : 2), S, DIP>(smA, smB, smC, res_pairs, chA, chB, chC, n_pairs,
                                                     lane, ex2, total);
            break;
          default:
            sweep_frame_any<S, S, DIP>(smA, smB, smC, res_pairs, chA, chB, chC, n_pairs, lane, ex2, total);
            break;
        }
      } else if (resident) {  // whole frame in shared memory
        switch (na) {
          case 1: sweep_f32x2<1, S, DIP>(nullptr, nullptr, nullptr, 0, smA, smB, smC, n_pairs, lane, ex2, total); break;
          case 2: sweep_f32x2<2, S, DIP>(nullptr, nullptr, nullptr, 0, smA, smB, smC, n_pairs, lane, ex2, total); break;
          case 3: sweep_f32x2<(S > 2 ? 3 : 2), S, DIP>(nullptr, nullptr, nullptr, 0, smA, smB, smC, n_pairs, lane, ex2, total); break;
          default: sweep_f32x2<S, S, DIP>(nullptr, nullptr, nullptr, 0, smA, smB, smC, n_pairs, lane, ex2, total); break;
        }
      } else {  // every pair from global memory
        switch (na) {
          case 1: sweep_f32x2<1, S, DIP>(nullptr, nullptr, nullptr, 0, chA, chB, chC, n_pairs, lane, ex2, total); break;
          case 2: sweep_f32x2<2, S, DIP>(nullptr, nullptr, nullptr, 0, chA, chB, chC, n_pairs, lane, ex2, total); break;
          case 3: sweep_f32x2<(S > 2 ? 3 : 2), S, DIP>(nullptr, nullptr, nullptr, 0, chA, chB, chC, n_pairs, lane, ex2, total); break;
          default: sweep_f32x2<S, S, DIP>(nullptr, nullptr, nullptr, 0, chA, chB, chC, n_pairs, lane, ex2, total); break;
        }
      }
      // component c of slot rank e sits in lanes (3e + c) << (5 - LV) and up
      float Ef[3];
      const int rk = my_rank >= 0 ? my_rank : 0;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        Ef[c] = __shfl_sync(0xffffffffu, total, (3 * rk + c) << (S == 4 ? 1 : 2));
      if (my_rank >= 0) {
        // step vector in FP32 (the factor k does not change the direction)
        const float n2 = __fmaf_rn(Ef[0], Ef[0], __fmaf_rn(Ef[1], Ef[1], __fmul_rn(Ef[2], Ef[2])));
        const float s = __fdiv_rn(static_cast<float>(fc.step), __fsqrt_rn(n2));
#pragma unroll
        for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + static_cast<double>(__fmul_rn(Ef[c], s));
      }
    } else {
      double ex[S][3];
#pragma unroll
      for (int e = 0; e < S; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) ex[e][c] = __shfl_sync(0xffffffffu, sl.pos[c], src_of[e]);
      double Es[S][3];
      if constexpr (DIP) {
        const Dipole64* g = reinterpret_cast<const Dipole64*>(chA);
        switch (na) {
          case 1: sweep_dipole_f64<1, S>(g, n_pad, lane, ex, Es); break;
          case 2: sweep_dipole_f64<2, S>(g, n_pad, lane, ex, Es); break;
          case 3: sweep_dipole_f64<(S > 2 ? 3 : 2), S>(g, n_pad, lane, ex, Es); break;
          default: sweep_dipole_f64<S, S>(g, n_pad, lane, ex, Es); break;
        }
      } else {
        const Charge64* g = reinterpret_cast<const Charge64*>(chA);
        switch (na) {
          case 1: sweep_f64<1, S>(g, n_pad, lane, ex, Es); break;
          case 2: sweep_f64<2, S>(g, n_pad, lane, ex, Es); break;
          case 3: sweep_f64<(S > 2 ? 3 : 2), S>(g, n_pad, lane, ex, Es); break;
          default: sweep_f64<S, S>(g, n_pad, lane, ex, Es); break;
        }
      }
      if (my_rank >= 0) {
        double E[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int e = 0; e < S; ++e)
          if (e == my_rank)
#pragma unroll
            for (int c = 0; c < 3; ++c) E[c] = Es[e][c];
        const double n = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
#pragma unroll
        for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + fc.step * E[c] / n;
      }
    }

    if (my_rank >= 0) {
      if (slot_advance<PREC == kFP32C>(sl, *my_rec, nx, p, fc)) {
        const int li = atomicAdd(queue, 1);
        slot_load(sl, *my_rec, li < fc.n_lines ? static_cast<int>(fc.line_off + li) : -1, p);
      }
    }
    __syncwarp();
  }
}

// Frames are visited in table order; a CTA stays on a frame while its line
// queue lasts, then moves on (after its own warps are done, so the shared
// copy of the charges can be replaced).  Frames thus overlap only at their
// tails and every frame switch costs a CTA one line's latency at most.
// DIP: the sources are point dipoles (FP32C: three 16-byte pair blocks per
// frame; FP64: Dipole64 records) instead of point charges.  RES: residency
// mode of the launch's frames (kResNone, kResWhole, kResAny).
template <int PREC, int RES, int S, bool DIP>
__global__ void __launch_bounds__(kTopoThreads, 1) topo_kernel(TopoParams p, TopoFrame frame0) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_skip;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  SlotRec* recs = reinterpret_cast<SlotRec*>(smem_raw);  // [kTopoWarps][S]
  const size_t rec_bytes = sizeof(SlotRec) * kTopoWarps * S;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + rec_bytes);
  ulonglong2* sm_ch = reinterpret_cast<ulonglong2*>(smem_raw + rec_bytes + 128);
  SlotRec* my_rec = recs + warp * S + (lane < S ? lane : 0);
  const int n_frames = p.frames ? p.n_frames : 1;
  uint32_t load_parity = 0;
  if (RES != kResNone && threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }

  for (int f = 0; f < n_frames; ++f) {
    const TopoFrame fr = p.frames ? p.frames[f] : frame0;
    int* queue = p.queue + f;
    __syncthreads();  // the CTA's warps are done with the previous frame
    if (threadIdx.x == 0) s_skip = (*reinterpret_cast<volatile int*>(queue) >= fr.n_lines) ? 1 : 0;
    __syncthreads();
    if (s_skip) continue;
    // sources in shared memory.  kResAny: the frame's first fr.resident
    // sources -- all of them, or a prefix of whole Kahan runs when the frame
    // exceeds shared memory -- copied block by block.  Otherwise whole frames
    // (the host launches kResWhole only when every resident frame is entirely
    // so) in one contiguous copy of the packed blocks: written as the
    // block-wise copy, that kernel was compiled to a schedule 6% slower on
    // the 8,000-charge workload.
    int res = 0;
    bool resident = false;
    if constexpr (RES == kResAny) {
      res = fr.resident;
      if (res > 0) {
        if (threadIdx.x == 0) {
          const uint32_t blk = static_cast<uint32_t>(res / 2) * 16u;  // bytes of one block's prefix
          const int n_blk = DIP ? 3 : 2;
          mbar_arrive_expect_tx(bar, blk * n_blk);
          const char* src = static_cast<const char*>(p.packed) + fr.packed_off * 16;
          constexpr uint32_t kChunk = 32768;
          for (int b = 0; b < n_blk; ++b) {  // block b of the frame starts at b * n_pad/2 pairs
            const char* bs = src + static_cast<size_t>(b) * (fr.n_pad / 2) * 16;
            char* bd = reinterpret_cast<char*>(sm_ch) + static_cast<size_t>(b) * blk;
            for (uint32_t off = 0; off < blk; off += kChunk)
              bulk_g2s(bd + off, bs + off, min(kChunk, blk - off), bar);
          }
        }
        const bool mine = mbar_wait(bar, load_parity, p.status);
        load_parity ^= 1u;
        if (!__syncthreads_and(mine)) return;
      }
    } else {
      resident = RES == kResWhole && fr.resident;
      if (resident) {
        if (threadIdx.x == 0) {
          const uint32_t total = static_cast<uint32_t>(fr.n_pad) * (DIP ? 24u : 16u);
          mbar_arrive_expect_tx(bar, total);
          const char* src = static_cast<const char*>(p.packed) + fr.packed_off * 16;
          constexpr uint32_t kChunk = 32768;
          for (uint32_t off = 0; off < total; off += kChunk)
            bulk_g2s(reinterpret_cast<char*>(sm_ch) + off, src + off, min(kChunk, total - off), bar);
        }
        const bool mine = mbar_wait(bar, load_parity, p.status);
        load_parity ^= 1u;
        if (!__syncthreads_and(mine)) return;
      }
    }
    FrameCtx fc;
    fc.line_off = fr.line_off;
    fc.n_lines = fr.n_lines;
    fc.step = fr.step;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      fc.half[k] = fr.half[k];
      fc.hf[k] = static_cast<float>(fr.half[k]);
    }
    const size_t elem = (PREC == kFP32C) ? 16 : 32;
    const ulonglong2* gA = reinterpret_cast<const ulonglong2*>(
        static_cast<const char*>(p.packed) + fr.packed_off * elem);
    const ulonglong2* gB = gA + fr.n_pad / 2;
    const ulonglong2* gC = DIP ? gA + fr.n_pad : nullptr;
    if constexpr (RES == kResAny) {
      const ulonglong2* sC = DIP ? sm_ch + res : nullptr;
      run_frame<PREC, S, DIP, RES>(p, fc, queue, gA, gB, gC, sm_ch, sm_ch + res / 2, sC, false,
                                   res / 2, fr.n_pad, my_rec, lane);
    } else {
      const ulonglong2* sC = DIP ? sm_ch + fr.n_pad : nullptr;
      run_frame<PREC, S, DIP, RES>(p, fc, queue, gA, gB, gC, sm_ch, sm_ch + fr.n_pad / 2, sC, resident,
                                   0, fr.n_pad, my_rec, lane);
    }
  }
}

// ---------------------------------------------------------------------------
// Serving engine: continuous batching of streamline requests.
// ---------------------------------------------------------------------------
// Warps claim chunks of lines from a ring the host appends to while the
// kernel runs; a slot that finishes a line takes the next line of the warp's
// chunk (or of a newly claimed chunk, possibly of another frame), so requests
// arriving while others are in flight are admitted as slots free up.  Each
// step the warp sweeps the charges once per distinct frame among its active
// slots.  Charges are read from global memory (L2).
//
// Lifetime of a launch: a warp without lines polls for chunks, and stays while
// any warp of the launch has lines or claims happen, so work published later
// finds every warp of the launch (a launch whose idle warps had left would
// serve it with the few warps still busy, while the next launch waits behind
// it).  Once no warp has had lines and nothing was claimed for kEngineIdleNs,
// the first warp to see it closes the launch: no warp claims again, and each
// ends when its lines are done.  Work published after that goes to the next
// launch, which the host keeps queued.
constexpr int kEngineThreads = 256;
constexpr int kEngineWarps = kEngineThreads / 32;
constexpr unsigned long long kEngineIdleNs = 50000000ull;      // launch idle 50 ms: it closes
constexpr unsigned long long kEngineMaxWaitNs = 60000000000ull;  // bound on one idle wait (60 s)

__device__ __forceinline__ int ld_acquire_sys(const int* p) {
  int v;
  asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Claims the next published chunk; -1 when none is published.  The claim
// counter lives in device memory (L2 atomics); every failed CAS means another
// warp advanced it, so the loop ends within the number of published chunks.
// The host sees claims through a monotonic mirror in host-mapped memory.
__device__ int engine_claim(const EngineParams& E) {
  for (int tries = 0; tries < (1 << 20); ++tries) {
    const int t = ld_acquire_sys(E.tail);
    const int h = *reinterpret_cast<volatile int*>(E.head);
    if (h >= t) return -1;
    if (atomicCAS(E.head, h, h + 1) == h) {
      atomicMax_system(E.head_mirror, h + 1);
      return h;
    }
  }
  return -1;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Idle wait of a warp with no line (lane 0 only): polls for a chunk with a
// sleep growing from 20 to 320 us.  Returns the claimed chunk, or -1 once the
// launch is closed -- by this warp when neither a busy warp nor a claim was
// seen for kEngineIdleNs, or after kEngineMaxWaitNs in any case.
__device__ int engine_idle_wait(const EngineParams& E) {
  const unsigned long long t0 = globaltimer_ns();
  unsigned long long quiet_since = t0;
  int last_head = ld_volatile(E.head);
  unsigned sleep_ns = 20000;
  for (;;) {
    if (ld_volatile(E.closing)) return -1;
    const int got = engine_claim(E);
    if (got >= 0) return got;
    const unsigned long long now = globaltimer_ns();
    const int h = ld_volatile(E.head);
    if (ld_volatile(E.busy) > 0 || h != last_head) {
      quiet_since = now;
      last_head = h;
    } else if (now - quiet_since > kEngineIdleNs) {
      atomicExch(E.closing, 1);
      return -1;
    }
    if (now - t0 > kEngineMaxWaitNs) {
      atomicExch(E.closing, 1);
      return -1;
    }
    __nanosleep(sleep_ns);
    if (sleep_ns < 320000) sleep_ns *= 2;
  }
}

__device__ __forceinline__ EngineChunk engine_read_chunk(const EngineParams& E, int idx) {
  const volatile EngineChunk* c = E.chunks + (idx % E.chunk_capacity);
  EngineChunk r;
  r.frame = c->frame;
  r.request = c->request;
  r.line_begin = c->line_begin;
  r.line_end = c->line_end;
  r.step = c->step;
  r.half[0] = c->half[0];
  r.half[1] = c->half[1];
  r.half[2] = c->half[2];
  return r;
}

// slot_load for lines the host wrote while the kernel may run: read past L1.
__device__ void engine_slot_load(Slot& sl, SlotRec& rec, int line, const TopoParams& p) {
  sl.line = line;
  const double* s = p.starts + 3 * static_cast<int64_t>(line);
  double st[3];
  for (int k = 0; k < 3; ++k) rec.x0[k] = st[k] = __ldcg(s + k);
  set_pos(sl, st);
  sl.cap = max(__ldcg(p.n_iter + line), 0);
  if (sl.cap > kMaxLineCap) {
    atomicCAS(p.status, kDevOk, kDevBadCap);
    sl.cap = 0;
  }
  sl.steps = 0;
  if (sl.cap > 0) {
    sl.phase = kMain;
  } else {
    sl.phase = kStart1;
    for (int k = 0; k < 3; ++k) rec.xend[k] = st[k];
  }
}

// Per-slot request context, kept in shared memory (read once per step).
struct EngineSlotCtx {
  long long off;  // the frame's first packed element
  int frame;
  int req;
  int n_pad;
  int pad_;
  double step;
  double half[3];
};

template <int PREC, int S>
__global__ void __launch_bounds__(kEngineThreads, 2) engine_kernel(EngineParams E) {
  __shared__ SlotRec recs[kEngineWarps][S];
  __shared__ EngineSlotCtx sctx[kEngineWarps][S];
  __shared__ EngineChunk wchunk[kEngineWarps];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  SlotRec& rec = recs[warp][lane < S ? lane : 0];
  EngineSlotCtx& my = sctx[warp][lane < S ? lane : 0];
  const size_t elem = (PREC == kFP32C) ? 16 : 32;
  if (lane < S) my.frame = -1;

  Slot sl;
  sl.line = -1;
  sl.phase = kMain;
  sl.steps = sl.cap = 0;
  sl.pos[0] = sl.pos[1] = sl.pos[2] = 0.0;
  sl.posf[0] = sl.posf[1] = sl.posf[2] = 0.f;
  int c_next = 0, c_end = 0;  // the warp's chunk cursor (uniform across the warp)
  int backoff = 0;            // steps to wait before claiming again after an empty queue
  bool counted = false;       // this warp is counted in E.busy (uniform)
  __syncwarp();

  for (;;) {
    // refill idle slots, claiming chunks as needed
    unsigned need = __ballot_sync(0xffffffffu, lane < S && sl.line < 0);
    const bool all_idle = __popc(need) == S;
    if (all_idle && counted && c_next >= c_end) {  // no line held or left in the chunk
      if (lane == 0) atomicSub(E.busy, 1);
      counted = false;
    }
    if (backoff > 0 && !all_idle) {
      --backoff;
      need = (c_next < c_end) ? need : 0u;  // only lines of the current chunk
    }
    bool took = false;  // a line was given to a slot in this pass
    while (need) {
      if (c_next >= c_end) {
        int got = -1;
        if (lane == 0) {
          if (!ld_volatile(E.closing)) got = engine_claim(E);
          if (got < 0 && all_idle && !took) got = engine_idle_wait(E);
          if (got >= 0 && !counted) atomicAdd(E.busy, 1);
          if (got >= 0) wchunk[warp] = engine_read_chunk(E, got);
        }
        got = __shfl_sync(0xffffffffu, got, 0);
        __syncwarp();
        if (got < 0) {
          backoff = 8;
          break;
        }
        counted = true;
        c_next = wchunk[warp].line_begin;
        c_end = wchunk[warp].line_end;
        continue;
      }
      const int target = __ffs(need) - 1;
      const int line = c_next++;
      if (lane == target) {
        const EngineChunk& ch = wchunk[warp];
        // frame slots are reused while the kernel runs: read the table past L1
        my.off = __ldcg(&E.frames[ch.frame].packed_off);
        my.frame = ch.frame;
        my.req = ch.request;
        my.n_pad = __ldcg(&E.frames[ch.frame].n_pad);
        my.step = ch.step;
        for (int k = 0; k < 3; ++k) my.half[k] = ch.half[k];
        engine_slot_load(sl, rec, line, E.p);
      }
      took = true;
      need &= ~(1u << target);
      __syncwarp();
    }
    const unsigned active = __ballot_sync(0xffffffffu, lane < S && sl.line >= 0);
    if (active == 0) break;

    double nx[3] = {0.0, 0.0, 0.0};
    unsigned remaining = active;
    while (remaining) {
      const int leader = __ffs(remaining) - 1;
      const EngineSlotCtx& L = sctx[warp][leader];
      const int f = L.frame;
      const unsigned group =
          __ballot_sync(0xffffffffu, lane < S && sl.line >= 0 && my.frame == f) & remaining;
      remaining &= ~group;
      const int na = __popc(group);
      const int n_pad = L.n_pad;
      const ulonglong2* gA = reinterpret_cast<const ulonglong2*>(
          static_cast<const char*>(E.p.packed) + L.off * static_cast<long long>(elem));
      const ulonglong2* gB = gA + n_pad / 2;
      int src_of[S];
      int my_rank = -1;
      {
        unsigned m = group;
#pragma unroll
        for (int e = 0; e < S; ++e) {
          src_of[e] = m ? (__ffs(m) - 1) : 0;
          if (m) m &= m - 1;
          if (src_of[e] == lane && e < na) my_rank = e;
        }
      }
      if constexpr (PREC == kFP32C) {
        uint64_t ex2[S][3];
#pragma unroll
        for (int e = 0; e < S; ++e)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float v = __shfl_sync(0xffffffffu, sl.posf[c], src_of[e]);
            ex2[e][c] = pk2(v, v);
          }
        float total;
        const int n_pairs = n_pad / 2;
        switch (na) {
          case 1: sweep_f32x2<1, S>(nullptr, nullptr, nullptr, 0, gA, gB, nullptr, n_pairs, lane, ex2, total); break;
          case 2: sweep_f32x2<2, S>(nullptr, nullptr, nullptr, 0, gA, gB, nullptr, n_pairs, lane, ex2, total); break;
          case 3: sweep_f32x2<(S > 2 ? 3 : 2), S>(nullptr, nullptr, nullptr, 0, gA, gB, nullptr, n_pairs, lane, ex2, total); break;
          default: sweep_f32x2<S, S>(nullptr, nullptr, nullptr, 0, gA, gB, nullptr, n_pairs, lane, ex2, total); break;
        }
        float Ef[3];
        const int rk = my_rank >= 0 ? my_rank : 0;
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Ef[c] = __shfl_sync(0xffffffffu, total, (3 * rk + c) << (S == 4 ? 1 : 2));
        if (my_rank >= 0) {
          const float n2 =
              __fmaf_rn(Ef[0], Ef[0], __fmaf_rn(Ef[1], Ef[1], __fmul_rn(Ef[2], Ef[2])));
          const float st = __fdiv_rn(static_cast<float>(my.step), __fsqrt_rn(n2));
#pragma unroll
          for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + static_cast<double>(__fmul_rn(Ef[c], st));
        }
      } else {
        double ex[S][3];
#pragma unroll
        for (int e = 0; e < S; ++e)
#pragma unroll
          for (int c = 0; c < 3; ++c) ex[e][c] = __shfl_sync(0xffffffffu, sl.pos[c], src_of[e]);
        double Es[S][3];
        const Charge64* g = reinterpret_cast<const Charge64*>(gA);
        switch (na) {
          case 1: sweep_f64<1, S>(g, n_pad, lane, ex, Es); break;
          case 2: sweep_f64<2, S>(g, n_pad, lane, ex, Es); break;
          case 3: sweep_f64<(S > 2 ? 3 : 2), S>(g, n_pad, lane, ex, Es); break;
          default: sweep_f64<S, S>(g, n_pad, lane, ex, Es); break;
        }
        if (my_rank >= 0) {
          double Ev[3] = {0.0, 0.0, 0.0};
#pragma unroll
          for (int e = 0; e < S; ++e)
            if (e == my_rank)
#pragma unroll
              for (int c = 0; c < 3; ++c) Ev[c] = Es[e][c];
          const double n = sqrt(Ev[0] * Ev[0] + Ev[1] * Ev[1] + Ev[2] * Ev[2]);
#pragma unroll
          for (int c = 0; c < 3; ++c) nx[c] = sl.pos[c] + my.step * Ev[c] / n;
        }
      }
    }

    if (lane < S && sl.line >= 0) {
      FrameCtx fc;
      fc.line_off = 0;
      fc.n_lines = 0;
      fc.step = my.step;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        fc.half[k] = my.half[k];
        fc.hf[k] = static_cast<float>(my.half[k]);
      }
      if (slot_advance<PREC == kFP32C>(sl, rec, nx, E.p, fc)) {
        __threadfence_system();  // the line's results before its completion count
        atomicAdd_system(E.done + my.req, 1);
        sl.line = -1;
      }
    }
    __syncwarp();
  }
}

__global__ void pack_pairs_kernel(int64_t n, int64_t n_pad, const double* __restrict__ x,
                                  const double* __restrict__ q, float4* __restrict__ out) {
  const int64_t n_pairs = n_pad / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pairs;
       p += (int64_t)gridDim.x * blockDim.x) {
    float c[2][4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t i = 2 * p + h;
      if (i < n) {
        c[h][0] = static_cast<float>(x[3 * i]);
        c[h][1] = static_cast<float>(x[3 * i + 1]);
        c[h][2] = static_cast<float>(x[3 * i + 2]);
        c[h][3] = static_cast<float>(q[i]);
      } else {  // zero charge far outside any box
        c[h][0] = c[h][1] = c[h][2] = 1.0e4f;
        c[h][3] = 0.f;
      }
    }
    out[p] = make_float4(c[0][0], c[1][0], c[0][1], c[1][1]);            // A
    out[n_pairs + p] = make_float4(c[0][2], c[1][2], c[0][3], c[1][3]);  // B
  }
}

// Dynamic shared memory: slot records, the mbarrier, and the resident sources
// (16 bytes per FP32C charge, 24 per FP32C dipole).
// Dipoles, FP32C: A[p] = {x, x', y, y'}, B[p] = {z, z', 3 mu_x, 3 mu_x'},
// C[p] = {mu_y, mu_y', mu_z, mu_z'} for the pair (2p, 2p + 1); padding =
// zero moments far outside any box (they add exactly 0).
__global__ void pack_dipole_pairs_kernel(int64_t n, int64_t n_pad, const double* __restrict__ x,
                                         const double* __restrict__ mu, float4* __restrict__ out) {
  const int64_t n_pairs = n_pad / 2;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_pairs;
       p += (int64_t)gridDim.x * blockDim.x) {
    float c[2][6];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t i = 2 * p + h;
      const bool in = i < n;
      c[h][0] = in ? static_cast<float>(x[3 * i]) : 1.0e4f;
      c[h][1] = in ? static_cast<float>(x[3 * i + 1]) : 1.0e4f;
      c[h][2] = in ? static_cast<float>(x[3 * i + 2]) : 1.0e4f;
      c[h][3] = in ? static_cast<float>(3.0 * mu[3 * i]) : 0.f;
      c[h][4] = in ? static_cast<float>(mu[3 * i + 1]) : 0.f;
      c[h][5] = in ? static_cast<float>(mu[3 * i + 2]) : 0.f;
    }
    out[p] = make_float4(c[0][0], c[1][0], c[0][1], c[1][1]);
    out[n_pairs + p] = make_float4(c[0][2], c[1][2], c[0][3], c[1][3]);
    out[2 * n_pairs + p] = make_float4(c[0][4], c[1][4], c[0][5], c[1][5]);
  }
}

__global__ void pack_dipole64_kernel(int64_t n, int64_t n_pad, const double* __restrict__ x,
                                     const double* __restrict__ mu, Dipole64* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad;
       i += (int64_t)gridDim.x * blockDim.x) {
    Dipole64 d;
    if (i < n) {
      d.x = x[3 * i]; d.y = x[3 * i + 1]; d.z = x[3 * i + 2];
      d.mx = mu[3 * i]; d.my = mu[3 * i + 1]; d.mz = mu[3 * i + 2];
    } else {
      d.x = d.y = d.z = 1.0e4;
      d.mx = d.my = d.mz = 0.0;
    }
    out[i] = d;
  }
}

size_t topo_smem_bytes(int S, int max_resident_pad, bool dip = false) {
  return sizeof(SlotRec) * kTopoWarps * S + 128 +
         static_cast<size_t>(max_resident_pad) * (dip ? 24 : 16);
}

template <int PREC, int RES, int S, bool DIP>
cudaError_t launch_topo_t(const TopoParams& p, const TopoFrame& f0, int total_lines, int num_sms,
                          cudaStream_t s) {
  const size_t smem = topo_smem_bytes(S, RES != kResNone ? p.max_resident_pad : 0, DIP);
  cudaError_t err = cudaFuncSetAttribute(topo_kernel<PREC, RES, S, DIP>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
  if (err != cudaSuccess) return err;
  int per_sm = 1;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, topo_kernel<PREC, RES, S, DIP>,
                                                      kTopoThreads, smem);
  if (err != cudaSuccess) return err;
  per_sm = std::max(per_sm, 1);
  const int max_useful = (total_lines + kTopoWarps * S - 1) / (kTopoWarps * S);
  const int grid = std::max(1, std::min(num_sms * per_sm, max_useful));
  topo_kernel<PREC, RES, S, DIP><<<grid, kTopoThreads, smem, s>>>(p, f0);
  return cudaGetLastError();
}

__global__ void pack_frames_kernel(int prec, const TopoFrame* __restrict__ frames,
                                   const int64_t* __restrict__ src, const double* __restrict__ x,
                                   const double* __restrict__ q, void* __restrict__ packed) {
  const int f = blockIdx.y;
  const TopoFrame fr = frames[f];
  const int64_t off = src[2 * f], n = src[2 * f + 1];
  const double* fx = x + 3 * off;
  const double* fq = q + off;
  if (prec == kFP32C) {
    float4* out = static_cast<float4*>(packed) + fr.packed_off;
    const int64_t n_pairs = fr.n_pad / 2;
    for (int64_t pp = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pp < n_pairs;
         pp += (int64_t)gridDim.x * blockDim.x) {
      float c[2][4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t i = 2 * pp + h;
        if (i < n) {
          c[h][0] = static_cast<float>(fx[3 * i]);
          c[h][1] = static_cast<float>(fx[3 * i + 1]);
          c[h][2] = static_cast<float>(fx[3 * i + 2]);
          c[h][3] = static_cast<float>(fq[i]);
        } else {
          c[h][0] = c[h][1] = c[h][2] = 1.0e4f;
          c[h][3] = 0.f;
        }
      }
      out[pp] = make_float4(c[0][0], c[1][0], c[0][1], c[1][1]);
      out[n_pairs + pp] = make_float4(c[0][2], c[1][2], c[0][3], c[1][3]);
    }
  } else {
    Charge64* out = static_cast<Charge64*>(packed) + fr.packed_off;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < fr.n_pad;
         i += (int64_t)gridDim.x * blockDim.x) {
      Charge64 c;
      if (i < n) {
        c.x = fx[3 * i];
        c.y = fx[3 * i + 1];
        c.z = fx[3 * i + 2];
        c.q = fq[i];
      } else {
        c.x = c.y = c.z = 1.0e4;
        c.q = 0.0;
      }
      out[i] = c;
    }
  }
}

}  // namespace

int topo_charge_pad(int prec) { return prec == kFP32C ? kChargePad32 : kChargePad64; }

int engine_threads() { return kEngineThreads; }

// ctas = SMs x CTAs per SM (1 or 2; a CTA takes half of an SM's registers).
// At one CTA per SM the engine runs beside grid launches: its SMs keep the
// largest shared-memory carveout so grid blocks (33 KB of staged charge
// tiles) fit next to it.
cudaError_t launch_engine(int prec, const EngineParams& e, int ctas, cudaStream_t s) {
  cudaError_t err;
  if (prec == kFP32C) {
    err = cudaFuncSetAttribute(engine_kernel<kFP32C, 4>,
                               cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (err != cudaSuccess) return err;
    engine_kernel<kFP32C, 4><<<ctas, kEngineThreads, 0, s>>>(e);
  } else {
    err = cudaFuncSetAttribute(engine_kernel<kFP64, 4>,
                               cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (err != cudaSuccess) return err;
    engine_kernel<kFP64, 4><<<ctas, kEngineThreads, 0, s>>>(e);
  }
  return cudaGetLastError();
}

// Charges (or dipoles) of a frame held in shared memory: all of them when the
// frame fits, else the largest prefix of whole Kahan runs (32 x kLanePairs
// pairs) that fits; 0 for FP64.
int topo_resident_count(int prec, int source, int n_pad) {
  const int limit = static_cast<int>(topo_resident_limit(prec, source));
  if (limit <= 0) return 0;
  if (n_pad <= limit) return n_pad;
  constexpr int kRun = 2 * 32 * kLanePairs;
  return (limit / kRun) * kRun;
}

size_t topo_resident_limit(int prec, int source) {
  if (prec != kFP32C) return 0;  // FP64 sources are read from global memory (L2)
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t fixed = topo_smem_bytes(4, 0) + 256;  // + static shared memory
  if (optin <= static_cast<int>(fixed)) return 0;
  size_t n = (static_cast<size_t>(optin) - fixed) / (source == kDipoles ? 24 : 16);
  return (n / kChargePad32) * kChargePad32;
}

cudaError_t launch_pack_dipoles(int prec, int64_t n, int64_t n_pad, const double* x,
                                const double* mu, void* packed, cudaStream_t s) {
  if (n_pad <= 0) return cudaSuccess;
  if (prec == kFP32C) {
    const int blocks = static_cast<int>(std::min<int64_t>((n_pad / 2 + 255) / 256, 4096));
    pack_dipole_pairs_kernel<<<blocks, 256, 0, s>>>(n, n_pad, x, mu, static_cast<float4*>(packed));
  } else {
    const int blocks = static_cast<int>(std::min<int64_t>((n_pad + 255) / 256, 4096));
    pack_dipole64_kernel<<<blocks, 256, 0, s>>>(n, n_pad, x, mu, static_cast<Dipole64*>(packed));
  }
  return cudaGetLastError();
}

size_t topo_source_bytes(int prec, int source) {
  if (source == kDipoles) return prec == kFP32C ? 24 : sizeof(Dipole64);
  return prec == kFP32C ? 16 : sizeof(Charge64);
}

cudaError_t launch_pack_topo(int prec, int64_t n, int64_t n_pad, const double* x, const double* q,
                             void* packed, cudaStream_t s) {
  if (prec != kFP32C) return launch_pack_charges(prec, n, n_pad, x, q, packed, s);
  if (n_pad <= 0) return cudaSuccess;
  const int blocks = static_cast<int>(std::min<int64_t>((n_pad / 2 + 255) / 256, 4096));
  pack_pairs_kernel<<<blocks, 256, 0, s>>>(n, n_pad, x, q, static_cast<float4*>(packed));
  return cudaGetLastError();
}

cudaError_t launch_pack_topo_frames(int prec, int n_frames, const TopoFrame* d_frames,
                                    const int64_t* d_src, const double* x, const double* q,
                                    void* packed, int max_pairs, cudaStream_t s) {
  if (n_frames <= 0) return cudaSuccess;
  const int bx = std::max(1, std::min((max_pairs + 255) / 256, 256));
  pack_frames_kernel<<<dim3(bx, n_frames), 256, 0, s>>>(prec, d_frames, d_src, x, q, packed);
  return cudaGetLastError();
}

template <int PREC, int RES, bool DIP = false>
cudaError_t launch_topo_s(const TopoParams& p, const TopoFrame& f0, int total_lines, int num_sms,
                          cudaStream_t s, int slots) {
  return slots == 2 ? launch_topo_t<PREC, RES, 2, DIP>(p, f0, total_lines, num_sms, s)
                    : launch_topo_t<PREC, RES, 4, DIP>(p, f0, total_lines, num_sms, s);
}

// FP32C launch by residency mode; FP64 frames are never resident.
template <bool DIP>
cudaError_t launch_topo_mode(int prec, int mode, const TopoParams& p, const TopoFrame& f0,
                             int num_sms, cudaStream_t s, int slots) {
  if (prec == kFP64) return launch_topo_s<kFP64, kResNone, DIP>(p, f0, p.n_lines, num_sms, s, slots);
  if (mode == kResWhole) return launch_topo_s<kFP32C, kResWhole, DIP>(p, f0, p.n_lines, num_sms, s, slots);
  if (mode == kResAny) return launch_topo_s<kFP32C, kResAny, DIP>(p, f0, p.n_lines, num_sms, s, slots);
  return launch_topo_s<kFP32C, kResNone, DIP>(p, f0, p.n_lines, num_sms, s, slots);
}

// Single frame: p.packed holds round_up(n_charges, topo_charge_pad(prec)) charges
// packed by launch_pack_topo (the tail being zero charges far from the box).
cudaError_t launch_topo(int prec, const TopoParams& p_in, int num_sms, cudaStream_t s) {
  if (p_in.n_lines <= 0) return cudaSuccess;
  TopoParams p = p_in;
  const int pad = topo_charge_pad(prec);
  TopoFrame f0;
  f0.packed_off = 0;
  f0.line_off = 0;
  f0.n_pad = ((std::max(p.n_charges, 1) + pad - 1) / pad) * pad;
  f0.n_lines = p.n_lines;
  f0.resident = topo_resident_count(prec, p.source, f0.n_pad);
  f0.pad_ = 0;
  f0.step = p.step;
  for (int k = 0; k < 3; ++k) f0.half[k] = p.half[k];
  p.frames = nullptr;
  p.n_frames = 1;
  p.max_resident_pad = f0.resident;
  const int slots = tuned_topo_slots(prec, f0.resident == f0.n_pad, p.n_lines);
  const int mode = f0.resident == 0 ? kResNone : (f0.resident == f0.n_pad ? kResWhole : kResAny);
  if (p.source == kDipoles) return launch_topo_mode<true>(prec, mode, p, f0, num_sms, s, slots);
  return launch_topo_mode<false>(prec, mode, p, f0, num_sms, s, slots);
}

cudaError_t launch_topo_frames(int prec, const TopoParams& p, int num_sms, cudaStream_t s) {
  if (p.n_frames <= 0 || p.n_lines <= 0) return cudaSuccess;
  TopoFrame dummy{};
  const int slots = tuned_topo_slots(prec, p.all_resident != 0, p.n_lines);
  // kResWhole when no frame is partly resident (all_resident: every frame whole)
  const int mode = p.max_resident_pad <= 0 ? kResNone : (p.all_resident ? kResWhole : kResAny);
  return launch_topo_mode<false>(prec, mode, p, dummy, num_sms, s, slots);
}

}  // namespace cpetgb

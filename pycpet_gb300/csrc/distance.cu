// distance.cu -- all-pairs distance matrices over many topology histograms or
// volume fields: the clustering front end that consumes the streamline and
// volume results.
//
// Replaces construct_distance_matrix (CPET/utils/calculator.py:1003-1015: a
// scikit-learn pairwise_distances call with the numpy metric distance_numpy,
// calculator.py:975-978) and construct_distance_matrix_volume
// (calculator.py:1042-1058, a Python double loop over field pairs):
//   chi2   D[i][j] = 1/2 sum_k (a_k - b_k)^2 / (a_k + b_k), terms whose
//          a_k + b_k == 0 contribute nothing (distance_numpy's where= mask);
//   field  D[i][j] = sum_p |f_i[p] - f_j[p]|, the Euclidean norm of the
//          3-vector difference at each grid point, summed over the points.
// Both are symmetric with a zero diagonal.
//
// One CTA computes a 64 x 64 tile of the upper triangle (tiles below the
// diagonal return at once) and writes it and its mirror image.  When there are
// too few tiles to fill the GPU (fewer than about four per SM) the features are
// split over several CTAs per tile whose partial sums are added afterwards in
// split order, so the result does not depend on scheduling.  The features
// (histogram bins or grid points) stream through shared memory in chunks of
// 32 bins or 8-16 points, transposed so that for one feature a thread reads
// its 4 rows and 4 columns as broadcast loads; each thread owns 4 x 4 matrix
// entries.
//   FP64   every operation in IEEE double; the per-point norm is formed as
//          numpy forms it, (dx*dx + dy*dy) + dz*dz then sqrt, with no fused
//          multiply-add, so only the order of the final sum differs.
//   FP32C  values rounded to FP32 once before the launch; chi2 terms use the
//          MUFU reciprocal (two columns per packed f32x2 instruction), field
//          terms the MUFU reciprocal square root; each staged chunk is summed
//          plainly and Kahan-added (Kahan 1965) into a running (sum,
//          compensation) pair.
// The term of (i, j) equals the term of (j, i) bit for bit in both forms, so
// a tile on the diagonal writes an exactly symmetric block.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kTile = 64;      // matrix rows / columns per CTA
constexpr int kThreads = 256;  // 16 x 16 threads, 4 x 4 entries each

// Features staged per step: 32 histogram bins, or 16 (FP32) / 8 (FP64) grid
// points, keeping both staged tiles at or under 33 KB.
template <typename Real, int NC>
constexpr int chunk_of() {
  return NC == 1 ? 32 : (sizeof(Real) == 4 ? 16 : 8);
}

__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

__device__ __forceinline__ float rcp_mufu(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <typename Real>
struct Acc;  // running sum of one matrix entry
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ void add(double t) { s = __dadd_rn(s, t); }
  __device__ double value() const { return s; }
};
template <>
struct Acc<float> {
  float s = 0.f, c = 0.f;
  __device__ void add(float t) { kahan_add(s, c, t); }
  __device__ double value() const { return static_cast<double>(s) - static_cast<double>(c); }
};

// One staged feature of one row: a histogram bin, or a grid point's vector
// padded to 4 components so that it is a single (FP32) or double (FP64)
// vector load.
template <typename Real, int NC>
struct Feat;
template <typename Real>
struct Feat<Real, 1> {
  Real v;
};
template <typename Real>
struct alignas(4 * sizeof(Real)) Feat<Real, 3> {
  Real x, y, z, w;
};

__device__ __forceinline__ double chi2_term(double a, double b) {
  const double s = __dadd_rn(a, b);
  const double d = __dsub_rn(a, b);
  return s != 0.0 ? __ddiv_rn(__dmul_rn(d, d), s) : 0.0;
}
__device__ __forceinline__ float chi2_term(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float d = __fsub_rn(a, b);
  const float r = s != 0.f ? rcp_mufu(s) : 0.f;
  return __fmul_rn(__fmul_rn(d, d), r);
}

template <typename Real>
__device__ __forceinline__ Real term(const Feat<Real, 1>& a, const Feat<Real, 1>& b) {
  return chi2_term(a.v, b.v);
}
__device__ __forceinline__ double term(const Feat<double, 3>& a, const Feat<double, 3>& b) {
  const double dx = __dsub_rn(a.x, b.x), dy = __dsub_rn(a.y, b.y), dz = __dsub_rn(a.z, b.z);
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}
__device__ __forceinline__ float term(const Feat<float, 3>& a, const Feat<float, 3>& b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
  return __fmul_rn(r2, rsqrt_mufu(fmaxf(r2, 1e-37f)));  // r2 == 0 gives 0
}

template <typename Real, int NC>
__device__ __forceinline__ void load_feat(Feat<Real, NC>& f, const double* p, bool ok) {
  if constexpr (NC == 1) {
    f.v = ok ? static_cast<Real>(p[0]) : Real(0);
  } else {
    f.x = ok ? static_cast<Real>(p[0]) : Real(0);
    f.y = ok ? static_cast<Real>(p[1]) : Real(0);
    f.z = ok ? static_cast<Real>(p[2]) : Real(0);
    f.w = Real(0);
  }
}

// KIND 0: chi2 over `feat` bins of rows of `src` ([n][feat] doubles).
// KIND 1: field norm over `feat` points of rows of `src` ([n][feat][3] doubles).
// blockIdx.z = feature split: features [z * per, min(feat, (z+1) * per)).
// With one split the CTA writes the final matrix (halved for chi2, zero
// diagonal); with several it writes its partial sums to part[z][n][n].
template <typename Real, int KIND>
__global__ void __launch_bounds__(kThreads)
    distance_kernel(int n, int feat, int per, const void* __restrict__ src_raw,
                    double* __restrict__ out, double* __restrict__ part_out) {
  constexpr int NC = KIND == 0 ? 1 : 3;  // components per feature
  constexpr int kChunk = chunk_of<Real, NC>();
  using F = Feat<Real, NC>;
  const int ib = blockIdx.y, jb = blockIdx.x;
  if (ib > jb) return;  // lower triangle: the mirror of a computed tile
  __shared__ F sA[kChunk][kTile + 1];
  __shared__ F sB[kChunk][kTile + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int i0 = ib * kTile, j0 = jb * kTile;
  const int64_t row_len = int64_t(feat) * NC;
  const int kb = blockIdx.z * per, ke = min(feat, kb + per);

  Acc<Real> acc[4][4];
  for (int k0 = kb; k0 < ke; k0 += kChunk) {
    __syncthreads();  // previous chunk consumed
    // stage rows i0.. and j0.. for features k0 .. k0+kChunk-1 (zero outside)
    for (int e = tid; e < kTile * kChunk; e += kThreads) {
      const int k = e % kChunk, row = e / kChunk, kk = k0 + k;
      const bool in = kk < ke;
      if constexpr (sizeof(Real) == 4) {  // FP32C: rows converted once to Feat<float, NC>
        const F* src = static_cast<const F*>(src_raw);
        const F zero{};
        sA[k][row] = (in && i0 + row < n) ? src[int64_t(i0 + row) * feat + kk] : zero;
        sB[k][row] = (in && j0 + row < n) ? src[int64_t(j0 + row) * feat + kk] : zero;
      } else {
        const double* src = static_cast<const double*>(src_raw);
        load_feat<Real, NC>(sA[k][row], src + (i0 + row) * row_len + int64_t(kk) * NC, in && i0 + row < n);
        load_feat<Real, NC>(sB[k][row], src + (j0 + row) * row_len + int64_t(kk) * NC, in && j0 + row < n);
      }
    }
    __syncthreads();
    Real part[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) part[r][c] = Real(0);
    const int kn = min(kChunk, ke - k0);
    if constexpr (KIND == 0 && sizeof(Real) == 4) {
      // chi2 in packed pairs of columns: one f32x2 instruction for two terms
      uint64_t p2[4][2];
#pragma unroll
      for (int r = 0; r < 4; ++r) p2[r][0] = p2[r][1] = 0ull;
#pragma unroll 4
      for (int k = 0; k < kn; ++k) {
        float a[4];
        uint64_t b2[2];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = reinterpret_cast<const float&>(sA[k][ty + 16 * r]);
        b2[0] = pk2(reinterpret_cast<const float&>(sB[k][tx]), reinterpret_cast<const float&>(sB[k][tx + 16]));
        b2[1] = pk2(reinterpret_cast<const float&>(sB[k][tx + 32]), reinterpret_cast<const float&>(sB[k][tx + 48]));
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const uint64_t aa = pk2(a[r], a[r]);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint64_t s2 = add2(aa, b2[h]);
            const uint64_t d2 = sub2(aa, b2[h]);
            float s0, s1;
            upk2(s2, s0, s1);
            const uint64_t rr = pk2(s0 != 0.f ? rcp_mufu(s0) : 0.f, s1 != 0.f ? rcp_mufu(s1) : 0.f);
            p2[r][h] = fma2(mul2(d2, d2), rr, p2[r][h]);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float lo, hi;
          upk2(p2[r][h], lo, hi);
          part[r][2 * h] = reinterpret_cast<Real&>(lo);
          part[r][2 * h + 1] = reinterpret_cast<Real&>(hi);
        }
    } else {
#pragma unroll 4
    for (int k = 0; k < kn; ++k) {
      F a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        a[r] = sA[k][ty + 16 * r];
        b[r] = sB[k][tx + 16 * r];
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const Real t = term(a[r], b[c]);
          if constexpr (sizeof(Real) == 8)
            part[r][c] = __dadd_rn(part[r][c], t);
          else
            part[r][c] = __fadd_rn(part[r][c], t);
        }
    }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c].add(part[r][c]);
  }

  double* dst = part_out ? part_out + int64_t(blockIdx.z) * n * n : out;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
      if (i >= n || j >= n) continue;
      double v = acc[r][c].value();
      if (!part_out) {
        if (KIND == 0) v *= 0.5;
        if (i == j) v = 0.0;
      }
      dst[int64_t(i) * n + j] = v;
      if (ib != jb) dst[int64_t(j) * n + i] = v;
    }
}

// FP32C staging source: every value rounded to float once (a field point
// padded to 4 components), instead of in every CTA that stages the row.
template <int NC>
__global__ void to_f32_kernel(int64_t n_feat, const double* __restrict__ in,
                              Feat<float, NC>* __restrict__ out) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n_feat;
       i += int64_t(gridDim.x) * blockDim.x)
    load_feat<float, NC>(out[i], in + i * NC, true);
}

// Sum of the feature splits in split order (deterministic); chi2 halved;
// zero diagonal.
__global__ void distance_reduce_kernel(int kind, int n, int splits, const double* __restrict__ part,
                                       double* __restrict__ out) {
  const int64_t nn = int64_t(n) * n;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < nn;
       e += int64_t(gridDim.x) * blockDim.x) {
    double v = part[e];
    for (int z = 1; z < splits; ++z) v = __dadd_rn(v, part[z * nn + e]);
    if (kind == 0) v *= 0.5;
    if (e / n == e % n) v = 0.0;
    out[e] = v;
  }
}

}  // namespace

int distance_splits(int n, int feat, int num_sms) {
  const int nb = (n + kTile - 1) / kTile;
  const int64_t tiles = int64_t(nb) * (nb + 1) / 2;
  const int64_t want = 4LL * num_sms;  // about four CTAs per SM
  if (tiles >= want || feat < 256) return 1;
  int s = static_cast<int>((want + tiles - 1) / tiles);
  return std::max(1, std::min(s, feat / 64));  // at least 64 features per split
}

size_t distance_f32_bytes(int kind, int n, int feat) {
  return size_t(n) * size_t(feat) * (kind == 0 ? sizeof(float) : sizeof(Feat<float, 3>));
}

cudaError_t launch_distance_matrix(int prec, int kind, int n, int feat, const double* src,
                                   double* out, int splits, double* partial, void* f32_rows,
                                   cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (prec != kFP64 && int64_t(n) * feat > 0) {
    const int64_t nf = int64_t(n) * feat;
    const int blocks = static_cast<int>(std::min<int64_t>((nf + 255) / 256, 8192));
    if (kind == 0)
      to_f32_kernel<1><<<blocks, 256, 0, s>>>(nf, src, static_cast<Feat<float, 1>*>(f32_rows));
    else
      to_f32_kernel<3><<<blocks, 256, 0, s>>>(nf, src, static_cast<Feat<float, 3>*>(f32_rows));
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  const int nb = (n + kTile - 1) / kTile;
  if (splits < 1 || feat == 0) splits = 1;
  const int per = (feat + splits - 1) / splits;
  double* pout = splits > 1 ? partial : nullptr;
  const dim3 grid(nb, nb, splits);
  if (prec == kFP64) {
    if (kind == 0)
      distance_kernel<double, 0><<<grid, kThreads, 0, s>>>(n, feat, per, src, out, pout);
    else
      distance_kernel<double, 1><<<grid, kThreads, 0, s>>>(n, feat, per, src, out, pout);
  } else {
    if (kind == 0)
      distance_kernel<float, 0><<<grid, kThreads, 0, s>>>(n, feat, per, f32_rows, out, pout);
    else
      distance_kernel<float, 1><<<grid, kThreads, 0, s>>>(n, feat, per, f32_rows, out, pout);
  }
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || splits == 1) return err;
  const int64_t nn = int64_t(n) * n;
  const int blocks = static_cast<int>(std::min<int64_t>((nn + 255) / 256, 4096));
  distance_reduce_kernel<<<blocks, 256, 0, s>>>(kind, n, splits, partial, out);
  return cudaGetLastError();
}

}  // namespace cpetgb

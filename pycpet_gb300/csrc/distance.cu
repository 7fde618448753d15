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
// diagonal return at once) and writes it and its mirror image.  The features
// (histogram bins or grid points) stream through shared memory in chunks of
// 32 bins or 8-16 points, transposed so that for one feature a thread reads
// its 4 rows and 4 columns as broadcast loads; each thread owns 4 x 4 matrix
// entries.
//   FP64   every operation in IEEE double; the per-point norm is formed as
//          numpy forms it, (dx*dx + dy*dy) + dz*dz then sqrt, with no fused
//          multiply-add, so only the order of the final sum differs.
//   FP32C  values rounded to FP32 as they are staged; chi2 terms use the MUFU
//          reciprocal, field terms the MUFU reciprocal square root; each
//          staged chunk is summed plainly and Kahan-added (Kahan 1965)
//          into a running (sum, compensation) pair.
// The term of (i, j) equals the term of (j, i) bit for bit in both forms, so
// a tile on the diagonal writes an exactly symmetric block.
#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kTile = 64;      // matrix rows / columns per CTA
constexpr int kThreads = 256;  // 16 x 16 threads, 4 x 4 entries each

// Features staged per step: 32 histogram bins, 16 (FP32) or 8 (FP64) grid
// points of 3 components, keeping both staged tiles under 48 KB.
template <typename Real, int NC>
constexpr int chunk_of() {
  return NC == 1 ? 32 : (sizeof(Real) == 4 ? 16 : 8);
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

__device__ __forceinline__ double norm_term(double ax, double ay, double az, double bx, double by,
                                            double bz) {
  const double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
  return sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}
__device__ __forceinline__ float norm_term(float ax, float ay, float az, float bx, float by,
                                           float bz) {
  const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
  return __fmul_rn(r2, rsqrt_mufu(fmaxf(r2, 1e-37f)));  // r2 == 0 gives 0
}

// KIND 0: chi2 over `feat` bins of rows of `src` ([n][feat] doubles).
// KIND 1: field norm over `feat` points of rows of `src` ([n][feat][3] doubles).
template <typename Real, int KIND>
__global__ void __launch_bounds__(kThreads)
    distance_kernel(int n, int feat, const double* __restrict__ src, double* __restrict__ out) {
  constexpr int NC = KIND == 0 ? 1 : 3;  // components per feature
  constexpr int kChunk = chunk_of<Real, NC>();
  const int ib = blockIdx.y, jb = blockIdx.x;
  if (ib > jb) return;  // lower triangle: the mirror of a computed tile
  __shared__ Real sA[NC][kChunk][kTile + 1];
  __shared__ Real sB[NC][kChunk][kTile + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int i0 = ib * kTile, j0 = jb * kTile;
  const int64_t row_len = int64_t(feat) * NC;

  Acc<Real> acc[4][4];
  for (int k0 = 0; k0 < feat; k0 += kChunk) {
    __syncthreads();  // previous chunk consumed
    // stage rows i0.. and j0.. for features k0 .. k0+kChunk-1 (zero outside the matrix)
    for (int e = tid; e < kTile * kChunk * NC; e += kThreads) {
      const int comp = e % NC, k = (e / NC) % kChunk, row = e / (NC * kChunk);
      const int kk = k0 + k;
      double va = 0.0, vb = 0.0;
      if (kk < feat) {
        if (i0 + row < n) va = src[(i0 + row) * row_len + int64_t(kk) * NC + comp];
        if (j0 + row < n) vb = src[(j0 + row) * row_len + int64_t(kk) * NC + comp];
      }
      sA[comp][k][row] = static_cast<Real>(va);
      sB[comp][k][row] = static_cast<Real>(vb);
    }
    __syncthreads();
    Real part[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) part[r][c] = Real(0);
    const int kn = min(kChunk, feat - k0);
#pragma unroll 4
    for (int k = 0; k < kn; ++k) {
      Real a[NC][4], b[NC][4];
#pragma unroll
      for (int q = 0; q < NC; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          a[q][r] = sA[q][k][ty + 16 * r];
          b[q][r] = sB[q][k][tx + 16 * r];
        }
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          Real t;
          if constexpr (KIND == 0)
            t = chi2_term(a[0][r], b[0][c]);
          else
            t = norm_term(a[0][r], a[1][r], a[2][r], b[0][c], b[1][c], b[2][c]);
          if constexpr (sizeof(Real) == 8)
            part[r][c] = __dadd_rn(part[r][c], t);
          else
            part[r][c] = __fadd_rn(part[r][c], t);
        }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c].add(part[r][c]);
  }

#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
      if (i >= n || j >= n) continue;
      double v = acc[r][c].value();
      if (KIND == 0) v *= 0.5;
      if (i == j) v = 0.0;
      out[int64_t(i) * n + j] = v;
      if (ib != jb) out[int64_t(j) * n + i] = v;
    }
}

}  // namespace

cudaError_t launch_distance_matrix(int prec, int kind, int n, int feat, const double* src,
                                   double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int nb = (n + kTile - 1) / kTile;
  const dim3 grid(nb, nb);
  if (prec == kFP64) {
    if (kind == 0)
      distance_kernel<double, 0><<<grid, kThreads, 0, s>>>(n, feat, src, out);
    else
      distance_kernel<double, 1><<<grid, kThreads, 0, s>>>(n, feat, src, out);
  } else {
    if (kind == 0)
      distance_kernel<float, 0><<<grid, kThreads, 0, s>>>(n, feat, src, out);
    else
      distance_kernel<float, 1><<<grid, kThreads, 0, s>>>(n, feat, src, out);
  }
  return cudaGetLastError();
}

}  // namespace cpetgb

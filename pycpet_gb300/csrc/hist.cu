// hist.cu -- 2-D histogram of per-line (distance, curvature) values (K4).
//
// Replaces the np.histogram2d call of make_histograms
// (CPET/utils/calculator.py:702-707), with numpy's binning rules reproduced
// exactly so that both sides give identical integer counts for identical
// values:
//   * edges = linspace(lo, hi, nbins + 1): delta = hi - lo, step = delta/nbins,
//     edge[i] = i*step + lo, edge[nbins] = hi (each operation rounded once,
//     no fused multiply-add);
//   * a degenerate range lo == hi is widened to [lo - 0.5, hi + 0.5];
//   * bin index = (number of edges <= x) - 1, a value equal to the last edge
//     goes to the last bin, values outside [lo, hi] and NaNs are dropped.
// A range bound given as NaN is taken from the data (min or max of that
// column, as make_histograms does with np.min / np.max, lines 664-667); a
// non-finite data bound sets the status word and no counts are produced.
// The set form bins many value sets (one per .top file of make_histograms,
// lines 689-711) with one binning in a single launch and can normalise each
// set's counts to sum 1.
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kRangeThreads = 1024;
constexpr int kBinThreads = 256;
constexpr int kMaxSharedBins = 8192;

__device__ __forceinline__ double linspace_at(double lo, double step, int i) {
  return __dadd_rn(__dmul_rn(static_cast<double>(i), step), lo);
}

// One block: resolve auto bounds, build both edge arrays.
__global__ void __launch_bounds__(kRangeThreads)
    hist_range_kernel(int n, const double* __restrict__ vals, int nb0, int nb1, double lo0,
                      double hi0, double lo1, double hi1, double* __restrict__ edges,
                      int* __restrict__ status) {
  __shared__ double red[4][kRangeThreads / 32];
  __shared__ double bounds[4];
  double mn0 = INFINITY, mx0 = -INFINITY, mn1 = INFINITY, mx1 = -INFINITY;
  bool nan0 = false, nan1 = false;
  const bool need = isnan(lo0) || isnan(hi0) || isnan(lo1) || isnan(hi1);
  if (need) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double a = vals[2 * i], b = vals[2 * i + 1];
      nan0 |= isnan(a);
      nan1 |= isnan(b);
      mn0 = fmin(mn0, a); mx0 = fmax(mx0, a);
      mn1 = fmin(mn1, b); mx1 = fmax(mx1, b);
    }
  }
  const int any0 = __syncthreads_or(nan0), any1 = __syncthreads_or(nan1);
  for (int off = 16; off >= 1; off >>= 1) {
    mn0 = fmin(mn0, __shfl_xor_sync(0xffffffffu, mn0, off));
    mx0 = fmax(mx0, __shfl_xor_sync(0xffffffffu, mx0, off));
    mn1 = fmin(mn1, __shfl_xor_sync(0xffffffffu, mn1, off));
    mx1 = fmax(mx1, __shfl_xor_sync(0xffffffffu, mx1, off));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = mn0; red[1][w] = mx0; red[2][w] = mn1; red[3][w] = mx1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kRangeThreads / 32; ++k) {
      red[0][0] = fmin(red[0][0], red[0][k]); red[1][0] = fmax(red[1][0], red[1][k]);
      red[2][0] = fmin(red[2][0], red[2][k]); red[3][0] = fmax(red[3][0], red[3][k]);
    }
    double b[4] = {lo0, hi0, lo1, hi1};
    // np.min / np.max propagate NaN; an empty column gives no finite bound.
    if (isnan(b[0])) b[0] = any0 ? NAN : red[0][0];
    if (isnan(b[1])) b[1] = any0 ? NAN : red[1][0];
    if (isnan(b[2])) b[2] = any1 ? NAN : red[2][0];
    if (isnan(b[3])) b[3] = any1 ? NAN : red[3][0];
    bool bad = false;
    for (int d = 0; d < 2; ++d) {
      double lo = b[2 * d], hi = b[2 * d + 1];
      if (!isfinite(lo) || !isfinite(hi) || lo > hi) bad = true;
      if (lo == hi) {  // numpy widens a zero-width range
        lo = __dsub_rn(lo, 0.5);
        hi = __dadd_rn(hi, 0.5);
      }
      bounds[2 * d] = lo;
      bounds[2 * d + 1] = hi;
    }
    if (bad) atomicCAS(status, kDevOk, kDevBadArgument);
  }
  __syncthreads();
  if (*(volatile int*)status != kDevOk) return;
  for (int d = 0; d < 2; ++d) {
    const int nb = d == 0 ? nb0 : nb1;
    double* e = edges + (d == 0 ? 0 : nb0 + 1);
    const double lo = bounds[2 * d], hi = bounds[2 * d + 1];
    const double step = __ddiv_rn(__dsub_rn(hi, lo), static_cast<double>(nb));
    for (int i = threadIdx.x; i <= nb; i += blockDim.x) e[i] = (i == nb) ? hi : linspace_at(lo, step, i);
  }
}

// Index of x's bin among nb bins with edges e[0..nb], or -1 when dropped.
__device__ __forceinline__ int bin_of(double x, const double* e, int nb) {
  if (isnan(x)) return -1;
  // count of edges <= x (upper bound), edges non-decreasing
  int lo = 0, hi = nb + 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (e[mid] <= x)
      lo = mid + 1;
    else
      hi = mid;
  }
  int idx = lo;
  if (x == e[nb]) idx -= 1;
  if (idx <= 0 || idx > nb) return -1;
  return idx - 1;
}

__global__ void __launch_bounds__(kBinThreads)
    hist_bin_kernel(int n, const double* __restrict__ vals, int nb0, int nb1,
                    const double* __restrict__ edges, unsigned long long* __restrict__ counts,
                    const int* __restrict__ status, int shared_bins) {
  extern __shared__ unsigned char sraw[];
  if (*status != kDevOk) return;
  double* e0 = reinterpret_cast<double*>(sraw);
  double* e1 = e0 + nb0 + 1;
  unsigned int* sh = reinterpret_cast<unsigned int*>(e1 + nb1 + 1);
  const int nbins = nb0 * nb1;
  for (int i = threadIdx.x; i <= nb0; i += blockDim.x) e0[i] = edges[i];
  for (int i = threadIdx.x; i <= nb1; i += blockDim.x) e1[i] = edges[nb0 + 1 + i];
  if (shared_bins)
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int b0 = bin_of(vals[2 * i], e0, nb0);
    const int b1 = bin_of(vals[2 * i + 1], e1, nb1);
    if (b0 < 0 || b1 < 0) continue;
    if (shared_bins)
      atomicAdd(&sh[b0 * nb1 + b1], 1u);
    else
      atomicAdd(&counts[b0 * nb1 + b1], 1ull);
  }
  if (!shared_bins) return;
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (sh[i]) atomicAdd(&counts[i], static_cast<unsigned long long>(sh[i]));
}

// Many value sets with one binning: set f = blockIdx.y holds the values
// [off[f], off[f + 1]) and counts into counts[f][nb0 * nb1].
__global__ void __launch_bounds__(kBinThreads)
    hist_bin_sets_kernel(const int64_t* __restrict__ off, const double* __restrict__ vals, int nb0,
                         int nb1, const double* __restrict__ edges,
                         unsigned long long* __restrict__ counts, const int* __restrict__ status,
                         int shared_bins) {
  extern __shared__ unsigned char sraw[];
  if (*status != kDevOk) return;
  double* e0 = reinterpret_cast<double*>(sraw);
  double* e1 = e0 + nb0 + 1;
  unsigned int* sh = reinterpret_cast<unsigned int*>(e1 + nb1 + 1);
  const int nbins = nb0 * nb1;
  const int f = blockIdx.y;
  const int64_t begin = off[f], end = off[f + 1];
  unsigned long long* cf = counts + int64_t(f) * nbins;
  for (int i = threadIdx.x; i <= nb0; i += blockDim.x) e0[i] = edges[i];
  for (int i = threadIdx.x; i <= nb1; i += blockDim.x) e1[i] = edges[nb0 + 1 + i];
  if (shared_bins)
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
  for (int64_t i = begin + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < end;
       i += int64_t(gridDim.x) * blockDim.x) {
    const int b0 = bin_of(vals[2 * i], e0, nb0);
    const int b1 = bin_of(vals[2 * i + 1], e1, nb1);
    if (b0 < 0 || b1 < 0) continue;
    if (shared_bins)
      atomicAdd(&sh[b0 * nb1 + b1], 1u);
    else
      atomicAdd(&cf[b0 * nb1 + b1], 1ull);
  }
  if (!shared_bins) return;
  __syncthreads();
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    if (sh[i]) atomicAdd(&cf[i], static_cast<unsigned long long>(sh[i]));
}

// hists[f][b] = counts[f][b] / sum_b counts[f][b] in IEEE double: the integer
// total is exact, so this is make_histograms' a / np.sum(a) bit for bit
// (CPET/utils/calculator.py:709-711); an empty set gives NaN as numpy does.
__global__ void __launch_bounds__(kBinThreads)
    hist_normalise_kernel(int nbins, const unsigned long long* __restrict__ counts,
                          double* __restrict__ hists) {
  __shared__ unsigned long long red[kBinThreads / 32];
  const int f = blockIdx.x;
  const unsigned long long* cf = counts + int64_t(f) * nbins;
  unsigned long long t = 0;
  for (int i = threadIdx.x; i < nbins; i += blockDim.x) t += cf[i];
  for (int o = 16; o >= 1; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  unsigned long long total = 0;
  for (int w = 0; w < kBinThreads / 32; ++w) total += red[w];
  const double dt = static_cast<double>(total);
  for (int i = threadIdx.x; i < nbins; i += blockDim.x)
    hists[int64_t(f) * nbins + i] = __ddiv_rn(static_cast<double>(cf[i]), dt);
}

}  // namespace

// Many sets, one binning: range {lo0, hi0, lo1, hi1} finite (host); d_off the
// device copy of the set offsets [n_sets + 1]; counts [n_sets][nb0*nb1] zeroed;
// hists (optional) receives the normalised histograms.
cudaError_t launch_hist2d_sets(int n_sets, const int64_t* d_off, int64_t max_set,
                               const double* vals, int nb0, int nb1, const double* range,
                               double* edges, unsigned long long* counts, double* hists,
                               int* status, cudaStream_t s) {
  if (n_sets <= 0) return cudaSuccess;
  hist_range_kernel<<<1, kRangeThreads, 0, s>>>(0, vals, nb0, nb1, range[0], range[1], range[2],
                                                range[3], edges, status);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const int nbins = nb0 * nb1;
  size_t smem = sizeof(double) * (nb0 + nb1 + 2);
  const int shared_bins =
      (nbins <= kMaxSharedBins && smem + sizeof(unsigned int) * nbins <= 48 * 1024) ? 1 : 0;
  if (shared_bins) smem += sizeof(unsigned int) * nbins;
  if (smem > 48 * 1024) return cudaErrorInvalidValue;  // callers keep nb0 + nb1 <= 4096
  const int64_t per = (max_set + kBinThreads * 4 - 1) / (kBinThreads * 4);
  const int bx = static_cast<int>(per < 1 ? 1 : (per > 64 ? 64 : per));
  hist_bin_sets_kernel<<<dim3(bx, n_sets), kBinThreads, smem, s>>>(d_off, vals, nb0, nb1, edges,
                                                                   counts, status, shared_bins);
  err = cudaGetLastError();
  if (err != cudaSuccess || !hists) return err;
  hist_normalise_kernel<<<n_sets, kBinThreads, 0, s>>>(nbins, counts, hists);
  return cudaGetLastError();
}

// range: {lo0, hi0, lo1, hi1} on the host; NaN = from the data.
// counts (nb0*nb1, row-major over (distance bin, curvature bin)) must be zeroed.
cudaError_t launch_hist2d(int n, const double* vals, int nb0, int nb1, const double* range,
                          double* edges, unsigned long long* counts, int* status,
                          cudaStream_t s) {
  hist_range_kernel<<<1, kRangeThreads, 0, s>>>(n, vals, nb0, nb1, range[0], range[1], range[2],
                                                range[3], edges, status);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  const int nbins = nb0 * nb1;
  size_t smem = sizeof(double) * (nb0 + nb1 + 2);
  const int shared_bins =
      (nbins <= kMaxSharedBins && smem + sizeof(unsigned int) * nbins <= 48 * 1024) ? 1 : 0;
  if (shared_bins) smem += sizeof(unsigned int) * nbins;
  if (smem > 48 * 1024) return cudaErrorInvalidValue;  // callers keep nb0 + nb1 <= 4096
  int blocks = (n + kBinThreads - 1) / kBinThreads;
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  hist_bin_kernel<<<blocks, kBinThreads, smem, s>>>(n, vals, nb0, nb1, edges, counts, status,
                                                    shared_bins);
  return cudaGetLastError();
}

}  // namespace cpetgb

// format.cu -- fixed-point text of volume outputs, formatted on the GPU.
//
// Replaces the body of save_numpy_as_dat (CPET/utils/io.py:50-109), which
// writes the (P,6) float32 field or (P,4) float16 potential rows of a volume
// with numpy.savetxt(fmt="%.3f"): per row the values formatted as "%.3f",
// joined by single spaces, ended by "\n".  At 51^3 points per frame this text
// formatting costs about a thousand times the field evaluation itself.
//
// Exactness: "%.3f" of a float32 value (widened to double, as numpy hands it
// to Python's formatter) is its exact binary value rounded to three decimals,
// ties to even.  For |v| < 2^24, v * 1000 is exact in double (a 24-bit
// significand times a 10-bit integer), so rint() of it is the correctly
// rounded value in thousandths.  Every float32 of magnitude >= 2^24 is an
// integer; it is printed exactly from its significand and exponent with
// 128-bit integer arithmetic, followed by ".000".  NaN prints as "nan", the
// infinities as "inf" / "-inf", and a negative value that rounds to zero keeps
// its sign ("-0.000"), as Python's formatting does.
//
// Three passes: the length of every row, an exclusive scan of the lengths,
// then every row written at its offset.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 8;  // rows per thread in the scan
constexpr int kScanTile = kScanThreads * kScanItems;

// Decimal digits of an unsigned 128-bit integer (at least 1).
__device__ __forceinline__ int digits128(unsigned __int128 v) {
  int d = 1;
  while (v >= 10) {
    v /= 10;
    ++d;
  }
  return d;
}

struct Fixed3 {
  int kind;                 // 0 finite, 1 nan, 2 +inf, 3 -inf
  bool neg;
  unsigned __int128 ip;     // integer part
  int frac;                 // thousandths 0..999
};

__device__ __forceinline__ Fixed3 decompose(float f) {
  Fixed3 r;
  r.kind = 0;
  r.neg = signbit(f);
  r.ip = 0;
  r.frac = 0;
  if (isnan(f)) {
    r.kind = 1;
    return r;
  }
  if (isinf(f)) {
    r.kind = r.neg ? 3 : 2;
    return r;
  }
  const double a = fabs(static_cast<double>(f));
  if (a < 16777216.0) {  // 2^24: a * 1000 exact, below 2^34
    const uint64_t n = static_cast<uint64_t>(rint(a * 1000.0));
    r.ip = n / 1000;
    r.frac = static_cast<int>(n % 1000);
  } else {  // an integer: significand << exponent
    int e;
    const double m = frexp(a, &e);                           // a = m 2^e, m in [0.5, 1)
    const uint64_t sig = static_cast<uint64_t>(ldexp(m, 24));  // 24-bit integer
    r.ip = static_cast<unsigned __int128>(sig) << (e - 24);
  }
  return r;
}

__device__ __forceinline__ int fixed3_len(float f) {
  const Fixed3 r = decompose(f);
  if (r.kind == 1 || r.kind == 2) return 3;
  if (r.kind == 3) return 4;
  return (r.neg ? 1 : 0) + digits128(r.ip) + 4;
}

__device__ __forceinline__ char* fixed3_write(float f, char* o) {
  const Fixed3 r = decompose(f);
  if (r.kind == 1) {
    o[0] = 'n'; o[1] = 'a'; o[2] = 'n';
    return o + 3;
  }
  if (r.kind >= 2) {
    if (r.kind == 3) *o++ = '-';
    o[0] = 'i'; o[1] = 'n'; o[2] = 'f';
    return o + 3;
  }
  if (r.neg) *o++ = '-';
  const int nd = digits128(r.ip);
  unsigned __int128 v = r.ip;
  for (int k = nd - 1; k >= 0; --k) {
    o[k] = static_cast<char>('0' + static_cast<int>(v % 10));
    v /= 10;
  }
  o += nd;
  o[0] = '.';
  o[1] = static_cast<char>('0' + r.frac / 100);
  o[2] = static_cast<char>('0' + (r.frac / 10) % 10);
  o[3] = static_cast<char>('0' + r.frac % 10);
  return o + 4;
}

__global__ void row_len_kernel(int64_t n_rows, int n_cols, const float* __restrict__ v,
                               int64_t* __restrict__ len) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows;
       r += int64_t(gridDim.x) * blockDim.x) {
    int64_t l = n_cols;  // n_cols - 1 separators + the newline
    for (int c = 0; c < n_cols; ++c) l += fixed3_len(v[r * n_cols + c]);
    len[r] = l;
  }
}

// In-place exclusive scan of x[0..n) tile by tile; tile sums to sums[].
__global__ void __launch_bounds__(kScanThreads)
    scan_tiles_kernel(int64_t n, int64_t* __restrict__ x, int64_t* __restrict__ sums) {
  __shared__ int64_t warp_tot[kScanThreads / 32];
  const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
  int64_t loc[kScanItems];
  int64_t t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    loc[k] = (base + k < n) ? x[base + k] : 0;
    t += loc[k];
  }
  // inclusive scan of the thread totals across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int64_t w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_tot[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  int64_t run = inc - t + (warp > 0 ? warp_tot[warp - 1] : 0);  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) x[base + k] = run;
    run += loc[k];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = run;
}

__global__ void add_tile_offsets_kernel(int64_t n, int64_t* __restrict__ x,
                                        const int64_t* __restrict__ tile_off) {
  const int64_t tile = blockIdx.x;
  const int64_t add = tile_off[tile];
  for (int64_t i = tile * kScanTile + threadIdx.x; i < min(n, (tile + 1) * kScanTile);
       i += blockDim.x)
    x[i] += add;
}

__global__ void write_rows_kernel(int64_t n_rows, int n_cols, const float* __restrict__ v,
                                  const int64_t* __restrict__ off, char* __restrict__ out) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows;
       r += int64_t(gridDim.x) * blockDim.x) {
    char* o = out + off[r];
    for (int c = 0; c < n_cols; ++c) {
      if (c) *o++ = ' ';
      o = fixed3_write(v[r * n_cols + c], o);
    }
    *o = '\n';
  }
}

}  // namespace

// Exclusive scan of n int64 values in place (recursive over tile sums).
// scratch holds at least scan_scratch_i64(n) values.
cudaError_t scan_exclusive_i64(int64_t n, int64_t* x, int64_t* scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  scan_tiles_kernel<<<static_cast<unsigned>(tiles), kScanThreads, 0, s>>>(n, x, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || tiles == 1) return e;
  e = scan_exclusive_i64(tiles, scratch, scratch + tiles, s);
  if (e != cudaSuccess) return e;
  add_tile_offsets_kernel<<<static_cast<unsigned>(tiles), 256, 0, s>>>(n, x, scratch);
  return cudaGetLastError();
}

int64_t scan_scratch_i64(int64_t n) {
  int64_t total = 0;
  while (n > 1) {
    n = (n + kScanTile - 1) / kScanTile;
    total += n;
  }
  return total + 1;
}

int64_t fixed3_scan_scratch(int64_t n) { return scan_scratch_i64(n); }

// offsets [n_rows + 1] and scan scratch (fixed3_scan_scratch) in device memory;
// offsets[n_rows] receives the total length.
cudaError_t launch_fixed3_offsets(int64_t n_rows, int n_cols, const float* v, int64_t* offsets,
                                  int64_t* scratch, cudaStream_t s) {
  if (n_rows <= 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);
  const int blocks = static_cast<int>(std::min<int64_t>((n_rows + 255) / 256, 8192));
  row_len_kernel<<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // offsets[n_rows] = 0 joins the scan so it ends up as the total
  e = cudaMemsetAsync(offsets + n_rows, 0, sizeof(int64_t), s);
  if (e != cudaSuccess) return e;
  return scan_exclusive_i64(n_rows + 1, offsets, scratch, s);
}

cudaError_t launch_fixed3_write(int64_t n_rows, int n_cols, const float* v, const int64_t* offsets,
                                char* out, cudaStream_t s) {
  if (n_rows <= 0) return cudaSuccess;
  const int blocks = static_cast<int>(std::min<int64_t>((n_rows + 255) / 256, 8192));
  write_rows_kernel<<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets, out);
  return cudaGetLastError();
}

}  // namespace cpetgb

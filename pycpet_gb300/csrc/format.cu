// format.cu -- text of volume and topology outputs, formatted on the GPU.
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
// "%.18e" (numpy.savetxt's default format, which writes every topology result
// to a .top file, CPET/source/CPET.py:123): a float32 value v = m * 2^e,
// widened exactly to double, printed with 19 significant digits, correctly
// rounded, ties to even, as d.dddddddddddddddddde+XX.  The digits are
// D = round(v * 10^(18 - E)) with E = floor(log10 v), computed exactly in
// integers: for 10^(18-E) >= 1, v * 10^k = m * 5^k * 2^(e+k), with m * 5^k held
// in 192 bits (k <= 63: float32 values reach down to 1.4e-45), shifted and
// rounded by its discarded bits; for v >= 10^19 (an integer below 2^128) by a
// 128-bit division by 10^(E-18).  E is estimated from the binary exponent and
// corrected by one when D falls outside [10^18, 10^19).  The method is the
// exact big-integer conversion of Steele & White / Gay ("Correctly rounded
// binary-decimal and decimal-binary conversions", 1990) specialised to float32.
// NaN prints as "nan" whatever its sign, the infinities as "inf" / "-inf",
// zeros as "0.000000000000000000e+00" with the sign kept.
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

struct FmtFixed3 {
  static __device__ __forceinline__ int len(float f) { return fixed3_len(f); }
  static __device__ __forceinline__ char* write(float f, char* o) { return fixed3_write(f, o); }
};

// ---- "%.18e" ----------------------------------------------------------------
// 192-bit unsigned integer, little-endian 64-bit limbs.
struct U192 {
  uint64_t w[3];
};

__device__ __forceinline__ void mul_small(U192& a, uint32_t f) {
  unsigned __int128 carry = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const unsigned __int128 p = static_cast<unsigned __int128>(a.w[i]) * f + carry;
    a.w[i] = static_cast<uint64_t>(p);
    carry = p >> 64;
  }
}
__device__ __forceinline__ bool bit_of(const U192& a, int i) {  // 0 <= i < 192
  return (a.w[i >> 6] >> (i & 63)) & 1ull;
}
__device__ __forceinline__ bool any_below(const U192& a, int i) {  // a bit below bit i set?
  for (int l = 0; l < 3 && 64 * l < i; ++l) {
    const int nb = min(64, i - 64 * l);
    const uint64_t mask = nb == 64 ? ~0ull : ((1ull << nb) - 1);
    if (a.w[l] & mask) return true;
  }
  return false;
}
// a >> r (0 < r < 192) and a << r (0 <= r < 192; false when bits fall off)
__device__ __forceinline__ void shr(U192& a, int r) {
  U192 o = {{0, 0, 0}};
  const int q = r >> 6, b = r & 63;
  for (int i = 0; i + q < 3; ++i) {
    o.w[i] = a.w[i + q] >> b;
    if (b && i + q + 1 < 3) o.w[i] |= a.w[i + q + 1] << (64 - b);
  }
  a = o;
}
__device__ __forceinline__ bool shl(U192& a, int r) {
  if (r == 0) return true;
  U192 o = {{0, 0, 0}};
  const int q = r >> 6, b = r & 63;
  for (int i = 2; i >= 0; --i) {
    if (i - q < 0) break;
    o.w[i] = a.w[i - q] << b;
    if (b && i - q - 1 >= 0) o.w[i] |= a.w[i - q - 1] >> (64 - b);
  }
  U192 back = o;
  shr(back, r);
  const bool ok = back.w[0] == a.w[0] && back.w[1] == a.w[1] && back.w[2] == a.w[2];
  a = o;
  return ok;
}

constexpr uint64_t kTen18 = 1000000000000000000ull;
constexpr uint64_t kTen19 = 10000000000000000000ull;

// floor(m 2^e 10^k) into d and how the discarded part compares with one half
// (cmp: -1 below, 0 equal, +1 above).  Returns 0 when d is in [1e18, 1e19),
// -1 when below, +1 when at or above 1e19.
__device__ int scaled_digits(uint32_t m, int e, int k, uint64_t& d, int& cmp) {
  cmp = -1;
  if (k >= 0) {
    U192 n = {{m, 0, 0}};
    for (int i = 0; i < k; ++i) mul_small(n, 5);
    const int s = e + k;  // m 10^k 2^e = (m 5^k) 2^(e+k)
    if (s >= 0) {
      if (!shl(n, s)) return 1;
    } else {
      const int r = -s;
      if (r >= 192) {
        d = 0;
        return -1;
      }
      const bool half = bit_of(n, r - 1);
      const bool sticky = r >= 2 && any_below(n, r - 1);
      cmp = half ? (sticky ? 1 : 0) : -1;
      shr(n, r);
    }
    if (n.w[1] || n.w[2] || n.w[0] >= kTen19) return 1;
    d = n.w[0];
    return d < kTen18 ? -1 : 0;
  }
  // v >= 10^19: an integer m 2^e (e >= 40, below 2^128), divided by 10^(-k)
  unsigned __int128 p = 1;
  for (int i = 0; i < -k; ++i) p *= 10;
  const unsigned __int128 v = static_cast<unsigned __int128>(m) << e;
  const unsigned __int128 q = v / p, r2 = 2 * (v % p);
  cmp = r2 > p ? 1 : (r2 == p ? 0 : -1);
  if (q >= kTen19) return 1;
  d = static_cast<uint64_t>(q);
  return d < kTen18 ? -1 : 0;
}

struct Sci18 {
  int kind;   // 0 finite, 1 nan, 2 +inf, 3 -inf
  bool neg;
  uint64_t d; // 19 significant digits (0 for a zero)
  int exp10;
};

__device__ Sci18 sci18(float f) {
  Sci18 r;
  r.kind = 0;
  r.neg = signbit(f);
  r.d = 0;
  r.exp10 = 0;
  if (isnan(f)) {
    r.kind = 1;
    return r;
  }
  if (isinf(f)) {
    r.kind = r.neg ? 3 : 2;
    return r;
  }
  const uint32_t bits = __float_as_uint(f);
  const uint32_t be = (bits >> 23) & 0xffu, frac = bits & 0x7fffffu;
  if (be == 0 && frac == 0) return r;  // zero
  const uint32_t m = be ? (frac | 0x800000u) : frac;
  const int e = be ? static_cast<int>(be) - 150 : -149;
  const int exp2 = e + (31 - __clz(static_cast<int>(m)));  // floor(log2 v)
  int E = static_cast<int>(floor(exp2 * 0.30102999566398120));
  uint64_t d = 0;
  int cmp = -1;
  for (int tries = 0; tries < 3; ++tries) {  // E_est is exact or one below
    const int c = scaled_digits(m, e, 18 - E, d, cmp);
    if (c == 0) break;
    E += c;
  }
  if (cmp > 0 || (cmp == 0 && (d & 1ull))) {
    if (++d == kTen19) {
      d = kTen18;
      ++E;
    }
  }
  r.d = d;
  r.exp10 = E;
  return r;
}

struct FmtSci18 {
  static __device__ __forceinline__ int len(float f) {
    const Sci18 r = sci18(f);
    if (r.kind == 1 || r.kind == 2) return 3;
    if (r.kind == 3) return 4;
    return (r.neg ? 1 : 0) + 24;  // d.<18>e+XX (|exponent| < 100 for float32)
  }
  static __device__ __forceinline__ char* write(float f, char* o) {
    const Sci18 r = sci18(f);
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
    uint64_t d = r.d;
    for (int k = 19; k >= 0; --k) {  // o[0] digit, o[1] '.', o[2..19] digits
      if (k == 1) continue;
      o[k] = static_cast<char>('0' + static_cast<int>(d % 10));
      d /= 10;
    }
    o[1] = '.';
    o[20] = 'e';
    o[21] = r.exp10 < 0 ? '-' : '+';
    const int a = r.exp10 < 0 ? -r.exp10 : r.exp10;
    o[22] = static_cast<char>('0' + a / 10);
    o[23] = static_cast<char>('0' + a % 10);
    return o + 24;
  }
};

template <class Fmt>
__global__ void row_len_kernel(int64_t n_rows, int n_cols, const float* __restrict__ v,
                               int64_t* __restrict__ len) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows;
       r += int64_t(gridDim.x) * blockDim.x) {
    int64_t l = n_cols;  // n_cols - 1 separators + the newline
    for (int c = 0; c < n_cols; ++c) l += Fmt::len(v[r * n_cols + c]);
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

template <class Fmt>
__global__ void write_rows_kernel(int64_t n_rows, int n_cols, const float* __restrict__ v,
                                  const int64_t* __restrict__ off, char* __restrict__ out) {
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < n_rows;
       r += int64_t(gridDim.x) * blockDim.x) {
    char* o = out + off[r];
    for (int c = 0; c < n_cols; ++c) {
      if (c) *o++ = ' ';
      o = Fmt::write(v[r * n_cols + c], o);
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
// offsets[n_rows] receives the total length.  fmt: kTextFixed3 or kTextSci18.
cudaError_t launch_text_offsets(int fmt, int64_t n_rows, int n_cols, const float* v,
                                int64_t* offsets, int64_t* scratch, cudaStream_t s) {
  if (n_rows <= 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);
  const int blocks = static_cast<int>(std::min<int64_t>((n_rows + 255) / 256, 8192));
  if (fmt == kTextSci18)
    row_len_kernel<FmtSci18><<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets);
  else
    row_len_kernel<FmtFixed3><<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // offsets[n_rows] = 0 joins the scan so it ends up as the total
  e = cudaMemsetAsync(offsets + n_rows, 0, sizeof(int64_t), s);
  if (e != cudaSuccess) return e;
  return scan_exclusive_i64(n_rows + 1, offsets, scratch, s);
}

cudaError_t launch_text_write(int fmt, int64_t n_rows, int n_cols, const float* v,
                              const int64_t* offsets, char* out, cudaStream_t s) {
  if (n_rows <= 0) return cudaSuccess;
  const int blocks = static_cast<int>(std::min<int64_t>((n_rows + 255) / 256, 8192));
  if (fmt == kTextSci18)
    write_rows_kernel<FmtSci18><<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets, out);
  else
    write_rows_kernel<FmtFixed3><<<blocks, 256, 0, s>>>(n_rows, n_cols, v, offsets, out);
  return cudaGetLastError();
}

}  // namespace cpetgb

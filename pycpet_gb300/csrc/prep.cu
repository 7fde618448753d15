// prep.cu -- frame preparation on the device: residue radius filter,
// rotation into the box frame, box filter, box shift, compaction.
//
// Restates the per-frame preparation of PyCPET's calculator
// (CPET/source/calculator.py:239-251, 341-371) for charges already parsed:
//   1. filter_radius_whole_residue (CPET/utils/io.py:283-338): a residue is
//      kept when any of its atoms lies strictly within `radius` of the centre
//      (lab frame; |x - c| formed as numpy.linalg.norm forms it); a residue is
//      a run of consecutive atoms with the same (resid, resnum);
//   2. rotation (calculator.py:341-346): x <- (x - c) @ inv(T) (or x - c when
//      no basis is given);
//   3. filter_in_box (io.py:422-475): drop atoms strictly inside the box of
//      half-widths d.  The reference subtracts the centre a second time from
//      the already centred coordinates (calculator.py:349-358 passes
//      self.center to a function that recentres); that is kept, so the test
//      is on x - c after the rotation;
//   4. box shift (calculator.py:369-371): x <- x - shift;
// and the survivors are written in their original order (a scan of keep
// flags), ready for the field and streamline kernels.  All arithmetic IEEE
// double with single roundings (no fused multiply-add).
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kPrepThreads = 256;

// run start flags: 1 where (resid, resnum) differs from the previous atom
__global__ void run_start_kernel(int n, const int32_t* __restrict__ resid,
                                 const int32_t* __restrict__ resnum, int64_t* __restrict__ flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = (i == 0 || resid[i] != resid[i - 1] || resnum[i] != resnum[i - 1]) ? 1 : 0;
}

// After an exclusive scan of the start flags, run(i) = scan[i] + flag[i] - 1;
// a residue is kept when any atom is strictly within the radius.
__global__ void radius_kernel(int n, const double* __restrict__ x, double cx, double cy, double cz,
                              double radius, const int64_t* __restrict__ run_scan,
                              const int32_t* __restrict__ resid, const int32_t* __restrict__ resnum,
                              int* __restrict__ run_keep) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double dx = __dsub_rn(x[3 * i], cx), dy = __dsub_rn(x[3 * i + 1], cy),
                 dz = __dsub_rn(x[3 * i + 2], cz);
    const double r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    if (r < radius) {
      const bool start = i == 0 || resid[i] != resid[i - 1] || resnum[i] != resnum[i - 1];
      atomicOr(&run_keep[run_scan[i] + (start ? 1 : 0) - 1], 1);
    }
  }
}

struct PrepGeom {
  double c[3];
  double inv[9];     // row-major inv(T); identity when no basis
  double half[3];
  double shift[3];
  int rotate, box;
};

__device__ __forceinline__ void to_box(const double* x, const PrepGeom& g, double y[3]) {
  const double d0 = __dsub_rn(x[0], g.c[0]), d1 = __dsub_rn(x[1], g.c[1]), d2 = __dsub_rn(x[2], g.c[2]);
  if (!g.rotate) {
    y[0] = d0; y[1] = d1; y[2] = d2;
    return;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
    y[j] = __dadd_rn(__dadd_rn(__dmul_rn(d0, g.inv[j]), __dmul_rn(d1, g.inv[3 + j])),
                     __dmul_rn(d2, g.inv[6 + j]));
}

__global__ void keep_kernel(int n, const double* __restrict__ x, PrepGeom g, int radius_on,
                            const int64_t* __restrict__ run_scan, const int32_t* __restrict__ resid,
                            const int32_t* __restrict__ resnum, const int* __restrict__ run_keep,
                            int64_t* __restrict__ keep) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool k = true;
    if (radius_on) {
      const bool start = i == 0 || resid[i] != resid[i - 1] || resnum[i] != resnum[i - 1];
      k = run_keep[run_scan[i] + (start ? 1 : 0) - 1] != 0;
    }
    if (k && g.box) {
      double y[3];
      to_box(x + 3 * i, g, y);
      bool inside = true;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double r = __dsub_rn(y[a], g.c[a]);  // the reference's second recentring
        inside = inside && (r > -g.half[a]) && (r < g.half[a]);
      }
      k = !inside;
    }
    keep[i] = k ? 1 : 0;
  }
}

__global__ void compact_kernel(int n, const double* __restrict__ x, const double* __restrict__ q,
                               PrepGeom g, const int64_t* __restrict__ pos,
                               double* __restrict__ x_out, double* __restrict__ q_out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (pos[i + 1] == pos[i]) continue;  // dropped
    const int64_t o = pos[i];
    double y[3];
    to_box(x + 3 * i, g, y);
#pragma unroll
    for (int a = 0; a < 3; ++a) x_out[3 * o + a] = __dsub_rn(y[a], g.shift[a]);
    q_out[o] = q[i];
  }
}

int blocks_for(int n) { return std::max(1, std::min((n + kPrepThreads - 1) / kPrepThreads, 8192)); }

}  // namespace

size_t prep_scratch_bytes(int n) {
  return sizeof(int64_t) * (2 * (size_t(n) + 1) + size_t(scan_scratch_i64(int64_t(n) + 1))) +
         sizeof(int) * (size_t(n) + 1);
}

cudaError_t launch_prepare_frame(int n, const double* x, const double* q, const int32_t* resid,
                                 const int32_t* resnum, const double* center, const double* inv,
                                 double radius, const double* half, const double* shift,
                                 double* x_out, double* q_out, void* scratch, int64_t* d_count,
                                 cudaStream_t s) {
  int64_t* runs = static_cast<int64_t*>(scratch);       // [n + 1]
  int64_t* keep = runs + (n + 1);                        // [n + 1]
  int64_t* scan_tmp = keep + (n + 1);                    // scan scratch
  int* run_keep = reinterpret_cast<int*>(scan_tmp + scan_scratch_i64(int64_t(n) + 1));
  PrepGeom g;
  for (int a = 0; a < 3; ++a) {
    g.c[a] = center[a];
    g.half[a] = half ? half[a] : 0.0;
    g.shift[a] = shift ? shift[a] : 0.0;
  }
  for (int k = 0; k < 9; ++k) g.inv[k] = inv ? inv[k] : (k % 4 == 0 ? 1.0 : 0.0);
  g.rotate = inv ? 1 : 0;
  g.box = half ? 1 : 0;
  const int radius_on = radius > 0.0 ? 1 : 0;
  const int b = blocks_for(n);
  cudaError_t e = cudaSuccess;
  if (radius_on) {
    run_start_kernel<<<b, kPrepThreads, 0, s>>>(n, resid, resnum, runs);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_exclusive_i64(n, runs, scan_tmp, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(run_keep, 0, sizeof(int) * (size_t(n) + 1), s);
    if (e == cudaSuccess) {
      radius_kernel<<<b, kPrepThreads, 0, s>>>(n, x, center[0], center[1], center[2], radius, runs,
                                               resid, resnum, run_keep);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) return e;
  keep_kernel<<<b, kPrepThreads, 0, s>>>(n, x, g, radius_on, runs, resid, resnum, run_keep, keep);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemsetAsync(keep + n, 0, sizeof(int64_t), s);
  if (e == cudaSuccess) e = scan_exclusive_i64(int64_t(n) + 1, keep, scan_tmp, s);
  if (e != cudaSuccess) return e;
  compact_kernel<<<b, kPrepThreads, 0, s>>>(n, x, q, g, keep, x_out, q_out);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_count, keep + n, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  return e;
}

}  // namespace cpetgb

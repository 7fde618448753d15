// noalloc.cu -- streamlines without any device allocation.
//
// cpetgb_topo_lines allocates its scratch (the packed charge array and the
// work-queue counter) from the stream-ordered pool on every call.  Some callers
// cannot let a library allocate device memory: an application whose device
// memory is reserved up front by its own allocator (a PyTorch process whose
// caching allocator holds the budget, an engine with a fixed arena), where an
// extra cudaMallocAsync can fail or fragment that budget, or a long-running
// service that forbids allocation after start-up so its footprint never moves.
// For them this file provides cpetgb_topo_lines_noalloc: the same kernels, with
// their scratch in one fixed array below that is part of the library image.
//
//  * The array is a file-scope __device__ variable: every GPU that loads this
//    library holds kNoAllocBytes (about 512 KiB) for as long as the process
//    lives.  It fits a frame of at most kNoAllocMaxCharges charges.
//  * Host code cannot use the array's name as an address (on the host it names
//    a stand-in object).  The device address is looked up once per device with
//    cudaGetSymbolAddress, with that device current, on the first call made on
//    that device; make that first call before any stream capture.
//  * All calls share the array and it keeps the last call's contents; each call
//    clears its queue counter and status word before its kernels run.  Calls
//    whose work overlaps on the GPU (other streams, other host threads) race on
//    the array: issue them in order on one stream.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "cpetgb.h"
#include "kernels.cuh"

namespace cpetgb {
namespace {

constexpr int kNoAllocMaxCharges = 16384;
constexpr size_t kNoAllocChargeBytes = size_t(kNoAllocMaxCharges) * sizeof(Charge64);
constexpr size_t kNoAllocBytes = kNoAllocChargeBytes + 256;  // + queue counter, status word

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDev = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kMaxDev] = {};

}  // namespace
}  // namespace cpetgb

using namespace cpetgb;

extern "C" int cpetgb_topo_lines_noalloc(int precision, int n_lines, int n_charges,
                                         const double* starts, const int32_t* n_iter, double step,
                                         const double* half_dims, const double* x, const double* q,
                                         double* result, double* ends, int32_t* steps,
                                         void* stream) {
  if (precision != CPETGB_FP64 && precision != CPETGB_FP32C)
    return set_error(CPETGB_EINVAL, "bad precision");
  if (n_lines < 0 || n_charges < 0) return set_error(CPETGB_EINVAL, "negative line or charge count");
  if (n_charges > kNoAllocMaxCharges)
    return set_error(CPETGB_EINVAL,
                     "cpetgb_topo_lines_noalloc holds at most 16384 charges in its fixed scratch; "
                     "use cpetgb_topo_lines for larger frames");
  if (!half_dims) return set_error(CPETGB_EINVAL, "half_dims is NULL");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(half_dims[k]) || half_dims[k] < 0)
      return set_error(CPETGB_EINVAL, "half_dims must be finite and >= 0");
  if (!std::isfinite(step)) return set_error(CPETGB_EINVAL, "step must be finite");
  if (n_lines == 0) return CPETGB_OK;
  if (!starts || !n_iter || !result || (n_charges > 0 && (!x || !q)))
    return set_error(CPETGB_EINVAL, "NULL device pointer");

  int dev = -1, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
    cudaGetLastError();
    return set_error(CPETGB_ENODEV, "no usable CUDA device");
  }
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return set_error(CPETGB_ECUDA, "cudaGetSymbolAddress of the fixed scratch failed");
      }
      g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    base = g_noalloc_ptr[dev];
  }
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return set_error(CPETGB_ENODEV, "cannot query the device");
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* counters = reinterpret_cast<int*>(base + kNoAllocChargeBytes);  // [0] queue, [1] status
  const int pad = topo_charge_pad(precision);
  const int64_t n_pad = ((std::max(n_charges, 1) + int64_t(pad) - 1) / pad) * pad;

  cudaError_t e = cudaMemsetAsync(counters, 0, 2 * sizeof(int), s);
  if (e == cudaSuccess) e = launch_pack_topo(precision, n_charges, n_pad, x, q, base, s);
  if (e == cudaSuccess) {
    TopoParams p;
    p.n_lines = n_lines;
    p.n_charges = n_charges;
    p.step = step;
    for (int k = 0; k < 3; ++k) p.half[k] = half_dims[k];
    p.starts = starts;
    p.n_iter = n_iter;
    p.packed = base;
    p.result = result;
    p.ends = ends;
    p.steps = steps;
    p.queue = counters;
    p.status = counters + 1;
    e = launch_topo(precision, p, sms, s);
  }
  int st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, counters + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(CPETGB_ECUDA, cudaGetErrorString(e));
  }
  if (st == kDevWaitTimeout) return set_error(CPETGB_ETIMEOUT, "a device-side wait exceeded its limit");
  if (st == kDevBadCap) return set_error(CPETGB_EINVAL, "a streamline step cap exceeds 2^24");
  if (st != kDevOk) return set_error(CPETGB_ECUDA, "device status word set");
  return CPETGB_OK;
}

// engine.cu -- host side of the streamline serving engine (C ABI cpetgb_engine_*).
//
// Continuous batching of streamline requests on one device:
//  * frames (charges) are packed once into a device pool and stay resident;
//  * a request's lines are copied into a device line store and published as
//    chunks in a ring the engine kernel's warps claim from while it runs;
//  * per-request completion counters live in host-mapped memory, updated by
//    the kernel with system-scope atomics, so the host polls without syncing;
//  * admission: a request is accepted only if its lines fit the line store,
//    its chunks fit the ring and a request slot is free; otherwise the call
//    returns CPETGB_EAGAIN and the caller retries after collecting others.
// Launch rule: after publishing, if fewer than two engine launches are in
// flight one more is queued on the engine stream.  A running kernel takes the
// new chunks as its slots free up (its idle warps stay while any of its warps
// has lines); once it has been idle for 50 ms it closes and ends, and a queued
// one starts, so work is never left unclaimed.  Storage released by collect/remove is reused only
// when no engine launch is in flight (the kernel may hold it in L1).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "cpetgb.h"
#include "kernels.cuh"

using namespace cpetgb;

namespace {

struct Range {
  int64_t begin, size;
};

// First-fit allocator over [0, capacity) with deferred reuse.
struct RangePool {
  int64_t capacity = 0;
  std::vector<Range> free_list, pending;
  void init(int64_t cap) {
    capacity = cap;
    free_list = {{0, cap}};
    pending.clear();
  }
  int64_t alloc(int64_t n) {
    for (size_t i = 0; i < free_list.size(); ++i) {
      if (free_list[i].size >= n) {
        const int64_t b = free_list[i].begin;
        free_list[i].begin += n;
        free_list[i].size -= n;
        if (free_list[i].size == 0) free_list.erase(free_list.begin() + i);
        return b;
      }
    }
    return -1;
  }
  void release(int64_t b, int64_t n) { pending.push_back({b, n}); }
  void recycle() {  // pending ranges become free; coalesce
    for (auto& r : pending) free_list.push_back(r);
    pending.clear();
    std::sort(free_list.begin(), free_list.end(),
              [](const Range& a, const Range& b) { return a.begin < b.begin; });
    std::vector<Range> merged;
    for (auto& r : free_list) {
      if (!merged.empty() && merged.back().begin + merged.back().size == r.begin)
        merged.back().size += r.size;
      else
        merged.push_back(r);
    }
    free_list.swap(merged);
  }
  int64_t free_total() const {
    int64_t t = 0;
    for (auto& r : free_list) t += r.size;
    return t;
  }
};

struct Request {
  bool used = false;
  int64_t line_begin = 0, n_lines = 0;
};

struct FrameSlot {
  bool used = false;
  int64_t begin = 0, n_pad = 0;
};

}  // namespace

struct cpetgb_engine {
  int device = -1, prec = CPETGB_FP32C, sms = 0;
  int ctas_per_sm = 1;  // 1: half of every SM's registers; 2: whole SMs
  int chunk_lines = 32;
  cudaStream_t run_stream = nullptr, copy_stream = nullptr;
  std::mutex mu;
  // device
  unsigned char* pool = nullptr;  // packed charges
  TopoFrame* d_frames = nullptr;
  double* starts = nullptr;
  int32_t* n_iter = nullptr;
  double* result = nullptr;
  int32_t* steps = nullptr;
  int* status = nullptr;
  int* d_head = nullptr;      // [0] claim counter, [1] busy warps, [2] closing flag (device)
  double* stage_x = nullptr;  // frame upload staging
  double* stage_q = nullptr;
  int64_t stage_cap = 0;
  // host-mapped
  EngineChunk* chunks = nullptr;
  int* counters = nullptr;  // [0] tail (published), [1] claims mirror
  int* done = nullptr;
  EngineChunk* d_chunks = nullptr;
  int* d_counters = nullptr;
  int* d_done = nullptr;
  int chunk_cap = 0, max_frames = 0, max_requests = 0;
  // bookkeeping
  RangePool charge_pool, line_pool;
  std::vector<FrameSlot> frames;
  std::vector<Request> requests;
  std::vector<cudaEvent_t> launches;  // engine launches possibly in flight
  int tail = 0;

  ~cpetgb_engine() {
    if (run_stream) cudaStreamSynchronize(run_stream);
    if (copy_stream) cudaStreamSynchronize(copy_stream);
    for (auto ev : launches) cudaEventDestroy(ev);
    for (void* p : {(void*)pool, (void*)d_frames, (void*)starts, (void*)n_iter, (void*)result,
                    (void*)steps, (void*)status, (void*)d_head, (void*)stage_x, (void*)stage_q})
      if (p) cudaFree(p);
    for (void* p : {(void*)chunks, (void*)counters, (void*)done})
      if (p) cudaFreeHost(p);
    if (run_stream) cudaStreamDestroy(run_stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
  }

  // Drops finished launch records; true when none is in flight.
  int in_flight() {
    std::vector<cudaEvent_t> keep;
    for (auto ev : launches) {
      if (cudaEventQuery(ev) == cudaSuccess)
        cudaEventDestroy(ev);
      else
        keep.push_back(ev);
    }
    cudaGetLastError();  // cudaErrorNotReady is not an error here
    launches.swap(keep);
    return static_cast<int>(launches.size());
  }

  void maybe_recycle() {
    if (in_flight() == 0) {
      charge_pool.recycle();
      line_pool.recycle();
    }
  }

  cudaError_t launch() {
    EngineParams E{};
    E.p.n_lines = 0;
    E.p.starts = starts;
    E.p.n_iter = n_iter;
    E.p.packed = pool;
    E.p.result = result;
    E.p.ends = nullptr;
    E.p.steps = steps;
    E.p.status = status;
    E.frames = d_frames;
    E.chunks = d_chunks;
    E.chunk_capacity = chunk_cap;
    E.tail = d_counters;
    E.head = d_head;
    E.head_mirror = d_counters + 1;
    E.done = d_done;
    E.busy = d_head + 1;
    E.closing = d_head + 2;
    // the launch's busy count and closing flag start at 0 (stream-ordered after
    // the previous launch)
    cudaError_t e = cudaMemsetAsync(d_head + 1, 0, 2 * sizeof(int), run_stream);
    if (e == cudaSuccess) e = launch_engine(prec, E, sms * ctas_per_sm, run_stream);
    if (e != cudaSuccess) return e;
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
    e = cudaEventRecord(ev, run_stream);
    launches.push_back(ev);
    return e;
  }

  cudaError_t kick() {
    const int published = __atomic_load_n(counters, __ATOMIC_ACQUIRE);
    const int claimed = __atomic_load_n(counters + 1, __ATOMIC_ACQUIRE);
    const int n = in_flight();
    if (published > claimed && n < 2) return launch();
    return cudaSuccess;
  }
};

namespace {

int efail(int code, const char* msg) { return set_error(code, msg); }

int ecuda(cudaError_t e, const char* what) {
  cudaGetLastError();
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return set_error(e == cudaErrorMemoryAllocation ? CPETGB_ENOMEM : CPETGB_ECUDA, buf);
}

#define ECK(expr, what)                               \
  do {                                                \
    cudaError_t e_ = (expr);                          \
    if (e_ != cudaSuccess) return ecuda(e_, what);    \
  } while (0)

size_t elem_size(int prec) { return prec == CPETGB_FP32C ? 16 : 32; }

}  // namespace

extern "C" {

int cpetgb_engine_create(cpetgb_engine** out, int precision, int64_t charge_capacity,
                         int64_t line_capacity, int max_frames, int max_requests,
                         int chunk_lines) {
  if (!out) return efail(CPETGB_EINVAL, "engine pointer is NULL");
  *out = nullptr;
  if (precision != CPETGB_FP32C && precision != CPETGB_FP64)
    return efail(CPETGB_EINVAL, "bad precision");
  if (charge_capacity <= 0 || line_capacity <= 0 || line_capacity > INT32_MAX || max_frames <= 0 ||
      max_requests <= 0 || chunk_lines <= 0)
    return efail(CPETGB_EINVAL, "engine capacities must be positive");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return efail(CPETGB_ENODEV, "no CUDA device available");
  }
  cpetgb_engine* e = new cpetgb_engine();
  e->prec = precision;
  e->chunk_lines = chunk_lines;
  e->max_frames = max_frames;
  e->max_requests = max_requests;
  e->chunk_cap = static_cast<int>(std::min<int64_t>(line_capacity / 4 + max_requests, 1 << 24));
  const int pad = topo_charge_pad(precision);
  charge_capacity = ((charge_capacity + pad - 1) / pad) * pad;
  cudaError_t err = cudaGetDevice(&e->device);
  if (err == cudaSuccess)
    err = cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, e->device);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->run_stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaMalloc(&e->pool, size_t(charge_capacity) * elem_size(precision));
  if (err == cudaSuccess) err = cudaMalloc(&e->d_frames, sizeof(TopoFrame) * max_frames);
  if (err == cudaSuccess) err = cudaMalloc(&e->starts, sizeof(double) * 3 * line_capacity);
  if (err == cudaSuccess) err = cudaMalloc(&e->n_iter, sizeof(int32_t) * line_capacity);
  if (err == cudaSuccess) err = cudaMalloc(&e->result, sizeof(double) * 2 * line_capacity);
  if (err == cudaSuccess) err = cudaMalloc(&e->steps, sizeof(int32_t) * line_capacity);
  if (err == cudaSuccess) err = cudaMalloc(&e->status, sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(e->status, 0, sizeof(int));
  if (err == cudaSuccess) err = cudaMalloc(&e->d_head, 3 * sizeof(int));
  if (err == cudaSuccess) err = cudaMemset(e->d_head, 0, 3 * sizeof(int));
  if (err == cudaSuccess)
    err = cudaHostAlloc(&e->chunks, sizeof(EngineChunk) * e->chunk_cap, cudaHostAllocMapped);
  if (err == cudaSuccess) err = cudaHostAlloc(&e->counters, sizeof(int) * 2, cudaHostAllocMapped);
  if (err == cudaSuccess) err = cudaHostAlloc(&e->done, sizeof(int) * max_requests, cudaHostAllocMapped);
  if (err == cudaSuccess) err = cudaHostGetDevicePointer(&e->d_chunks, e->chunks, 0);
  if (err == cudaSuccess) err = cudaHostGetDevicePointer(&e->d_counters, e->counters, 0);
  if (err == cudaSuccess) err = cudaHostGetDevicePointer(&e->d_done, e->done, 0);
  if (err != cudaSuccess) {
    delete e;
    return ecuda(err, "engine allocation");
  }
  e->counters[0] = e->counters[1] = 0;
  std::memset(e->done, 0, sizeof(int) * max_requests);
  e->charge_pool.init(charge_capacity);
  e->line_pool.init(line_capacity);
  e->frames.assign(max_frames, FrameSlot{});
  e->requests.assign(max_requests, Request{});
  *out = e;
  return CPETGB_OK;
}

int cpetgb_engine_destroy(cpetgb_engine* e) {
  delete e;
  return CPETGB_OK;
}

// Packs a frame's charges (HOST x[n][3], q[n]) into the pool; *frame_id names it.
int cpetgb_engine_add_frame(cpetgb_engine* e, int n_charges, const double* x, const double* q,
                            int* frame_id) {
  if (!e || !frame_id || n_charges < 0 || (n_charges > 0 && (!x || !q)))
    return efail(CPETGB_EINVAL, "bad frame arguments");
  std::lock_guard<std::mutex> lock(e->mu);
  int slot = -1;
  for (int i = 0; i < e->max_frames; ++i)
    if (!e->frames[i].used) {
      slot = i;
      break;
    }
  if (slot < 0) return efail(CPETGB_EAGAIN, "all frame slots are in use");
  const int pad = topo_charge_pad(e->prec);
  const int64_t n_pad = ((std::max(n_charges, 1) + int64_t(pad) - 1) / pad) * pad;
  e->maybe_recycle();
  const int64_t begin = e->charge_pool.alloc(n_pad);
  if (begin < 0) return efail(CPETGB_EAGAIN, "the charge pool is full");
  if (n_charges > e->stage_cap) {
    if (e->stage_x) cudaFree(e->stage_x);
    if (e->stage_q) cudaFree(e->stage_q);
    e->stage_x = e->stage_q = nullptr;
    e->stage_cap = 0;
    ECK(cudaMalloc(&e->stage_x, sizeof(double) * 3 * n_charges), "frame staging");
    ECK(cudaMalloc(&e->stage_q, sizeof(double) * n_charges), "frame staging");
    e->stage_cap = n_charges;
  }
  ECK(cudaMemcpyAsync(e->stage_x, x, sizeof(double) * 3 * n_charges, cudaMemcpyHostToDevice,
                      e->copy_stream), "frame upload");
  ECK(cudaMemcpyAsync(e->stage_q, q, sizeof(double) * n_charges, cudaMemcpyHostToDevice,
                      e->copy_stream), "frame upload");
  void* dst = e->pool + begin * elem_size(e->prec);
  ECK(launch_pack_topo(e->prec, n_charges, n_pad, e->stage_x, e->stage_q, dst, e->copy_stream),
      "frame pack");
  TopoFrame fr{};
  fr.packed_off = begin;
  fr.n_pad = static_cast<int32_t>(n_pad);
  ECK(cudaMemcpyAsync(e->d_frames + slot, &fr, sizeof fr, cudaMemcpyHostToDevice, e->copy_stream),
      "frame table");
  ECK(cudaStreamSynchronize(e->copy_stream), "frame upload");
  e->frames[slot] = {true, begin, n_pad};
  *frame_id = slot;
  return CPETGB_OK;
}

int cpetgb_engine_remove_frame(cpetgb_engine* e, int frame_id) {
  if (!e) return efail(CPETGB_EINVAL, "engine is NULL");
  std::lock_guard<std::mutex> lock(e->mu);
  if (frame_id < 0 || frame_id >= e->max_frames || !e->frames[frame_id].used)
    return efail(CPETGB_EINVAL, "no such frame");
  e->charge_pool.release(e->frames[frame_id].begin, e->frames[frame_id].n_pad);
  e->frames[frame_id].used = false;
  return CPETGB_OK;
}

// Admits a request: HOST starts[n][3] and n_iter[n]; half_dims HOST[3].
// Returns CPETGB_EAGAIN when the line store, the chunk ring or the request
// slots are full (retry after collecting finished requests).
int cpetgb_engine_submit(cpetgb_engine* e, int frame_id, int n_lines, const double* starts,
                         const int32_t* n_iter, double step, const double* half_dims,
                         int* request_id) {
  if (!e || !request_id || n_lines <= 0 || !starts || !n_iter || !half_dims)
    return efail(CPETGB_EINVAL, "bad request arguments");
  if (!std::isfinite(step)) return efail(CPETGB_EINVAL, "step must be finite");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(half_dims[k]) || half_dims[k] < 0)
      return efail(CPETGB_EINVAL, "half-widths must be finite and >= 0");
  std::lock_guard<std::mutex> lock(e->mu);
  if (frame_id < 0 || frame_id >= e->max_frames || !e->frames[frame_id].used)
    return efail(CPETGB_EINVAL, "no such frame");
  int rid = -1;
  for (int i = 0; i < e->max_requests; ++i)
    if (!e->requests[i].used) {
      rid = i;
      break;
    }
  if (rid < 0) return efail(CPETGB_EAGAIN, "all request slots are in use");
  // chunk size: spread the request over every warp of the engine (at least one
  // warp's line slots per chunk, at most chunk_lines)
  const int warps = e->sms * e->ctas_per_sm * (engine_threads() / 32);
  const int cl = std::max(4, std::min(e->chunk_lines, n_lines / std::max(warps, 1)));
  const int n_chunks = (n_lines + cl - 1) / cl;
  const int claimed = __atomic_load_n(e->counters + 1, __ATOMIC_ACQUIRE);
  if (e->tail - claimed + n_chunks > e->chunk_cap) return efail(CPETGB_EAGAIN, "the chunk ring is full");
  e->maybe_recycle();
  const int64_t lb = e->line_pool.alloc(n_lines);
  if (lb < 0) return efail(CPETGB_EAGAIN, "the line store is full");
  ECK(cudaMemcpyAsync(e->starts + 3 * lb, starts, sizeof(double) * 3 * n_lines,
                      cudaMemcpyHostToDevice, e->copy_stream), "line upload");
  ECK(cudaMemcpyAsync(e->n_iter + lb, n_iter, sizeof(int32_t) * n_lines, cudaMemcpyHostToDevice,
                      e->copy_stream), "line upload");
  ECK(cudaStreamSynchronize(e->copy_stream), "line upload");
  e->requests[rid] = {true, lb, n_lines};
  __atomic_store_n(e->done + rid, 0, __ATOMIC_RELAXED);
  for (int c = 0; c < n_chunks; ++c) {
    EngineChunk& ch = e->chunks[(e->tail + c) % e->chunk_cap];
    ch.frame = frame_id;
    ch.request = rid;
    ch.line_begin = static_cast<int32_t>(lb + int64_t(c) * cl);
    ch.line_end = static_cast<int32_t>(std::min<int64_t>(lb + n_lines, lb + int64_t(c + 1) * cl));
    ch.step = step;
    for (int k = 0; k < 3; ++k) ch.half[k] = half_dims[k];
  }
  e->tail += n_chunks;
  __atomic_store_n(e->counters, e->tail, __ATOMIC_RELEASE);  // publish
  ECK(e->kick(), "engine launch");
  *request_id = rid;
  return CPETGB_OK;
}

// 1 when all lines of the request are done, 0 while pending, < 0 on error.
int cpetgb_engine_poll(cpetgb_engine* e, int request_id) {
  if (!e) return efail(CPETGB_EINVAL, "engine is NULL");
  std::lock_guard<std::mutex> lock(e->mu);
  if (request_id < 0 || request_id >= e->max_requests || !e->requests[request_id].used)
    return efail(CPETGB_EINVAL, "no such request");
  const int n = e->in_flight();
  const int d = __atomic_load_n(e->done + request_id, __ATOMIC_ACQUIRE);
  if (d >= e->requests[request_id].n_lines) return 1;
  if (n == 0) {  // no launch in flight: unclaimed work needs one, else something failed
    int st = 0;
    ECK(cudaMemcpy(&st, e->status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
    if (st == kDevBadCap) return efail(CPETGB_EINVAL, "a streamline step cap exceeds 2^24");
    if (st != kDevOk) return efail(CPETGB_ECUDA, "device status word set");
    const int published = __atomic_load_n(e->counters, __ATOMIC_ACQUIRE);
    const int claimed = __atomic_load_n(e->counters + 1, __ATOMIC_ACQUIRE);
    if (published <= claimed)
      return efail(CPETGB_ECUDA, "the engine stopped before finishing the request");
    ECK(e->kick(), "engine launch");
  }
  return 0;
}

// Copies a finished request's results (HOST result[n][2], steps[n] or NULL) and frees it.
int cpetgb_engine_collect(cpetgb_engine* e, int request_id, double* result, int32_t* steps) {
  if (!e || !result) return efail(CPETGB_EINVAL, "bad collect arguments");
  std::lock_guard<std::mutex> lock(e->mu);
  if (request_id < 0 || request_id >= e->max_requests || !e->requests[request_id].used)
    return efail(CPETGB_EINVAL, "no such request");
  Request& r = e->requests[request_id];
  if (__atomic_load_n(e->done + request_id, __ATOMIC_ACQUIRE) < r.n_lines)
    return efail(CPETGB_EINVAL, "request is not finished");
  ECK(cudaMemcpyAsync(result, e->result + 2 * r.line_begin, sizeof(double) * 2 * r.n_lines,
                      cudaMemcpyDeviceToHost, e->copy_stream), "result download");
  if (steps)
    ECK(cudaMemcpyAsync(steps, e->steps + r.line_begin, sizeof(int32_t) * r.n_lines,
                        cudaMemcpyDeviceToHost, e->copy_stream), "result download");
  ECK(cudaStreamSynchronize(e->copy_stream), "result download");
  e->line_pool.release(r.line_begin, r.n_lines);
  r.used = false;
  return CPETGB_OK;
}

// Engine CTAs per SM from the next launch on: 1 leaves half of every SM's
// registers to grid launches on other streams; 2 gives the engine whole SMs.
int cpetgb_engine_set_ctas_per_sm(cpetgb_engine* e, int ctas_per_sm) {
  if (!e) return efail(CPETGB_EINVAL, "engine is NULL");
  if (ctas_per_sm != 1 && ctas_per_sm != 2) return efail(CPETGB_EINVAL, "ctas_per_sm must be 1 or 2");
  std::lock_guard<std::mutex> lock(e->mu);
  e->ctas_per_sm = ctas_per_sm;
  return CPETGB_OK;
}

// Waits until every engine launch has ended.
int cpetgb_engine_drain(cpetgb_engine* e) {
  if (!e) return efail(CPETGB_EINVAL, "engine is NULL");
  ECK(cudaStreamSynchronize(e->run_stream), "engine drain");
  std::lock_guard<std::mutex> lock(e->mu);
  e->in_flight();
  e->maybe_recycle();
  return CPETGB_OK;
}

}  // extern "C"

// api.cu -- the C ABI of libcpetgb.so (declared in include/cpetgb.h).
//
// Host-side responsibilities: argument validation, the per-device context
// (SM count, a library stream for host-memory calls, the device status word),
// stream-ordered scratch memory (cudaMallocAsync on the call's stream),
// host<->device staging for CPETGB_HOST calls, the work decomposition of the
// grid kernels (point tiles x charge splits, largest first), and the mapping
// of device-side status words to return codes.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "cpetgb.h"
#include "kernels.cuh"

using namespace cpetgb;

namespace {

constexpr int kVersion = 10000;  // 1.0.0
constexpr int kMaxDevices = 64;

thread_local std::string g_err;
std::mutex g_mu;
std::atomic<int> g_default_prec{CPETGB_FP32C};
// FP32C field: points with |E| below this fraction of their frame's median |E|
// are recomputed in double-float arithmetic (0 turns the refinement off).
std::atomic<double> g_refine_tau{0.15};

struct Ctx {
  bool ready = false;
  int sms = 0;
  cudaStream_t stream = nullptr;  // used by CPETGB_HOST calls without a stream
  int* status = nullptr;          // device status word (DevStatus)
};
Ctx g_ctx[kMaxDevices];

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a sticky launch error of this thread
  const int code = (e == cudaErrorMemoryAllocation) ? CPETGB_ENOMEM : CPETGB_ECUDA;
  return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                          \
  do {                                          \
    cudaError_t e_ = (expr);                    \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

Ctx* context(int* rc) {
  int dev = -1, count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    *rc = fail(CPETGB_ENODEV, "no CUDA device available");
    return nullptr;
  }
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    *rc = fail(CPETGB_ENODEV, "cannot query the current CUDA device");
    return nullptr;
  }
  Ctx& c = g_ctx[dev];
  std::lock_guard<std::mutex> lock(g_mu);
  if (!c.ready) {
    cudaError_t e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c.status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c.status, 0, sizeof(int));
    if (e == cudaSuccess) {
      // Keep freed scratch in the device's stream-ordered pool.
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    }
    if (e != cudaSuccess) {
      *rc = cuda_fail(e, "device context setup");
      return nullptr;
    }
    c.ready = true;
  }
  *rc = CPETGB_OK;
  return &c;
}

// Stream-ordered scratch, released (to the pool) on the same stream.
struct Scratch {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t st) : s(st) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
  template <typename T>
  cudaError_t get(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* v = nullptr;
    cudaError_t e = cudaMallocAsync(&v, ((count * sizeof(T) + 255) / 256) * 256, s);
    if (e == cudaSuccess) {
      ptrs.push_back(v);
      *p = static_cast<T*>(v);
    }
    return e;
  }
};

template <typename T>
cudaError_t h2d(T** dst, Scratch& S, const T* src, size_t count) {
  cudaError_t e = S.get(dst, count);
  if (e == cudaSuccess && count)
    e = cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, S.s);
  return e;
}

// Waits for the stream and converts the device status word into a return code.
int finish(Ctx* c, cudaStream_t s) {
  CK(cudaStreamSynchronize(s), "stream synchronize");
  int st = 0;
  CK(cudaMemcpy(&st, c->status, sizeof(int), cudaMemcpyDeviceToHost), "status read");
  if (st != kDevOk) {
    cudaMemset(c->status, 0, sizeof(int));
    if (st == kDevWaitTimeout)
      return fail(CPETGB_ETIMEOUT, "a device-side wait exceeded its limit");
    if (st == kDevBadArgument)
      return fail(CPETGB_ERANGE, "histogram range is not finite or is inverted");
    if (st == kDevBadCap)
      return fail(CPETGB_EINVAL, "a streamline step cap exceeds %d", kMaxLineCap);
    return fail(CPETGB_ECUDA, "device status %d", st);
  }
  return CPETGB_OK;
}

bool valid_prec(int p) { return p == CPETGB_FP64 || p == CPETGB_FP32C; }
bool valid_mem(int m) { return m == CPETGB_HOST || m == CPETGB_DEVICE; }
size_t packed_size(int prec) { return prec == CPETGB_FP32C ? 16 : 32; }  // streamline layouts
constexpr size_t kGridRecord = 32;  // grid layouts: Charge64 or the duplicated FP32C record

// ---------------------------------------------------------------------------
// Grid work decomposition.
// ---------------------------------------------------------------------------
struct GridPlan {
  std::vector<GridItem> items;
  std::vector<GridFinal> finals;
  int n_slots = 0;
};

// ---------------------------------------------------------------------------
// Autotuner table: (operation, precision, class, size bucket) -> variant.
// Filled by pycpet_gb300.autotune (timed candidates), read at every launch.
// ---------------------------------------------------------------------------
std::mutex g_tune_mu;
std::map<int, int> g_tune;

constexpr int kOpGrid = 0, kOpTopo = 1;
// points per thread {4, 8} x work items per SM: variants 0-9 {4, 8, 16, 32, 64},
// 10-13 {128, 256} (numbered after the first ten so saved tables keep their meaning)
constexpr int kGridVariants = 14;
constexpr int kTopoVariants = 2;  // line slots per warp {4, 2}

int size_bucket(double v, double base) {
  if (!(v > base)) return 0;
  const int b = static_cast<int>(std::floor(std::log(v / base) / std::log(4.0)));
  return std::min(std::max(b, 0), 15);
}

int tune_key(int op, int prec, int cls, double size) {
  const int b = op == kOpGrid ? size_bucket(size, 1e6) : size_bucket(size, 1e3);
  return (op << 12) | (prec << 8) | ((cls & 15) << 4) | b;
}

int tune_lookup(int key) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(key);
  return it == g_tune.end() ? -1 : it->second;
}

// The variant for a launch: the entry of its own size bucket, else that of the
// nearest tuned bucket of the same (operation, precision, class), the smaller
// one on a tie; -1 when nothing of that class is tuned.
int tune_choose(int key) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune.find(key);
  if (it != g_tune.end()) return it->second;
  const int b = key & 15;
  for (int d = 1; d < 16; ++d) {
    for (int nb : {b - d, b + d}) {
      if (nb < 0 || nb > 15) continue;
      auto jt = g_tune.find((key & ~15) | nb);
      if (jt != g_tune.end()) return jt->second;
    }
  }
  return -1;
}

void plan_grid(int n_frames, const int64_t* desc, int sms, GridPlan& plan, int ppt,
               int items_per_sm) {
  const int tile = kGridThreads * ppt;
  // A CTA's time is proportional to its charge count alone: every thread
  // evaluates all of its point slots, valid or not.  Each frame's points are
  // cut into equal tiles, and charge ranges are split so that about
  // items_per_sm items of equal cost fall on each SM.
  auto n_tiles = [&](int64_t P) { return (P + tile - 1) / tile; };
  double total = 0.0;
  for (int f = 0; f < n_frames; ++f)
    total += double(n_tiles(desc[4 * f + 3])) * tile * double(desc[4 * f + 1]);
  const double target = std::max(1.0, total / (double(std::max(sms, 1)) * items_per_sm));
  for (int f = 0; f < n_frames; ++f) {
    const int64_t co = desc[4 * f + 0], n = desc[4 * f + 1];
    const int64_t po = desc[4 * f + 2], P = desc[4 * f + 3];
    const int64_t nt = n_tiles(P);
    for (int64_t ti = 0; ti < nt; ++ti) {
      const int64_t pb = ti * (P / nt) + std::min<int64_t>(ti, P % nt);
      const int pc = static_cast<int>(P / nt + (ti < P % nt ? 1 : 0));
      int64_t split = 1;
      if (n > 0) {
        split = static_cast<int64_t>(std::ceil(double(tile) * double(n) / target));
        split = std::max<int64_t>(1, std::min<int64_t>(split, std::max<int64_t>(1, n / 256)));
      }
      const int64_t chunk = n > 0 ? (n + split - 1) / split : 0;
      if (n > 0) split = (n + chunk - 1) / chunk;
      int slot_base = -1;
      if (split > 1) {
        slot_base = plan.n_slots;
        plan.n_slots += static_cast<int>(split);
        plan.finals.push_back(GridFinal{po + pb, pc, slot_base, static_cast<int32_t>(split), 0});
      }
      for (int64_t k = 0; k < split; ++k) {
        GridItem it;
        it.charge_off = co;
        it.point_off = po;
        it.p_begin = static_cast<int32_t>(pb);
        it.p_count = pc;
        it.n_begin = static_cast<int32_t>(k * chunk);
        it.n_count = static_cast<int32_t>(std::min<int64_t>(chunk, n - k * chunk));
        it.slot = split > 1 ? slot_base + static_cast<int32_t>(k) : -1;
        it.pad = 0;
        plan.items.push_back(it);
      }
    }
  }
  // longest first, so the last wave holds the shortest items
  std::stable_sort(plan.items.begin(), plan.items.end(),
                   [](const GridItem& a, const GridItem& b) { return a.n_count > b.n_count; });
}

// Entries the refinement list may need: every point of every frame (frames
// may share point ranges, so this is the sum, not the extent).
int64_t refine_list_len(int n_frames, const int64_t* desc) {
  int64_t n = 0;
  for (int f = 0; f < n_frames; ++f) n += desc[4 * f + 3];
  return std::max<int64_t>(n, 1);
}

int64_t max_frame_points(int n_frames, const int64_t* desc) {
  int64_t m = 0;
  for (int f = 0; f < n_frames; ++f) m = std::max(m, desc[4 * f + 3]);
  return m;
}

double grid_pair_evals(int n_frames, const int64_t* desc) {
  double total = 0.0;
  for (int f = 0; f < n_frames; ++f) total += double(desc[4 * f + 1]) * double(desc[4 * f + 3]);
  return total;
}

int grid_batch_impl(int kind, int prec, int mem, int clamp, int n_frames, const int64_t* desc,
                    const double* pts, const double* x, const double* q, double* out,
                    void* stream) {
  if (kind != CPETGB_FIELD && kind != CPETGB_ESP) return fail(CPETGB_EINVAL, "bad grid kind %d", kind);
  if (!valid_prec(prec)) return fail(CPETGB_EINVAL, "bad precision %d", prec);
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (n_frames < 0 || (n_frames > 0 && !desc)) return fail(CPETGB_EINVAL, "bad frame table");
  int64_t tot_pts = 0, tot_ch = 0;
  for (int f = 0; f < n_frames; ++f) {
    const int64_t co = desc[4 * f], n = desc[4 * f + 1], po = desc[4 * f + 2], P = desc[4 * f + 3];
    if (co < 0 || n < 0 || po < 0 || P < 0 || n > INT_MAX || P > INT_MAX)
      return fail(CPETGB_EINVAL, "frame %d: negative or oversized offset/count", f);
    tot_pts = std::max(tot_pts, po + P);
    tot_ch = std::max(tot_ch, co + n);
  }
  if (tot_pts == 0) return CPETGB_OK;
  if (!pts || !out) return fail(CPETGB_EINVAL, "points/output pointer is NULL");
  if (tot_ch > 0 && (!x || !q)) return fail(CPETGB_EINVAL, "charge pointer is NULL");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;
  const int NC = kind == CPETGB_FIELD ? 3 : 1;

  GridPlan plan;
  int ppt = 4, ips = 8;
  tuned_grid_shape(prec, kind, grid_pair_evals(n_frames, desc), &ppt, &ips);
  plan_grid(n_frames, desc, c->sms, plan, ppt, ips);

  Scratch S(s);
  const double *dp = pts, *dx = x, *dq = q;
  double* dout = out;
  if (mem == CPETGB_HOST) {
    CK(h2d(const_cast<double**>(&dp), S, pts, size_t(tot_pts) * 3), "copy points");
    if (tot_ch) {
      CK(h2d(const_cast<double**>(&dx), S, x, size_t(tot_ch) * 3), "copy charge positions");
      CK(h2d(const_cast<double**>(&dq), S, q, size_t(tot_ch)), "copy charges");
    }
    CK(S.get(&dout, size_t(tot_pts) * NC), "alloc output");
  }
  unsigned char* packed = nullptr;
  GridItem* d_items = nullptr;
  GridFinal* d_fin = nullptr;
  double* partial = nullptr;
  CK(S.get(&packed, size_t(std::max<int64_t>(tot_ch, 1)) * kGridRecord), "alloc packed charges");
  CK(h2d(&d_items, S, plan.items.data(), plan.items.size()), "copy work items");
  if (!plan.finals.empty()) {
    CK(h2d(&d_fin, S, plan.finals.data(), plan.finals.size()), "copy split table");
    CK(S.get(&partial, size_t(plan.n_slots) * kGridSlotPts * 3), "alloc partial sums");
  }
  if (reinterpret_cast<uintptr_t>(packed) % 16 != 0)  // bulk async copies need 16-byte sources
    return fail(CPETGB_ECUDA, "scratch allocation is not 16-byte aligned");
  CK(launch_pack_charges(prec, tot_ch, tot_ch, dx, dq, packed, s), "pack charges");
  CK(launch_grid(prec, kind, clamp ? 1 : 0, ppt, static_cast<int>(plan.items.size()), d_items,
                 packed, dp, dout, partial, c->status, s),
     "grid kernel launch");
  CK(launch_grid_final(kind, static_cast<int>(plan.finals.size()), d_fin, partial, dout, s),
     "grid reduction launch");
  const double tau = g_refine_tau.load();
  // A frame of one or two points never has a point below tau x its lower
  // median, so launches of such frames only (point fields) skip the pass.
  if (kind == CPETGB_FIELD && prec == CPETGB_FP32C && tau > 0.0 && tot_ch > 0 &&
      max_frame_points(n_frames, desc) >= 3) {
    int64_t *d_desc = nullptr, *list = nullptr;
    int* count = nullptr;
    unsigned char* dfq = nullptr;
    int* hist = nullptr;
    CK(h2d(&d_desc, S, desc, size_t(n_frames) * 4), "copy frame table");
    CK(S.get(&list, size_t(refine_list_len(n_frames, desc)) * 2), "alloc refinement list");
    CK(S.get(&count, 1), "alloc refinement count");
    CK(S.get(&hist, size_t(grid_refine_hist_ints(n_frames))), "alloc magnitude histograms");
    CK(S.get(&dfq, size_t(tot_ch) * 32), "alloc double-float charges");
    CK(launch_grid_refine(n_frames, tot_ch, max_frame_points(n_frames, desc), d_desc, dp, dx, dq, dout,
                          clamp ? 1 : 0, tau, list, count, hist, dfq, c->sms, s),
       "field refinement launch");
  }
  if (mem == CPETGB_HOST) {
    CK(cudaMemcpyAsync(out, dout, size_t(tot_pts) * NC * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy output");
    return finish(c, s);
  }
  return CPETGB_OK;
}

// source = kCharges: q[N] charges; kDipoles: q is mu[N][3], the dipole moments.
int topo_impl(int prec, int mem, int L, int N, const double* starts, const int32_t* n_iter,
              double step, const double* half, const double* x, const double* q, double* result,
              double* ends, int32_t* steps, void* stream, int source = kCharges) {
  if (!valid_prec(prec)) return fail(CPETGB_EINVAL, "bad precision %d", prec);
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (L < 0 || N < 0) return fail(CPETGB_EINVAL, "negative line or charge count");
  if (!half) return fail(CPETGB_EINVAL, "half_dims is NULL");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(half[k]) || half[k] < 0)
      return fail(CPETGB_EINVAL, "half_dims[%d] must be finite and >= 0", k);
  if (!std::isfinite(step)) return fail(CPETGB_EINVAL, "step must be finite");
  if (L == 0) return CPETGB_OK;
  if (!starts || !n_iter || !result) return fail(CPETGB_EINVAL, "line pointer is NULL");
  if (N > 0 && (!x || !q)) return fail(CPETGB_EINVAL, "charge pointer is NULL");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;

  Scratch S(s);
  const double *ds = starts, *dx = x, *dq = q;
  const int32_t* dn = n_iter;
  double *dres = result, *dends = ends;
  int32_t* dsteps = steps;
  if (mem == CPETGB_HOST) {
    CK(h2d(const_cast<double**>(&ds), S, starts, size_t(L) * 3), "copy starts");
    CK(h2d(const_cast<int32_t**>(&dn), S, n_iter, size_t(L)), "copy n_iter");
    if (N) {
      CK(h2d(const_cast<double**>(&dx), S, x, size_t(N) * 3), "copy charge positions");
      CK(h2d(const_cast<double**>(&dq), S, q, size_t(N) * (source == kDipoles ? 3 : 1)),
         "copy charges");
    }
    CK(S.get(&dres, size_t(L) * 2), "alloc result");
    if (ends) CK(S.get(&dends, size_t(L) * 3), "alloc ends");
    if (steps) CK(S.get(&dsteps, size_t(L)), "alloc steps");
  }
  const int pad = topo_charge_pad(prec);
  const int64_t n_pad = ((std::max(N, 1) + int64_t(pad) - 1) / pad) * pad;
  unsigned char* packed = nullptr;
  int* queue = nullptr;
  CK(S.get(&packed, size_t(n_pad) * topo_source_bytes(prec, source)), "alloc packed charges");
  CK(S.get(&queue, 1), "alloc queue");
  CK(cudaMemsetAsync(queue, 0, sizeof(int), s), "zero queue");
  if (reinterpret_cast<uintptr_t>(packed) % 16 != 0)
    return fail(CPETGB_ECUDA, "scratch allocation is not 16-byte aligned");
  if (source == kDipoles)
    CK(launch_pack_dipoles(prec, N, n_pad, dx, dq, packed, s), "pack dipoles");
  else
    CK(launch_pack_topo(prec, N, n_pad, dx, dq, packed, s), "pack charges");
  TopoParams p;
  p.source = source;
  p.n_lines = L;
  p.n_charges = N;
  p.step = step;
  for (int k = 0; k < 3; ++k) p.half[k] = half[k];
  p.starts = ds;
  p.n_iter = dn;
  p.packed = packed;
  p.result = dres;
  p.ends = dends;
  p.steps = dsteps;
  p.queue = queue;
  p.status = c->status;
  CK(launch_topo(prec, p, c->sms, s), "topo kernel launch");
  if (mem == CPETGB_HOST) {
    CK(cudaMemcpyAsync(result, dres, size_t(L) * 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy result");
    if (ends)
      CK(cudaMemcpyAsync(ends, dends, size_t(L) * 3 * sizeof(double), cudaMemcpyDeviceToHost, s),
         "copy ends");
    if (steps)
      CK(cudaMemcpyAsync(steps, dsteps, size_t(L) * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
         "copy steps");
    return finish(c, s);
  }
  return CPETGB_OK;
}

struct TopoTables {
  std::vector<TopoFrame> frames;
  std::vector<int64_t> src;  // per frame {charge offset, charge count} into x/q
  int64_t tot_lines = 0, tot_ch = 0, packed_elems = 0;
  int max_res = 0, max_pairs = 0;
  bool all_resident = true;  // every frame entirely in shared memory (tuner class 1)
};

// Frame table of a streamline launch: padded sizes, packed offsets (FP32C
// frames occupy n_pad float4 -- the pair block A then B --, FP64 frames n_pad
// Charge64), how many charges of each frame stay resident in shared memory.
int build_topo_tables(int prec, int F, const int64_t* desc, const double* params, TopoTables& t) {
  if (!valid_prec(prec)) return fail(CPETGB_EINVAL, "bad precision %d", prec);
  if (F < 0 || (F > 0 && (!desc || !params))) return fail(CPETGB_EINVAL, "bad frame table");
  const int pad = topo_charge_pad(prec);
  t.frames.assign(F, TopoFrame{});
  t.src.assign(2 * size_t(F), 0);
  for (int f = 0; f < F; ++f) {
    const int64_t co = desc[4 * f], n = desc[4 * f + 1], lo = desc[4 * f + 2], L = desc[4 * f + 3];
    if (co < 0 || n < 0 || lo < 0 || L < 0 || n > INT_MAX / 2 || L > INT_MAX)
      return fail(CPETGB_EINVAL, "frame %d: negative or oversized offset/count", f);
    const double* pr = params + 4 * f;
    if (!std::isfinite(pr[0])) return fail(CPETGB_EINVAL, "frame %d: step must be finite", f);
    for (int k = 1; k < 4; ++k)
      if (!std::isfinite(pr[k]) || pr[k] < 0)
        return fail(CPETGB_EINVAL, "frame %d: half-widths must be finite and >= 0", f);
    TopoFrame& fr = t.frames[f];
    fr.n_pad = static_cast<int32_t>(((std::max<int64_t>(n, 1) + pad - 1) / pad) * pad);
    fr.packed_off = t.packed_elems;
    t.packed_elems += fr.n_pad;
    fr.line_off = lo;
    fr.n_lines = static_cast<int32_t>(L);
    fr.resident = topo_resident_count(prec, kCharges, fr.n_pad);
    fr.pad_ = 0;
    fr.step = pr[0];
    for (int k = 0; k < 3; ++k) fr.half[k] = pr[1 + k];
    t.max_res = std::max(t.max_res, int(fr.resident));
    if (fr.resident < fr.n_pad) t.all_resident = false;
    t.max_pairs = std::max(t.max_pairs, int(fr.n_pad));
    t.src[2 * f] = co;
    t.src[2 * f + 1] = n;
    t.tot_lines = std::max(t.tot_lines, lo + L);
    t.tot_ch = std::max(t.tot_ch, co + n);
  }
  if (t.tot_lines > INT_MAX) return fail(CPETGB_EINVAL, "too many lines");
  return CPETGB_OK;
}

int topo_batch_impl(int prec, int mem, int F, const int64_t* desc, const double* params,
                    const double* starts, const int32_t* n_iter, const double* x, const double* q,
                    double* result, double* ends, int32_t* steps, void* stream) {
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  TopoTables t;
  int rc0 = build_topo_tables(prec, F, desc, params, t);
  if (rc0 != CPETGB_OK) return rc0;
  std::vector<TopoFrame>& frames = t.frames;
  std::vector<int64_t>& src = t.src;
  const int64_t tot_lines = t.tot_lines, tot_ch = t.tot_ch, packed_elems = t.packed_elems;
  const int max_res = t.max_res, max_pairs = t.max_pairs;
  const bool all_resident = t.all_resident;
  if (tot_lines == 0) return CPETGB_OK;
  if (!starts || !n_iter || !result) return fail(CPETGB_EINVAL, "line pointer is NULL");
  if (tot_ch > 0 && (!x || !q)) return fail(CPETGB_EINVAL, "charge pointer is NULL");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;
  const size_t L = size_t(tot_lines);
  Scratch S(s);
  const double *ds = starts, *dx = x, *dq = q;
  const int32_t* dn = n_iter;
  double *dres = result, *dends = ends;
  int32_t* dsteps = steps;
  if (mem == CPETGB_HOST) {
    CK(h2d(const_cast<double**>(&ds), S, starts, L * 3), "copy starts");
    CK(h2d(const_cast<int32_t**>(&dn), S, n_iter, L), "copy n_iter");
    if (tot_ch) {
      CK(h2d(const_cast<double**>(&dx), S, x, size_t(tot_ch) * 3), "copy charge positions");
      CK(h2d(const_cast<double**>(&dq), S, q, size_t(tot_ch)), "copy charges");
    }
    CK(S.get(&dres, L * 2), "alloc result");
    if (ends) CK(S.get(&dends, L * 3), "alloc ends");
    if (steps) CK(S.get(&dsteps, L), "alloc steps");
  }
  unsigned char* packed = nullptr;
  TopoFrame* d_frames = nullptr;
  int64_t* d_src = nullptr;
  int* queues = nullptr;
  CK(S.get(&packed, size_t(std::max<int64_t>(packed_elems, 1)) * packed_size(prec)),
     "alloc packed charges");
  if (reinterpret_cast<uintptr_t>(packed) % 16 != 0)
    return fail(CPETGB_ECUDA, "scratch allocation is not 16-byte aligned");
  CK(h2d(&d_frames, S, frames.data(), frames.size()), "copy frame table");
  CK(h2d(&d_src, S, src.data(), src.size()), "copy frame sources");
  CK(S.get(&queues, size_t(F)), "alloc queues");
  CK(cudaMemsetAsync(queues, 0, sizeof(int) * size_t(F), s), "zero queues");
  CK(launch_pack_topo_frames(prec, F, d_frames, d_src, dx, dq, packed, max_pairs, s),
     "pack charges");
  TopoParams p{};
  p.n_lines = static_cast<int>(tot_lines);
  p.starts = ds;
  p.n_iter = dn;
  p.packed = packed;
  p.result = dres;
  p.ends = dends;
  p.steps = dsteps;
  p.queue = queues;
  p.status = c->status;
  p.frames = d_frames;
  p.n_frames = F;
  p.max_resident_pad = max_res;
  p.all_resident = all_resident ? 1 : 0;
  CK(launch_topo_frames(prec, p, c->sms, s), "topo kernel launch");
  if (mem == CPETGB_HOST) {
    CK(cudaMemcpyAsync(result, dres, L * 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy result");
    if (ends)
      CK(cudaMemcpyAsync(ends, dends, L * 3 * sizeof(double), cudaMemcpyDeviceToHost, s),
         "copy ends");
    if (steps)
      CK(cudaMemcpyAsync(steps, dsteps, L * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
         "copy steps");
    return finish(c, s);
  }
  return CPETGB_OK;
}

int hist_impl(int mem, int L, const double* result, int nb0, int nb1, const double* range,
              uint64_t* counts, double* edges, void* stream) {
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (L < 0 || nb0 < 1 || nb1 < 1 || nb0 + nb1 > 4096)
    return fail(CPETGB_EINVAL, "bad histogram shape (%d lines, %d x %d bins)", L, nb0, nb1);
  if (!range || !counts || (L > 0 && !result)) return fail(CPETGB_EINVAL, "NULL pointer");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;
  Scratch S(s);
  const double* dv = result;
  unsigned long long* dc = reinterpret_cast<unsigned long long*>(counts);
  double* de = edges;
  const size_t nbins = size_t(nb0) * nb1;
  if (mem == CPETGB_HOST) {
    if (L) CK(h2d(const_cast<double**>(&dv), S, result, size_t(L) * 2), "copy values");
    CK(S.get(&dc, nbins), "alloc counts");
  }
  if (mem == CPETGB_HOST || !edges) CK(S.get(&de, size_t(nb0 + nb1 + 2)), "alloc edges");
  CK(cudaMemsetAsync(dc, 0, nbins * sizeof(unsigned long long), s), "zero counts");
  CK(launch_hist2d(L, dv, nb0, nb1, range, de, dc, c->status, s), "histogram launch");
  if (mem == CPETGB_HOST) {
    CK(cudaMemcpyAsync(counts, dc, nbins * sizeof(uint64_t), cudaMemcpyDeviceToHost, s),
       "copy counts");
    if (edges)
      CK(cudaMemcpyAsync(edges, de, size_t(nb0 + nb1 + 2) * sizeof(double),
                         cudaMemcpyDeviceToHost, s),
         "copy edges");
    return finish(c, s);
  }
  return CPETGB_OK;
}

int hist_sets_impl(int mem, int n_sets, const int64_t* offsets, const double* values, int nb0,
                   int nb1, const double* range, uint64_t* counts, double* hists, void* stream) {
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (n_sets < 0 || nb0 < 1 || nb1 < 1 || nb0 + nb1 > 4096)
    return fail(CPETGB_EINVAL, "bad histogram shape (%d sets, %d x %d bins)", n_sets, nb0, nb1);
  if (n_sets == 0) return CPETGB_OK;
  if (!offsets || !range || (!counts && !hists)) return fail(CPETGB_EINVAL, "NULL pointer");
  if (offsets[0] != 0) return fail(CPETGB_EINVAL, "offsets[0] must be 0");
  int64_t max_set = 0;
  for (int f = 0; f < n_sets; ++f) {
    if (offsets[f + 1] < offsets[f]) return fail(CPETGB_EINVAL, "offsets decrease at set %d", f);
    max_set = std::max(max_set, offsets[f + 1] - offsets[f]);
  }
  const int64_t L = offsets[n_sets];
  if (L > 0 && !values) return fail(CPETGB_EINVAL, "values pointer is NULL");
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(range[k])) return fail(CPETGB_ERANGE, "histogram range must be finite");
  if (range[0] > range[1] || range[2] > range[3])
    return fail(CPETGB_ERANGE, "histogram range is inverted");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;
  Scratch S(s);
  const size_t nbins = size_t(nb0) * nb1, total = nbins * size_t(n_sets);
  const double* dv = values;
  unsigned long long* dc = reinterpret_cast<unsigned long long*>(counts);
  double* dh = hists;
  double* de = nullptr;
  int64_t* doff = nullptr;
  if (mem == CPETGB_HOST && L) CK(h2d(const_cast<double**>(&dv), S, values, size_t(L) * 2), "copy values");
  if (mem == CPETGB_HOST || !counts) CK(S.get(&dc, total), "alloc counts");
  if (mem == CPETGB_HOST && hists) CK(S.get(&dh, total), "alloc histograms");
  CK(S.get(&de, size_t(nb0 + nb1 + 2)), "alloc edges");
  CK(h2d(&doff, S, offsets, size_t(n_sets) + 1), "copy offsets");
  CK(cudaMemsetAsync(dc, 0, total * sizeof(unsigned long long), s), "zero counts");
  CK(launch_hist2d_sets(n_sets, doff, max_set, dv, nb0, nb1, range, de, dc, hists ? dh : nullptr,
                        c->status, s),
     "histogram launch");
  if (mem == CPETGB_HOST) {
    if (counts)
      CK(cudaMemcpyAsync(counts, dc, total * sizeof(uint64_t), cudaMemcpyDeviceToHost, s),
         "copy counts");
    if (hists)
      CK(cudaMemcpyAsync(hists, dh, total * sizeof(double), cudaMemcpyDeviceToHost, s),
         "copy histograms");
    return finish(c, s);
  }
  return CPETGB_OK;
}

int prepare_frame_impl(int mem, int n, const double* x, const double* q, const int32_t* resid,
                       const int32_t* resnum, const double* center, const double* inv,
                       double radius, const double* half, const double* shift, double* x_out,
                       double* q_out, int* n_out, void* stream) {
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (n < 0) return fail(CPETGB_EINVAL, "negative atom count");
  if (!center || !n_out) return fail(CPETGB_EINVAL, "center / n_out pointer is NULL");
  if (!std::isfinite(radius)) return fail(CPETGB_EINVAL, "radius must be finite (<= 0: no filter)");
  for (int k = 0; k < 3; ++k)
    if (!std::isfinite(center[k]) || (half && !(half[k] >= 0.0)) || (shift && !std::isfinite(shift[k])))
      return fail(CPETGB_EINVAL, "center, box half-widths and shift must be finite (half-widths >= 0)");
  if (inv)
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(inv[k])) return fail(CPETGB_EINVAL, "inverse basis must be finite");
  *n_out = 0;
  if (n == 0) return CPETGB_OK;
  if (!x || !q || !x_out || !q_out) return fail(CPETGB_EINVAL, "array pointer is NULL");
  if (radius > 0.0 && (!resid || !resnum))
    return fail(CPETGB_EINVAL, "the residue radius filter needs resid and resnum");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!s) s = c->stream;
  Scratch S(s);
  const double *dx = x, *dq = q;
  const int32_t *dr = resid, *dn = resnum;
  double *dxo = x_out, *dqo = q_out;
  if (mem == CPETGB_HOST) {
    CK(h2d(const_cast<double**>(&dx), S, x, size_t(n) * 3), "copy positions");
    CK(h2d(const_cast<double**>(&dq), S, q, size_t(n)), "copy charges");
    if (radius > 0.0) {
      CK(h2d(const_cast<int32_t**>(&dr), S, resid, size_t(n)), "copy resid");
      CK(h2d(const_cast<int32_t**>(&dn), S, resnum, size_t(n)), "copy resnum");
    }
    CK(S.get(&dxo, size_t(n) * 3), "alloc positions");
    CK(S.get(&dqo, size_t(n)), "alloc charges");
  }
  unsigned char* scratch = nullptr;
  int64_t* dcount = nullptr;
  CK(S.get(&scratch, prep_scratch_bytes(n)), "alloc scratch");
  CK(S.get(&dcount, 1), "alloc count");
  CK(launch_prepare_frame(n, dx, dq, dr, dn, center, inv, radius, half, shift, dxo, dqo, scratch,
                          dcount, s),
     "frame preparation");
  int64_t count = 0;
  CK(cudaMemcpyAsync(&count, dcount, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "read count");
  CK(cudaStreamSynchronize(s), "stream synchronize");
  *n_out = static_cast<int>(count);
  if (mem == CPETGB_HOST && count) {
    CK(cudaMemcpyAsync(x_out, dxo, size_t(count) * 3 * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy positions");
    CK(cudaMemcpyAsync(q_out, dqo, size_t(count) * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy charges");
    return finish(c, s);
  }
  return CPETGB_OK;
}

int format_text_impl(int fmt, int mem, int64_t n_rows, int n_cols, const float* values, char* text,
                     int64_t capacity, int64_t* length, void* stream) {
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (n_rows < 0 || n_cols < 1) return fail(CPETGB_EINVAL, "need n_rows >= 0 and n_cols >= 1");
  if (!length) return fail(CPETGB_EINVAL, "length pointer is NULL");
  if (n_rows > 0 && !values) return fail(CPETGB_EINVAL, "values pointer is NULL");
  if (n_rows > (int64_t(1) << 40) / n_cols) return fail(CPETGB_EINVAL, "matrix too large");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!s) s = c->stream;
  Scratch S(s);
  const float* dv = values;
  if (mem == CPETGB_HOST && n_rows)
    CK(h2d(const_cast<float**>(&dv), S, values, size_t(n_rows) * n_cols), "copy values");
  int64_t* off = nullptr;
  int64_t* scratch = nullptr;
  CK(S.get(&off, size_t(n_rows) + 1), "alloc offsets");
  CK(S.get(&scratch, size_t(fixed3_scan_scratch(n_rows + 1))), "alloc scan scratch");
  CK(launch_text_offsets(fmt, n_rows, n_cols, dv, off, scratch, s), "length pass");
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, off + n_rows, sizeof(int64_t), cudaMemcpyDeviceToHost, s), "read length");
  CK(cudaStreamSynchronize(s), "stream synchronize");
  *length = total;
  if (!text) return CPETGB_OK;
  if (capacity < total) return fail(CPETGB_ERANGE, "text buffer holds %lld bytes, %lld needed",
                                    (long long)capacity, (long long)total);
  char* dt = text;
  if (mem == CPETGB_HOST) CK(S.get(&dt, size_t(std::max<int64_t>(total, 1))), "alloc text");
  CK(launch_text_write(fmt, n_rows, n_cols, dv, off, dt, s), "write pass");
  if (mem == CPETGB_HOST) {
    if (total) CK(cudaMemcpyAsync(text, dt, size_t(total), cudaMemcpyDeviceToHost, s), "copy text");
    return finish(c, s);
  }
  return CPETGB_OK;
}

// kind 0: chi-square over histogram rows [n][feat]; kind 1: field rows [n][feat][3].
int distance_impl(int kind, int prec, int mem, int n, int feat, const double* src, double* out,
                  void* stream) {
  if (!valid_prec(prec)) return fail(CPETGB_EINVAL, "bad precision %d", prec);
  if (!valid_mem(mem)) return fail(CPETGB_EINVAL, "bad memory kind %d", mem);
  if (n < 0 || feat < 0) return fail(CPETGB_EINVAL, "negative matrix or feature count");
  if (n > 65535 * 64) return fail(CPETGB_EINVAL, "at most %d rows", 65535 * 64);
  if (n == 0) return CPETGB_OK;
  if (!out || (feat > 0 && !src)) return fail(CPETGB_EINVAL, "NULL pointer");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mem == CPETGB_HOST && !s) s = c->stream;
  Scratch S(s);
  const size_t nc = kind == 0 ? 1 : 3;
  const double* dsrc = src;
  double* dout = out;
  if (mem == CPETGB_HOST) {
    if (feat) CK(h2d(const_cast<double**>(&dsrc), S, src, size_t(n) * feat * nc), "copy rows");
    CK(S.get(&dout, size_t(n) * n), "alloc matrix");
  }
  const int splits = distance_splits(n, feat, c->sms);
  double* partial = nullptr;
  if (splits > 1) CK(S.get(&partial, size_t(splits) * n * n), "alloc partial sums");
  unsigned char* f32_rows = nullptr;
  if (prec != CPETGB_FP64 && feat > 0)
    CK(S.get(&f32_rows, distance_f32_bytes(kind, n, feat)), "alloc float rows");
  CK(launch_distance_matrix(prec, kind, n, feat, dsrc, dout, splits, partial, f32_rows, s),
     "distance launch");
  if (mem == CPETGB_HOST) {
    CK(cudaMemcpyAsync(out, dout, size_t(n) * n * sizeof(double), cudaMemcpyDeviceToHost, s),
       "copy matrix");
    return finish(c, s);
  }
  return CPETGB_OK;
}

std::vector<double> widen(const float* p, size_t n) {
  std::vector<double> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = p[i];
  return v;
}

template <typename T>
cudaError_t plan_alloc(std::vector<void*>& bufs, T** p, size_t count) {
  *p = nullptr;
  void* v = nullptr;
  cudaError_t e = cudaMalloc(&v, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) {
    bufs.push_back(v);
    *p = static_cast<T*>(v);
  }
  return e;
}

}  // namespace

// A prepared launch: device tables and scratch allocated once, the launch
// sequence captured into a CUDA graph and replayed by cpetgb_plan_launch.
struct cpetgb_plan {
  int device = -1;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> bufs;
  ~cpetgb_plan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : bufs) cudaFree(p);
  }
};

namespace {

// Captures `body` (launches on the capture stream) into plan->graph/exec.
template <typename Body>
int capture_plan(cpetgb_plan* pl, Body body) {
  cudaStream_t cs = nullptr;
  CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    return cuda_fail(e, "begin capture");
  }
  const int rc = body(cs);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);
  cudaStreamDestroy(cs);
  if (rc != CPETGB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  pl->graph = g;
  CK(cudaGraphInstantiate(&pl->exec, g, 0), "graph instantiate");
  return CPETGB_OK;
}

int grid_plan_impl(cpetgb_plan** out_plan, int kind, int prec, int clamp, int n_frames,
                   const int64_t* desc, const double* pts, const double* x, const double* q,
                   double* out) {
  if (!out_plan) return fail(CPETGB_EINVAL, "plan pointer is NULL");
  *out_plan = nullptr;
  if (kind != CPETGB_FIELD && kind != CPETGB_ESP) return fail(CPETGB_EINVAL, "bad grid kind %d", kind);
  if (!valid_prec(prec)) return fail(CPETGB_EINVAL, "bad precision %d", prec);
  if (n_frames < 0 || (n_frames > 0 && !desc)) return fail(CPETGB_EINVAL, "bad frame table");
  int64_t tot_pts = 0, tot_ch = 0;
  for (int f = 0; f < n_frames; ++f) {
    const int64_t co = desc[4 * f], n = desc[4 * f + 1], po = desc[4 * f + 2], P = desc[4 * f + 3];
    if (co < 0 || n < 0 || po < 0 || P < 0 || n > INT_MAX || P > INT_MAX)
      return fail(CPETGB_EINVAL, "frame %d: negative or oversized offset/count", f);
    tot_pts = std::max(tot_pts, po + P);
    tot_ch = std::max(tot_ch, co + n);
  }
  if (tot_pts > 0 && (!pts || !out)) return fail(CPETGB_EINVAL, "points/output pointer is NULL");
  if (tot_ch > 0 && (!x || !q)) return fail(CPETGB_EINVAL, "charge pointer is NULL");
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  GridPlan gp;
  int ppt = 4, ips = 8;
  tuned_grid_shape(prec, kind, grid_pair_evals(n_frames, desc), &ppt, &ips);
  plan_grid(n_frames, desc, c->sms, gp, ppt, ips);
  cpetgb_plan* pl = new cpetgb_plan();
  cudaGetDevice(&pl->device);
  unsigned char* packed = nullptr;
  GridItem* d_items = nullptr;
  GridFinal* d_fin = nullptr;
  double* partial = nullptr;
  cudaError_t e = plan_alloc(pl->bufs, &packed, size_t(std::max<int64_t>(tot_ch, 1)) * kGridRecord);
  if (e == cudaSuccess) e = plan_alloc(pl->bufs, &d_items, gp.items.size());
  if (e == cudaSuccess && !gp.items.empty())
    e = cudaMemcpy(d_items, gp.items.data(), gp.items.size() * sizeof(GridItem), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !gp.finals.empty()) {
    e = plan_alloc(pl->bufs, &d_fin, gp.finals.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(d_fin, gp.finals.data(), gp.finals.size() * sizeof(GridFinal),
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = plan_alloc(pl->bufs, &partial, size_t(gp.n_slots) * kGridSlotPts * 3);
  }
  if (e != cudaSuccess) {
    delete pl;
    return cuda_fail(e, "plan allocation");
  }
  const double tau = g_refine_tau.load();
  const bool refine = kind == CPETGB_FIELD && prec == CPETGB_FP32C && tau > 0.0 && tot_ch > 0 &&
                      max_frame_points(n_frames, desc) >= 3;
  int64_t *d_desc = nullptr, *list = nullptr;
  int* count = nullptr;
  unsigned char* dfq = nullptr;
  int* hist = nullptr;
  if (refine) {
    e = plan_alloc(pl->bufs, &d_desc, size_t(n_frames) * 4);
    if (e == cudaSuccess) e = plan_alloc(pl->bufs, &hist, size_t(grid_refine_hist_ints(n_frames)));
    if (e == cudaSuccess) e = plan_alloc(pl->bufs, &dfq, size_t(tot_ch) * 32);
    if (e == cudaSuccess)
      e = cudaMemcpy(d_desc, desc, size_t(n_frames) * 4 * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = plan_alloc(pl->bufs, &list, size_t(refine_list_len(n_frames, desc)) * 2);
    if (e == cudaSuccess) e = plan_alloc(pl->bufs, &count, 1);
    if (e == cudaSuccess) e = preload_grid_refine();
    if (e != cudaSuccess) {
      delete pl;
      return cuda_fail(e, "plan allocation");
    }
  }
  const int n_items = static_cast<int>(gp.items.size()), n_fin = static_cast<int>(gp.finals.size());
  e = preload_grid_kernels(prec, kind, clamp ? 1 : 0, ppt);
  if (e != cudaSuccess) {
    delete pl;
    return cuda_fail(e, "kernel load");
  }
  rc = capture_plan(pl, [&](cudaStream_t cs) -> int {
    CK(launch_pack_charges(prec, tot_ch, tot_ch, x, q, packed, cs), "pack charges");
    CK(launch_grid(prec, kind, clamp ? 1 : 0, ppt, n_items, d_items, packed, pts, out, partial,
                   c->status, cs),
       "grid kernel launch");
    CK(launch_grid_final(kind, n_fin, d_fin, partial, out, cs), "grid reduction launch");
    if (refine)
      CK(launch_grid_refine(n_frames, tot_ch, max_frame_points(n_frames, desc), d_desc, pts, x, q, out,
                            clamp ? 1 : 0, tau, list, count, hist, dfq, c->sms, cs),
         "field refinement launch");
    return CPETGB_OK;
  });
  if (rc != CPETGB_OK) {
    delete pl;
    return rc;
  }
  *out_plan = pl;
  return CPETGB_OK;
}

int topo_plan_impl(cpetgb_plan** out_plan, int prec, int F, const int64_t* desc,
                   const double* params, const double* starts, const int32_t* n_iter,
                   const double* x, const double* q, double* result, double* ends, int32_t* steps) {
  if (!out_plan) return fail(CPETGB_EINVAL, "plan pointer is NULL");
  *out_plan = nullptr;
  TopoTables t;
  int rc = build_topo_tables(prec, F, desc, params, t);
  if (rc != CPETGB_OK) return rc;
  if (t.tot_lines > 0 && (!starts || !n_iter || !result))
    return fail(CPETGB_EINVAL, "line pointer is NULL");
  if (t.tot_ch > 0 && (!x || !q)) return fail(CPETGB_EINVAL, "charge pointer is NULL");
  Ctx* c = context(&rc);
  if (!c) return rc;
  cpetgb_plan* pl = new cpetgb_plan();
  cudaGetDevice(&pl->device);
  unsigned char* packed = nullptr;
  TopoFrame* d_frames = nullptr;
  int64_t* d_src = nullptr;
  int* queues = nullptr;
  cudaError_t e =
      plan_alloc(pl->bufs, &packed, size_t(std::max<int64_t>(t.packed_elems, 1)) * packed_size(prec));
  if (e == cudaSuccess) e = plan_alloc(pl->bufs, &d_frames, t.frames.size());
  if (e == cudaSuccess) e = plan_alloc(pl->bufs, &d_src, t.src.size());
  if (e == cudaSuccess) e = plan_alloc(pl->bufs, &queues, size_t(std::max(F, 1)));
  if (e == cudaSuccess && F > 0)
    e = cudaMemcpy(d_frames, t.frames.data(), t.frames.size() * sizeof(TopoFrame),
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess && F > 0)
    e = cudaMemcpy(d_src, t.src.data(), t.src.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete pl;
    return cuda_fail(e, "plan allocation");
  }
  if (reinterpret_cast<uintptr_t>(packed) % 16 != 0) {
    delete pl;
    return fail(CPETGB_ECUDA, "plan allocation is not 16-byte aligned");
  }
  TopoParams p{};
  p.n_lines = static_cast<int>(t.tot_lines);
  p.starts = starts;
  p.n_iter = n_iter;
  p.packed = packed;
  p.result = result;
  p.ends = ends;
  p.steps = steps;
  p.queue = queues;
  p.status = c->status;
  p.frames = d_frames;
  p.n_frames = F;
  p.max_resident_pad = t.max_res;
  p.all_resident = t.all_resident ? 1 : 0;
  const int max_pairs = t.max_pairs;
  rc = capture_plan(pl, [&](cudaStream_t cs) -> int {
    CK(cudaMemsetAsync(queues, 0, sizeof(int) * size_t(std::max(F, 1)), cs), "zero queues");
    CK(launch_pack_topo_frames(prec, F, d_frames, d_src, x, q, packed, max_pairs, cs),
       "pack charges");
    CK(launch_topo_frames(prec, p, c->sms, cs), "topo kernel launch");
    return CPETGB_OK;
  });
  if (rc != CPETGB_OK) {
    delete pl;
    return rc;
  }
  *out_plan = pl;
  return CPETGB_OK;
}

}  // namespace

int cpetgb::set_error(int code, const char* msg) { return fail(code, "%s", msg); }

int cpetgb::tuned_topo_slots(int prec, bool resident, int n_lines) {
  const int v = tune_choose(tune_key(kOpTopo, prec, resident ? 1 : 0, double(n_lines)));
  return v == 1 ? 2 : 4;
}

void cpetgb::tuned_grid_shape(int prec, int kind, double pair_evals, int* ppt, int* items_per_sm) {
  int v = tune_choose(tune_key(kOpGrid, prec, kind, pair_evals));
  if (v < 0 || v >= kGridVariants) v = 1;  // untuned: 4 points per thread, 8 items per SM
  if (v >= 10) {
    *ppt = ((v - 10) / 2) == 1 ? 8 : 4;
    *items_per_sm = ((v - 10) % 2) == 0 ? 128 : 256;
    return;
  }
  static const int ips[5] = {4, 8, 16, 32, 64};
  *ppt = (v / 5) == 1 ? 8 : 4;
  *items_per_sm = ips[v % 5];
}

extern "C" {

int cpetgb_version(void) { return kVersion; }

int cpetgb_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return CPETGB_EINVAL;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return CPETGB_OK;
}

int cpetgb_device_sms(void) {
  int rc;
  Ctx* c = context(&rc);
  return c ? c->sms : rc;
}

int cpetgb_synchronize(void* stream) {
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  return finish(c, static_cast<cudaStream_t>(stream));
}

int cpetgb_check_wait_limit(double seconds) {
  if (!(seconds > 0.0) || seconds > 2.0)
    return fail(CPETGB_EINVAL, "wait limit must be in (0, 2] s, got %g", seconds);
  int rc;
  Ctx* c = context(&rc);
  if (!c) return rc;
  const unsigned long long ns = static_cast<unsigned long long>(seconds * 1e9);
  CK(launch_wait_limit_check(c->status, ns, c->stream), "wait check launch");
  return finish(c, c->stream);
}

int cpetgb_set_field_refinement(double tau) {
  if (!(tau >= 0.0) || !std::isfinite(tau) || tau > 1.0)
    return fail(CPETGB_EINVAL, "refinement threshold must be in [0, 1], got %g", tau);
  g_refine_tau.store(tau);
  return CPETGB_OK;
}

double cpetgb_field_refinement(void) { return g_refine_tau.load(); }

int cpetgb_set_default_precision(int precision) {
  if (!valid_prec(precision)) return fail(CPETGB_EINVAL, "bad precision %d", precision);
  g_default_prec.store(precision);
  return CPETGB_OK;
}

int cpetgb_get_default_precision(void) { return g_default_prec.load(); }

int cpetgb_field_grid(int precision, int mem, int n_points, int n_charges, const double* points,
                      const double* x, const double* q, int clamp, double* field, void* stream) {
  if (n_points < 0 || n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  const int64_t desc[4] = {0, n_charges, 0, n_points};
  return grid_batch_impl(CPETGB_FIELD, precision, mem, clamp, 1, desc, points, x, q, field, stream);
}

int cpetgb_esp_grid(int precision, int mem, int n_points, int n_charges, const double* points,
                    const double* x, const double* q, double* esp, void* stream) {
  if (n_points < 0 || n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  const int64_t desc[4] = {0, n_charges, 0, n_points};
  return grid_batch_impl(CPETGB_ESP, precision, mem, 0, 1, desc, points, x, q, esp, stream);
}

int cpetgb_grid_batch(int kind, int precision, int mem, int clamp, int n_frames,
                      const int64_t* desc, const double* points, const double* x,
                      const double* q, double* out, void* stream) {
  return grid_batch_impl(kind, precision, mem, clamp, n_frames, desc, points, x, q, out, stream);
}

int cpetgb_topo_lines(int precision, int mem, int n_lines, int n_charges, const double* starts,
                      const int32_t* n_iter, double step, const double* half_dims,
                      const double* x, const double* q, double* result, double* ends,
                      int32_t* steps, void* stream) {
  return topo_impl(precision, mem, n_lines, n_charges, starts, n_iter, step, half_dims, x, q,
                   result, ends, steps, stream);
}

int cpetgb_topo_dipole_lines(int precision, int mem, int n_lines, int n_dipoles,
                             const double* starts, const int32_t* n_iter, double step,
                             const double* half_dims, const double* x, const double* mu,
                             double* result, double* ends, int32_t* steps, void* stream) {
  return topo_impl(precision, mem, n_lines, n_dipoles, starts, n_iter, step, half_dims, x, mu,
                   result, ends, steps, stream, kDipoles);
}

int cpetgb_topo_batch(int precision, int mem, int n_frames, const int64_t* desc,
                      const double* params, const double* starts, const int32_t* n_iter,
                      const double* x, const double* q, double* result, double* ends,
                      int32_t* steps, void* stream) {
  return topo_batch_impl(precision, mem, n_frames, desc, params, starts, n_iter, x, q, result, ends,
                         steps, stream);
}

int cpetgb_grid_plan_create(cpetgb_plan** plan, int kind, int precision, int clamp, int n_frames,
                            const int64_t* desc, const double* points, const double* x,
                            const double* q, double* out) {
  return grid_plan_impl(plan, kind, precision, clamp, n_frames, desc, points, x, q, out);
}

int cpetgb_topo_plan_create(cpetgb_plan** plan, int precision, int n_frames, const int64_t* desc,
                            const double* params, const double* starts, const int32_t* n_iter,
                            const double* x, const double* q, double* result, double* ends,
                            int32_t* steps) {
  return topo_plan_impl(plan, precision, n_frames, desc, params, starts, n_iter, x, q, result, ends,
                        steps);
}

int cpetgb_tune_key(int op, int precision, int cls, double size) {
  if ((op != kOpGrid && op != kOpTopo) || !valid_prec(precision) || cls < 0 || cls > 15 ||
      !(size >= 0))
    return fail(CPETGB_EINVAL, "bad tuning key arguments");
  return tune_key(op, precision, cls, size);
}

int cpetgb_tune_variants(int op) {
  if (op == kOpGrid) return kGridVariants;
  if (op == kOpTopo) return kTopoVariants;
  return fail(CPETGB_EINVAL, "bad operation %d", op);
}

int cpetgb_topo_resident_limit(int precision, int dipoles) {
  if (!valid_prec(precision)) return fail(CPETGB_EINVAL, "bad precision %d", precision);
  int rc;
  if (!context(&rc)) return rc;
  return static_cast<int>(topo_resident_limit(precision, dipoles ? kDipoles : kCharges));
}

int cpetgb_tune_set(int key, int variant) {
  const int op = key >> 12;
  const int n = op == kOpGrid ? kGridVariants : (op == kOpTopo ? kTopoVariants : 0);
  if (key < 0 || variant < -1 || variant >= n) return fail(CPETGB_EINVAL, "bad tuning entry");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (variant < 0)
    g_tune.erase(key);
  else
    g_tune[key] = variant;
  return CPETGB_OK;
}

int cpetgb_tune_get(int key) { return tune_lookup(key); }

int cpetgb_plan_launch(cpetgb_plan* plan, void* stream) {
  if (!plan || !plan->exec) return fail(CPETGB_EINVAL, "plan is NULL or empty");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != plan->device)
    return fail(CPETGB_EINVAL, "plan belongs to device %d; current device is %d", plan->device, dev);
  CK(cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream)), "graph launch");
  return CPETGB_OK;
}

int cpetgb_plan_destroy(cpetgb_plan* plan) {
  delete plan;
  return CPETGB_OK;
}

int cpetgb_topo_hist2d(int mem, int n_lines, const double* result, int nb_dist, int nb_curv,
                       const double* range, uint64_t* counts, double* edges, void* stream) {
  return hist_impl(mem, n_lines, result, nb_dist, nb_curv, range, counts, edges, stream);
}

int cpetgb_prepare_frame(int mem, int n_atoms, const double* x, const double* q,
                         const int32_t* resid, const int32_t* resnum, const double* center,
                         const double* inv_basis, double radius, const double* box_half,
                         const double* box_shift, double* x_out, double* q_out, int* n_out,
                         void* stream) {
  return prepare_frame_impl(mem, n_atoms, x, q, resid, resnum, center, inv_basis, radius, box_half,
                            box_shift, x_out, q_out, n_out, stream);
}

int cpetgb_format_fixed3(int mem, int64_t n_rows, int n_cols, const float* values, char* text,
                         int64_t capacity, int64_t* length, void* stream) {
  return format_text_impl(kTextFixed3, mem, n_rows, n_cols, values, text, capacity, length, stream);
}

int cpetgb_format_sci18(int mem, int64_t n_rows, int n_cols, const float* values, char* text,
                        int64_t capacity, int64_t* length, void* stream) {
  return format_text_impl(kTextSci18, mem, n_rows, n_cols, values, text, capacity, length, stream);
}

int cpetgb_topo_hist2d_sets(int mem, int n_sets, const int64_t* offsets, const double* values,
                            int nb_dist, int nb_curv, const double* range, uint64_t* counts,
                            double* hists, void* stream) {
  return hist_sets_impl(mem, n_sets, offsets, values, nb_dist, nb_curv, range, counts, hists,
                        stream);
}

int cpetgb_chi2_distance_matrix(int precision, int mem, int n, int bins, const double* hists,
                                double* out, void* stream) {
  return distance_impl(0, precision, mem, n, bins, hists, out, stream);
}

int cpetgb_field_distance_matrix(int precision, int mem, int n, int n_points,
                                 const double* fields, double* out, void* stream) {
  return distance_impl(1, precision, mem, n, n_points, fields, out, stream);
}

// ---- float32 drop-ins ----------------------------------------------------

int cpetgb_compute_looped_field_p(int precision, int total_points, int n_charges,
                                  const float* x_0, const float* x, const float* Q, float* E) {
  if (total_points < 0 || n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  if (total_points == 0) return CPETGB_OK;
  if (!x_0 || !E || (n_charges && (!x || !Q))) return fail(CPETGB_EINVAL, "NULL pointer");
  auto p = widen(x_0, size_t(total_points) * 3);
  auto xx = widen(x, size_t(n_charges) * 3);
  auto qq = widen(Q, size_t(n_charges));
  std::vector<double> out(size_t(total_points) * 3);
  const int rc = cpetgb_field_grid(precision, CPETGB_HOST, total_points, n_charges,
                                   p.data(), xx.data(), qq.data(), 1, out.data(), nullptr);
  if (rc != CPETGB_OK) return rc;
  for (size_t i = 0; i < out.size(); ++i) E[i] = static_cast<float>(out[i]);
  return CPETGB_OK;
}

int cpetgb_compute_esp_grid_p(int precision, int total_points, int n_charges, const float* x_0,
                              const float* x, const float* Q, float* ESP) {
  if (total_points < 0 || n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  if (total_points == 0) return CPETGB_OK;
  if (!x_0 || !ESP || (n_charges && (!x || !Q))) return fail(CPETGB_EINVAL, "NULL pointer");
  auto p = widen(x_0, size_t(total_points) * 3);
  auto xx = widen(x, size_t(n_charges) * 3);
  auto qq = widen(Q, size_t(n_charges));
  std::vector<double> out(static_cast<size_t>(total_points));
  const int rc = cpetgb_esp_grid(precision, CPETGB_HOST, total_points, n_charges,
                                 p.data(), xx.data(), qq.data(), out.data(), nullptr);
  if (rc != CPETGB_OK) return rc;
  for (size_t i = 0; i < out.size(); ++i) ESP[i] = static_cast<float>(out[i]);
  return CPETGB_OK;
}

int cpetgb_calc_esp_base_p(int precision, float* ESP, const float* x_init, int n_charges,
                           const float* x, const float* Q) {
  if (!ESP || !x_init) return fail(CPETGB_EINVAL, "NULL pointer");
  float v = 0.f;
  const int rc = cpetgb_compute_esp_grid_p(precision, 1, n_charges, x_init, x, Q, &v);
  if (rc != CPETGB_OK) return rc;
  ESP[0] += v;
  return CPETGB_OK;
}

int cpetgb_calc_field_p(int precision, float* E, const float* x_init, int n_charges,
                        const float* x, const float* Q) {
  if (!E || !x_init) return fail(CPETGB_EINVAL, "NULL pointer");
  if (n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  double p[3] = {x_init[0], x_init[1], x_init[2]}, out[3];
  auto xx = widen(x, size_t(n_charges) * 3);
  auto qq = widen(Q, size_t(n_charges));
  const int rc = cpetgb_field_grid(precision, CPETGB_HOST, 1, n_charges, p, xx.data(),
                                   qq.data(), 0, out, nullptr);
  if (rc != CPETGB_OK) return rc;
  for (int k = 0; k < 3; ++k) E[k] = static_cast<float>(out[k]);
  return CPETGB_OK;
}

int cpetgb_thread_operation_batch_p(int precision, int n_lines, int n_charges,
                                    const int32_t* n_iter, float step_size, const float* x_0,
                                    const float* dimensions, const float* x, const float* Q,
                                    float* ret) {
  if (n_lines < 0 || n_charges < 0) return fail(CPETGB_EINVAL, "negative size");
  if (n_lines == 0) return CPETGB_OK;
  if (!n_iter || !x_0 || !dimensions || !ret || (n_charges && (!x || !Q)))
    return fail(CPETGB_EINVAL, "NULL pointer");
  auto s = widen(x_0, size_t(n_lines) * 3);
  auto xx = widen(x, size_t(n_charges) * 3);
  auto qq = widen(Q, size_t(n_charges));
  const double half[3] = {dimensions[0], dimensions[1], dimensions[2]};
  std::vector<double> res(size_t(n_lines) * 2);
  const int rc = cpetgb_topo_lines(precision, CPETGB_HOST, n_lines, n_charges,
                                   s.data(), n_iter, double(step_size), half, xx.data(),
                                   qq.data(), res.data(), nullptr, nullptr, nullptr);
  if (rc != CPETGB_OK) return rc;
  for (size_t i = 0; i < res.size(); ++i) ret[i] = static_cast<float>(res[i]);
  return CPETGB_OK;
}

int cpetgb_thread_operation_p(int precision, int n_charges, int n_iter, float step_size,
                              const float* x_0, const float* dimensions, const float* x,
                              const float* Q, float* ret) {
  const int32_t it = n_iter;
  return cpetgb_thread_operation_batch_p(precision, 1, n_charges, &it, step_size, x_0, dimensions,
                                         x, Q, ret);
}

int cpetgb_thread_operation_dipole_p(int precision, int n_dipoles, int n_iter, float step_size,
                                     const float* x_0, const float* dimensions, const float* x,
                                     const float* mu, float* ret) {
  if (n_dipoles < 0) return fail(CPETGB_EINVAL, "negative size");
  if (!x_0 || !dimensions || !ret || (n_dipoles && (!x || !mu)))
    return fail(CPETGB_EINVAL, "NULL pointer");
  auto s = widen(x_0, 3);
  auto xx = widen(x, size_t(n_dipoles) * 3);
  auto mm = widen(mu, size_t(n_dipoles) * 3);
  const double half[3] = {dimensions[0], dimensions[1], dimensions[2]};
  const int32_t it = n_iter;
  double res[2];
  const int rc = cpetgb_topo_dipole_lines(precision, CPETGB_HOST, 1, n_dipoles,
                                          s.data(), &it, double(step_size), half, xx.data(),
                                          mm.data(), res, nullptr, nullptr, nullptr);
  if (rc != CPETGB_OK) return rc;
  ret[0] = static_cast<float>(res[0]);
  ret[1] = static_cast<float>(res[1]);
  return CPETGB_OK;
}

// The reference-shaped entry points: the same calls in the library's default precision.
int cpetgb_compute_looped_field(int total_points, int n_charges, const float* x_0,
                                const float* x, const float* Q, float* E) {
  return cpetgb_compute_looped_field_p(g_default_prec.load(), total_points, n_charges, x_0, x, Q,
                                       E);
}

int cpetgb_compute_esp_grid(int total_points, int n_charges, const float* x_0, const float* x,
                            const float* Q, float* ESP) {
  return cpetgb_compute_esp_grid_p(g_default_prec.load(), total_points, n_charges, x_0, x, Q,
                                   ESP);
}

int cpetgb_calc_esp_base(float* ESP, const float* x_init, int n_charges, const float* x,
                         const float* Q) {
  return cpetgb_calc_esp_base_p(g_default_prec.load(), ESP, x_init, n_charges, x, Q);
}

int cpetgb_calc_field(float* E, const float* x_init, int n_charges, const float* x,
                      const float* Q) {
  return cpetgb_calc_field_p(g_default_prec.load(), E, x_init, n_charges, x, Q);
}

int cpetgb_thread_operation_batch(int n_lines, int n_charges, const int32_t* n_iter,
                                  float step_size, const float* x_0, const float* dimensions,
                                  const float* x, const float* Q, float* ret) {
  return cpetgb_thread_operation_batch_p(g_default_prec.load(), n_lines, n_charges, n_iter,
                                         step_size, x_0, dimensions, x, Q, ret);
}

int cpetgb_thread_operation(int n_charges, int n_iter, float step_size, const float* x_0,
                            const float* dimensions, const float* x, const float* Q,
                            float* ret) {
  return cpetgb_thread_operation_p(g_default_prec.load(), n_charges, n_iter, step_size, x_0,
                                   dimensions, x, Q, ret);
}

int cpetgb_thread_operation_dipole(int n_dipoles, int n_iter, float step_size, const float* x_0,
                                   const float* dimensions, const float* x, const float* mu,
                                   float* ret) {
  return cpetgb_thread_operation_dipole_p(g_default_prec.load(), n_dipoles, n_iter, step_size,
                                          x_0, dimensions, x, mu, ret);
}

}  // extern "C"

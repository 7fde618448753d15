// kernels.cuh -- launch interface between the C-ABI layer (api.cu) and the
// kernels (grid.cu, topo.cu, hist.cu).  Host-side declarations only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cpetgb {

enum Precision : int { kFP64 = 0, kFP32C = 1 };

// Status word written by kernels (device memory); 0 = fine, first error wins.
enum DevStatus : int {
  kDevOk = 0,
  kDevWaitTimeout = 1,   // an mbarrier wait exceeded its limit
  kDevBadArgument = 2,   // histogram range not finite or inverted
  kDevBadCap = 3,        // a streamline step cap above kMaxLineCap
};

// Largest accepted per-line step cap: keeps every streamline kernel bounded.
constexpr int kMaxLineCap = 1 << 24;
enum GridKind : int { kField = 0, kEsp = 1 };

// Packed charge layouts in HBM (positions relative to the box centre).
struct alignas(32) Charge64 {
  double x, y, z, q;
};
// Point dipole (FP64 streamline form): position and moment.
struct alignas(16) Dipole64 {
  double x, y, z, mx, my, mz;
};
static_assert(sizeof(Dipole64) == 48, "Dipole64 layout");
// Sources of a streamline launch.
enum Source : int { kCharges = 0, kDipoles = 1 };
// FP32C uses float4 {x, y, z, q}.

// One CTA of the grid kernel: a tile of up to kGridTilePts points of one frame
// against a contiguous range of that frame's charges.
struct GridItem {
  int64_t charge_off;  // first packed charge of the frame
  int64_t point_off;   // first point of the frame (points / output rows)
  int32_t p_begin;     // first point of this tile inside the frame
  int32_t p_count;     // points in this tile (<= kGridThreads * points per thread)
  int32_t n_begin;     // first charge of this item inside the frame
  int32_t n_count;     // charges of this item
  int32_t slot;        // partial-sum slot (>= 0), or -1 to write the final value
  int32_t pad;
};
static_assert(sizeof(GridItem) == 40, "GridItem layout");

// Reduction of the partial sums of one point tile over its charge splits.
struct GridFinal {
  int64_t out_row;     // first output row (frame point_off + p_begin)
  int32_t p_count;
  int32_t slot_base;   // partial slots slot_base .. slot_base + n_split - 1
  int32_t n_split;
  int32_t pad;
};
static_assert(sizeof(GridFinal) == 24, "GridFinal layout");

constexpr int kGridThreads = 128;
constexpr int kGridMaxPPT = 8;                              // points per thread: 4 or 8
constexpr int kGridSlotPts = kGridThreads * kGridMaxPPT;    // stride of a partial-sum slot

// grid.cu
// Packs x[n][3], q[n] for the grid kernels (32-byte records: Charge64, or the
// FP32C record with every component duplicated) and fills [n, n_pad) with zero
// charges placed far outside any box (they contribute exactly zero).
cudaError_t launch_pack_charges(int prec, int64_t n, int64_t n_pad, const double* x,
                                const double* q, void* packed, cudaStream_t s);
cudaError_t launch_grid(int prec, int kind, int clamp, int ppt, int n_items, const GridItem* items,
                        const void* packed, const double* points, double* out,
                        double* partial, int* status, cudaStream_t s);
// Loads the module code of the grid kernels (before a graph capture).
cudaError_t preload_grid_kernels(int prec, int kind, int clamp, int ppt);
cudaError_t launch_grid_final(int kind, int n_final, const GridFinal* fin,
                              const double* partial, double* out, cudaStream_t s);

// FP32C field refinement after the grid pass: points of each frame (desc rows
// {charge_off, n, point_off, P}, device memory; max_points = the largest P)
// whose |E| is below tau times the frame's median |E| are recomputed in
// double-float arithmetic from x/q (n_charges of them in all).  Scratch: list
// 2 int64 per point of the launch, count one int, hist
// grid_refine_hist_ints(n_frames) ints (both zeroed here), df_charges 32 bytes
// per charge.  tau <= 0: no-op.
cudaError_t launch_grid_refine(int n_frames, int64_t n_charges, int64_t max_points,
                               const int64_t* desc, const double* points, const double* x,
                               const double* q, double* out, int clamp, double tau, int64_t* list,
                               int* count, int* hist, void* df_charges, int num_sms, cudaStream_t s);
int64_t grid_refine_hist_ints(int n_frames);
cudaError_t preload_grid_refine();

// topo.cu
// One frame of a streamline launch (device table for multi-frame launches).
struct TopoFrame {
  int64_t packed_off;  // first packed element (FP32C: float4 index of the pair block; FP64: Charge64)
  int64_t line_off;    // first line of the frame in starts / n_iter / result
  int32_t n_pad;       // padded charge count (a multiple of topo_charge_pad(prec))
  int32_t n_lines;
  int32_t resident;    // charges staged in shared memory: n_pad, a prefix, or 0
  int32_t pad_;
  double step;
  double half[3];
};
static_assert(sizeof(TopoFrame) == 64, "TopoFrame layout");

struct TopoParams {
  int n_lines;
  int n_charges;
  double step;
  double half[3];
  const double* starts;      // [L][3]
  const int32_t* n_iter;     // [L]
  const void* packed;        // packed charges
  double* result;            // [L][2]  {distance, mean curvature}
  double* ends;              // [L][3] or null
  int32_t* steps;            // [L] or null (Euler steps of the main loop)
  int* queue;                // work-queue counter(s), one per frame (zeroed by the caller)
  int* status;
  const TopoFrame* frames;   // device frame table (multi-frame launches) or null
  int n_frames;              // frames in the table
  int max_resident_pad;      // largest TopoFrame::resident of the launch (shared-memory size)
  int all_resident = 0;      // 1: every frame entirely in shared memory (tuner class)
  int source = kCharges;     // kDipoles: packed holds dipoles (single-frame launches only)
};
// Single frame: p.frames == null, the frame is described by n_charges/step/half.
cudaError_t launch_topo(int prec, const TopoParams& p, int num_sms, cudaStream_t s);
// Multi-frame: p.frames/n_frames/queue[n_frames]/max_resident_pad set by the caller.
cudaError_t launch_topo_frames(int prec, const TopoParams& p, int num_sms, cudaStream_t s);
// Packs the charges of every frame of a table (host copy `frames`, device copy `d_frames`,
// source offsets src_off[f] into x/q) into the streamline layout.
cudaError_t launch_pack_topo_frames(int prec, int n_frames, const TopoFrame* d_frames,
                                    const int64_t* d_src, const double* x, const double* q,
                                    void* packed, int max_pairs, cudaStream_t s);
// max sources (charges or dipoles) held resident in shared memory
size_t topo_resident_limit(int prec, int source = kCharges);
// sources of a frame of n_pad held in shared memory: n_pad when it fits, else
// a prefix of whole Kahan runs; 0 for FP64 (TopoFrame::resident)
int topo_resident_count(int prec, int source, int n_pad);
// bytes per packed source (FP32C charge 16, dipole 24; FP64 charge 32, dipole 48)
size_t topo_source_bytes(int prec, int source);
// Packs point dipoles x[n][3], mu[n][3] in the streamline layout (single frame).
cudaError_t launch_pack_dipoles(int prec, int64_t n, int64_t n_pad, const double* x,
                                const double* mu, void* packed, cudaStream_t s);
int topo_charge_pad(int prec);         // packed charge arrays are padded to this multiple
// Packs charges in the streamline kernel's layout (FP32C: pair layout; FP64: Charge64).
cudaError_t launch_pack_topo(int prec, int64_t n, int64_t n_pad, const double* x, const double* q,
                             void* packed, cudaStream_t s);

// peaks.cu: one CTA whose bounded mbarrier wait can never be satisfied runs
// out after limit_ns and records kDevWaitTimeout in *status.
cudaError_t launch_wait_limit_check(int* status, unsigned long long limit_ns, cudaStream_t s);

// api.cu: records `msg` as the calling thread's last error and returns `code`.
int set_error(int code, const char* msg);

// Streamline serving engine (topo.cu kernel, engine.cu host side).
// A chunk of lines of one request; written by the host into host-mapped memory.
struct EngineChunk {
  int32_t frame;       // engine frame slot (index into the frame table)
  int32_t request;     // request slot (index into the done counters)
  int32_t line_begin;  // global line indices [line_begin, line_end)
  int32_t line_end;
  double step;
  double half[3];
};
static_assert(sizeof(EngineChunk) == 48, "EngineChunk layout");

struct EngineParams {
  TopoParams p;                 // line arrays (starts, n_iter, result, ends, steps) and status
  const TopoFrame* frames;      // frame table (packed_off, n_pad) in device memory
  const EngineChunk* chunks;    // chunk ring (host-mapped)
  int chunk_capacity;
  const int* tail;              // chunks published (host-mapped, written by the host)
  int* head;                    // chunks claimed (device memory)
  int* head_mirror;             // claims seen by the host (host-mapped, monotonic)
  int* done;                    // finished lines per request slot (host-mapped)
  int* busy;                    // warps of this launch holding lines (device memory, 0 at launch)
  int* closing;                 // 1 once this launch takes no more chunks (device memory, 0 at launch)
};
cudaError_t launch_engine(int prec, const EngineParams& e, int ctas, cudaStream_t s);
int engine_threads();

// api.cu: the tuned variants (autotuner table, defaults when untuned).
int tuned_topo_slots(int prec, bool resident, int n_lines);    // 2 or 4 line slots per warp
void tuned_grid_shape(int prec, int kind, double pair_evals, int* ppt, int* items_per_sm);

// hist.cu
cudaError_t launch_hist2d(int n, const double* vals, int nb0, int nb1, const double* range,
                          double* edges, unsigned long long* counts, int* status,
                          cudaStream_t s);
cudaError_t launch_hist2d_sets(int n_sets, const int64_t* d_off, int64_t max_set,
                               const double* vals, int nb0, int nb1, const double* range,
                               double* edges, unsigned long long* counts, double* hists,
                               int* status, cudaStream_t s);

// distance.cu: kind 0 = chi-square over histogram rows [n][feat]; kind 1 =
// summed Euclidean norms over field rows [n][feat][3]; out [n][n].
// prep.cu: residue radius filter, rotation, box filter, shift, compaction of one
// frame (device pointers; center/inv/half/shift on the host, inv/half/shift may
// be null); the survivor count lands in d_count (device int64).
size_t prep_scratch_bytes(int n);
cudaError_t launch_prepare_frame(int n, const double* x, const double* q, const int32_t* resid,
                                 const int32_t* resnum, const double* center, const double* inv,
                                 double radius, const double* half, const double* shift,
                                 double* x_out, double* q_out, void* scratch, int64_t* d_count,
                                 cudaStream_t s);

// format.cu: in-place exclusive scan of int64 values (scratch: scan_scratch_i64(n)).
int64_t scan_scratch_i64(int64_t n);
cudaError_t scan_exclusive_i64(int64_t n, int64_t* x, int64_t* scratch, cudaStream_t s);
// format.cu: text of a float32 matrix in numpy.savetxt's layout (values joined
// by single spaces, "\n" after each row), "%.3f" or "%.18e".
enum TextFormat : int { kTextFixed3 = 0, kTextSci18 = 1 };
int64_t fixed3_scan_scratch(int64_t n);
cudaError_t launch_text_offsets(int fmt, int64_t n_rows, int n_cols, const float* v,
                                int64_t* offsets, int64_t* scratch, cudaStream_t s);
cudaError_t launch_text_write(int fmt, int64_t n_rows, int n_cols, const float* v,
                              const int64_t* offsets, char* out, cudaStream_t s);

// splits > 1 (distance_splits) needs partial scratch of splits * n * n doubles.
// FP32C also needs f32_rows scratch of distance_f32_bytes(kind, n, feat) bytes.
int distance_splits(int n, int feat, int num_sms);
size_t distance_f32_bytes(int kind, int n, int feat);
cudaError_t launch_distance_matrix(int prec, int kind, int n, int feat, const double* src,
                                   double* out, int splits, double* partial, void* f32_rows,
                                   cudaStream_t s);

}  // namespace cpetgb

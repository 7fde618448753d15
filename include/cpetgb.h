/*
 * cpetgb.h -- C ABI of libcpetgb.so, the GB300 (sm_103a) implementation of
 * PyCPET's Coulomb hot path: field / potential on point sets, streamline
 * topology, and the topology histogram.
 *
 * Conventions
 *   - Every call returns an int status: CPETGB_OK (0) or a negative code;
 *     cpetgb_last_error() gives the message of the calling thread's last failure.
 *   - No exceptions cross this boundary and there is no CPU fallback: without a
 *     usable CUDA device every compute call returns CPETGB_ENODEV.
 *   - The caller owns every buffer.  `mem` says where the data pointers live:
 *     CPETGB_HOST (host memory; the call copies in, computes, copies out and
 *     returns when the results are in place) or CPETGB_DEVICE (device memory of
 *     the current device; the call is enqueued on `stream` and returns at once;
 *     cpetgb_synchronize(stream) waits and reports errors raised on the device).
 *   - Errors raised inside kernels (a bounded wait that ran out, a refused
 *     step cap or histogram range) go to one status word per device.  The next
 *     call that waits on the device -- cpetgb_synchronize or any CPETGB_HOST
 *     call, on whichever stream -- reports that status and clears it.  To tie
 *     such an error to the CPETGB_DEVICE call that raised it, call
 *     cpetgb_synchronize(stream) after that call, before other work.
 *   - `stream` is a cudaStream_t; NULL means the legacy default stream for
 *     CPETGB_DEVICE calls and a library-owned stream for CPETGB_HOST calls.
 *   - Coordinates are in Angstrom, charges in e, fields in V/A, potentials in
 *     V; charge positions are relative to the box centre (the reference
 *     calculator's frame after its rotation step, CPET/source/calculator.py:341-346).
 *   - Precision: CPETGB_FP64 = every operation in IEEE double (the plain
 *     drop-in); CPETGB_FP32C = FP32 pair terms with compensated (Kahan)
 *     accumulation across charge tiles, FP64 for streamline positions and the
 *     final curvature / distance.  FP32C fields are refined: the points where
 *     |E| is below a fraction (cpetgb_set_field_refinement, default 0.15) of
 *     their frame's median |E| -- where the pair terms cancel and FP32
 *     rounding is largest relative to |E| -- are recomputed in double-float
 *     arithmetic (pairs of floats, about 1e-12 relative per pair term).
 */
#ifndef CPETGB_H
#define CPETGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPETGB_OK 0
#define CPETGB_EINVAL (-1)   /* bad argument (size, pointer, enum) */
#define CPETGB_ENOMEM (-2)   /* device allocation failed */
#define CPETGB_ECUDA (-3)    /* CUDA runtime error */
#define CPETGB_ETIMEOUT (-4) /* a bounded device-side wait gave up */
#define CPETGB_ENODEV (-5)   /* no usable CUDA device */
#define CPETGB_ERANGE (-6)   /* non-finite or inverted histogram range */
#define CPETGB_EAGAIN (-7)   /* engine capacity in use: retry after collecting requests */

#define CPETGB_FP64 0
#define CPETGB_FP32C 1

#define CPETGB_HOST 0
#define CPETGB_DEVICE 1

#define CPETGB_FIELD 0
#define CPETGB_ESP 1

/* ---- library ------------------------------------------------------------ */
int cpetgb_version(void);
/* Copies the calling thread's last error message (NUL-terminated). */
int cpetgb_last_error(char* buf, size_t len);
/* Number of SMs of the current device, or a negative status. */
int cpetgb_device_sms(void);
/* Waits for `stream` and returns (then clears) the device-side status. */
int cpetgb_synchronize(void* stream);
/* Precision used by the float32 drop-in entry points below (default FP32C).
 * Process-wide; the *_p variants take the precision per call instead. */
int cpetgb_set_default_precision(int precision);
int cpetgb_get_default_precision(void);
/* FP32C field refinement threshold tau in [0, 1] (0 = off; default 0.15):
 * after the FP32C pass, every point of a frame with |E| < tau * (the frame's
 * median |E|, rounded down to 1/16 octave) is recomputed over all of the
 * frame's charges in double-float arithmetic (about 1e-12 per pair term).
 * Process-wide setting read when a call (or a plan, at creation) is made.  No
 * counterpart in the reference, whose field is plain float
 * (CPET/utils/math_module.c:405-451). */
int cpetgb_set_field_refinement(double tau);
double cpetgb_field_refinement(void);

/* Failure-path check of the device-side waits: runs one CTA whose bounded
 * mbarrier wait can never be satisfied (no copy is issued), with a limit of
 * `seconds` (0 < seconds <= 2) instead of the kernels' 2 s.  The wait runs out,
 * the kernel records the timeout in the device status word and returns, and
 * this call reports it like any other call: CPETGB_ETIMEOUT means the bounded
 * wait works (the device stays usable).  No counterpart in the reference,
 * whose CPU code has no device waits. */
int cpetgb_check_wait_limit(double seconds);
/* Pipe throughput microbenchmark on the current device (roofline denominators):
 * kind 0 FP32 FFMA flop/s, 1 FP64 DFMA flop/s, 2 MUFU rsqrt op/s, 3 FP32x2 FFMA2 flop/s,
 * 4 pair evaluations/s of the FP32C streamline sweep's inner loop alone. */
int cpetgb_measure_peak(int kind, double* ops_per_s);

/* ---- float32 drop-ins of the reference FFI (host buffers) ---------------- */
/* compute_looped_field: CPET/utils/math_module.c:405-451, bound by
 * CPET/utils/c_ops.py:151-159,250-263.  E[p] = k sum q (x0[p]-x)/|.|^3 with
 * r^2 clamped at 1e-6. */
int cpetgb_compute_looped_field(int total_points, int n_charges, const float* x_0,
                                const float* x, const float* Q, float* E);
/* calc_esp_base: math_module.c:453-486, c_ops.py:131-138,326-341.
 * ESP[0] += k sum q / |x_init - x|  (accumulates, like the reference). */
int cpetgb_calc_esp_base(float* ESP, const float* x_init, int n_charges, const float* x,
                         const float* Q);
/* calc_field: math_module.c:255-293, c_ops.py:113-120,360-375.  Unclamped. */
int cpetgb_calc_field(float* E, const float* x_init, int n_charges, const float* x,
                      const float* Q);
/* thread_operation: math_module.c:523-591, c_ops.py:85-95,281-302.
 * ret = {start-to-end distance, mean start/end curvature}. */
int cpetgb_thread_operation(int n_charges, int n_iter, float step_size, const float* x_0,
                            const float* dimensions, const float* x, const float* Q,
                            float* ret);
/* thread_operation_dipole: math_module.c:593-659, c_ops.py:96-110,304-325
 * (dipole moments mu[n_dipoles][3] instead of charges). */
int cpetgb_thread_operation_dipole(int n_dipoles, int n_iter, float step_size, const float* x_0,
                                   const float* dimensions, const float* x, const float* mu,
                                   float* ret);
/* All lines of compute_topo_complete_c_shared (CPET/source/calculator.py:675-712)
 * in one call: x_0[L][3], n_iter[L], ret[L][2] in start order. */
int cpetgb_thread_operation_batch(int n_lines, int n_charges, const int32_t* n_iter,
                                  float step_size, const float* x_0, const float* dimensions,
                                  const float* x, const float* Q, float* ret);
/* compute_ESP_on_grid's per-point loop (CPET/utils/calculator.py:450-475) in one
 * call: ESP[p] = k sum q / |x_0[p] - x|. */
int cpetgb_compute_esp_grid(int total_points, int n_charges, const float* x_0, const float* x,
                            const float* Q, float* ESP);

/* The same seven calls with the precision passed per call (CPETGB_FP64 or
 * CPETGB_FP32C) instead of read from the library default: callers that mix
 * precisions from several threads use these.  Arguments otherwise as above. */
int cpetgb_compute_looped_field_p(int precision, int total_points, int n_charges,
                                  const float* x_0, const float* x, const float* Q, float* E);
int cpetgb_calc_esp_base_p(int precision, float* ESP, const float* x_init, int n_charges,
                           const float* x, const float* Q);
int cpetgb_calc_field_p(int precision, float* E, const float* x_init, int n_charges,
                        const float* x, const float* Q);
int cpetgb_thread_operation_p(int precision, int n_charges, int n_iter, float step_size,
                              const float* x_0, const float* dimensions, const float* x,
                              const float* Q, float* ret);
int cpetgb_thread_operation_dipole_p(int precision, int n_dipoles, int n_iter, float step_size,
                                     const float* x_0, const float* dimensions, const float* x,
                                     const float* mu, float* ret);
int cpetgb_thread_operation_batch_p(int precision, int n_lines, int n_charges,
                                    const int32_t* n_iter, float step_size, const float* x_0,
                                    const float* dimensions, const float* x, const float* Q,
                                    float* ret);
int cpetgb_compute_esp_grid_p(int precision, int total_points, int n_charges, const float* x_0,
                              const float* x, const float* Q, float* ESP);

/* ---- general entry points (double buffers, host or device) --------------- */
/* Field at n_points points: points[P][3], x[N][3], q[N] -> field[P][3].
 * clamp != 0 applies compute_looped_field's r^2 >= 1e-6; clamp == 0 is calc_field. */
int cpetgb_field_grid(int precision, int mem, int n_points, int n_charges, const double* points,
                      const double* x, const double* q, int clamp, double* field, void* stream);
/* Potential at n_points points (calc_esp_base per point) -> esp[P]. */
int cpetgb_esp_grid(int precision, int mem, int n_points, int n_charges, const double* points,
                    const double* x, const double* q, double* esp, void* stream);
/* Many frames in one launch.  desc is a HOST array [n_frames][4] of int64:
 * {charge_offset, n_charges, point_offset, n_points} into x/q and points/out.
 * kind = CPETGB_FIELD (out[.][3]) or CPETGB_ESP (out[.]). */
int cpetgb_grid_batch(int kind, int precision, int mem, int clamp, int n_frames,
                      const int64_t* desc, const double* points, const double* x,
                      const double* q, double* out, void* stream);
/* Streamlines: starts[L][3], n_iter[L], half_dims (HOST, 3 half-widths).
 * result[L][2] = {distance, mean curvature} in start order; ends[L][3] (last
 * position) and steps[L] (Euler steps of the main loop) may be NULL. */
int cpetgb_topo_lines(int precision, int mem, int n_lines, int n_charges, const double* starts,
                      const int32_t* n_iter, double step, const double* half_dims,
                      const double* x, const double* q, double* result, double* ends,
                      int32_t* steps, void* stream);
/* Streamlines through the field of point dipoles (thread_operation_dipole,
 * CPET/utils/math_module.c:593-659, with the term of calc_field_base_dipole,
 * 335-371: r^-5 ((3 mu_x R_x + mu_y R_y + mu_z R_z) R - mu r^2), the factor 3
 * on the x term as the reference writes it).  mu[n_dipoles][3]; everything else
 * as cpetgb_topo_lines. */
int cpetgb_topo_dipole_lines(int precision, int mem, int n_lines, int n_dipoles,
                             const double* starts, const int32_t* n_iter, double step,
                             const double* half_dims, const double* x, const double* mu,
                             double* result, double* ends, int32_t* steps, void* stream);
/* Streamlines of many frames in one persistent launch.  desc is a HOST array
 * [n_frames][4] of int64 {charge_offset, n_charges, line_offset, n_lines} into
 * x/q and starts/n_iter/result/ends/steps; params is a HOST array
 * [n_frames][4] of double {step, half_x, half_y, half_z}.  Frames are worked
 * in table order; results as cpetgb_topo_lines, at each line's index. */
int cpetgb_topo_batch(int precision, int mem, int n_frames, const int64_t* desc,
                      const double* params, const double* starts, const int32_t* n_iter,
                      const double* x, const double* q, double* result, double* ends,
                      int32_t* steps, void* stream);
/* ---- autotuner table ------------------------------------------------------ */
/* Tile shapes are chosen per (operation, precision, class, size bucket):
 *   op 0 = grid sums: class = CPETGB_FIELD / CPETGB_ESP, size = pair evaluations
 *          of the launch (buckets of x4 from 1e6); variants 0..9 = points per
 *          thread {4, 8} x work items per SM {4, 8, 16, 32, 64} (v / 5, v % 5),
 *          10..13 = points per thread {4, 8} x {128, 256} items per SM
 *          ((v - 10) / 2, (v - 10) % 2) (default 1);
 *   op 1 = streamlines: class = 1 if the frame's charges stay in shared memory,
 *          size = lines (buckets of x4 from 1e3); variants 0..1 = line slots per
 *          warp {4, 2} (default 0).
 * A launch whose own bucket is untuned uses the nearest tuned bucket of the
 * same (operation, precision, class), else the default.
 * pycpet_gb300.autotune times the candidates and fills the table. */
int cpetgb_tune_key(int op, int precision, int cls, double size);
int cpetgb_tune_variants(int op);
/* Largest frame whose streamline sources are held in shared memory for the
 * whole launch on the current device (the tuner's class 1): point charges
 * (dipoles = 0) or point dipoles (dipoles = 1); 0 for FP64. */
int cpetgb_topo_resident_limit(int precision, int dipoles);
int cpetgb_tune_set(int key, int variant);   /* variant -1 removes the entry */
int cpetgb_tune_get(int key);                /* -1 when untuned */

/* ---- prepared launches (CUDA graphs) ------------------------------------ */
/* A plan binds DEVICE buffers once, builds the work decomposition and the
 * scratch (cudaMalloc, held until cpetgb_plan_destroy), and captures the launch
 * sequence (pack, kernel, reduction) into a CUDA graph.  cpetgb_plan_launch
 * replays it on `stream`, reading the bound inputs as they are at that time
 * (e.g. the next MD frame's coordinates written in place).  Arguments as
 * cpetgb_grid_batch / cpetgb_topo_batch with mem = CPETGB_DEVICE. */
typedef struct cpetgb_plan cpetgb_plan;
int cpetgb_grid_plan_create(cpetgb_plan** plan, int kind, int precision, int clamp, int n_frames,
                            const int64_t* desc, const double* points, const double* x,
                            const double* q, double* out);
int cpetgb_topo_plan_create(cpetgb_plan** plan, int precision, int n_frames, const int64_t* desc,
                            const double* params, const double* starts, const int32_t* n_iter,
                            const double* x, const double* q, double* result, double* ends,
                            int32_t* steps);
int cpetgb_plan_launch(cpetgb_plan* plan, void* stream);
int cpetgb_plan_destroy(cpetgb_plan* plan);

/* ---- streamline serving engine (continuous batching) --------------------- */
/* Frames stay resident in a device pool; each submitted request's lines are
 * published as chunks that a persistent kernel's warps claim while it runs, so
 * requests arriving while others are in flight are admitted as line slots free
 * up and their work overlaps on the device.  Results are the same as
 * cpetgb_topo_lines on the same inputs.  Capacities are fixed at creation; a
 * request that does not fit gets CPETGB_EAGAIN (admission control).  All data
 * pointers are HOST pointers.  One thread at a time per engine. */
typedef struct cpetgb_engine cpetgb_engine;
int cpetgb_engine_create(cpetgb_engine** engine, int precision, int64_t charge_capacity,
                         int64_t line_capacity, int max_frames, int max_requests,
                         int chunk_lines);
int cpetgb_engine_destroy(cpetgb_engine* engine);
int cpetgb_engine_add_frame(cpetgb_engine* engine, int n_charges, const double* x, const double* q,
                            int* frame_id);
int cpetgb_engine_remove_frame(cpetgb_engine* engine, int frame_id);
int cpetgb_engine_submit(cpetgb_engine* engine, int frame_id, int n_lines, const double* starts,
                         const int32_t* n_iter, double step, const double* half_dims,
                         int* request_id);
int cpetgb_engine_poll(cpetgb_engine* engine, int request_id);  /* 1 done, 0 pending */
int cpetgb_engine_collect(cpetgb_engine* engine, int request_id, double* result, int32_t* steps);
int cpetgb_engine_drain(cpetgb_engine* engine);
/* Engine CTAs per SM from its next launch on: 1 (default) takes half of every
 * SM's registers, so grid and point launches on other streams run beside the
 * engine; 2 gives the engine whole SMs (higher streamline throughput, but grid
 * launches wait until the engine's launch ends). */
int cpetgb_engine_set_ctas_per_sm(cpetgb_engine* engine, int ctas_per_sm);

/* Streamlines for callers that must not have device memory allocated on their
 * behalf (device memory reserved up front by their own allocator, or a fixed
 * footprint after start-up).  No counterpart in the reference.  Same arguments
 * and results as cpetgb_topo_lines with mem = CPETGB_DEVICE (every data pointer
 * a device pointer, half_dims on the host), but the scratch lives in a fixed
 * ~512 KiB device array inside the library, so at most 16384 charges (larger
 * frames return CPETGB_EINVAL).  No cudaMalloc/cudaFree is called.  The first
 * call on a device looks the array up (cudaGetSymbolAddress): make it before any
 * stream capture.  The call waits for `stream` and returns the device status.
 * All calls share the array: calls that overlap on the GPU race. */
int cpetgb_topo_lines_noalloc(int precision, int n_lines, int n_charges, const double* starts,
                              const int32_t* n_iter, double step, const double* half_dims,
                              const double* x, const double* q, double* result, double* ends,
                              int32_t* steps, void* stream);
/* 2-D histogram of result[L][2] with numpy.histogram2d's edges and binning.
 * range (HOST) = {dist_lo, dist_hi, curv_lo, curv_hi}; a NaN bound is taken
 * from the data (column min / max).  counts[nb_dist][nb_curv] (uint64) are
 * overwritten; edges (nb_dist+1 then nb_curv+1 doubles) may be NULL.
 * nb_dist + nb_curv <= 4096. */
int cpetgb_topo_hist2d(int mem, int n_lines, const double* result, int nb_dist, int nb_curv,
                       const double* range, uint64_t* counts, double* edges, void* stream);

/* ---- frame preparation ----------------------------------------------------- */
/* The per-frame preparation of PyCPET's calculator for parsed charges
 * (CPET/source/calculator.py:239-251, 341-371), on the device:
 *   radius > 0: filter_radius_whole_residue (CPET/utils/io.py:283-338) -- keep
 *     the residues (runs of consecutive atoms with equal resid and resnum, both
 *     int32 codes) with any atom strictly within `radius` of `center`;
 *   rotation x <- (x - center) @ inv_basis (row-major 3x3, HOST; NULL: x - center);
 *   box_half != NULL: filter_in_box (io.py:422-475) -- drop atoms strictly
 *     inside the box, tested on x - center after the rotation as the
 *     reference's call does (calculator.py:349-358);
 *   box_shift != NULL: x <- x - box_shift (calculator.py:369-371).
 * Survivors are written in input order to x_out[.][3], q_out; *n_out (HOST)
 * receives their count.  center, inv_basis, box_half, box_shift are HOST
 * arrays.  Synchronous: waits for `stream` to read the count. */
int cpetgb_prepare_frame(int mem, int n_atoms, const double* x, const double* q,
                         const int32_t* resid, const int32_t* resnum, const double* center,
                         const double* inv_basis, double radius, const double* box_half,
                         const double* box_shift, double* x_out, double* q_out, int* n_out,
                         void* stream);

/* ---- output text --------------------------------------------------------- */
/* The body of save_numpy_as_dat (CPET/utils/io.py:50-109): the rows of a
 * float32 matrix values[n_rows][n_cols] as numpy.savetxt(fmt="%.3f") writes
 * them (each value correctly rounded to 3 decimals, ties to even; single
 * spaces between values; "\n" after each row), formatted on the GPU.  *length
 * (HOST) receives the byte count; text (HOST or DEVICE per mem, not
 * NUL-terminated) is written when non-NULL and capacity >= *length, else
 * CPETGB_ERANGE.  Synchronous: waits for `stream` to read the length. */
int cpetgb_format_fixed3(int mem, int64_t n_rows, int n_cols, const float* values, char* text,
                         int64_t capacity, int64_t* length, void* stream);
/* The .top writer of the topology dispatcher (np.savetxt(path, hist),
 * CPET/source/CPET.py:119-123; numpy's default fmt "%.18e"): the rows of a
 * float32 matrix with every value printed to 19 significant digits, correctly
 * rounded from its exact binary value, ties to even, as Python formats it
 * ("nan", "inf", "-inf"; signed zeros kept); single spaces; "\n" after each
 * row.  At most 26 bytes per value.  Arguments and return as
 * cpetgb_format_fixed3. */
int cpetgb_format_sci18(int mem, int64_t n_rows, int n_cols, const float* values, char* text,
                        int64_t capacity, int64_t* length, void* stream);

/* ---- clustering front end: histograms and distance matrices -------------- */
/* Histograms of many (distance, curvature) sets with one binning, in one
 * launch; replaces the per-file np.histogram2d loop of make_histograms
 * (CPET/utils/calculator.py:689-711).  Set f is rows offsets[f] ..
 * offsets[f+1]-1 of values[L][2]; offsets is a HOST array [n_sets + 1]
 * (non-decreasing, offsets[0] = 0); range is a HOST {dist_lo, dist_hi,
 * curv_lo, curv_hi}, finite with lo <= hi (make_histograms passes the global
 * min / max).  counts [n_sets][nb_dist*nb_curv] (uint64) and hists (double,
 * each set divided by its total as make_histograms does, NaN for an empty set)
 * may each be NULL, not both.  nb_dist + nb_curv <= 4096. */
int cpetgb_topo_hist2d_sets(int mem, int n_sets, const int64_t* offsets, const double* values,
                            int nb_dist, int nb_curv, const double* range, uint64_t* counts,
                            double* hists, void* stream);
/* Chi-square distance matrix of n histograms (rows of hists[n][bins]):
 * out[i][j] = 1/2 sum_k (a_k - b_k)^2 / (a_k + b_k) over bins with
 * a_k + b_k != 0, zero diagonal, out [n][n].  Replaces construct_distance_matrix
 * with the metric distance_numpy (CPET/utils/calculator.py:975-978, 1003-1015). */
int cpetgb_chi2_distance_matrix(int precision, int mem, int n, int bins, const double* hists,
                                double* out, void* stream);
/* Distance matrix of n vector fields on a common grid (fields[n][n_points][3]):
 * out[i][j] = sum_p |f_i[p] - f_j[p]|, zero diagonal, out [n][n].  Replaces
 * construct_distance_matrix_volume (CPET/utils/calculator.py:1042-1058). */
int cpetgb_field_distance_matrix(int precision, int mem, int n, int n_points,
                                 const double* fields, double* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CPETGB_H */

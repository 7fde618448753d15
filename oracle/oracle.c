/*
 * oracle.c -- CPU restatement of PyCPET's Coulomb hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the test oracle of the CUDA library in
 * pycpet_gb300/csrc: only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it.  Nothing in the product path links or calls it.
 *
 * Two families of functions, each following the reference file:line it cites
 * (paths are inside the pujanajmera/pycpet project):
 *
 *   *_f64  precision oracle: the reference algorithm evaluated in IEEE double
 *          throughout (plain sequential sums, 1/sqrt via libm).
 *   *_f32  reference-arithmetic restatement: the same loops in the float/double
 *          mix the reference's C uses (float storage, libm pow/sqrt in double,
 *          float accumulation).  Used as the timed CPU baseline ("port") and to
 *          cross-check against the reference library built from source.
 *
 * Parity pins: tests/test_oracle.py checks these functions against the golden
 * fixtures in tests/golden (outputs of the reference's own C library and of
 * its shipped example outputs).
 *
 * Multi-threading: the *_mt batch drivers split lines (or grid points) over
 * POSIX threads with a shared atomic counter, the in-process analogue of the
 * reference's multiprocessing.Pool fan-out (CPET/source/calculator.py:690-697).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_COULOMB_K 14.3996451 /* V*A/e, CPET/utils/math_module.c:412 */

/* ------------------------------------------------------------------------- */
/* FP64 precision oracle                                                      */
/* ------------------------------------------------------------------------- */

/* Field at one point.  clamp != 0 reproduces the r^2 >= 1e-6 softening of
 * compute_looped_field (math_module.c:431-436); clamp == 0 is the unsoftened
 * form of calc_field / calc_field_base (math_module.c:255-333). */
static void field_at_f64(const double p[3], int N, const double* x, const double* q,
                         int clamp, double E[3]) {
  double ex = 0.0, ey = 0.0, ez = 0.0;
  for (int j = 0; j < N; ++j) {
    double dx = p[0] - x[3 * j + 0];
    double dy = p[1] - x[3 * j + 1];
    double dz = p[2] - x[3 * j + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    if (clamp && r2 < 1e-6) r2 = 1e-6;
    double rinv = 1.0 / sqrt(r2);
    double s = q[j] * rinv * rinv * rinv;
    ex += s * dx;
    ey += s * dy;
    ez += s * dz;
  }
  E[0] = ORACLE_COULOMB_K * ex;
  E[1] = ORACLE_COULOMB_K * ey;
  E[2] = ORACLE_COULOMB_K * ez;
}

/* Potential at one point: calc_esp_base (math_module.c:453-486), no softening. */
static double esp_at_f64(const double p[3], int N, const double* x, const double* q) {
  double acc = 0.0;
  for (int j = 0; j < N; ++j) {
    double dx = p[0] - x[3 * j + 0];
    double dy = p[1] - x[3 * j + 1];
    double dz = p[2] - x[3 * j + 2];
    acc += q[j] / sqrt(dx * dx + dy * dy + dz * dz);
  }
  return ORACLE_COULOMB_K * acc;
}

/* compute_looped_field (math_module.c:405-451) over P points, clamp selectable
 * (clamp=0 gives calc_field, math_module.c:255-293, at each point). */
void oracle_field_grid_f64(int P, int N, const double* pts, const double* x, const double* q,
                           double* E, int clamp) {
  for (int i = 0; i < P; ++i) field_at_f64(pts + 3 * i, N, x, q, clamp, E + 3 * i);
}

/* compute_ESP_on_grid (CPET/utils/calculator.py:450-475) = calc_esp_base per point. */
void oracle_esp_grid_f64(int P, int N, const double* pts, const double* x, const double* q,
                         double* phi) {
  for (int i = 0; i < P; ++i) phi[i] = esp_at_f64(pts + 3 * i, N, x, q);
}

/* propagate_topo (math_module.c:489-503): x <- x + h * E/|E| with the
 * unsoftened field of calc_field_base (math_module.c:296-333). */
static void step_f64(const double p[3], int N, const double* x, const double* q, double h,
                     double out[3]) {
  double E[3];
  field_at_f64(p, N, x, q, 0, E);
  double n = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
  for (int k = 0; k < 3; ++k) out[k] = p[k] + h * E[k] / n;
}

/* curve (math_module.c:108-121): |v1 x v2| / |v1|^3. */
static double curve_f64(const double a[3], const double b[3]) {
  double c0 = a[1] * b[2] - a[2] * b[1];
  double c1 = a[2] * b[0] - a[0] * b[2];
  double c2 = a[0] * b[1] - a[1] * b[0];
  double nc = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  return nc / (na * na * na);
}

static int outside_box(const double p[3], const double d[3]) {
  /* strict test of thread_operation (math_module.c:539-546) */
  return p[0] < -d[0] || p[0] > d[0] || p[1] < -d[1] || p[1] > d[1] || p[2] < -d[2] ||
         p[2] > d[2];
}

/* thread_operation (math_module.c:523-591) for one streamline, in FP64.
 * ret = {start-to-end distance, mean of start and end curvature}; end = the
 * last position (first one outside the box, or the one after n_iter steps).
 * Returns the number of Euler steps taken inside the main loop. */
int oracle_topo_line_f64(int N, int n_iter, double h, const double x0[3], const double dims[3],
                         const double* x, const double* q, double ret[2], double end[3]) {
  double cur[3] = {x0[0], x0[1], x0[2]};
  int steps = 0;
  for (int i = 0; i < n_iter; ++i) {
    double nxt[3];
    step_f64(cur, N, x, q, h, nxt);
    memcpy(cur, nxt, sizeof cur);
    ++steps;
    if (outside_box(cur, dims)) break;
  }
  double a1[3], a2[3], b1[3], b2[3];
  step_f64(x0, N, x, q, h, a1);
  step_f64(a1, N, x, q, h, a2);
  step_f64(cur, N, x, q, h, b1);
  step_f64(b1, N, x, q, h, b2);
  double v1[3], v2[3], w1[3], w2[3];
  for (int k = 0; k < 3; ++k) {
    v1[k] = a1[k] - x0[k];
    v2[k] = a2[k] - 2.0 * a1[k] + x0[k];
    w1[k] = b1[k] - cur[k];
    w2[k] = b2[k] - 2.0 * b1[k] + cur[k];
  }
  double c0 = curve_f64(v1, v2), c1 = curve_f64(w1, w2);
  double dd = 0.0;
  for (int k = 0; k < 3; ++k) dd += (x0[k] - cur[k]) * (x0[k] - cur[k]);
  ret[0] = sqrt(dd);           /* euclidean_dist, math_module.c:99-105 */
  ret[1] = 0.5 * (c0 + c1);    /* curve_mean, math_module.c:584 */
  if (end) memcpy(end, cur, sizeof cur);
  return steps;
}

/* FP32 restatement lives in oracle_ref32.c (built with the reference wheel's flags). */
void oracle_field_grid_f32(int P, int N, const float* pts, const float* x, const float* q,
                           float* E);
void oracle_esp_grid_f32(int P, int N, const float* pts, const float* x, const float* q,
                         float* phi);
int oracle_topo_line_f32(int N, int n_iter, float h, const float x0[3], const float dims[3],
                         const float* x, const float* q, float ret[2], float end[3]);

/* ------------------------------------------------------------------------- */
/* Multi-threaded batch drivers                                               */
/* ------------------------------------------------------------------------- */

typedef struct {
  int kind; /* 0 topo f64, 1 topo f32, 2 field f64, 3 field f32, 4 esp f64, 5 esp f32 */
  int n_items, N, clamp;
  const int* n_iter;
  double h64;
  float h32;
  const void* x0;   /* start points / grid points */
  const void* dims;
  const void* x;
  const void* q;
  void* ret;
  void* ends;
  int* steps;
  int chunk;
  volatile int next;
} job_t;

static void* worker(void* arg) {
  job_t* J = (job_t*)arg;
  for (;;) {
    int b = __atomic_fetch_add(&J->next, J->chunk, __ATOMIC_RELAXED);
    if (b >= J->n_items) break;
    int e = b + J->chunk < J->n_items ? b + J->chunk : J->n_items;
    for (int i = b; i < e; ++i) {
      switch (J->kind) {
        case 0: {
          const double* s = (const double*)J->x0 + 3 * i;
          double* e3 = J->ends ? (double*)J->ends + 3 * i : NULL;
          int st = oracle_topo_line_f64(J->N, J->n_iter[i], J->h64, s, (const double*)J->dims,
                                        (const double*)J->x, (const double*)J->q,
                                        (double*)J->ret + 2 * i, e3);
          if (J->steps) J->steps[i] = st;
        } break;
        case 1: {
          const float* s = (const float*)J->x0 + 3 * i;
          float* e3 = J->ends ? (float*)J->ends + 3 * i : NULL;
          int st = oracle_topo_line_f32(J->N, J->n_iter[i], J->h32, s, (const float*)J->dims,
                                        (const float*)J->x, (const float*)J->q,
                                        (float*)J->ret + 2 * i, e3);
          if (J->steps) J->steps[i] = st;
        } break;
        case 2:
          field_at_f64((const double*)J->x0 + 3 * i, J->N, (const double*)J->x,
                       (const double*)J->q, J->clamp, (double*)J->ret + 3 * i);
          break;
        case 3:
          oracle_field_grid_f32(1, J->N, (const float*)J->x0 + 3 * i, (const float*)J->x,
                                (const float*)J->q, (float*)J->ret + 3 * i);
          break;
        case 4:
          ((double*)J->ret)[i] =
              esp_at_f64((const double*)J->x0 + 3 * i, J->N, (const double*)J->x,
                         (const double*)J->q);
          break;
        case 5:
          oracle_esp_grid_f32(1, J->N, (const float*)J->x0 + 3 * i, (const float*)J->x,
                              (const float*)J->q, (float*)J->ret + i);
          break;
      }
    }
  }
  return NULL;
}

static void run_job(job_t* J, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  if (n_threads > 512) n_threads = 512;
  J->next = 0;
  if (n_threads == 1) {
    worker(J);
    return;
  }
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
  int started = 0;
  for (int t = 0; t < n_threads; ++t)
    if (pthread_create(&th[t], NULL, worker, J) == 0) ++started;
  if (started == 0) worker(J);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(th);
}

/* Batch of streamlines (compute_topo_complete_c_shared, CPET/source/calculator.py:675-712). */
void oracle_topo_lines_f64_mt(int L, int N, const int* n_iter, double h, const double* x0,
                              const double* dims, const double* x, const double* q, double* ret,
                              double* ends, int* steps, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 0; J.n_items = L; J.N = N; J.n_iter = n_iter; J.h64 = h; J.x0 = x0; J.dims = dims;
  J.x = x; J.q = q; J.ret = ret; J.ends = ends; J.steps = steps; J.chunk = 1;
  run_job(&J, n_threads);
}

void oracle_topo_lines_f32_mt(int L, int N, const int* n_iter, float h, const float* x0,
                              const float* dims, const float* x, const float* q, float* ret,
                              float* ends, int* steps, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 1; J.n_items = L; J.N = N; J.n_iter = n_iter; J.h32 = h; J.x0 = x0; J.dims = dims;
  J.x = x; J.q = q; J.ret = ret; J.ends = ends; J.steps = steps; J.chunk = 1;
  run_job(&J, n_threads);
}

void oracle_field_grid_f64_mt(int P, int N, const double* pts, const double* x, const double* q,
                              double* E, int clamp, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 2; J.n_items = P; J.N = N; J.clamp = clamp; J.x0 = pts; J.x = x; J.q = q; J.ret = E;
  J.chunk = 16;
  run_job(&J, n_threads);
}

void oracle_field_grid_f32_mt(int P, int N, const float* pts, const float* x, const float* q,
                              float* E, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 3; J.n_items = P; J.N = N; J.x0 = pts; J.x = x; J.q = q; J.ret = E; J.chunk = 16;
  run_job(&J, n_threads);
}

void oracle_esp_grid_f64_mt(int P, int N, const double* pts, const double* x, const double* q,
                            double* phi, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 4; J.n_items = P; J.N = N; J.x0 = pts; J.x = x; J.q = q; J.ret = phi; J.chunk = 16;
  run_job(&J, n_threads);
}

void oracle_esp_grid_f32_mt(int P, int N, const float* pts, const float* x, const float* q,
                            float* phi, int n_threads) {
  job_t J;
  memset(&J, 0, sizeof J);
  J.kind = 5; J.n_items = P; J.N = N; J.x0 = pts; J.x = x; J.q = q; J.ret = phi; J.chunk = 16;
  run_job(&J, n_threads);
}

/*
 * oracle_cluster.c -- CPU restatement of PyCPET's clustering distance matrices.
 *
 * TEST INFRASTRUCTURE ONLY (the test oracle of pycpet_gb300/csrc/distance.cu):
 * only tests/ and the CPU-baseline leg of bench.py load it.
 *
 *   oracle_chi2_matrix_f64   construct_distance_matrix with the metric
 *                            distance_numpy (CPET/utils/calculator.py:975-978,
 *                            1003-1015): D[i][j] = sum over bins with
 *                            a + b != 0 of (a - b)^2 / (a + b), halved; the
 *                            diagonal set to zero (1011-1012).
 *   oracle_field_matrix_f64  construct_distance_matrix_volume
 *                            (calculator.py:1042-1058): D[i][j] = sum over
 *                            points of the Euclidean norm of f_i - f_j, the
 *                            norm formed as numpy.linalg.norm forms it,
 *                            sqrt((dx*dx + dy*dy) + dz*dz).
 * IEEE double, sequential sums in feature order; rows of the upper triangle
 * are split over POSIX threads (a shared atomic row counter) and mirrored.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>

typedef struct {
  int kind, n, feat, nthreads;
  const double* src;
  double* out;
  volatile int next;
} cjob_t;

static double chi2_pair(const double* a, const double* b, int bins) {
  double s = 0.0;
  for (int k = 0; k < bins; ++k) {
    const double num = (a[k] - b[k]) * (a[k] - b[k]);
    const double den = a[k] + b[k];
    if (den != 0.0) s += num / den;
  }
  return s / 2.0;
}

static double field_pair(const double* a, const double* b, int points) {
  double s = 0.0;
  for (int p = 0; p < points; ++p) {
    const double dx = a[3 * p] - b[3 * p], dy = a[3 * p + 1] - b[3 * p + 1],
                 dz = a[3 * p + 2] - b[3 * p + 2];
    s += sqrt((dx * dx + dy * dy) + dz * dz);
  }
  return s;
}

static void* cworker(void* arg) {
  cjob_t* J = (cjob_t*)arg;
  const int64_t row = (int64_t)J->feat * (J->kind == 0 ? 1 : 3);
  for (;;) {
    const int i = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (i >= J->n) break;
    J->out[(int64_t)i * J->n + i] = 0.0;
    for (int j = i + 1; j < J->n; ++j) {
      const double* a = J->src + i * row;
      const double* b = J->src + j * row;
      const double v = J->kind == 0 ? chi2_pair(a, b, J->feat) : field_pair(a, b, J->feat);
      J->out[(int64_t)i * J->n + j] = v;
      J->out[(int64_t)j * J->n + i] = v;
    }
  }
  return 0;
}

static void run(int kind, int n, int feat, const double* src, double* out, int threads) {
  cjob_t J = {kind, n, feat, threads, src, out, 0};
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t t[256];
  for (int k = 1; k < threads; ++k) pthread_create(&t[k], 0, cworker, &J);
  cworker(&J);
  for (int k = 1; k < threads; ++k) pthread_join(t[k], 0);
}

void oracle_chi2_matrix_f64(int n, int bins, const double* hists, double* out, int threads) {
  run(0, n, bins, hists, out, threads);
}

void oracle_field_matrix_f64(int n, int points, const double* fields, double* out, int threads) {
  run(1, n, points, fields, out, threads);
}

/*
 * oracle_dipole.c -- CPU restatement of PyCPET's dipole streamline path.
 *
 * TEST INFRASTRUCTURE ONLY (the test oracle of the dipole form of
 * pycpet_gb300/csrc/topo.cu): only tests/ and bench.py's CPU-baseline leg load it.
 *
 * thread_operation_dipole (CPET/utils/math_module.c:593-659) is
 * thread_operation (523-591) with the step of propagate_topo_dipole
 * (506-520): the field of point dipoles from calc_field_base_dipole (335-371),
 *   E_c += k r^-5 ((3 mu_x R_x + mu_y R_y + mu_z R_z) R_c - mu_c r^2),
 * R = p - x_i.  The factor 3 multiplies the x term only, as the reference's
 * expression is written (math_module.c:362-364); the restatement keeps it.
 * The line semantics (at most n_iter steps, stop at the first position
 * strictly outside the box and keep it, two extra steps from the start and
 * from the end point, mean curvature, start-to-end distance) are the charge
 * path's, restated here in IEEE double.  The float form (the reference's own
 * arithmetic) is in oracle_ref32.c.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <string.h>

#define DIPOLE_K 14.3996451 /* V*A/e, math_module.c:343 */

static void dipole_field_f64(const double p[3], int N, const double* x, const double* mu,
                             double E[3]) {
  double ex = 0.0, ey = 0.0, ez = 0.0;
  for (int j = 0; j < N; ++j) {
    const double R0 = p[0] - x[3 * j], R1 = p[1] - x[3 * j + 1], R2 = p[2] - x[3 * j + 2];
    const double m0 = mu[3 * j], m1 = mu[3 * j + 1], m2 = mu[3 * j + 2];
    const double r2 = R0 * R0 + R1 * R1 + R2 * R2;
    const double r = sqrt(r2);
    const double r5 = 1.0 / (r2 * r2 * r);
    const double dot = 3.0 * m0 * R0 + m1 * R1 + m2 * R2;
    ex += r5 * (dot * R0 - m0 * r2);
    ey += r5 * (dot * R1 - m1 * r2);
    ez += r5 * (dot * R2 - m2 * r2);
  }
  E[0] = DIPOLE_K * ex;
  E[1] = DIPOLE_K * ey;
  E[2] = DIPOLE_K * ez;
}

static void dipole_step_f64(const double p[3], int N, const double* x, const double* mu,
                            double h, double out[3]) {
  double E[3];
  dipole_field_f64(p, N, x, mu, E);
  const double n = sqrt(E[0] * E[0] + E[1] * E[1] + E[2] * E[2]);
  for (int k = 0; k < 3; ++k) out[k] = p[k] + h * E[k] / n;
}

static double curve64(const double a[3], const double b[3]) {
  const double c0 = a[1] * b[2] - a[2] * b[1], c1 = a[2] * b[0] - a[0] * b[2],
               c2 = a[0] * b[1] - a[1] * b[0];
  const double na = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  return sqrt(c0 * c0 + c1 * c1 + c2 * c2) / (na * na * na);
}

/* thread_operation_dipole (math_module.c:593-659) for one line in FP64;
 * returns the Euler steps of the main loop. */
int oracle_topo_line_dipole_f64(int N, int n_iter, double h, const double x0[3],
                                const double dims[3], const double* x, const double* mu,
                                double ret[2], double end[3]) {
  double cur[3] = {x0[0], x0[1], x0[2]};
  int steps = 0;
  for (int i = 0; i < n_iter; ++i) {
    double nxt[3];
    dipole_step_f64(cur, N, x, mu, h, nxt);
    memcpy(cur, nxt, sizeof cur);
    ++steps;
    if (cur[0] < -dims[0] || cur[0] > dims[0] || cur[1] < -dims[1] || cur[1] > dims[1] ||
        cur[2] < -dims[2] || cur[2] > dims[2])
      break;
  }
  double a1[3], a2[3], b1[3], b2[3], v1[3], v2[3], w1[3], w2[3];
  dipole_step_f64(x0, N, x, mu, h, a1);
  dipole_step_f64(a1, N, x, mu, h, a2);
  dipole_step_f64(cur, N, x, mu, h, b1);
  dipole_step_f64(b1, N, x, mu, h, b2);
  double dd = 0.0;
  for (int k = 0; k < 3; ++k) {
    v1[k] = a1[k] - x0[k];
    v2[k] = a2[k] - 2.0 * a1[k] + x0[k];
    w1[k] = b1[k] - cur[k];
    w2[k] = b2[k] - 2.0 * b1[k] + cur[k];
    dd += (x0[k] - cur[k]) * (x0[k] - cur[k]);
  }
  ret[0] = sqrt(dd);
  ret[1] = 0.5 * (curve64(v1, v2) + curve64(w1, w2));
  if (end) memcpy(end, cur, sizeof cur);
  return steps;
}

int oracle_topo_line_dipole_f32(int N, int n_iter, float h, const float x0[3], const float dims[3],
                                const float* x, const float* mu, float ret[2], float end[3]);

typedef struct {
  int f32, L, N;
  const int* n_iter;
  double h;
  const void *x0, *dims, *x, *mu;
  void *ret, *ends;
  int* steps;
  volatile int next;
} djob_t;

static void* dworker(void* arg) {
  djob_t* J = (djob_t*)arg;
  for (;;) {
    const int i = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (i >= J->L) break;
    int st;
    if (J->f32)
      st = oracle_topo_line_dipole_f32(J->N, J->n_iter[i], (float)J->h, (const float*)J->x0 + 3 * i,
                                       (const float*)J->dims, (const float*)J->x,
                                       (const float*)J->mu, (float*)J->ret + 2 * i,
                                       J->ends ? (float*)J->ends + 3 * i : 0);
    else
      st = oracle_topo_line_dipole_f64(J->N, J->n_iter[i], J->h, (const double*)J->x0 + 3 * i,
                                       (const double*)J->dims, (const double*)J->x,
                                       (const double*)J->mu, (double*)J->ret + 2 * i,
                                       J->ends ? (double*)J->ends + 3 * i : 0);
    if (J->steps) J->steps[i] = st;
  }
  return 0;
}

static void drun(djob_t* J, int threads) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t t[256];
  int started = 1;
  for (int k = 1; k < threads; ++k)
    if (pthread_create(&t[started], 0, dworker, J) == 0) ++started;
  dworker(J);
  for (int k = 1; k < started; ++k) pthread_join(t[k], 0);
}

/* compute_topo_complete_c_shared_dipole (CPET/source/calculator.py:714-749):
 * every line of a start-point set, FP64 (f32 = 0) or the reference's float
 * arithmetic (f32 = 1; arrays then float32 and h rounded to float). */
void oracle_topo_lines_dipole_mt(int f32, int L, int N, const int* n_iter, double h, const void* x0,
                                 const void* dims, const void* x, const void* mu, void* ret,
                                 void* ends, int* steps, int threads) {
  djob_t J;
  memset(&J, 0, sizeof J);
  J.f32 = f32; J.L = L; J.N = N; J.n_iter = n_iter; J.h = h; J.x0 = x0; J.dims = dims; J.x = x;
  J.mu = mu; J.ret = ret; J.ends = ends; J.steps = steps;
  drun(&J, threads);
}

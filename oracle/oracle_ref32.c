/*
 * oracle_ref32.c -- the reference's float arithmetic for the Coulomb hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.c).  Compiled with the flags of the
 * reference's Linux wheel (-O3 -funroll-loops -ffast-math, pyproject.toml:55-61,
 * minus -march=native so it builds the same on x86 and Arm), because it is the
 * timed CPU baseline ("port") of bench.py as well as a cross-check of the
 * reference library built from source.
 */
#include <math.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Reference-arithmetic FP32 restatement                                      */
/* ------------------------------------------------------------------------- */

/* compute_looped_field (math_module.c:405-451): float storage, r^2 clamped at
 * 1e-6f, 1/sqrtf, float accumulation of factor*q*r^-3*R in charge order. */
void oracle_field_grid_f32(int P, int N, const float* pts, const float* x, const float* q,
                           float* E) {
  const float k = 14.3996451f;
  for (int i = 0; i < P; ++i) {
    float ex = 0.f, ey = 0.f, ez = 0.f;
    for (int j = 0; j < N; ++j) {
      float dx = pts[3 * i + 0] - x[3 * j + 0];
      float dy = pts[3 * i + 1] - x[3 * j + 1];
      float dz = pts[3 * i + 2] - x[3 * j + 2];
      float r2 = fmaxf(dx * dx + dy * dy + dz * dz, 1e-6f);
      float rinv = 1.0f / sqrtf(r2);
      float s = k * q[j] * (rinv * rinv * rinv);
      ex += s * dx;
      ey += s * dy;
      ez += s * dz;
    }
    E[3 * i + 0] = ex;
    E[3 * i + 1] = ey;
    E[3 * i + 2] = ez;
  }
}

/* calc_field_base / calc_field (math_module.c:255-333): r from a double
 * sqrt of the squared components, r^-3 via double pow, float products. */
static void field_at_f32(const float p[3], int N, const float* x, const float* q, float E[3]) {
  const float k = 14.3996451f;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  for (int j = 0; j < N; ++j) {
    float R0 = p[0] - x[3 * j + 0];
    float R1 = p[1] - x[3 * j + 1];
    float R2 = p[2] - x[3 * j + 2];
    float rn = (float)sqrt((double)R0 * R0 + (double)R1 * R1 + (double)R2 * R2);
    float r3 = (float)(1.0 / ((double)rn * rn * rn));
    float s = k * r3 * q[j];
    ex += s * R0;
    ey += s * R1;
    ez += s * R2;
  }
  E[0] = ex;
  E[1] = ey;
  E[2] = ez;
}

void oracle_point_field_f32(int P, int N, const float* pts, const float* x, const float* q,
                            float* E) {
  for (int i = 0; i < P; ++i) field_at_f32(pts + 3 * i, N, x, q, E + 3 * i);
}

/* calc_esp_base (math_module.c:453-486) at P points. */
void oracle_esp_grid_f32(int P, int N, const float* pts, const float* x, const float* q,
                         float* phi) {
  const float k = 14.3996451f;
  for (int i = 0; i < P; ++i) {
    float acc = 0.f;
    for (int j = 0; j < N; ++j) {
      float R0 = pts[3 * i + 0] - x[3 * j + 0];
      float R1 = pts[3 * i + 1] - x[3 * j + 1];
      float R2 = pts[3 * i + 2] - x[3 * j + 2];
      float rn = (float)sqrt((double)R0 * R0 + (double)R1 * R1 + (double)R2 * R2);
      acc += k * (float)(1.0 / rn) * q[j];
    }
    phi[i] = acc;
  }
}

static void step_f32(const float p[3], int N, const float* x, const float* q, float h,
                     float out[3]) {
  float E[3];
  field_at_f32(p, N, x, q, E);
  float n = (float)sqrt((double)E[0] * E[0] + (double)E[1] * E[1] + (double)E[2] * E[2]);
  for (int k = 0; k < 3; ++k) out[k] = p[k] + h * E[k] / n;
}

static float curve_f32(const float a[3], const float b[3]) {
  float c0 = a[1] * b[2] - a[2] * b[1];
  float c1 = a[2] * b[0] - a[0] * b[2];
  float c2 = a[0] * b[1] - a[1] * b[0];
  float nc = (float)sqrt((double)c0 * c0 + (double)c1 * c1 + (double)c2 * c2);
  float na = (float)sqrt((double)a[0] * a[0] + (double)a[1] * a[1] + (double)a[2] * a[2]);
  return (float)(nc / ((double)na * na * na));
}

static int outside_box_f32(const float p[3], const float d[3]) {
  return p[0] < -d[0] || p[0] > d[0] || p[1] < -d[1] || p[1] > d[1] || p[2] < -d[2] ||
         p[2] > d[2];
}

/* thread_operation (math_module.c:523-591) in the reference's float arithmetic. */
int oracle_topo_line_f32(int N, int n_iter, float h, const float x0[3], const float dims[3],
                         const float* x, const float* q, float ret[2], float end[3]) {
  float cur[3] = {x0[0], x0[1], x0[2]};
  int steps = 0;
  for (int i = 0; i < n_iter; ++i) {
    float nxt[3];
    step_f32(cur, N, x, q, h, nxt);
    memcpy(cur, nxt, sizeof cur);
    ++steps;
    if (outside_box_f32(cur, dims)) break;
  }
  float a1[3], a2[3], b1[3], b2[3];
  step_f32(x0, N, x, q, h, a1);
  step_f32(a1, N, x, q, h, a2);
  step_f32(cur, N, x, q, h, b1);
  step_f32(b1, N, x, q, h, b2);
  float v1[3], v2[3], w1[3], w2[3];
  for (int k = 0; k < 3; ++k) {
    v1[k] = a1[k] - x0[k];
    v2[k] = a2[k] - 2 * a1[k] + x0[k];
    w1[k] = b1[k] - cur[k];
    w2[k] = b2[k] - 2 * b1[k] + cur[k];
  }
  float cm = (curve_f32(v1, v2) + curve_f32(w1, w2)) / 2;
  float s = 0.f;
  for (int k = 0; k < 3; ++k) s += (float)pow(fabsf(x0[k] - cur[k]), 2);
  ret[0] = (float)sqrt(s);
  ret[1] = cm;
  if (end) memcpy(end, cur, sizeof cur);
  return steps;
}


/* calc_field_base_dipole (math_module.c:335-371) in the reference's
 * arithmetic: float R, r from a double sqrt of double squares, r^2 and r^-5
 * through double pow rounded to float, float products and sums; the factor 3
 * on the x term only, as written there. */
static void dipole_field_f32(const float p[3], int N, const float* x, const float* mu, float E[3]) {
  const float k = 14.3996451f;
  float ex = 0.f, ey = 0.f, ez = 0.f;
  for (int j = 0; j < N; ++j) {
    float R0 = p[0] - x[3 * j], R1 = p[1] - x[3 * j + 1], R2 = p[2] - x[3 * j + 2];
    float rn = (float)sqrt(pow(R0, 2) + pow(R1, 2) + pow(R2, 2));
    float r2 = (float)pow(rn, 2);
    float r5 = (float)pow(rn, -5);
    const float* m = mu + 3 * j;
    float dot = 3 * m[0] * R0 + m[1] * R1 + m[2] * R2;
    ex += k * r5 * (dot * R0 - m[0] * r2);
    ey += k * r5 * (dot * R1 - m[1] * r2);
    ez += k * r5 * (dot * R2 - m[2] * r2);
  }
  E[0] = ex;
  E[1] = ey;
  E[2] = ez;
}

static void dipole_step_f32(const float p[3], int N, const float* x, const float* mu, float h,
                            float out[3]) {
  float E[3];
  dipole_field_f32(p, N, x, mu, E);
  float n = (float)sqrt(pow(E[0], 2) + pow(E[1], 2) + pow(E[2], 2));
  for (int k = 0; k < 3; ++k) out[k] = p[k] + h * E[k] / n;
}

/* thread_operation_dipole (math_module.c:593-659) in the reference's float arithmetic. */
int oracle_topo_line_dipole_f32(int N, int n_iter, float h, const float x0[3], const float dims[3],
                                const float* x, const float* mu, float ret[2], float end[3]) {
  float cur[3] = {x0[0], x0[1], x0[2]};
  int steps = 0;
  for (int i = 0; i < n_iter; ++i) {
    float nxt[3];
    dipole_step_f32(cur, N, x, mu, h, nxt);
    memcpy(cur, nxt, sizeof cur);
    ++steps;
    if (outside_box_f32(cur, dims)) break;
  }
  float a1[3], a2[3], b1[3], b2[3];
  dipole_step_f32(x0, N, x, mu, h, a1);
  dipole_step_f32(a1, N, x, mu, h, a2);
  dipole_step_f32(cur, N, x, mu, h, b1);
  dipole_step_f32(b1, N, x, mu, h, b2);
  float v1[3], v2[3], w1[3], w2[3];
  for (int k = 0; k < 3; ++k) {
    v1[k] = a1[k] - x0[k];
    v2[k] = a2[k] - 2 * a1[k] + x0[k];
    w1[k] = b1[k] - cur[k];
    w2[k] = b2[k] - 2 * b1[k] + cur[k];
  }
  float cm = (curve_f32(v1, v2) + curve_f32(w1, w2)) / 2;
  float s = 0.f;
  for (int k = 0; k < 3; ++k) s += (float)pow(fabsf(x0[k] - cur[k]), 2);
  ret[0] = (float)sqrt(s);
  ret[1] = cm;
  if (end) memcpy(end, cur, sizeof cur);
  return steps;
}

/*
 * girih CPU oracle -- TEST INFRASTRUCTURE ONLY (see girih_oracle.h).
 *
 * Restates, in the same floating-point evaluation order, the girih reference's
 * serial operators (src/verification.c:315-479 and 786-819), its
 * initialisation (src/utils.c:436-496, 605-697) and its ping-pong time loop
 * (src/verification.c:281-284).  Must be compiled with -ffp-contract=off so
 * that no multiply-add is fused: the reference's serial build (-O0, x86-64
 * SSE2) rounds every product and every sum separately.
 */
#include "girih_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdint.h>

#define BOUNDARY_SRC (100.1) /* BOUNDARY_SRC_VAL, src/data_structures.h:195 */

int go_op_info(int op, int *radius, int *time_order, int *n_coef, int *coef_is_array) {
  int r, to, nc, arr;
  switch (op) { /* src/kernels/stencils.c:260-271 (radius, time order) */
    case GO_OP_STAR25_CONST_LEAPFROG: r = 4; to = 2; nc = 5; arr = 0; break;
    case GO_OP_STAR7_CONST: r = 1; to = 1; nc = 2; arr = 0; break;
    case GO_OP_STAR7_VAR: r = 1; to = 1; nc = 2; arr = 1; break;          /* 1 + r arrays */
    case GO_OP_STAR7_VAR_AXSYM: r = 1; to = 1; nc = 4; arr = 1; break;    /* 1 + 3r */
    case GO_OP_STAR25_VAR_AXSYM: r = 4; to = 1; nc = 13; arr = 1; break;  /* 1 + 3r */
    case GO_OP_STAR7_VAR_NOSYM: r = 1; to = 1; nc = 7; arr = 1; break;    /* 1 + 6r */
    case GO_OP_BOX27_CONST: r = 1; to = 1; nc = 4; arr = 0; break;
    case GO_OP_STAR7_CONST_LEAPFROG: r = 1; to = 2; nc = 2; arr = 0; break;
    default: return -1;
  }
  if (radius) *radius = r;
  if (time_order) *time_order = to;
  if (n_coef) *n_coef = nc;
  if (coef_is_array) *coef_is_array = arr;
  return 0;
}

void go_default_coefs(double out[11]) {
  /* param_default, src/utils.c:116-119 */
  static const double c[11] = {-0.28472, 0.16000, -0.02000, 0.00254, -0.00018, -0.18472,
                               0.19,     -0.0500, 0.00554,  -0.0009, 0.00354};
  for (int i = 0; i < 11; i++) out[i] = c[i];
}

/* ---------------------------------------------------------------- init */

void go_fill_ref(int op, int nx, int ny, int nz, int pnx, double *U1, double *U2, double *U3,
                 double *coef) {
  int r, to, nc, arr;
  if (go_op_info(op, &r, &to, &nc, &arr)) return;
  const int64_t nny = ny + 2 * r, nnz = nz + 2 * r;
  const int64_t ln = (int64_t)pnx * nny * nnz;
  double g[11];
  go_default_coefs(g);

  for (int64_t i = 0; i < ln; i++) {
    U1[i] = 0.0;
    U2[i] = 0.0;
    if (to == 2 && U3) U3[i] = 0.0;
  }
  /* interior ramp, utils.c:631-647 (single rank: gb = 0, xb = r, xe = nx + r) */
  for (int64_t k = r; k < nz + r; k++)
    for (int64_t j = r; j < ny + r; j++)
      for (int64_t i = r; i < nx + r; i++) {
        double rr = 1.0 / 3 * (1.0 * i / nx + 1.0 * j / ny + 1.0 * k / nz);
        int64_t idx = (k * nny + j) * pnx + i;
        U1[idx] = rr * 1.845703;
        U2[idx] = rr * 1.845703;
        if (to == 2 && U3) U3[idx] = rr * 1.845703;
      }
  /* boundary sources on the first and last x planes, utils.c:674-695 */
  for (int64_t k = 0; k < nnz; k++)
    for (int64_t j = 0; j < nny; j++) {
      int64_t row = (k * nny + j) * pnx;
      U1[row] += BOUNDARY_SRC;
      U2[row] += BOUNDARY_SRC;
      U1[row + nx + 2 * r - 1] += BOUNDARY_SRC;
      U2[row + nx + 2 * r - 1] += BOUNDARY_SRC;
    }
  /* coefficients, init_coeff utils.c:436-496 */
  if (!coef) return;
  if (!arr) {
    for (int i = 0; i <= r; i++) coef[i] = g[i];
    return;
  }
  switch (op) {
    case GO_OP_STAR7_VAR:
      for (int m = 0; m <= r; m++)
        for (int64_t i = 0; i < ln; i++) coef[i + m * ln] = g[m];
      break;
    case GO_OP_STAR7_VAR_AXSYM:
    case GO_OP_STAR25_VAR_AXSYM:
      for (int64_t i = 0; i < ln; i++) coef[i] = g[0];
      for (int d = 0; d < r; d++)
        for (int ax = 0; ax < 3; ax++)
          for (int64_t i = 0; i < ln; i++) coef[i + ln + 3 * d * ln + ax * ln] = g[d + 1];
      break;
    case GO_OP_STAR7_VAR_NOSYM:
      for (int64_t i = 0; i < ln; i++) coef[i] = g[0];
      for (int d = 0; d < r; d++)
        for (int ax = 0; ax < 3; ax++)
          for (int64_t i = 0; i < ln; i++) {
            coef[i + ln + 6 * d * ln + 2 * ax * ln] = g[d + 1];
            coef[i + ln + 6 * d * ln + (2 * ax + 1) * ln] = g[d + 1];
          }
      break;
  }
}

static uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double go_seeded_value(uint64_t seed, uint32_t stream, uint64_t idx, double lo, double hi) {
  uint64_t key = splitmix64(seed ^ ((uint64_t)stream * 0xD1B54A32D192ED03ULL));
  uint64_t h = splitmix64(key + idx);
  double u = (double)(h >> 11) * 0x1.0p-53;
  double d = hi - lo;
  double m = d * u;
  return lo + m;
}

static double seeded_maybe_f32(uint64_t seed, uint32_t stream, uint64_t idx, double lo, double hi,
                               int round_f32) {
  double v = go_seeded_value(seed, stream, idx, lo, hi);
  return round_f32 ? (double)(float)v : v;
}

void go_fill_seeded(int op, int nx, int ny, int nz, int pnx, uint64_t seed, double f_lo,
                    double f_hi, double r_lo, double r_hi, double c_lo, double c_hi, double *U1,
                    double *U2, double *U3, double *coef, int round_f32, int nthreads) {
  int r, to, nc, arr;
  if (go_op_info(op, &r, &to, &nc, &arr)) return;
  const int64_t nnx = nx + 2 * r, nny = ny + 2 * r, nnz = nz + 2 * r;
  const int64_t ln = (int64_t)pnx * nny * nnz;
  int nth = nthreads < 1 ? 1 : nthreads;
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int64_t k = 0; k < nnz; k++)
    for (int64_t j = 0; j < nny; j++)
      for (int64_t i = 0; i < pnx; i++) {
        int64_t idx = (k * nny + j) * pnx + i;
        int in = i < nnx;
        uint64_t g = (uint64_t)((k * nny + j) * nnx + i);
        double f = in ? seeded_maybe_f32(seed, 0, g, f_lo, f_hi, round_f32) : 0.0;
        U1[idx] = f;
        U2[idx] = f;
        if (to == 2 && U3) U3[idx] = in ? seeded_maybe_f32(seed, 1, g, r_lo, r_hi, round_f32) : 0.0;
        if (arr && coef)
          for (int m = 0; m < nc; m++)
            coef[idx + m * ln] =
                in ? seeded_maybe_f32(seed, 2 + (uint32_t)m, g, c_lo, c_hi, round_f32) : 0.0;
      }
}

/* ---------------------------------------------------------------- operators */

#define IDX(i, j, k) (((int64_t)(k) * nny + (j)) * pnx + (i))
#define V(i, j, k) v[IDX(i, j, k)]
#define COEF(m, i, j, k) coef[IDX(i, j, k) + (int64_t)(m) * ln]

/* Each body is the serial reference operator with the same association of
 * sums and products.  The comments give the reference lines restated. */

static void step_star25_const_leapfrog(int nx, int ny, int nz, int pnx, const double *coef,
                                       double *u, const double *v, const double *roc2, int nth) {
  const int64_t nny = ny + 8;
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 4; k < nz + 4; k++)
    for (int j = 4; j < ny + 4; j++)
      for (int i = 4; i < nx + 4; i++) {
        /* verification.c:330-350 */
        double lap = coef[0] * V(i, j, k)
                   + coef[1] * (V(i + 1, j, k) + V(i - 1, j, k))
                   + coef[1] * (V(i, j + 1, k) + V(i, j - 1, k))
                   + coef[1] * (V(i, j, k + 1) + V(i, j, k - 1))
                   + coef[2] * (V(i + 2, j, k) + V(i - 2, j, k))
                   + coef[2] * (V(i, j + 2, k) + V(i, j - 2, k))
                   + coef[2] * (V(i, j, k + 2) + V(i, j, k - 2))
                   + coef[3] * (V(i + 3, j, k) + V(i - 3, j, k))
                   + coef[3] * (V(i, j + 3, k) + V(i, j - 3, k))
                   + coef[3] * (V(i, j, k + 3) + V(i, j, k - 3))
                   + coef[4] * (V(i + 4, j, k) + V(i - 4, j, k))
                   + coef[4] * (V(i, j + 4, k) + V(i, j - 4, k))
                   + coef[4] * (V(i, j, k + 4) + V(i, j, k - 4));
        int64_t c = IDX(i, j, k);
        u[c] = 2. * v[c] - u[c] + roc2[c] * lap;
      }
}

static void step_star7_const_leapfrog(int nx, int ny, int nz, int pnx, const double *coef,
                                      double *u, const double *v, const double *roc2, int nth) {
  const int64_t nny = ny + 2;
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* operator 0's update (verification.c:330-350) with radius 1 */
        double lap = coef[0] * V(i, j, k)
                   + coef[1] * (V(i + 1, j, k) + V(i - 1, j, k))
                   + coef[1] * (V(i, j + 1, k) + V(i, j - 1, k))
                   + coef[1] * (V(i, j, k + 1) + V(i, j, k - 1));
        int64_t c = IDX(i, j, k);
        u[c] = 2. * v[c] - u[c] + roc2[c] * lap;
      }
}

static void step_star7_const(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                             const double *v, int nth) {
  const int64_t nny = ny + 2;
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* verification.c:367-370 */
        u[IDX(i, j, k)] = coef[0] * V(i, j, k)
                        + coef[1] * (V(i + 1, j, k) + V(i - 1, j, k))
                        + coef[1] * (V(i, j + 1, k) + V(i, j - 1, k))
                        + coef[1] * (V(i, j, k + 1) + V(i, j, k - 1));
      }
}

static void step_star7_var(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                           const double *v, int nth) {
  const int64_t nny = ny + 2, ln = (int64_t)pnx * nny * (nz + 2);
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* verification.c:390-393 */
        u[IDX(i, j, k)] = COEF(0, i, j, k) * V(i, j, k)
                        + COEF(1, i, j, k) * (V(i + 1, j, k) + V(i - 1, j, k))
                        + COEF(1, i, j, k) * (V(i, j + 1, k) + V(i, j - 1, k))
                        + COEF(1, i, j, k) * (V(i, j, k + 1) + V(i, j, k - 1));
      }
}

static void step_star7_var_axsym(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                                 const double *v, int nth) {
  const int64_t nny = ny + 2, ln = (int64_t)pnx * nny * (nz + 2);
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* verification.c:413-416 */
        u[IDX(i, j, k)] = COEF(0, i, j, k) * V(i, j, k)
                        + COEF(1, i, j, k) * (V(i + 1, j, k) + V(i - 1, j, k))
                        + COEF(2, i, j, k) * (V(i, j + 1, k) + V(i, j - 1, k))
                        + COEF(3, i, j, k) * (V(i, j, k + 1) + V(i, j, k - 1));
      }
}

static void step_star25_var_axsym(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                                  const double *v, int nth) {
  const int64_t nny = ny + 8, ln = (int64_t)pnx * nny * (nz + 8);
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 4; k < nz + 4; k++)
    for (int j = 4; j < ny + 4; j++)
      for (int i = 4; i < nx + 4; i++) {
        /* verification.c:437-449 */
        u[IDX(i, j, k)] = COEF(0, i, j, k) * V(i, j, k)
                        + COEF(1, i, j, k) * (V(i + 1, j, k) + V(i - 1, j, k))
                        + COEF(2, i, j, k) * (V(i, j + 1, k) + V(i, j - 1, k))
                        + COEF(3, i, j, k) * (V(i, j, k + 1) + V(i, j, k - 1))
                        + COEF(4, i, j, k) * (V(i + 2, j, k) + V(i - 2, j, k))
                        + COEF(5, i, j, k) * (V(i, j + 2, k) + V(i, j - 2, k))
                        + COEF(6, i, j, k) * (V(i, j, k + 2) + V(i, j, k - 2))
                        + COEF(7, i, j, k) * (V(i + 3, j, k) + V(i - 3, j, k))
                        + COEF(8, i, j, k) * (V(i, j + 3, k) + V(i, j - 3, k))
                        + COEF(9, i, j, k) * (V(i, j, k + 3) + V(i, j, k - 3))
                        + COEF(10, i, j, k) * (V(i + 4, j, k) + V(i - 4, j, k))
                        + COEF(11, i, j, k) * (V(i, j + 4, k) + V(i, j - 4, k))
                        + COEF(12, i, j, k) * (V(i, j, k + 4) + V(i, j, k - 4));
      }
}

static void step_star7_var_nosym(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                                 const double *v, int nth) {
  const int64_t nny = ny + 2, ln = (int64_t)pnx * nny * (nz + 2);
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* verification.c:468-474 */
        u[IDX(i, j, k)] = COEF(0, i, j, k) * V(i, j, k)
                        + COEF(1, i, j, k) * V(i - 1, j, k)
                        + COEF(2, i, j, k) * V(i + 1, j, k)
                        + COEF(3, i, j, k) * V(i, j - 1, k)
                        + COEF(4, i, j, k) * V(i, j + 1, k)
                        + COEF(5, i, j, k) * V(i, j, k - 1)
                        + COEF(6, i, j, k) * V(i, j, k + 1);
      }
}

static void step_box27_const(int nx, int ny, int nz, int pnx, const double *coef, double *u,
                             const double *v, int nth) {
  const int64_t nny = ny + 2;
  (void)nth;
#pragma omp parallel for num_threads(nth) if (nth > 1) schedule(static)
  for (int k = 1; k < nz + 1; k++)
    for (int j = 1; j < ny + 1; j++)
      for (int i = 1; i < nx + 1; i++) {
        /* verification.c:797-815 */
        u[IDX(i, j, k)] = coef[0] * V(i, j, k)
            + coef[1] * (V(i + 1, j, k) + V(i - 1, j, k))
            + coef[1] * (V(i, j + 1, k) + V(i, j - 1, k))
            + coef[1] * (V(i, j, k + 1) + V(i, j, k - 1))
            + coef[2] * (V(i + 1, j, k - 1) + V(i - 1, j, k - 1))
            + coef[2] * (V(i, j + 1, k - 1) + V(i, j - 1, k - 1))
            + coef[2] * (V(i + 1, j + 1, k) + V(i - 1, j - 1, k))
            + coef[2] * (V(i + 1, j - 1, k) + V(i - 1, j + 1, k))
            + coef[2] * (V(i + 1, j, k + 1) + V(i - 1, j, k + 1))
            + coef[2] * (V(i, j + 1, k + 1) + V(i, j - 1, k + 1))
            + coef[3] * (V(i + 1, j + 1, k + 1) + V(i - 1, j - 1, k - 1))
            + coef[3] * (V(i + 1, j - 1, k + 1) + V(i - 1, j + 1, k - 1))
            + coef[3] * (V(i - 1, j - 1, k + 1) + V(i + 1, j + 1, k - 1))
            + coef[3] * (V(i - 1, j + 1, k + 1) + V(i + 1, j - 1, k - 1));
      }
}

int go_step(int op, int nx, int ny, int nz, int pnx, const double *coef, double *u,
            const double *v, const double *roc2, int nthreads) {
  int r;
  if (go_op_info(op, &r, 0, 0, 0)) return -1;
  if (nx < 1 || ny < 1 || nz < 1 || pnx < nx + 2 * r) return -2;
  int nth = nthreads < 1 ? 1 : nthreads;
  switch (op) {
    case GO_OP_STAR25_CONST_LEAPFROG:
      step_star25_const_leapfrog(nx, ny, nz, pnx, coef, u, v, roc2, nth); break;
    case GO_OP_STAR7_CONST: step_star7_const(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_STAR7_VAR: step_star7_var(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_STAR7_VAR_AXSYM: step_star7_var_axsym(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_STAR25_VAR_AXSYM: step_star25_var_axsym(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_STAR7_VAR_NOSYM: step_star7_var_nosym(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_BOX27_CONST: step_box27_const(nx, ny, nz, pnx, coef, u, v, nth); break;
    case GO_OP_STAR7_CONST_LEAPFROG:
      step_star7_const_leapfrog(nx, ny, nz, pnx, coef, u, v, roc2, nth); break;
  }
  return 0;
}

int go_run(int op, int nx, int ny, int nz, int pnx, int nt, double *U1, double *U2,
           const double *U3, const double *coef, int nthreads) {
  for (int it = 0; it < nt; it += 2) {
    int e = go_step(op, nx, ny, nz, pnx, coef, U1, U2, U3, nthreads);
    if (e) return e;
    go_step(op, nx, ny, nz, pnx, coef, U2, U1, U3, nthreads);
  }
  return 0;
}

int go_run_source(int op, int nx, int ny, int nz, int pnx, int nt, double *U1, double *U2,
                  const double *U3, const double *coef, const int pt[3], const double *source,
                  int nsrc, int nthreads) {
  int r;
  if (go_op_info(op, &r, 0, 0, 0)) return -1;
  const int n[3] = {nx, ny, nz};
  for (int a = 0; a < 3; a++)
    if (pt[a] < r || pt[a] >= n[a] + r) return -3;
  const int64_t nny = ny + 2 * r;
  const int64_t at = IDX(pt[0], pt[1], pt[2]);
  for (int it = 0; it < nt; it += 2) {
    int e = go_step(op, nx, ny, nz, pnx, coef, U1, U2, U3, nthreads);
    if (e) return e;
    if (it < nsrc) U1[at] += source[it];
    go_step(op, nx, ny, nz, pnx, coef, U2, U1, U3, nthreads);
    if (it + 1 < nsrc) U2[at] += source[it + 1];
  }
  return 0;
}

void go_norms(const double *a, const double *b, int nx, int ny, int nz, int pnx, int r,
              double out[4]) {
  const int64_t nny = ny + 2 * r;
  double me = 0, mb = 0, se = 0, sb = 0;
  for (int k = r; k < nz + r; k++)
    for (int j = r; j < ny + r; j++)
      for (int i = r; i < nx + r; i++) {
        int64_t c = IDX(i, j, k);
        double e = fabs(a[c] - b[c]), bb = fabs(b[c]);
        if (e > me || e != e) me = e;
        if (bb > mb) mb = bb;
        se += e * e;
        sb += bb * bb;
      }
  out[0] = me; out[1] = mb; out[2] = se; out[3] = sb;
}

/*
 * CPU oracle: plain-C restatement of aphros's projection-step hot path.
 * TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline); the product
 * library never links or calls it.  See aphros_oracle.h for conventions.
 *
 * Compile with -ffp-contract=off: the reference is built for x86-64 without
 * FMA, so contracted multiply-adds (the default for GCC on aarch64) would
 * change the last bits of the results.
 */
#include "aphros_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <time.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* helpers                                                             */
/* ------------------------------------------------------------------ */

static inline int wrap(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}
static inline int64_t cidx(const int n[3], int i, int j, int k) {
  return (int64_t)wrap(i, n[0]) +
         (int64_t)n[0] * ((int64_t)wrap(j, n[1]) + (int64_t)n[1] * wrap(k, n[2]));
}
static inline double sqr(double a) { return a * a; }
static inline double cube(double a) { return a * a * a; }
/* std::min(a, b) / std::max(a, b) semantics (first argument wins ties and
 * NaN comparisons), as used throughout the reference. */
static inline double stdmin(double a, double b) { return (b < a) ? b : a; }
static inline double stdmax(double a, double b) { return (a < b) ? b : a; }

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ------------------------------------------------------------------ */
/* Poisson / projection                                                */
/* ------------------------------------------------------------------ */

void orc_mixture_density(
    int64_t ncells, const double* alpha, double rho1, double rho2,
    double* rho) {
  /* kernel/hydro.ipp:1818-1821: a2 = vf, a1 = 1 - a2, rho = rho1*a1+rho2*a2 */
  for (int64_t c = 0; c < ncells; ++c) {
    const double a2 = alpha[c];
    const double a1 = 1 - a2;
    rho[c] = rho1 * a1 + rho2 * a2;
  }
}

void orc_face_density(const int n[3], const double* rho, double* rho_f[3]) {
  /* approx_eb.h:351-363: inv = 1/rho; face = (inv[cp] + inv[cm]) * 0.5
   * (approx_eb.ipp:831); result 1/face. */
  for (int d = 0; d < 3; ++d) {
    for (int k = 0; k < n[2]; ++k)
      for (int j = 0; j < n[1]; ++j)
        for (int i = 0; i < n[0]; ++i) {
          const int64_t cp = cidx(n, i, j, k);
          const int64_t cm =
              cidx(n, i - (d == 0), j - (d == 1), k - (d == 2));
          const double invp = 1 / rho[cp];
          const double invm = 1 / rho[cm];
          rho_f[d][cp] = 1 / ((invp + invm) * 0.5);
        }
  }
}

void orc_surface_tension(
    const int n[3], double h, const double* u, const double* kappa,
    double sigma, double* ffst[3]) {
  /* util/hydro.ipp:1289-1310 (volume fraction of the mesh is 1) */
  for (int d = 0; d < 3; ++d) {
    for (int k = 0; k < n[2]; ++k)
      for (int j = 0; j < n[1]; ++j)
        for (int i = 0; i < n[0]; ++i) {
          const int64_t cp = cidx(n, i, j, k);
          const int64_t cm =
              cidx(n, i - (d == 0), j - (d == 1), k - (d == 2));
          const double um = stdmax(0., stdmin(1., u[cm] / 1.));
          const double up = stdmax(0., stdmin(1., u[cp] / 1.));
          const double ga = (up - um) / h;
          if (ga != 0.) {
            double kk = (fabs(um - 0.5) < fabs(up - 0.5) ? kappa[cm] : kappa[cp]);
            kk = (isnan(kk) ? 0 : kk);
            ffst[d][cp] += ga * kk * sigma;
          }
        }
  }
}

void orc_face_flux_with_force(
    const int n[3], double h, double dt, double* const vstar[3],
    double* const febp[3], double* const rho_f[3], double* vout[3]) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  const double area = h * h;
  for (int d = 0; d < 3; ++d)
    for (int64_t c = 0; c < nc; ++c) {
      double v = vstar[d][c];
      if (febp) v += febp[d][c] / rho_f[d][c] * dt * area;
      vout[d][c] = v;
    }
}

void orc_assemble_projection(
    const int n[3], double h, double dt, double* const rho_f[3],
    double* const vflux[3], const double* src, double* expr8, double* fk[3],
    double* fv[3]) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  const double area = h * h;
  const double vol = (h * h) * h;
  const double ainv = 1 / h; /* approx_eb.ipp:1442 a = 1/h */
  /* Face expressions (proj.ipp:343-360).  GradientImplicit gives
   * (-a, a, 0); multiplied by (-area/rho_f*dt), then v* added to [2].
   * e0 = -a*kk, e1 = a*kk with kk = -area/rho_f*dt, so e1 = -e0 exactly. */
  double* e0f[3];
  for (int d = 0; d < 3; ++d) {
    e0f[d] = (double*)malloc(sizeof(double) * nc);
    for (int64_t c = 0; c < nc; ++c) {
      const double kk = -area / rho_f[d][c] * dt;
      e0f[d][c] = -ainv * kk;
      if (fk) fk[d][c] = e0f[d][c];
      if (fv) fv[d][c] = vflux[d][c];
    }
  }
  /* GetFluxSum (proj.ipp:367-383): for q = xm,xp,ym,yp,zm,zp
   * v = ffe * outward (-1 for minus faces), AppendExpr:
   * sum[0] += v[1 - q%2]; sum[1+q] += v[q%2]; sum[7] += v[2]. */
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        double* e = expr8 + 8 * c;
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 6; ++q) {
          const int d = q / 2;
          const int64_t f =
              (q % 2 == 0)
                  ? c
                  : cidx(n, i + (d == 0), j + (d == 1), k + (d == 2));
          const double fe0 = e0f[d][f];
          const double fe1 = -fe0;
          const double fe2 = vflux[d][f];
          double v0, v1, v2;
          if (q % 2 == 0) {
            v0 = -fe0;
            v1 = -fe1;
            v2 = -fe2;
          } else {
            v0 = fe0;
            v1 = fe1;
            v2 = fe2;
          }
          const double vv[2] = {v0, v1};
          s[0] += vv[1 - q % 2];
          s[1 + q] += vv[q % 2];
          s[7] += v2;
        }
        if (src) s[7] -= src[c] * vol;
        memcpy(e, s, sizeof(s));
      }
  for (int d = 0; d < 3; ++d) free(e0f[d]);
}

void orc_remove_rhs_mean(int64_t ncells, double* expr8) {
  double sum = 0;
  for (int64_t c = 0; c < ncells; ++c) sum += expr8[8 * c + 7];
  const double mean = sum / ncells;
  for (int64_t c = 0; c < ncells; ++c) expr8[8 * c + 7] -= mean;
}

/* y = A x (+ e7 when with_rhs), the loop of linear.ipp:47-53 / 66-72:
 * u = x[c]*e[0] (+ e.back()); u += x[nb_q]*e[1+q] for q in 0..5. */
static inline double apply_cell(
    const int n[3], const double* e, const double* x, int i, int j, int k,
    int with_rhs) {
  const int64_t c = cidx(n, i, j, k);
  double u = x[c] * e[0];
  if (with_rhs) u += e[7];
  u += x[cidx(n, i - 1, j, k)] * e[1];
  u += x[cidx(n, i + 1, j, k)] * e[2];
  u += x[cidx(n, i, j - 1, k)] * e[3];
  u += x[cidx(n, i, j + 1, k)] * e[4];
  u += x[cidx(n, i, j, k - 1)] * e[5];
  u += x[cidx(n, i, j, k + 1)] * e[6];
  return u;
}

double orc_residual(
    const int n[3], const double* expr8, const double* x, double* r) {
  double s = 0;
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        const double u = apply_cell(n, expr8 + 8 * c, x, i, j, k, 1);
        if (r) r[c] = -u;
        s += u * u;
      }
  return s;
}

typedef struct {
  double* x;
  double* r;
  double* p;
  double* lp;
} cg_vec;

/* One CG iteration body (stages iter, iter2, iter3 of linear.ipp:64-101).
 * Returns dot_r (after update); writes dot_r_prev and max_r. */
static double cg_iteration(
    const int n[3], const double* expr8, cg_vec* v, double* dot_r_prev_out,
    double* max_r_out) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  double dot_r_prev = 0, dot_p_lp = 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        v->lp[c] = apply_cell(n, expr8 + 8 * c, v->p, i, j, k, 0);
      }
#pragma omp parallel for schedule(static) reduction(+ : dot_r_prev, dot_p_lp)
  for (int64_t c = 0; c < nc; ++c) {
    dot_r_prev += sqr(v->r[c]);
    dot_p_lp += v->p[c] * v->lp[c];
  }
  const double alpha = dot_r_prev / (dot_p_lp + 1e-100);
  double dot_r = 0, max_r = 0;
#pragma omp parallel for schedule(static) reduction(+ : dot_r) reduction(max : max_r)
  for (int64_t c = 0; c < nc; ++c) {
    v->x[c] += alpha * v->p[c];
    v->r[c] -= alpha * v->lp[c];
    dot_r += sqr(v->r[c]);
    max_r = stdmax(max_r, fabs(v->r[c]));
  }
  const double beta = dot_r / (dot_r_prev + 1e-100);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    v->p[c] = v->r[c] + beta * v->p[c];
  }
  *dot_r_prev_out = dot_r_prev;
  *max_r_out = max_r;
  return dot_r;
}

orc_info orc_cg_solve(
    const int n[3], double cellvol, const double* expr8, const double* x0,
    double* x, double tol, int miniter, int maxiter, int maxnorm,
    double* res_hist, int nthreads) {
  set_threads(nthreads);
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  cg_vec v;
  v.x = (double*)malloc(sizeof(double) * nc);
  v.r = (double*)malloc(sizeof(double) * nc);
  v.p = (double*)malloc(sizeof(double) * nc);
  v.lp = (double*)malloc(sizeof(double) * nc);
  /* stage init (linear.ipp:42-58) */
  if (x0)
    memcpy(v.x, x0, sizeof(double) * nc);
  else
    memset(v.x, 0, sizeof(double) * nc);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        v.r[c] = -apply_cell(n, expr8 + 8 * c, v.x, i, j, k, 1);
      }
  memcpy(v.p, v.r, sizeof(double) * nc);
  orc_info info = {0, 0};
  int iter = 0;
  for (;;) {
    double drp, maxr;
    const double dot_r = cg_iteration(n, expr8, &v, &drp, &maxr);
    /* stage check (linear.ipp:102-114) */
    info.residual = maxnorm ? maxr / cellvol : sqrt(dot_r / cellvol);
    ++iter;
    info.iter = iter;
    if (res_hist) res_hist[iter - 1] = info.residual;
    if (iter >= miniter && (iter > maxiter || info.residual < tol)) break;
  }
  memcpy(x, v.x, sizeof(double) * nc);
  free(v.x);
  free(v.r);
  free(v.p);
  free(v.lp);
  return info;
}

double orc_cg_time_iters(
    const int n[3], const double* expr8, double* x, int iters, int nthreads) {
  set_threads(nthreads);
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  cg_vec v;
  v.x = x;
  v.r = (double*)malloc(sizeof(double) * nc);
  v.p = (double*)malloc(sizeof(double) * nc);
  v.lp = (double*)malloc(sizeof(double) * nc);
  const double t0 = now_s();
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        v.r[c] = -apply_cell(n, expr8 + 8 * c, v.x, i, j, k, 1);
      }
  memcpy(v.p, v.r, sizeof(double) * nc);
  for (int it = 0; it < iters; ++it) {
    double drp, maxr;
    cg_iteration(n, expr8, &v, &drp, &maxr);
  }
  const double t1 = now_s();
  free(v.r);
  free(v.p);
  free(v.lp);
  return t1 - t0;
}

void orc_flux_correct(
    const int n[3], double* const fk[3], double* const fv[3], const double* p,
    double* vout[3]) {
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < n[2]; ++k)
      for (int j = 0; j < n[1]; ++j)
        for (int i = 0; i < n[0]; ++i) {
          const int64_t cp = cidx(n, i, j, k);
          const int64_t cm =
              cidx(n, i - (d == 0), j - (d == 1), k - (d == 2));
          const double e0 = fk[d][cp];
          const double e1 = -e0;
          vout[d][cp] = p[cm] * e0 + p[cp] * e1 + fv[d][cp];
        }
}

void orc_acceleration(
    const int n[3], double h, const double* p, double* const rho_f[3],
    double* const febp[3], double* acc) {
  /* proj.ipp:408-433 with UEmbed::Gradient (approx_eb.ipp:882-890) and
   * AverageGradient (approx_eb.ipp:1530-1544). */
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        double s[3] = {0, 0, 0};
        for (int q = 0; q < 6; ++q) {
          const int d = q / 2;
          const int64_t f =
              (q % 2 == 0)
                  ? c
                  : cidx(n, i + (d == 0), j + (d == 1), k + (d == 2));
          const int64_t cm =
              (q % 2 == 0) ? cidx(n, i - (d == 0), j - (d == 1), k - (d == 2))
                           : c;
          const int64_t cp = f;
          const double gp = (p[cp] - p[cm]) / h;
          const double fb = febp ? febp[d][f] : 0.;
          const double a = (fb - gp) / rho_f[d][f];
          for (int e = 0; e < 3; ++e) s[e] += (e == d ? 1. : 0.) * (a * 0.5);
        }
        acc[3 * c + 0] = s[0];
        acc[3 * c + 1] = s[1];
        acc[3 * c + 2] = s[2];
      }
}

/* ------------------------------------------------------------------ */
/* PLIC geometry, solver/reconst.h                                     */
/* ------------------------------------------------------------------ */

double orc_solve_cubic(double a, double b, double c, double d, int k) {
  /* reconst.h:38-49 */
  double p = (3. * a * c - b * b) / (3. * a * a);
  p = stdmin(p, 0.);
  const double q =
      (2. * cube(b) - 9. * a * b * c + 27. * a * a * d) / (27. * cube(a));
  double r = 3. * q * sqrt(-3. / p) / (2. * p);
  r = stdmax(-1., stdmin(1., r));
  const double t =
      2. * sqrt(-p / 3.) * cos(1. / 3. * acos(r) - 2. * M_PI * k / 3.);
  return t - b / (3. * a);
}

/* three-element sort of reconst.h:76-86 */
static inline void sort3(double v[3]) {
  double t;
  if (v[1] < v[0]) { t = v[0]; v[0] = v[1]; v[1] = t; }
  if (v[2] < v[1]) { t = v[1]; v[1] = v[2]; v[2] = t; }
  if (v[1] < v[0]) { t = v[0]; v[0] = v[1]; v[1] = t; }
}

/* reconst.h:140-168, n sorted ascending, -0.5*sum(n) <= a <= 0 */
static double line_u0(const double n[3], double a) {
  const double nx = n[0], ny = n[1], nz = n[2];
  const double f = a + 0.5 * (nx + ny + nz);
  if (f <= 0) return 0;
  if (nx >= f) return cube(f) / (6 * nx * ny * nz);
  if (ny >= f) return (3 * sqr(f) - 3 * f * nx + sqr(nx)) / (6 * ny * nz);
  if (nz >= f) {
    if (nx + ny >= f) {
      return (3 * sqr(f) - 3 * f * nx + sqr(nx) -
              stdmin(1., (f - ny) / nx) * sqr(f - ny)) /
             (6 * ny * nz);
    }
    return (2 * f - nx - ny) / (2 * nz);
  }
  return (cube(f) - cube(f - nx) - cube(f - ny) - cube(f - nz)) /
         (6 * nx * ny * nz);
}

/* reconst.h:183-195 GetLineU1 */
static double line_u1(const double n0[3], double a) {
  double n[3] = {fabs(n0[0]), fabs(n0[1]), fabs(n0[2])};
  sort3(n);
  const double s = ((0 + n[0]) + n[1]) + n[2]; /* Vect::sum */
  a = stdmax(-0.5 * s, stdmin(0.5 * s, a)); /* Clip */
  if (a < 0) return line_u0(n, a);
  return 1 - line_u0(n, -a);
}

double orc_line_u(const double n[3], double a, const double h[3]) {
  /* reconst.h:201-203: GetLineU1(n * h, a) */
  const double nh[3] = {n[0] * h[0], n[1] * h[1], n[2] * h[2]};
  return line_u1(nh, a);
}

/* reconst.h:218-250, n sorted ascending, 0 <= u <= 0.5 */
static double line_a0(const double n[3], double u) {
  const double nx = n[0], ny = n[1], nz = n[2];
  double f;
  if (6. * ny * nz * u < sqr(nx)) {
    f = pow(6. * nx * ny * nz * u, 1. / 3.);
  } else if (6. * ny * nz * u < 3. * sqr(ny) - 3 * nx * ny + sqr(nx)) {
    f = 0.5 * nx + sqrt(2. * ny * nz * u - sqr(nx) / 12.);
  } else if (nz > nx + ny) {
    if (2. * nz * u < nx + ny) {
      f = orc_solve_cubic(
          1., -3. * (nx + ny), 3. * (sqr(nx) + sqr(ny)),
          -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u, 1);
    } else {
      f = nz * u + 0.5 * (nx + ny);
    }
  } else {
    if (6. * nx * ny * nz * u < -cube(nz) + 3. * sqr(nz) * (nx + ny) -
                                    3. * nz * (sqr(nx) + sqr(ny)) + cube(nx) +
                                    cube(ny)) {
      f = orc_solve_cubic(
          1., -3. * (nx + ny), 3. * (sqr(nx) + sqr(ny)),
          -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u, 1);
    } else {
      f = orc_solve_cubic(
          2., -3. * (nx + ny + nz), 3. * (sqr(nx) + sqr(ny) + sqr(nz)),
          -(cube(nx) + cube(ny) + cube(nz)) + 6. * nx * ny * nz * u, 1);
    }
  }
  return f - 0.5 * (nx + ny + nz);
}

double orc_line_a(const double n0[3], double u, const double h[3]) {
  /* reconst.h:264-285: GetLineA1(n * h, u) */
  double n[3] = {fabs(n0[0] * h[0]), fabs(n0[1] * h[1]), fabs(n0[2] * h[2])};
  sort3(n);
  u = stdmax(0., stdmin(1., u));
  if (u <= 0.5) return line_a0(n, u);
  return -line_a0(n, 1 - u);
}

double orc_line_vol(
    const double n0[3], double a, const double h[3], double dx, int d) {
  /* reconst.h:318-324 GetLineVol and 290-312 GetLineVol0 */
  double n[3] = {n0[0], n0[1], n0[2]};
  if (dx < 0.) {
    n[d] = -n[d];
    dx = -dx;
  }
  double hh[3] = {h[0], h[1], h[2]};
  hh[d] = dx;
  double dc[3] = {0, 0, 0};
  dc[d] = (h[d] - dx) * 0.5;
  const double ndc = ((0 + n[0] * dc[0]) + n[1] * dc[1]) + n[2] * dc[2];
  const double aa = a - ndc;
  const double uu = orc_line_u(n, aa, hh);
  const double vv = (hh[0] * hh[1]) * hh[2];
  double r = uu * vv;
  r = stdmin(r, orc_line_u(n, a, h) * ((h[0] * h[1]) * h[2]));
  return r;
}

double orc_line_flux(
    const double n[3], double a, const double h[3], double q, double dt,
    int d) {
  /* reconst.h:371-379 */
  const double s = ((h[0] * h[1]) * h[2]) / h[d];
  const double dx = q / s * dt;
  double v = orc_line_vol(n, a, h, dx, d);
  if (q < 0.) v = -v;
  return v / dt;
}

/* ------------------------------------------------------------------ */
/* VOF                                                                 */
/* ------------------------------------------------------------------ */

static inline int is_interface(double u) { return u > 0 && u < 1; }

void orc_normal_cell(const double u3[27], double nout[3]) {
#define Q(dx, dy, dz) u3[((dx) + 1) + 3 * ((dy) + 1) + 9 * ((dz) + 1)]
  /* normal.ipp:100-125: the 27-point Youngs gradient, terms accumulated in
   * lexicographic (dx,dy,dz) order with weights 1,2,4. */
  double nn[3];
  int started[3] = {0, 0, 0};
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const double q = Q(dx, dy, dz);
        const int o[3] = {dx, dy, dz};
        for (int e = 0; e < 3; ++e) {
          if (o[e] == 0) continue;
          const int t1 = o[(e + 1) % 3], t2 = o[(e + 2) % 3];
          const double w = (double)(o[e] * (t1 == 0 ? 2 : 1) * (t2 == 0 ? 2 : 1));
          if (!started[e]) {
            nn[e] = w * q;
            started[e] = 1;
          } else {
            nn[e] += w * q;
          }
        }
      }
  {
    const double s = ((0 + fabs(nn[0])) + fabs(nn[1])) + fabs(nn[2]);
    const double ms = -s;
    nn[0] /= ms;
    nn[1] /= ms;
    nn[2] /= ms;
  }
  /* normal.ipp:283-312 UpdateNormalHeight (3D, force_overwrite = false) */
  double best[3] = {0, 0, 0};
  int bdz = 0;
  for (int dz = 0; dz < 3; ++dz) {
    const int dx = (dz + 1) % 3;
    const int dy = (dz + 2) % 3;
    int oz[3] = {0, 0, 0};
    oz[dz] = 1;
    int ox[3] = {0, 0, 0};
    ox[dx] = 1;
    int oy[3] = {0, 0, 0};
    oy[dy] = 1;
#define HH(s0, s1, s2)                                                   \
  ((Q((s0) - oz[0], (s1) - oz[1], (s2) - oz[2]) + Q((s0), (s1), (s2))) + \
   Q((s0) + oz[0], (s1) + oz[1], (s2) + oz[2]))
    double m[3];
    m[dx] = HH(ox[0], ox[1], ox[2]) - HH(-ox[0], -ox[1], -ox[2]);
    m[dy] = HH(oy[0], oy[1], oy[2]) - HH(-oy[0], -oy[1], -oy[2]);
    m[dz] = (Q(oz[0], oz[1], oz[2]) - Q(-oz[0], -oz[1], -oz[2]) > 0 ? 2 : -2);
#undef HH
    const double s = ((0 + fabs(m[0])) + fabs(m[1])) + fabs(m[2]);
    const double ms = -s;
    m[0] /= ms;
    m[1] /= ms;
    m[2] /= ms;
    if (fabs(best[bdz]) < fabs(m[dz])) {
      best[0] = m[0];
      best[1] = m[1];
      best[2] = m[2];
      bdz = dz;
    }
  }
  if (fabs(best[bdz]) < fabs(nn[bdz])) {
    nn[0] = best[0];
    nn[1] = best[1];
    nn[2] = best[2];
  }
  nout[0] = nn[0];
  nout[1] = nn[1];
  nout[2] = nn[2];
#undef Q
}

void orc_vof_reconstruct(
    const int n[3], const double h[3], const double* u, uint8_t* mask,
    double* nrm, double* a) {
  const double nan = NAN;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        const int m = is_interface(u[c]);
        if (mask) mask[c] = (uint8_t)m;
        if (!m) {
          nrm[3 * c + 0] = nan;
          nrm[3 * c + 1] = nan;
          nrm[3 * c + 2] = nan;
          a[c] = nan;
          continue;
        }
        double u3[27];
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
              u3[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] =
                  u[cidx(n, i + dx, j + dy, k + dz)];
        double nn[3];
        orc_normal_cell(u3, nn);
        nrm[3 * c + 0] = nn[0];
        nrm[3 * c + 1] = nn[1];
        nrm[3 * c + 2] = nn[2];
        a[c] = orc_line_a(nn, u[c], h);
      }
}

void orc_vof_sweep(
    const int n[3], const double h[3], double* u, const double* ffv, int d,
    const double* nrm, const double* a, const double* u0, double dt,
    double clipth) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  double* ffvu = (double*)malloc(sizeof(double) * nc);
  /* fluxes (vof.ipp:228-256): face between cm = c - e_d and cp = c */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t f = cidx(n, i, j, k);
        const int64_t cm = cidx(n, i - (d == 0), j - (d == 1), k - (d == 2));
        const double v = ffv[f];
        const double v0 = v / 1.; /* area fraction 1 */
        const int64_t c = (v > 0) ? cm : f;
        const double* nn = nrm + 3 * c;
        const double sq = ((0 + sqr(nn[0])) + sqr(nn[1])) + sqr(nn[2]);
        if (u[c] > 0 && u[c] < 1 && sq > 0) {
          ffvu[f] = orc_line_flux(nn, a[c], h, v0, dt, d);
        } else {
          ffvu[f] = v0 * u[c];
        }
      }
  /* update (vof.ipp:287-326), weymouth */
  const double vol = (h[0] * h[1]) * h[2];
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        const int64_t fp = cidx(n, i + (d == 0), j + (d == 1), k + (d == 2));
        const int64_t fm = c;
        const double ds =
            (ffv[fp] / (1 + 1e-16) - ffv[fm] / (1 + 1e-16)) * dt / vol;
        const double dl = (ffvu[fp] - ffvu[fm]) * dt / vol;
        const double uu = (u0[c] < 0.5 ? 0 : 1);
        double w = u[c];
        w += uu * ds - dl;
        if (!(w >= clipth)) {
          w = 0;
        } else if (!(w <= 1 - clipth)) {
          w = 1;
        }
        u[c] = w;
      }
  free(ffvu);
}

void orc_vof_step(
    const int n[3], const double h[3], double* u, double* const ffv[3],
    double dt, double clipth, int count, int reconstruct_first, uint8_t* mask,
    double* nrm, double* a) {
  orc_vof_step_src(n, h, u, ffv, NULL, dt, clipth, count, reconstruct_first,
                   mask, nrm, a);
}

void orc_vof_step_src(
    const int n[3], const double h[3], double* u, double* const ffv[3],
    const double* src, double dt, double clipth, int count,
    int reconstruct_first, uint8_t* mask, double* nrm, double* a) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  if (reconstruct_first) orc_vof_reconstruct(n, h, u, mask, nrm, a);
  if (src) {
    /* vof.ipp:510-513: uc = um + dt * fcs * (1 - um) */
    for (int64_t c = 0; c < nc; ++c) {
      const double um = u[c];
      u[c] = um + dt * src[c] * (1 - um);
    }
  }
  double* u0 = (double*)malloc(sizeof(double) * nc);
  memcpy(u0, u, sizeof(double) * nc);
  int dd[3];
  /* vof.ipp:428-435 */
  if (count % 3 == 0) {
    dd[0] = 0; dd[1] = 1; dd[2] = 2;
  } else if (count % 3 == 1) {
    dd[0] = 1; dd[1] = 2; dd[2] = 0;
  } else {
    dd[0] = 2; dd[1] = 0; dd[2] = 1;
  }
  for (int id = 0; id < 3; ++id) {
    const int d = dd[id];
    orc_vof_sweep(n, h, u, ffv[d], d, nrm, a, u0, dt, clipth);
    orc_vof_reconstruct(n, h, u, mask, nrm, a);
  }
  free(u0);
}

/* ------------------------------------------------------------------ */
/* Height functions, util/height.h and solver/curv.ipp                */
/* ------------------------------------------------------------------ */

double orc_height_good_n(const double* uu, int si, double nn) {
  /* util/height.h:19-62 */
  const int sih = si / 2;
  int ic = sih;
  while (ic < si && !is_interface(uu[ic])) {
    if (ic > sih)
      ic = si - ic - 1;
    else
      ic = si - ic;
  }
  if (ic >= si) return NAN;
  int im = ic;
  while (im >= 0 && is_interface(uu[im])) --im;
  if (im < 0) return NAN;
  int ip = ic;
  while (ip < si && is_interface(uu[ip])) ++ip;
  if (ip >= si) return NAN;
  if ((uu[ip] - uu[im]) * nn < 0) {
    double s = 0;
    for (int i = im; i <= ip; ++i) s += uu[i];
    return s + (double)im * uu[im] + (double)(si - ip - 1) * uu[ip];
  }
  return NAN;
}

double orc_height_good(const double* uu, int si) {
  /* util/height.h:69-124 */
  const int sih = si / 2;
  const int ic = sih;
  if (!is_interface(uu[ic])) return NAN;
  int im = ic;
  while (im >= 0 && is_interface(uu[im])) --im;
  if (im < 0) return NAN;
  int ip = ic;
  while (ip < si && is_interface(uu[ip])) ++ip;
  if (ip >= si) return NAN;
  if (uu[ip] != uu[im]) {
    double s = 0.;
    for (int i = im; i <= ip; ++i) s += uu[i];
    s += (double)im * uu[im] + (double)(si - ip - 1) * uu[ip];
    if (uu[im] == 0) s = si - s;
    s -= si * 0.5;
    return s;
  }
  return NAN;
}

void orc_heights_curvature(
    const int n[3], const double h[3], const double* u, const double* nrm,
    double* kappa, double* hgt_out) {
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  double* du2 = (double*)malloc(sizeof(double) * 3 * nc);
  double* du4 = (double*)malloc(sizeof(double) * 3 * nc);
  double* hgt = hgt_out ? hgt_out : (double*)malloc(sizeof(double) * 3 * nc);
  /* CalcDiff2 (curv.ipp:100-134) with all colours equal:
   * du2 = 0 + (-1)*u[c-2d] + (+1)*u[c+2d] */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        for (int d = 0; d < 3; ++d) {
          const int o[3] = {d == 0, d == 1, d == 2};
          double s = 0;
          s += -1 * u[cidx(n, i - 2 * o[0], j - 2 * o[1], k - 2 * o[2])];
          s += 1 * u[cidx(n, i + 2 * o[0], j + 2 * o[1], k + 2 * o[2])];
          du2[3 * c + d] = s;
        }
      }
  /* CalcDiff4 (curv.ipp:140-174) */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        for (int d = 0; d < 3; ++d) {
          const int o[3] = {d == 0, d == 1, d == 2};
          double s = 0;
          s += -1 * du2[3 * cidx(n, i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]) + d];
          s += 1 * du2[3 * cidx(n, i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]) + d];
          du4[3 * c + d] = s;
        }
      }
  /* CalcHeight (curv.ipp:185-254), S = 2, 13-cell column */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        hgt[3 * c + 0] = NAN;
        hgt[3 * c + 1] = NAN;
        hgt[3 * c + 2] = NAN;
        if (!is_interface(u[c])) continue;
        const int w[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
          const int o[3] = {d == 0, d == 1, d == 2};
#define NB(s) cidx(n, i + (s)*o[0], j + (s)*o[1], k + (s)*o[2])
          double uu[13];
          const int sih = 6;
          uu[sih] = u[c];
          uu[sih - 1] = u[NB(-1)];
          uu[sih + 1] = u[NB(1)];
          uu[sih - 2] = u[NB(-2)];
          uu[sih + 2] = u[NB(2)];
          for (int s = 0; s < 2; ++s) {
            const int q = (s + 1) * 2;
            const int ia = q + 1;
            const int ib = q + 2;
            const double* fcdu = (s == 0) ? du2 : du4;
            uu[sih - ia] = uu[sih - ia + 2 * q] - fcdu[3 * NB(-1) + d];
            uu[sih + ia] = uu[sih + ia - 2 * q] + fcdu[3 * NB(1) + d];
            uu[sih - ib] = uu[sih - ib + 2 * q] - fcdu[3 * NB(-2) + d];
            uu[sih + ib] = uu[sih + ib - 2 * q] + fcdu[3 * NB(2) + d];
          }
#undef NB
          const double off = orc_height_good(uu, 13);
          /* cell centre as MeshCartesian computes it (geom/mesh.ipp:205-206)
           * for a block at the origin: (low + h/2) + w*h */
          const double center = (0. + h[d] * 0.5) + (double)w[d] * h[d];
          hgt[3 * c + d] = center + off * h[d];
        }
      }
  /* CalcCurvHeight (curv.ipp:261-356) */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = cidx(n, i, j, k);
        kappa[c] = NAN;
        if (!is_interface(u[c])) continue;
        const double* nn = nrm + 3 * c;
        const double an[3] = {fabs(nn[0]), fabs(nn[1]), fabs(nn[2])};
        int dn = 0;
        for (int e = 1; e < 3; ++e)
          if (an[e] > an[dn]) dn = e;
        const int dx = (dn + 1) % 3;
        const int dy = (dn + 2) % 3;
        const double lx = h[dx];
        const double ly = h[dy];
        int on[3] = {0, 0, 0}, ox[3] = {0, 0, 0}, oy[3] = {0, 0, 0};
        on[dn] = 1;
        ox[dx] = 1;
        oy[dy] = 1;
        /* hh(cb): nearest interfacial cell along dn among shifts
         * 0,+1,-1,+2,-2 (curv.ipp:287-307) */
        double hv[3][3];
        for (int sy = -1; sy <= 1; ++sy)
          for (int sx = -1; sx <= 1; ++sx) {
            const int bi = i + sx * ox[0] + sy * oy[0];
            const int bj = j + sx * ox[1] + sy * oy[1];
            const int bk = k + sx * ox[2] + sy * oy[2];
            static const int shifts[5] = {0, 1, -1, 2, -2};
            double r = NAN;
            for (int t = 0; t < 5; ++t) {
              const int s = shifts[t];
              const int64_t cn =
                  cidx(n, bi + s * on[0], bj + s * on[1], bk + s * on[2]);
              if (is_interface(u[cn])) {
                r = hgt[3 * cn + dn];
                break;
              }
            }
            hv[sy + 1][sx + 1] = r;
          }
        const double hcc = hv[1][1];
        const double hmc = hv[1][0];
        const double hpc = hv[1][2];
        const double hcm = hv[0][1];
        const double hcp = hv[2][1];
        const double hmm = hv[0][0];
        const double hmp = hv[2][0];
        const double hpm = hv[0][2];
        const double hpp = hv[2][2];
        const double hx = (hpc - hmc) / (2 * lx);
        const double hy = (hcp - hcm) / (2 * ly);
        const double fl = 0.2;
        const double hxx = ((hpm - 2 * hcm + hmm) * fl + (hpc - 2 * hcc + hmc) +
                            (hpp - 2 * hcp + hmp) * fl) /
                           ((1 + 2 * fl) * lx * lx);
        const double hyy = ((hmp - 2 * hmc + hmm) * fl + (hcp - 2 * hcc + hcm) +
                            (hpp - 2 * hpc + hpm) * fl) /
                           ((1 + 2 * fl) * ly * ly);
        const double hxy = ((hpp - hmp) - (hpm - hmm)) / (4 * lx * ly);
        double kk =
            (2 * hx * hy * hxy - (sqr(hy) + 1) * hxx - (sqr(hx) + 1) * hyy) /
            pow(sqr(hx) + sqr(hy) + 1, 3. / 2.);
        if (nn[dn] < 0) kk *= -1;
        kappa[c] = kk;
      }
  free(du2);
  free(du4);
  if (!hgt_out) free(hgt);
}

/* ------------------------------------------------------------------------
 * Connected-component colours of the volume fraction, one block, periodic:
 * the union-find recolouring of Vof::MakeIteration (src/solver/vof.ipp:
 * 546-578) with UVof::Imp::RecolorUnionFind (src/util/vof.ipp:982-1150):
 *   resetcolor  gas cells (u > 0.5) get colour 0, others none (-1);
 *   recolor     26-connected gas cells form components; each takes the
 *               smallest unique initial colour in it, i.e. the ordinal of
 *               its first cell in x-fastest order (InitUniqueColors,
 *               util/vof.ipp:824-870); PairToMap (util/vof.ipp:612-650)
 *               maps each component to the previous colour of its first
 *               cell, in the order of the cells with two halo layers, that
 *               has one; ReduceColor (util/vof.ipp:740-803) keeps that
 *               colour unless taken, else gives the next unused one;
 *   propagate   cells without colour with 0 < u take the colour of a face
 *               neighbour with larger u, faces in the mesh's order
 *               (direction-major, x-fastest; geom/blockface.h:29-48), halo
 *               cells holding the values from before the pass.
 * cl_prev: colours before resetcolor; cl: result.
 * ------------------------------------------------------------------------ */

static int64_t uf_find(int64_t* p, int64_t x) {
  while (p[x] != x) {
    p[x] = p[p[x]];
    x = p[x];
  }
  return x;
}

static int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

#define XIDX(i, j, k) ((int64_t)(i) + (int64_t)nx * ((int64_t)(j) + (int64_t)ny * (int64_t)(k)))

void orc_recolor(const int n[3], const double* u, const double* cl_prev, double* cl) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const int64_t N = (int64_t)nx * ny * nz;
  int64_t* p = (int64_t*)malloc(sizeof(int64_t) * N);
  for (int64_t c = 0; c < N; ++c) p[c] = u[c] > 0.5 ? c : -1;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int64_t c = XIDX(i, j, k);
        if (p[c] < 0) continue;
        for (int dk = -1; dk <= 1; ++dk)
          for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
              const int64_t cn = XIDX(wrapi(i + di, nx), wrapi(j + dj, ny), wrapi(k + dk, nz));
              if (p[cn] < 0) continue;
              int64_t a = uf_find(p, c), b = uf_find(p, cn);
              if (a != b) {
                if (a < b) p[b] = a;  /* the smaller root stays: root = min */
                else p[a] = b;
              }
            }
      }
  /* components in order of their roots (first cells) */
  int64_t ncomp = 0;
  int64_t* slot = (int64_t*)malloc(sizeof(int64_t) * N);
  for (int64_t c = 0; c < N; ++c) {
    slot[c] = -1;
    if (p[c] >= 0) p[c] = uf_find(p, c);
    if (p[c] == c) slot[c] = ncomp++;
  }
  double* stable = (double*)malloc(sizeof(double) * (ncomp + 1));
  char* has = (char*)calloc(ncomp + 1, 1);
  /* PairToMap over the cells with two halo layers */
  for (int k = -2; k < nz + 2; ++k)
    for (int j = -2; j < ny + 2; ++j)
      for (int i = -2; i < nx + 2; ++i) {
        const int64_t c = XIDX(wrapi(i, nx), wrapi(j, ny), wrapi(k, nz));
        if (p[c] < 0 || cl_prev[c] == -1) continue;
        const int64_t s = slot[p[c]];
        if (!has[s]) {
          has[s] = 1;
          stable[s] = cl_prev[c];
        }
      }
  /* ReduceColor: colours in increasing order of the components' keys */
  double next = 0;
  for (int64_t s = 0; s < ncomp; ++s)
    if (has[s] && stable[s] > next) next = stable[s];
  next += 1;
  double* color = (double*)malloc(sizeof(double) * (ncomp + 1));
  /* used colours: a sorted list is enough for the sizes of the tests */
  double* used = (double*)malloc(sizeof(double) * (ncomp + 1));
  int64_t nused = 0;
  for (int64_t s = 0; s < ncomp; ++s) {
    int taken = 0;
    if (has[s])
      for (int64_t q = 0; q < nused; ++q)
        if (used[q] == stable[s]) taken = 1;
    if (!has[s] || taken) {
      color[s] = next;
      next += 1;
    } else {
      color[s] = stable[s];
    }
    used[nused++] = color[s];
  }
  for (int64_t c = 0; c < N; ++c) cl[c] = p[c] >= 0 ? color[slot[p[c]]] : -1;
  /* propagate */
  double* pre = (double*)malloc(sizeof(double) * N);
  memcpy(pre, cl, sizeof(double) * N);
  for (int d = 0; d < 3; ++d) {
    const int e[3] = {d == 0, d == 1, d == 2};
    for (int k = 0; k < nz + e[2]; ++k)
      for (int j = 0; j < ny + e[1]; ++j)
        for (int i = 0; i < nx + e[0]; ++i) {
          const int w[3] = {i, j, k};
          /* the two cells of the face: c0 = w - e_d, c1 = w; a cell outside
             the block is a halo copy of its periodic image, with the values
             from before the pass, local to this face */
          double clh[2], uh[2];
          int64_t cc[2];
          for (int q = 0; q < 2; ++q) {
            int v[3] = {w[0] - (q == 0 ? e[0] : 0), w[1] - (q == 0 ? e[1] : 0),
                        w[2] - (q == 0 ? e[2] : 0)};
            const int out = v[d] < 0 || v[d] >= n[d];
            for (int a = 0; a < 3; ++a) v[a] = wrapi(v[a], n[a]);
            const int64_t c = XIDX(v[0], v[1], v[2]);
            cc[q] = out ? -1 : c;
            clh[q] = out ? pre[c] : cl[c];
            uh[q] = u[c];
          }
          for (int q = 0; q < 2; ++q) {
            const int o = 1 - q;
            const double clc = cc[q] >= 0 ? cl[cc[q]] : clh[q];
            const double cln = cc[o] >= 0 ? cl[cc[o]] : clh[o];
            if (clc == -1 && uh[q] > 0 && uh[o] > uh[q] && cln != -1) {
              if (cc[q] >= 0) cl[cc[q]] = cln;
              else clh[q] = cln;
            }
          }
        }
  }
  free(pre);
  free(used);
  free(color);
  free(has);
  free(stable);
  free(slot);
  free(p);
}

/* ------------------------------------------------------------------------
 * BCG face predictor of a cell field on a periodic mesh of cubic cells:
 * UEmbed::InterpolateBcg (src/solver/approx_eb.ipp:753-821) without
 * boundary conditions, with UEmbed::Gradient (approx_eb.ipp:882-890).
 * Faces of direction d are stored at the index of their plus cell
 * (between c - e_d and c).  u: cell field; vflux: face volume fluxes;
 * src: cell source (the acceleration component); out: face values.
 * ------------------------------------------------------------------------ */
void orc_interpolate_bcg(const int n[3], double h, const double* u,
                         const double* const vflux[3], const double* src, double dt,
                         double* const out[3]) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const int64_t N = (int64_t)nx * ny * nz;
  const double area = h * h;
  /* face gradients (u(cp) - u(cm)) / h */
  double* g[3];
  for (int d = 0; d < 3; ++d) {
    g[d] = (double*)malloc(sizeof(double) * N);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int64_t c = XIDX(i, j, k);
          const int64_t cm = XIDX(wrapi(i - (d == 0), nx), wrapi(j - (d == 1), ny),
                                  wrapi(k - (d == 2), nz));
          g[d][c] = (u[c] - u[cm]) / h;
        }
  }
  for (int d0 = 0; d0 < 3; ++d0)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int64_t cp = XIDX(i, j, k);
          const int ci[3] = {wrapi(i - (d0 == 0), nx), wrapi(j - (d0 == 1), ny),
                             wrapi(k - (d0 == 2), nz)};
          const int64_t cm = XIDX(ci[0], ci[1], ci[2]);
          const double v = vflux[d0][cp];
          const double sgn = v > 0 ? 1 : -1;
          /* upwind cell and its coordinates */
          const int64_t c = sgn > 0 ? cm : cp;
          const int w[3] = {sgn > 0 ? ci[0] : i, sgn > 0 ? ci[1] : j, sgn > 0 ? ci[2] : k};
          double ut = (src[cm] + src[cp]) * 0.5;
          double ux = 0;
          int d = d0;
          {
            /* faces of the upwind cell in -d (its own index) and +d */
            const int64_t fm = c;
            const int64_t fp = XIDX(wrapi(w[0] + (d == 0), nx), wrapi(w[1] + (d == 1), ny),
                                    wrapi(w[2] + (d == 2), nz));
            ux += (g[d][fm] + g[d][fp]) * 0.5;
            const double vel = v / area;
            ut -= ux * vel;
          }
          for (int t = 0; t < 2; ++t) {
            d = (d + 1) % 3;
            const int64_t fm = c;
            const int64_t fp = XIDX(wrapi(w[0] + (d == 0), nx), wrapi(w[1] + (d == 1), ny),
                                    wrapi(w[2] + (d == 2), nz));
            const double vel = (vflux[d][fm] + vflux[d][fp]) / (area + area);
            ut -= g[d][vel > 0 ? fm : fp] * vel;
          }
          out[d0][cp] = u[c] + ux * (sgn * 0.5 * h) + ut * (0.5 * dt);
        }
  for (int d = 0; d < 3; ++d) free(g[d]);
}

/* ------------------------------------------------------------------------
 * One time step of the projection fluid solver Proj (src/solver/proj.ipp)
 * with the default ProjPar (BCG advection, implicit diffusion, one
 * iteration per step, conjugate solver), periodic, no forces or sources:
 * StartStep (proj.ipp:309-322), MakeIteration (:455-603), FinishStep
 * (:604-613).  State, all in/out: vel (3 blocks of N, the velocity), p
 * (pressure), ppred (pressure of the predictor projection, the next
 * step's guess), flux (3 face blocks, the volume fluxes of the time
 * layer); first: the first step (t = 0: initial pressure, proj.ipp:
 * 111-127).  rho, mu: cell density and dynamic viscosity.  Every linear
 * system is solved by orc_cg_solve (the conjugate solver) to tol.
 * Returns the total CG iteration count.
 * ------------------------------------------------------------------------ */

/* face values (u[cp] + u[cm]) * 0.5 of a cell field (approx_eb.ipp:
 * 828-836) dotted with the face surface (proj.ipp:64-67) */
static void fl_face_flux(const int n[3], double area, const double* vel, double* const out[3]) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const int64_t N = (int64_t)nx * ny * nz;
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int64_t cp = XIDX(i, j, k);
          const int64_t cm = XIDX(wrapi(i - (d == 0), nx), wrapi(j - (d == 1), ny),
                                  wrapi(k - (d == 2), nz));
          double sum = 0;
          for (int e = 0; e < 3; ++e) {
            const double v = (vel[e * N + cp] + vel[e * N + cm]) * 0.5;
            sum += (v - 0.) * (e == d ? area : 0.);
          }
          out[d][cp] = sum;
        }
}

/* Proj::Project (proj.ipp:384-407): assembly, CG from the guess in p,
 * corrected fluxes in place */
static int fl_project(const int n[3], double h, double* const rho_f[3], double* p,
                      double* const ffv[3], double dt, double tol, int maxiter, int nthreads) {
  const int64_t N = (int64_t)n[0] * n[1] * n[2];
  double* e = (double*)malloc(sizeof(double) * 8 * N);
  double* fk[3];
  double* fv[3];
  for (int d = 0; d < 3; ++d) {
    fk[d] = (double*)malloc(sizeof(double) * N);
    fv[d] = (double*)malloc(sizeof(double) * N);
  }
  orc_assemble_projection(n, h, dt, rho_f, ffv, NULL, e, fk, fv);
  const orc_info info = orc_cg_solve(n, h * h * h, e, p, p, tol, 0, maxiter, 0, NULL, nthreads);
  orc_flux_correct(n, fk, fv, p, (double**)ffv);
  for (int d = 0; d < 3; ++d) {
    free(fk[d]);
    free(fv[d]);
  }
  free(e);
  return info.iter;
}

void orc_fluid_init(const int n[3], double h, const double* vel, double* flux[3]) {
  const double V = (h * h) * h;
  fl_face_flux(n, V / h, vel, flux);
}

int orc_fluid_step(const int n[3], double h, double dt, const double* rho, const double* mu,
                   double* vel, double* p, double* ppred, double* flux[3], int first,
                   double tol, int maxiter, int nthreads) {
  const int nx = n[0], ny = n[1], nz = n[2];
  const int64_t N = (int64_t)nx * ny * nz;
  const double V = (h * h) * h;
  const double area = V / h;
  int iters = 0;
  double* rho_f[3];
  double* mu_f[3];
  double* ffv[3];
  double* ffu[3];
  for (int d = 0; d < 3; ++d) {
    rho_f[d] = (double*)malloc(sizeof(double) * N);
    mu_f[d] = (double*)malloc(sizeof(double) * N);
    ffv[d] = (double*)malloc(sizeof(double) * N);
    ffu[d] = (double*)malloc(sizeof(double) * N);
  }
  orc_face_density(n, rho, rho_f);
  for (int d = 0; d < 3; ++d)
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int64_t cp = XIDX(i, j, k);
          const int64_t cm = XIDX(wrapi(i - (d == 0), nx), wrapi(j - (d == 1), ny),
                                  wrapi(k - (d == 2), nz));
          mu_f[d][cp] = (mu[cp] + mu[cm]) * 0.5;
        }
  double* vi = (double*)malloc(sizeof(double) * 3 * N);   /* iteration layer */
  double* acc = (double*)malloc(sizeof(double) * 3 * N);  /* AoS */
  double* accd = (double*)malloc(sizeof(double) * N);
  double* guess = (double*)malloc(sizeof(double) * 3 * N);
  memcpy(vi, vel, sizeof(double) * 3 * N);
  for (int d = 0; d < 3; ++d) memcpy(ffv[d], flux[d], sizeof(double) * N);
  if (first) {
    /* CalcInitialPressure: face velocity of the iteration layer plus the
       (zero) balanced force, projected with dt */
    fl_face_flux(n, area, vi, ffv);
    for (int d = 0; d < 3; ++d)
      for (int64_t c = 0; c < N; ++c) ffv[d][c] += 0. / rho_f[d][c] * dt * area;
    iters += fl_project(n, h, rho_f, p, ffv, dt, tol, maxiter, nthreads);
  }
  orc_acceleration(n, h, p, rho_f, NULL, acc);
  /* predicted fluxes: BCG face velocities of the time layer with its fluxes */
  {
    /* orc_interpolate_bcg writes one face block per direction; the three
       components of the face velocity come from three calls */
    double* comp[3][3];
    for (int e = 0; e < 3; ++e)
      for (int d = 0; d < 3; ++d) comp[e][d] = (double*)malloc(sizeof(double) * N);
    for (int e = 0; e < 3; ++e) {
      for (int64_t c = 0; c < N; ++c) accd[c] = acc[3 * c + e];
      orc_interpolate_bcg(n, h, vel + e * N, (const double* const*)flux, accd, dt, comp[e]);
    }
    for (int d = 0; d < 3; ++d)
      for (int64_t c = 0; c < N; ++c) {
        double sum = 0;
        for (int e = 0; e < 3; ++e) sum += (comp[e][d][c] - 0.) * (e == d ? area : 0.);
        ffv[d][c] = sum;
      }
    for (int e = 0; e < 3; ++e)
      for (int d = 0; d < 3; ++d) free(comp[e][d]);
  }
  iters += fl_project(n, h, rho_f, ppred, ffv, dt * 0.5, tol, maxiter, nthreads);
  /* advection (proj.ipp:128-190): BCG face values with the predicted
     fluxes, flux sum, explicit update from the time layer */
  memcpy(vi, vel, sizeof(double) * 3 * N);
  for (int d = 0; d < 3; ++d) {
    for (int64_t c = 0; c < N; ++c) accd[c] = acc[3 * c + d];
    orc_interpolate_bcg(n, h, vi + d * N, (const double* const*)ffv, accd, dt, ffu);
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          const int64_t c = XIDX(i, j, k);
          double sum = 0;
          for (int q = 0; q < 6; ++q) {
            const int dd = q / 2;
            const int64_t f = (q % 2 == 0)
                                  ? c
                                  : XIDX(wrapi(i + (dd == 0), nx), wrapi(j + (dd == 1), ny),
                                         wrapi(k + (dd == 2), nz));
            const double fl = -ffu[dd][f] * ffv[dd][f];
            sum += fl * (double)(-1 + (q % 2) * 2);
          }
          vi[d * N + c] = vel[d * N + c] + sum * dt / V;
        }
  }
  for (int d = 0; d < 3; ++d)
    for (int64_t c = 0; c < N; ++c) vi[d * N + c] += acc[3 * c + d] * dt;
  /* implicit diffusion (proj.ipp:241-307), guess = velocity after
     advection, one iteration */
  memcpy(guess, vi, sizeof(double) * 3 * N);
  {
    double* e = (double*)malloc(sizeof(double) * 8 * N);
    double* x = (double*)malloc(sizeof(double) * N);
    const double a = 1 / h;
    for (int d = 0; d < 3; ++d) {
      const double* g = guess + d * N;
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            const int64_t c = XIDX(i, j, k);
            double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (int q = 0; q < 6; ++q) {
              const int dd = q / 2;
              const int64_t f = (q % 2 == 0)
                                    ? c
                                    : XIDX(wrapi(i + (dd == 0), nx), wrapi(j + (dd == 1), ny),
                                           wrapi(k + (dd == 2), nz));
              const int64_t fcm =
                  (q % 2 == 0) ? XIDX(wrapi(i - (dd == 0), nx), wrapi(j - (dd == 1), ny),
                                      wrapi(k - (dd == 2), nz))
                               : c;
              const int64_t fcp = f;
              /* GradientImplicit(fcu, ...) (approx_eb.ipp:1471-1480) */
              double fe[3] = {-a, a, 0};
              const double grad = (g[fcp] - g[fcm]) / h;
              const double ev = g[fcm] * fe[0] + g[fcp] * fe[1] + fe[2];
              fe[2] += grad - ev;
              const double o = (double)(-1 + (q % 2) * 2);
              double v[3];
              for (int t = 0; t < 3; ++t) v[t] = fe[t] * mu_f[dd][f] * area * o;
              s[0] += v[1 - q % 2];
              s[1 + q] += v[q % 2];
              s[7] += v[2];
            }
            double* ec = e + 8 * c;
            for (int t = 0; t < 8; ++t) ec[t] = -s[t];
            double td[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            td[0] = 1 / dt;
            td[7] = -vi[d * N + c] / dt;
            for (int t = 0; t < 8; ++t) ec[t] += td[t] * V * rho[c];
          }
      iters += orc_cg_solve(n, V, e, g, x, tol, 0, maxiter, 0, NULL, nthreads).iter;
      memcpy(vi + d * N, x, sizeof(double) * N);
    }
    free(x);
    free(e);
  }
  /* face acceleration: remove the old acceleration, face fluxes, project */
  for (int d = 0; d < 3; ++d)
    for (int64_t c = 0; c < N; ++c) vi[d * N + c] -= acc[3 * c + d] * dt;
  fl_face_flux(n, area, vi, ffv);
  for (int d = 0; d < 3; ++d)
    for (int64_t c = 0; c < N; ++c) ffv[d][c] += 0. / rho_f[d][c] * dt * area;
  iters += fl_project(n, h, rho_f, p, ffv, dt, tol, maxiter, nthreads);
  /* cell acceleration */
  orc_acceleration(n, h, p, rho_f, NULL, acc);
  for (int d = 0; d < 3; ++d)
    for (int64_t c = 0; c < N; ++c) vi[d * N + c] += acc[3 * c + d] * dt;
  /* FinishStep: the iteration layer becomes the time layer */
  memcpy(vel, vi, sizeof(double) * 3 * N);
  for (int d = 0; d < 3; ++d) memcpy(flux[d], ffv[d], sizeof(double) * N);
  free(guess);
  free(accd);
  free(acc);
  free(vi);
  for (int d = 0; d < 3; ++d) {
    free(rho_f[d]);
    free(mu_f[d]);
    free(ffv[d]);
    free(ffu[d]);
  }
  return iters;
}

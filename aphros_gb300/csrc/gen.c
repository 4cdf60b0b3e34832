/*
 * Synthetic workload generator for the projection-step hot path: bubble
 * fields and predicted face fluxes of the configurations the library is
 * benchmarked and tested on.  Host code, shared by the tests, the benchmark
 * and the serving demo so that the GPU path and the CPU oracle always see
 * identical inputs.  Not part of the drop-in C ABI.
 *
 * Volume fractions: exact sphere/cell overlap volume, in the role of
 * aphros's `GetSphereOverlap` (overlap/overlap.cpp:12-41, used by
 * func/init.ipp:72-84).  Our own method: the overlap volume is the integral
 * over z of the area of the disc rho(z)=sqrt(R^2-z^2) intersected with the
 * cell's xy rectangle.  The area has a closed form by inclusion-exclusion
 * over quadrant areas of the disc; the z integral is split at the radii
 * where the disc touches a rectangle edge line or corner, and each piece is
 * integrated with 20-point Gauss-Legendre after the substitution
 * z = a + (b-a)*(3t^2-2t^3), which smooths the (z-z0)^{1/2} and
 * (z-z0)^{3/2} endpoint behaviour.  Accuracy is ~1e-13 of the cell volume.
 *
 * Face fluxes: u* = Taylor-Green field sampled at face centres plus i.i.d.
 * Gaussian noise of standard deviation `noise` per face, drawn from a
 * counter-based generator (splitmix64 of seed and face number, Box-Muller),
 * multiplied by the face area (flux = u*.S).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------- counter-based random numbers ---------------- */

static inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
/* uniform in (0,1], 53 bits */
static inline double u01(uint64_t key, uint64_t ctr) {
  const uint64_t r = splitmix64(splitmix64(key) ^ splitmix64(ctr * 2 + 1));
  return ((r >> 11) + 1) * (1.0 / 9007199254740992.0);
}
static inline double normal01(uint64_t key, uint64_t ctr) {
  const double a = u01(key, 2 * ctr);
  const double b = u01(key, 2 * ctr + 1);
  return sqrt(-2.0 * log(a)) * cos(2.0 * M_PI * b);
}

double aphgen_uniform(uint64_t seed, uint64_t ctr) { return u01(seed, ctr); }
double aphgen_normal(uint64_t seed, uint64_t ctr) { return normal01(seed, ctr); }

/* ---------------- disc / rectangle areas ---------------- */

/* primitive of sqrt(r^2-X^2) */
static inline double prim(double X, double r) {
  if (X >= r) return 0.25 * M_PI * r * r;
  if (X <= -r) return -0.25 * M_PI * r * r;
  return 0.5 * (X * sqrt(r * r - X * X) + r * r * asin(X / r));
}
/* area of disc(r) with Y >= t */
static inline double cap(double t, double r) {
  if (t >= r) return 0;
  if (t <= -r) return M_PI * r * r;
  return 2.0 * (prim(r, r) - prim(t, r));
}
/* area of disc(r) with X >= x, Y >= y for x,y >= 0 */
static inline double corner(double x, double y, double r) {
  if (x * x + y * y >= r * r) return 0;
  const double X1 = sqrt(r * r - y * y);
  return prim(X1, r) - prim(x, r) - y * (X1 - x);
}
/* area of disc(r) with X >= x, Y >= y, any signs */
static inline double quad(double x, double y, double r) {
  if (x >= 0 && y >= 0) return corner(x, y, r);
  if (x < 0 && y >= 0) return cap(y, r) - corner(-x, y, r);
  if (x >= 0 && y < 0) return cap(x, r) - corner(x, -y, r);
  return M_PI * r * r - cap(-x, r) - cap(-y, r) + corner(-x, -y, r);
}
static inline double clampd(double v, double lo, double hi) {
  return v < lo ? lo : (v > hi ? hi : v);
}
static double disc_rect(double x0, double x1, double y0, double y1, double r) {
  if (r <= 0) return 0;
  x0 = clampd(x0, -r, r);
  x1 = clampd(x1, -r, r);
  y0 = clampd(y0, -r, r);
  y1 = clampd(y1, -r, r);
  if (x1 <= x0 || y1 <= y0) return 0;
  const double a =
      quad(x0, y0, r) - quad(x1, y0, r) - quad(x0, y1, r) + quad(x1, y1, r);
  return a > 0 ? a : 0;
}

/* ---------------- Gauss-Legendre nodes ---------------- */

#define GLN 20
static double gl_x[GLN], gl_w[GLN];
static int gl_ready = 0;

static void gl_init(void) {
  if (gl_ready) return;
  for (int i = 0; i < GLN; ++i) {
    double x = cos(M_PI * (i + 0.75) / (GLN + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = x;
      for (int k = 2; k <= GLN; ++k) {
        const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      const double dp = GLN * (x * p1 - p0) / (x * x - 1);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) {
        gl_w[i] = 2 / ((1 - x * x) * dp * dp);
        break;
      }
      gl_w[i] = 2 / ((1 - x * x) * dp * dp);
    }
    gl_x[i] = x;
  }
  gl_ready = 1;
}

static int cmpd(const void* a, const void* b) {
  const double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* Volume of the box [x0,x1]x[y0,y1]x[z0,z1] inside the sphere of radius R
 * centred at the origin. */
double aphgen_box_sphere(
    double x0, double x1, double y0, double y1, double z0, double z1,
    double R) {
  /* quick classification */
  double dn = 0, df = 0;
  const double lo[3] = {x0, y0, z0}, hi[3] = {x1, y1, z1};
  for (int d = 0; d < 3; ++d) {
    const double c = clampd(0, lo[d], hi[d]);
    dn += c * c;
    const double m = fmax(lo[d] * lo[d], hi[d] * hi[d]);
    df += m;
  }
  const double vol = (x1 - x0) * (y1 - y0) * (z1 - z0);
  if (dn >= R * R) return 0;
  if (df <= R * R) return vol;
  gl_init();
  const double za = fmax(z0, -R), zb = fmin(z1, R);
  if (zb <= za) return 0;
  /* breakpoints: rho(z) = |x_i|, |y_j|, sqrt(x_i^2+y_j^2) */
  double bp[32];
  int nb = 0;
  bp[nb++] = za;
  bp[nb++] = zb;
  const double xs[2] = {x0, x1}, ys[2] = {y0, y1};
  double d2[8];
  int nd = 0;
  for (int i = 0; i < 2; ++i) d2[nd++] = xs[i] * xs[i];
  for (int i = 0; i < 2; ++i) d2[nd++] = ys[i] * ys[i];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) d2[nd++] = xs[i] * xs[i] + ys[j] * ys[j];
  for (int i = 0; i < nd; ++i) {
    if (d2[i] < R * R) {
      const double z = sqrt(R * R - d2[i]);
      if (z > za && z < zb) bp[nb++] = z;
      if (-z > za && -z < zb) bp[nb++] = -z;
    }
  }
  if (0 > za && 0 < zb) bp[nb++] = 0;
  qsort(bp, nb, sizeof(double), cmpd);
  double s = 0;
  for (int b = 0; b + 1 < nb; ++b) {
    const double a = bp[b], L = bp[b + 1] - bp[b];
    if (L <= 0) continue;
    double part = 0;
    for (int g = 0; g < GLN; ++g) {
      const double t = 0.5 * (gl_x[g] + 1);
      const double zt = a + L * t * t * (3 - 2 * t);
      const double jac = L * 6 * t * (1 - t);
      const double rr = R * R - zt * zt;
      const double rho = rr > 0 ? sqrt(rr) : 0;
      part += gl_w[g] * 0.5 * jac * disc_rect(x0, x1, y0, y1, rho);
    }
    s += part;
  }
  if (s < 0) s = 0;
  if (s > vol) s = vol;
  return s;
}

/* Adds the gas volume fraction of `ns` spheres (centres c[3*s], radii r[s],
 * in a periodic box of nx*ny*nz cells of size h) to alpha, then clips alpha
 * to [0,1].  Periodic images are taken into account. */
void aphgen_alpha_spheres(
    int nx, int ny, int nz, double h, int ns, const double* c, const double* r,
    double* alpha) {
  const int n[3] = {nx, ny, nz};
  const double cellvol = h * h * h;
  gl_init();
  for (int s = 0; s < ns; ++s) {
    const double R = r[s];
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = (int)floor((c[3 * s + d] - R) / h) - 1;
      hi[d] = (int)floor((c[3 * s + d] + R) / h) + 1;
      if (hi[d] - lo[d] + 1 > n[d]) { /* sphere wider than box: clamp */
        lo[d] = (int)floor(c[3 * s + d] / h) - n[d] / 2;
        hi[d] = lo[d] + n[d] - 1;
      }
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const double x0 = i * h - c[3 * s + 0], x1 = (i + 1) * h - c[3 * s + 0];
          const double y0 = j * h - c[3 * s + 1], y1 = (j + 1) * h - c[3 * s + 1];
          const double z0 = k * h - c[3 * s + 2], z1 = (k + 1) * h - c[3 * s + 2];
          const double v = aphgen_box_sphere(x0, x1, y0, y1, z0, z1, R);
          if (v <= 0) continue;
          const int ii = ((i % nx) + nx) % nx;
          const int jj = ((j % ny) + ny) % ny;
          const int kk = ((k % nz) + nz) % nz;
          const int64_t idx = ii + (int64_t)nx * (jj + (int64_t)ny * kk);
          const double add = (v >= cellvol) ? 1.0 : v / cellvol;
          alpha[idx] += add;
        }
  }
  const int64_t nc = (int64_t)nx * ny * nz;
#pragma omp parallel for
  for (int64_t i = 0; i < nc; ++i) {
    if (alpha[i] > 1) alpha[i] = 1;
    if (alpha[i] < 0) alpha[i] = 0;
  }
}

/* Seeded non-overlapping sphere placement in the unit periodic cube:
 * radii uniform in [rmin,rmax], centres uniform, rejected when closer than
 * r1+r2+gap to any accepted sphere (minimum-image distance).  Returns the
 * number placed (<= ns when the box is too crowded after many attempts). */
int aphgen_place_spheres(
    uint64_t seed, int ns, double rmin, double rmax, double gap, double* c,
    double* r) {
  uint64_t ctr = 0;
  int placed = 0;
  for (int attempt = 0; attempt < 200000 && placed < ns; ++attempt) {
    const double rr = rmin + (rmax - rmin) * u01(seed, ctr++);
    double cc[3];
    for (int d = 0; d < 3; ++d) cc[d] = u01(seed, ctr++);
    int ok = 1;
    for (int q = 0; q < placed && ok; ++q) {
      double d2 = 0;
      for (int d = 0; d < 3; ++d) {
        double dd = fabs(cc[d] - c[3 * q + d]);
        if (dd > 0.5) dd = 1 - dd;
        d2 += dd * dd;
      }
      const double lim = rr + r[q] + gap;
      if (d2 < lim * lim) ok = 0;
    }
    if (!ok) continue;
    for (int d = 0; d < 3; ++d) c[3 * placed + d] = cc[d];
    r[placed] = rr;
    ++placed;
  }
  return placed;
}

/* Face fluxes u*.S of the Taylor-Green field (amplitude U) plus Gaussian
 * noise (standard deviation `noise`, seed) in a periodic cube of n^3 cells
 * and size n*h.  flux[d] has nx*ny*nz entries: the face between cell c-e_d
 * and c.  Noise counter of a face = d*ncells + cell index. */
void aphgen_tg_flux(
    int nx, int ny, int nz, double h, double U, double noise, uint64_t seed,
    double* fx, double* fy, double* fz) {
  const int n[3] = {nx, ny, nz};
  const int64_t nc = (int64_t)nx * ny * nz;
  const double Lx = nx * h, Ly = ny * h, Lz = nz * h;
  const double L[3] = {Lx, Ly, Lz};
  /* 1-D tables: s/c at face coordinates (i*h) and cell centres (i+.5)h */
  double* sf[3];
  double* cf[3];
  double* sc[3];
  double* cc[3];
  for (int d = 0; d < 3; ++d) {
    sf[d] = (double*)malloc(sizeof(double) * n[d]);
    cf[d] = (double*)malloc(sizeof(double) * n[d]);
    sc[d] = (double*)malloc(sizeof(double) * n[d]);
    cc[d] = (double*)malloc(sizeof(double) * n[d]);
    for (int i = 0; i < n[d]; ++i) {
      const double xf = 2 * M_PI * (i * h) / L[d];
      const double xc = 2 * M_PI * ((i + 0.5) * h) / L[d];
      sf[d][i] = sin(xf);
      cf[d][i] = cos(xf);
      sc[d][i] = sin(xc);
      cc[d][i] = cos(xc);
    }
  }
  const double area = h * h;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int64_t c = i + (int64_t)nx * (j + (int64_t)ny * k);
        /* x-face at (i h, (j+.5)h, (k+.5)h) */
        const double ux = U * sf[0][i] * cc[1][j] * cc[2][k];
        /* y-face at ((i+.5)h, j h, (k+.5)h) */
        const double vy = -U * cc[0][i] * sf[1][j] * cc[2][k];
        double nxv = 0, nyv = 0, nzv = 0;
        if (noise > 0) {
          nxv = noise * normal01(seed, (uint64_t)(0 * nc + c));
          nyv = noise * normal01(seed, (uint64_t)(1 * nc + c));
          nzv = noise * normal01(seed, (uint64_t)(2 * nc + c));
        }
        fx[c] = (ux + nxv) * area;
        fy[c] = (vy + nyv) * area;
        fz[c] = (0.0 + nzv) * area;
      }
  for (int d = 0; d < 3; ++d) {
    free(sf[d]);
    free(cf[d]);
    free(sc[d]);
    free(cc[d]);
  }
}

/* Uniform velocity face fluxes (used by the advection golden case). */
void aphgen_uniform_flux(
    int nx, int ny, int nz, double h, double vx, double vy, double vz,
    double* fx, double* fy, double* fz) {
  const int64_t nc = (int64_t)nx * ny * nz;
  const double area = h * h;
  for (int64_t c = 0; c < nc; ++c) {
    /* Vect::dot with the face surface (S,0,0), (0,S,0), (0,0,S) */
    fx[c] = ((0 + vx * area) + vy * 0.) + vz * 0.;
    fy[c] = ((0 + vx * 0.) + vy * area) + vz * 0.;
    fz[c] = ((0 + vx * 0.) + vy * 0.) + vz * area;
  }
}

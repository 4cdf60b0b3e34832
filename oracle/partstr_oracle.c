/* Particle-string curvature of aphros -- C restatement (TEST INFRASTRUCTURE:
 * the checker of the device kernel, never part of the product path).
 *
 * curvature::Particles (src/solver/curv.ipp:29-54) with PartStrMeshM
 * (src/solver/partstrmeshm.ipp:36-395) and PartStr (src/solver/partstr.h:
 * 57-646), one layer, periodic domain without embedded boundaries or contact
 * angles, dim 3.  Every expression keeps the reference's association order
 * (generic::Vect sums start from 0, src/geom/vect.h:255-380; Reconst
 * helpers, src/solver/reconst.h:20-130, 486-640, 748-780); compile with
 * -ffp-contract=off.  Pinned against the reference's own Particles
 * estimator through oracle/_ref/ref_harness (tests/test_oracle_pins.py). */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "aphros_oracle.h"

#define PS_MAXNP 31   /* particles per string at most */
#define PS_MAXSEG 125 /* interface segments per string: one per stencil cell */

typedef struct {
  double x, y;
} V2;

static V2 v2(double x, double y) {
  V2 r = {x, y};
  return r;
}
static V2 v2add(V2 a, V2 b) { return v2(a.x + b.x, a.y + b.y); }
static V2 v2sub(V2 a, V2 b) { return v2(a.x - b.x, a.y - b.y); }
static V2 v2mul(V2 a, double k) { return v2(a.x * k, a.y * k); }
static double v2dot(V2 a, V2 b) {
  double s = 0;
  s += a.x * b.x;
  s += a.y * b.y;
  return s;
}
static double v2sqrnorm(V2 a) {
  double s = 0;
  s += a.x * a.x;
  s += a.y * a.y;
  return s;
}
static double v2norm(V2 a) { return sqrt(v2sqrnorm(a)); }
static double v2cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
static double v2norminf(V2 a) {
  double r = 0;
  const double ax = fabs(a.x), ay = fabs(a.y);
  r = r < ax ? ax : r; /* std::max(r, |a_i|) */
  r = r < ay ? ay : r;
  return r;
}
/* rotation by pi/2, by the angle of unit vector e, by minus that angle
 * (partstr.h:418-433) */
static V2 v2rr(V2 x) { return v2(-x.y, x.x); }
static V2 v2re(V2 x, V2 e) { return v2(x.x * e.x - x.y * e.y, x.x * e.y + x.y * e.x); }
static V2 v2rem(V2 x, V2 e) { return v2(x.x * e.x + x.y * e.y, -x.x * e.y + x.y * e.x); }

static double v3dot(const double* a, const double* b) {
  double s = 0;
  s += a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}
static double v3norm(const double* a) { return sqrt(v3dot(a, a)); }
static void v3cross(const double* a, const double* b, double* r) {
  const double r0 = a[1] * b[2] - a[2] * b[1];
  const double r1 = a[2] * b[0] - a[0] * b[2];
  const double r2 = a[0] * b[1] - a[1] * b[0];
  r[0] = r0;
  r[1] = r1;
  r[2] = r2;
}

/* Reconst::GetCutPoly0 for 3D (reconst.h:523-588): polygon of the plane
 * n.x = a cut by the unit cell centred at 0, 0 <= nx <= ny <= nz, a <= 0. */
static int cut_poly0(const double* n, double a, double xx[6][3]) {
  int k = 0;
  const double f = a + 0.5 * (((0 + n[0]) + n[1]) + n[2]);
  const double nx = n[0], ny = n[1], nz = n[2];
#define P(x0, x1, x2)            \
  do {                           \
    xx[k][0] = -0.5 + (x0);      \
    xx[k][1] = -0.5 + (x1);      \
    xx[k][2] = -0.5 + (x2);      \
    ++k;                         \
  } while (0)
  if (f <= 0) {
    P(0., 0., 0.);
    P(0., 0., 0.);
    P(0., 0., 0.);
  } else if (nx >= f) {
    P(f / nx, 0., 0.);
    P(0., f / ny, 0.);
    P(0., 0., f / nz);
  } else if (ny >= f) {
    P(1., 0., (f - nx) / nz);
    P(1., (f - nx) / ny, 0.);
    P(0., f / ny, 0.);
    P(0., 0., f / nz);
  } else if (nz >= f) {
    if (nx + ny >= f) {
      P(1., 0., (f - nx) / nz);
      P(1., (f - nx) / ny, 0.);
      P((f - ny) / nx, 1., 0.);
      P(0., 1., (f - ny) / nz);
      P(0., 0., f / nz);
    } else {
      P(0., 0., f / nz);
      P(1., 0., (f - nx) / nz);
      P(1., 1., (f - nx - ny) / nz);
      P(0., 1., (f - ny) / nz);
    }
  } else {
    P(1., 0., (f - nx) / nz);
    P(1., (f - nx) / ny, 0.);
    P((f - ny) / nx, 1., 0.);
    P(0., 1., (f - ny) / nz);
    P(0., (f - nz) / ny, 1.);
    P((f - nz) / nx, 0., 1.);
  }
#undef P
  return k;
}

/* GetCutPoly2 (reconst.h:600-638): the polygon of the plane (n, a) in the
 * cell of size h centred at 0; Argsort of three values as reconst.h:100-114 */
static int cut_poly2(const double* n0in, double a, const double* h, double xx[6][3]) {
  double n0[3] = {n0in[0] * h[0], n0in[1] * h[1], n0in[2] * h[2]};
  if (a > 0) {
    n0[0] = -n0[0];
    n0[1] = -n0[1];
    n0[2] = -n0[2];
    a = -a;
  }
  const double n[3] = {fabs(n0[0]), fabs(n0[1]), fabs(n0[2])};
  double v[3] = {n[0], n[1], n[2]};
  int r[3] = {0, 1, 2};
#define SWAP(p, q)          \
  do {                      \
    double tv = v[p];       \
    v[p] = v[q];            \
    v[q] = tv;              \
    int tr = r[p];          \
    r[p] = r[q];            \
    r[q] = tr;              \
  } while (0)
  if (v[1] < v[0]) SWAP(0, 1);
  if (v[2] < v[1]) SWAP(1, 2);
  if (v[1] < v[0]) SWAP(0, 1);
#undef SWAP
  const double ns[3] = {n[r[0]], n[r[1]], n[r[2]]};
  const int k = cut_poly0(ns, a, xx);
  for (int q = 0; q < k; ++q) {
    const double t[3] = {xx[q][0], xx[q][1], xx[q][2]};
    for (int d = 0; d < 3; ++d) xx[q][r[d]] = t[d];
    for (int d = 0; d < 3; ++d)
      if (n0[d] < 0.) xx[q][d] *= -1.;
    for (int d = 0; d < 3; ++d) xx[q][d] *= h[d];
  }
  return k;
}

/* Reconst::GetInterPoly (reconst.h:748-765): the first two crossings of
 * the polygon's edges with the plane through xc with normal n */
static int inter_poly(double xx[6][3], int sx, const double* xc, const double* n,
                      double e[2][3]) {
  int j = 0;
  for (int i = 0; i < sx; ++i) {
    const int ip = (i + 1) % sx;
    const double* x0 = xx[i];
    const double* x1 = xx[ip];
    const double d0[3] = {x0[0] - xc[0], x0[1] - xc[1], x0[2] - xc[2]};
    const double d1[3] = {x1[0] - xc[0], x1[1] - xc[1], x1[2] - xc[2]};
    if ((v3dot(n, d0) > 0.) != (v3dot(n, d1) > 0.)) {
      const double a[3] = {xc[0] - x0[0], xc[1] - x0[1], xc[2] - x0[2]};
      const double b[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
      const double l = v3dot(a, n) / v3dot(b, n);
      for (int d = 0; d < 3; ++d) e[j][d] = x0[d] + b[d] * l;
      if (++j == 2) return 1;
    }
  }
  return 0;
}

typedef struct {
  double o[3], ux[3], uy[3];
} Basis;

/* PartStrMeshM::Imp::GetPlaneBasis, dim 3 (partstrmeshm.ipp:166-195) */
static void plane_basis(const double* xc, const double* n, double a, double an,
                        const double* h, Basis* B) {
  const double na[3] = {fabs(n[0]), fabs(n[1]), fabs(n[2])};
  int d = 0;
  for (int i = 1; i < 3; ++i)
    if (na[i] < na[d]) d = i;
  double xd[3] = {0, 0, 0};
  xd[d] = 1.;
  double t0[3], t1[3];
  v3cross(n, xd, t0);
  double nn = v3norm(t0);
  for (int i = 0; i < 3; ++i) t0[i] /= nn;
  v3cross(n, t0, t1);
  nn = v3norm(t1);
  for (int i = 0; i < 3; ++i) t1[i] /= nn;
  const double ca = cos(an), sa = sin(an);
  double t[3];
  for (int i = 0; i < 3; ++i) t[i] = t0[i] * ca + t1[i] * sa;
  nn = v3norm(t);
  for (int i = 0; i < 3; ++i) t[i] /= nn;
  /* origin: cell centre plus the mean of the PLIC polygon */
  double xx[6][3];
  const int k = cut_poly2(n, a, h, xx);
  double c[3] = {0, 0, 0};
  for (int q = 0; q < k; ++q)
    for (int i = 0; i < 3; ++i) c[i] += xx[q][i];
  for (int i = 0; i < 3; ++i) c[i] /= (double)k;
  const double nl = v3norm(n);
  for (int i = 0; i < 3; ++i) {
    B->o[i] = xc[i] + c[i];
    B->ux[i] = t[i];
    B->uy[i] = n[i] / nl;
  }
}

static V2 plane_coords(const double* x, const Basis* B) {
  const double d[3] = {x[0] - B->o[0], x[1] - B->o[1], x[2] - B->o[2]};
  return v2(v3dot(d, B->ux), v3dot(d, B->uy));
}

/* AppendInterface, dim 3 (partstrmeshm.ipp:222-257): the segment of cell
 * (xc, n, a) in the section plane, oriented by the normal. */
static int append_interface(const Basis* B, const double* xc, double a, const double* n,
                            const double* h, V2* seg) {
  double xx[6][3];
  const int k = cut_poly2(n, a, h, xx);
  for (int q = 0; q < k; ++q)
    for (int i = 0; i < 3; ++i) xx[q][i] += xc[i];
  double uz[3];
  v3cross(B->ux, B->uy, uz);
  double e[2][3];
  if (!inter_poly(xx, k, B->o, uz, e)) return 0;
  const double on[3] = {B->o[0] + n[0], B->o[1] + n[1], B->o[2] + n[2]};
  const V2 pn = plane_coords(on, B);
  V2 p0 = plane_coords(e[0], B), p1 = plane_coords(e[1], B);
  if (v2cross(pn, v2sub(p1, p0)) < 0) {
    const V2 t = p0;
    p0 = p1;
    p1 = t;
  }
  seg[0] = p0;
  seg[1] = p1;
  return 1;
}

/* Reconst::GetNearest (reconst.h:65-69) with Clip = max(0, min(1, k)) */
static V2 nearest(V2 x, V2 x0, V2 x1) {
  const V2 l = v2sub(x1, x0);
  const double k = v2dot(l, v2sub(x, x0)) / v2sqrnorm(l);
  const double m = k < 1. ? k : 1.;  /* std::min(1, k) */
  const double c = 0. < m ? m : 0.;  /* std::max(0, m) */
  return v2add(x0, v2mul(l, c));
}

/* PartStr::PartK (partstr.h:258-275) */
static double part_k(const V2* xx, int sx) {
  const int i = (sx - 1) / 2;
  const V2 dm = v2sub(xx[i], xx[i - 1]);
  const V2 dp = v2sub(xx[i + 1], xx[i]);
  const double lm = v2norm(dm), lp = v2norm(dp);
  const double lmp = lm * lp;
  double k = sqrt(2. * (lmp - v2dot(dm, dp))) / lmp;
  if (v2cross(dm, dp) > 0.) k = -k;
  return k;
}

/* PartStr::SegCirc (partstr.h:280-290) */
static double seg_circ(double k, double l, double d) {
  d = l < d ? l : d;
  const double il = 1. / l;
  k = il < k ? il : k;
  const double a1 = 1. - (k * l) * (k * l);
  const double a2 = 1. - (k * d) * (k * d);
  return k * (l * l - d * d) / (sqrt(a1) + sqrt(a2));
}

/* PartStr::InterfaceForce (partstr.h:300-385), all lines of two nodes */
static void interface_force(const V2* xx, int sx, const V2* lx, int nseg, double segcirc,
                            V2* ff) {
  for (int i = 0; i < sx; ++i) ff[i] = v2(0., 0.);
  if (nseg == 0) return;
  const double crv = part_k(xx, sx);
  for (int i = 0; i < sx; ++i) {
    const V2 x = xx[i];
    V2 e0 = v2(0., 0.), e1 = v2(0., 0.);
    double dn = DBL_MAX;
    for (int l = 0; l < nseg; ++l) {
      const V2 y = nearest(x, lx[2 * l], lx[2 * l + 1]);
      const double d = v2sqrnorm(v2sub(y, x));
      if (d < dn) {
        dn = d;
        e0 = lx[2 * l];
        e1 = lx[2 * l + 1];
      }
    }
    V2 xn = nearest(x, e0, e1);
    if (segcirc != 0.) {
      V2 nv = v2sub(e1, e0);
      nv = v2(nv.y, -nv.x);
      const double nn = v2norm(nv);
      if (!(nn < 1e-10)) {
        nv = v2(nv.x / nn, nv.y / nn);
        const V2 xc = v2mul(v2add(e0, e1), 0.5);
        const double dc = v2norm(v2sub(xn, xc));
        const double mdc = v2norm(v2sub(xc, e0));
        double s = seg_circ(crv, mdc, dc);
        s *= segcirc;
        xn = v2add(xn, v2mul(nv, s));
      }
    }
    ff[i] = v2add(ff[i], v2sub(xn, x));
  }
}

/* PartStr::ApplyConstraints (partstr.h:395-646) */
static void apply_constraints(const V2* xx, int sx, double relax, int dn, V2* ff) {
  V2 xxn[PS_MAXNP], xa[PS_MAXNP], dd[PS_MAXNP];
  for (int i = 0; i < sx; ++i) ff[i] = v2mul(ff[i], relax);
  for (int i = 0; i < sx; ++i) xxn[i] = xx[i];
  const int ic = (sx - 1) / 2;
  if (dn) {
    V2 dx = v2(0., 0.);
    for (int i = 0; i < sx; ++i) dx = v2add(dx, ff[i]);
    dx = v2(dx.x / (double)sx, dx.y / (double)sx);
    dx.x = 0.;
    for (int i = 0; i < sx; ++i) {
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
    }
  } else {
    V2 dx = v2(0., 0.);
    dx.y += ff[ic].y;
    for (int i = 0; i < sx; ++i) {
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
    }
  }
  /* alpha: rotation of the whole string about the centre */
  {
    xa[ic] = v2(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      int i = ic + q;
      xa[i] = v2add(xa[i - 1], v2rr(v2sub(xxn[i], xxn[i - 1])));
      i = ic - q;
      xa[i] = v2sub(xa[i + 1], v2rr(v2sub(xxn[i + 1], xxn[i])));
    }
    double fa = 0., na = 0.;
    for (int i = 0; i < sx; ++i) {
      fa += v2dot(ff[i], xa[i]);
      na += v2dot(xa[i], xa[i]);
    }
    const double da = fa / na;
    const V2 ea = v2(cos(da), sin(da));
    dd[ic] = v2(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = v2sub(xxn[ic + q], xxn[ic + q - 1]);
      dd[ic - q] = v2sub(xxn[ic - q + 1], xxn[ic - q]);
    }
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = v2re(dd[ic + q], ea);
      dd[ic - q] = v2re(dd[ic - q], ea);
    }
    for (int q = 1; q <= ic; ++q) {
      int i = ic + q;
      V2 dx = v2sub(v2add(xxn[i - 1], dd[i]), xxn[i]);
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
      i = ic - q;
      dx = v2sub(v2sub(xxn[i + 1], dd[i]), xxn[i]);
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
    }
  }
  /* theta: bending, the angle between consecutive segments */
  {
    V2* xt = xa;
    xt[ic] = v2(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      const double w = (double)q - 0.5;
      int i = ic + q;
      xt[i] = v2add(xt[i - 1], v2mul(v2rr(v2sub(xxn[i], xxn[i - 1])), w));
      i = ic - q;
      xt[i] = v2add(xt[i + 1], v2mul(v2rr(v2sub(xxn[i + 1], xxn[i])), w));
    }
    double ft = 0., nt = 0.;
    for (int i = 0; i < sx; ++i) {
      ft += v2dot(ff[i], xt[i]);
      nt += v2dot(xt[i], xt[i]);
    }
    const double dt = ft / nt;
    const V2 eth = v2(cos(dt), sin(dt));
    const V2 et = v2re(eth, eth);
    dd[ic] = v2(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = v2sub(xxn[ic + q], xxn[ic + q - 1]);
      dd[ic - q] = v2sub(xxn[ic - q + 1], xxn[ic - q]);
    }
    V2 e = eth;
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = v2re(dd[ic + q], e);
      dd[ic - q] = v2rem(dd[ic - q], e);
      e = v2re(e, et);
    }
    for (int q = 1; q <= ic; ++q) {
      int i = ic + q;
      V2 dx = v2sub(v2add(xxn[i - 1], dd[i]), xxn[i]);
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
      i = ic - q;
      dx = v2sub(v2sub(xxn[i + 1], dd[i]), xxn[i]);
      xxn[i] = v2add(xxn[i], dx);
      ff[i] = v2sub(ff[i], dx);
    }
  }
  for (int i = 0; i < sx; ++i) ff[i] = v2sub(xxn[i], xx[i]);
}

/* One string: seed (PartStr::Add, partstr.h:82-92, centre 0, tangent
 * (1, 0)), iterate (Run0 with Iter, partstr.h:110-157), curvature. */
static double run_string(const OrcPartPar* p, double hc, const V2* lx, int nseg,
                         int* iters) {
  V2 xx[PS_MAXNP], ff[PS_MAXNP];
  const int np = p->np;
  const double leq = p->leq * hc / (double)(np - 1);
  for (int i = 0; i < np; ++i) xx[i] = v2(0. + 1. * (((double)i - (np - 1) * 0.5) * leq),
                                         0. + 0. * (((double)i - (np - 1) * 0.5) * leq));
  int it;
  for (it = 0; it < p->itermax; ++it) {
    interface_force(xx, np, lx, nseg, p->segcirc, ff);
    apply_constraints(xx, np, p->relax, p->dn, ff);
    for (int i = 0; i < np; ++i) xx[i] = v2add(xx[i], ff[i]);
    double r = 0.;
    for (int i = 0; i < np; ++i) {
      const double m = v2norminf(ff[i]);
      r = r < m ? m : r;
    }
    r /= hc * p->relax;
    if (r < p->tol) break;
  }
  if (iters) *iters = it;
  return part_k(xx, np);
}

static int64_t pidx(const int n[3], int i, int j, int k) {
  i = ((i % n[0]) + n[0]) % n[0];
  j = ((j % n[1]) + n[1]) % n[1];
  k = ((k % n[2]) + n[2]) % n[2];
  return (int64_t)i + (int64_t)n[0] * ((int64_t)j + (int64_t)n[1] * k);
}

static int interfacial(double u) { return u > 0 && u < 1; }

void orc_part_default(OrcPartPar* p) {
  /* the defaults of deploy/scripts/sim_base.conf (part_*) */
  p->np = 7;
  p->ns = 3;
  p->leq = 4;
  p->relax = 0.5;
  p->tol = 1e-5;
  p->itermax = 20;
  p->segcirc = 0;
  p->dn = 0;
}

int orc_curv_particles(const int n[3], double h, const double* u, const double* nrm,
                       const double* pa, const double* cl, const OrcPartPar* p,
                       double* kappa, int nthreads) {
  if (p->np < 3 || p->np > PS_MAXNP || p->np % 2 == 0 || p->ns < 1) return -1;
  (void)nthreads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const double hv[3] = {h, h, h};
  const double half = h * 0.5;
  const int64_t nc = (int64_t)n[0] * n[1] * n[2];
  for (int64_t c = 0; c < nc; ++c) kappa[c] = NAN;
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const int64_t c = pidx(n, i, j, k);
        if (!interfacial(u[c]) || (cl && cl[c] == -1.)) continue;
        const double xc[3] = {(0. + half) + (double)i * h, (0. + half) + (double)j * h,
                              (0. + half) + (double)k * h};
        V2 lx[2 * PS_MAXSEG];
        double ksum = 0.;
        for (int s = 0; s < p->ns; ++s) {
          const double an = (double)s * M_PI / (double)p->ns;
          Basis B;
          plane_basis(xc, nrm + 3 * c, pa[c], an, hv, &B);
          int nseg = 0;
          /* Stencil5 in the mesh's order: x fastest, offsets -2..2 */
          for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
              for (int dx = -2; dx <= 2; ++dx) {
                const int64_t cn = pidx(n, i + dx, j + dy, k + dz);
                if (!interfacial(u[cn]) || (cl && cl[cn] != cl[c])) continue;
                const double xn[3] = {(0. + half) + (double)(i + dx) * h,
                                      (0. + half) + (double)(j + dy) * h,
                                      (0. + half) + (double)(k + dz) * h};
                if (append_interface(&B, xn, pa[cn], nrm + 3 * cn, hv, lx + 2 * nseg))
                  ++nseg;
              }
          ksum += run_string(p, h, lx, nseg, NULL);
        }
        ksum /= (double)p->ns;
        ksum *= 2.;
        kappa[c] = ksum;
      }
  return 0;
}

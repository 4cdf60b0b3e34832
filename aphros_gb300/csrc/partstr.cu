// Particle-string curvature of the resident volume fraction:
// curvature::Particles (src/solver/curv.ipp:29-54) with PartStrMeshM
// (src/solver/partstrmeshm.ipp:36-395) and PartStr (src/solver/partstr.h:
// 57-646), for one layer of a periodic domain without embedded boundaries
// or contact angles, dim 3, no colours (the single-field Vof hands the
// estimator no colour field, src/solver/vof.ipp:746-749), and the Hybrid
// estimator (curv.ipp:525-560: heights, then particles where the heights
// give no curvature).
//
// One thread per (interfacial cell, string): the section plane at angle
// s*pi/ns through the cell's PLIC centre, the segments where that plane
// cuts the PLIC polygons of the interfacial cells of the 5x5x5 stencil
// (mesh order, x fastest; cell centres unwrapped, data wrapped), a string
// of np particles relaxed by the interface force and the rotation and
// bending constraints until the correction falls below tol (at most itermax
// iterations), then the curvature of its three middle particles; a second
// pass averages the strings of each cell (times 2: two principal
// directions).
//
// Every expression keeps the reference's association order (generic::Vect
// sums start from 0, src/geom/vect.h:255-380), and the file is compiled
// with -fmad=false: the only differences to the reference come from the
// device's cos and sin (section angle, constraint rotations), which are not
// correctly rounded in every case.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace aphgpu {
namespace {

constexpr int kPsMaxNp = 15;    // particles per string at most
constexpr int kPsMaxSeg = 125;  // segments per string: one per stencil cell

struct V2 {
  double x, y;
};
__device__ __forceinline__ V2 Mk(double x, double y) { return V2{x, y}; }
__device__ __forceinline__ V2 Add(V2 a, V2 b) { return Mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V2 Sub(V2 a, V2 b) { return Mk(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ V2 Mul(V2 a, double k) { return Mk(a.x * k, a.y * k); }
__device__ __forceinline__ double Dot(V2 a, V2 b) {
  double s = 0;
  s += a.x * b.x;
  s += a.y * b.y;
  return s;
}
__device__ __forceinline__ double Norm(V2 a) { return sqrt(Dot(a, a)); }
__device__ __forceinline__ double Cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
// rotations by pi/2, by the angle of unit vector e, by minus that angle
__device__ __forceinline__ V2 Rr(V2 x) { return Mk(-x.y, x.x); }
__device__ __forceinline__ V2 Re(V2 x, V2 e) {
  return Mk(x.x * e.x - x.y * e.y, x.x * e.y + x.y * e.x);
}
__device__ __forceinline__ V2 Rem(V2 x, V2 e) {
  return Mk(x.x * e.x + x.y * e.y, -x.x * e.y + x.y * e.x);
}

__device__ __forceinline__ double Dot3(const double* a, const double* b) {
  double s = 0;
  s += a[0] * b[0];
  s += a[1] * b[1];
  s += a[2] * b[2];
  return s;
}
__device__ __forceinline__ double Norm3(const double* a) { return sqrt(Dot3(a, a)); }
__device__ __forceinline__ void Cross3(const double* a, const double* b, double* r) {
  const double r0 = a[1] * b[2] - a[2] * b[1];
  const double r1 = a[2] * b[0] - a[0] * b[2];
  const double r2 = a[0] * b[1] - a[1] * b[0];
  r[0] = r0;
  r[1] = r1;
  r[2] = r2;
}

// Reconst::GetCutPoly0, 3D (reconst.h:523-588): the plane n.x = a cut by
// the unit cell centred at 0, 0 <= nx <= ny <= nz, a <= 0
__device__ int CutPoly0(const double* n, double a, double xx[6][3]) {
  int k = 0;
  const double f = a + 0.5 * (((0 + n[0]) + n[1]) + n[2]);
  const double nx = n[0], ny = n[1], nz = n[2];
  auto P = [&](double x0, double x1, double x2) {
    xx[k][0] = -0.5 + x0;
    xx[k][1] = -0.5 + x1;
    xx[k][2] = -0.5 + x2;
    ++k;
  };
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
  return k;
}

// GetCutPoly2 (reconst.h:600-638): the polygon of plane (n, a) in the cell
// of size h centred at 0 (Argsort of three values as reconst.h:100-114)
__device__ int CutPoly2(const double* nin, double a, double h, double xx[6][3]) {
  double n0[3] = {nin[0] * h, nin[1] * h, nin[2] * h};
  if (a > 0) {
    n0[0] = -n0[0];
    n0[1] = -n0[1];
    n0[2] = -n0[2];
    a = -a;
  }
  const double n[3] = {fabs(n0[0]), fabs(n0[1]), fabs(n0[2])};
  double v0 = n[0], v1 = n[1], v2 = n[2];
  int r0 = 0, r1 = 1, r2 = 2;
  if (v1 < v0) {
    double t = v0; v0 = v1; v1 = t;
    int q = r0; r0 = r1; r1 = q;
  }
  if (v2 < v1) {
    double t = v1; v1 = v2; v2 = t;
    int q = r1; r1 = r2; r2 = q;
  }
  if (v1 < v0) {
    double t = v0; v0 = v1; v1 = t;
    int q = r0; r0 = r1; r1 = q;
  }
  const int r[3] = {r0, r1, r2};
  const double ns[3] = {n[r0], n[r1], n[r2]};
  const int k = CutPoly0(ns, a, xx);
  for (int q = 0; q < k; ++q) {
    const double t[3] = {xx[q][0], xx[q][1], xx[q][2]};
    for (int d = 0; d < 3; ++d) xx[q][r[d]] = t[d];
    for (int d = 0; d < 3; ++d)
      if (n0[d] < 0.) xx[q][d] *= -1.;
    for (int d = 0; d < 3; ++d) xx[q][d] *= h;
  }
  return k;
}

struct Basis {
  double o[3], ux[3], uy[3];
};

// PartStrMeshM::Imp::GetPlaneBasis, dim 3 (partstrmeshm.ipp:166-195)
__device__ void PlaneBasis(const double* xc, const double* n, int k, const double (*xx)[3],
                           double an, Basis& B) {
  const double na[3] = {fabs(n[0]), fabs(n[1]), fabs(n[2])};
  int d = 0;
  if (na[1] < na[d]) d = 1;
  if (na[2] < na[d]) d = 2;
  const double xd[3] = {d == 0 ? 1. : 0., d == 1 ? 1. : 0., d == 2 ? 1. : 0.};
  double t0[3], t1[3];
  Cross3(n, xd, t0);
  double nn = Norm3(t0);
  for (int i = 0; i < 3; ++i) t0[i] /= nn;
  Cross3(n, t0, t1);
  nn = Norm3(t1);
  for (int i = 0; i < 3; ++i) t1[i] /= nn;
  const double ca = cos(an), sa = sin(an);
  double t[3];
  for (int i = 0; i < 3; ++i) t[i] = t0[i] * ca + t1[i] * sa;
  nn = Norm3(t);
  for (int i = 0; i < 3; ++i) t[i] /= nn;
  double c[3] = {0, 0, 0};
  for (int q = 0; q < k; ++q)
    for (int i = 0; i < 3; ++i) c[i] += xx[q][i];
  for (int i = 0; i < 3; ++i) c[i] /= (double)k;
  const double nl = Norm3(n);
  for (int i = 0; i < 3; ++i) {
    B.o[i] = xc[i] + c[i];
    B.ux[i] = t[i];
    B.uy[i] = n[i] / nl;
  }
}

__device__ __forceinline__ V2 PlaneCoords(const double* x, const Basis& B) {
  const double d[3] = {x[0] - B.o[0], x[1] - B.o[1], x[2] - B.o[2]};
  return Mk(Dot3(d, B.ux), Dot3(d, B.uy));
}

// AppendInterface, dim 3 (partstrmeshm.ipp:222-257) with
// Reconst::GetInterPoly (reconst.h:748-765)
// (the cell's polygon xx0, k vertices relative to its centre, made once per
// call by KPartPolys)
__device__ bool AppendInterface(const Basis& B, const double* uz, const double* xc, int k,
                                const double (*xx0)[3], const double* n, V2* seg) {
  double xx[6][3];
  for (int q = 0; q < k; ++q)
    for (int i = 0; i < 3; ++i) xx[q][i] = xx0[q][i] + xc[i];
  double e[2][3];
  int j = 0;
  for (int i = 0; i < k && j < 2; ++i) {
    const int ip = (i + 1) % k;
    const double d0[3] = {xx[i][0] - B.o[0], xx[i][1] - B.o[1], xx[i][2] - B.o[2]};
    const double d1[3] = {xx[ip][0] - B.o[0], xx[ip][1] - B.o[1], xx[ip][2] - B.o[2]};
    if ((Dot3(uz, d0) > 0.) != (Dot3(uz, d1) > 0.)) {
      const double p[3] = {B.o[0] - xx[i][0], B.o[1] - xx[i][1], B.o[2] - xx[i][2]};
      const double q[3] = {xx[ip][0] - xx[i][0], xx[ip][1] - xx[i][1], xx[ip][2] - xx[i][2]};
      const double l = Dot3(p, uz) / Dot3(q, uz);
      for (int dd = 0; dd < 3; ++dd) e[j][dd] = xx[i][dd] + q[dd] * l;
      ++j;
    }
  }
  if (j < 2) return false;
  const double on[3] = {B.o[0] + n[0], B.o[1] + n[1], B.o[2] + n[2]};
  const V2 pn = PlaneCoords(on, B);
  V2 p0 = PlaneCoords(e[0], B), p1 = PlaneCoords(e[1], B);
  if (Cross(pn, Sub(p1, p0)) < 0) {
    const V2 t = p0;
    p0 = p1;
    p1 = t;
  }
  seg[0] = p0;
  seg[1] = p1;
  return true;
}

// Reconst::GetNearest (reconst.h:65-69), Clip as max(0, min(1, k))
__device__ __forceinline__ V2 Nearest(V2 x, V2 x0, V2 x1) {
  const V2 l = Sub(x1, x0);
  const double k = Dot(l, Sub(x, x0)) / Dot(l, l);
  const double m = k < 1. ? k : 1.;
  const double c = 0. < m ? m : 0.;
  return Add(x0, Mul(l, c));
}

// PartStr::PartK (partstr.h:258-275)
__device__ double PartK(const V2* xx, int sx) {
  const int i = (sx - 1) / 2;
  const V2 dm = Sub(xx[i], xx[i - 1]);
  const V2 dp = Sub(xx[i + 1], xx[i]);
  const double lm = Norm(dm), lp = Norm(dp);
  const double lmp = lm * lp;
  double k = sqrt(2. * (lmp - Dot(dm, dp))) / lmp;
  if (Cross(dm, dp) > 0.) k = -k;
  return k;
}

// PartStr::SegCirc (partstr.h:280-290)
__device__ double SegCirc(double k, double l, double d) {
  d = l < d ? l : d;
  const double il = 1. / l;
  k = il < k ? il : k;
  const double a1 = 1. - (k * l) * (k * l);
  const double a2 = 1. - (k * d) * (k * d);
  return k * (l * l - d * d) / (sqrt(a1) + sqrt(a2));
}

// A segment of the interface line: its ends x0, x1, its vector l = x1 - x0
// and l.l, computed once per string with the operations GetNearest performs
// on every call (reconst.h:65-69).
struct Seg {
  V2 x0, x1, l;
  double ll;
};

// GetNearest with the segment's cached vector and squared length
__device__ __forceinline__ V2 NearestSeg(V2 x, const Seg& s) {
  const double k = Dot(s.l, Sub(x, s.x0)) / s.ll;
  const double m = k < 1. ? k : 1.;
  const double c = 0. < m ? m : 0.;
  return Add(s.x0, Mul(s.l, c));
}

// PartStr::InterfaceForce (partstr.h:300-385)
__device__ void InterfaceForce(const V2* xx, int sx, const Seg* sg, int nseg, double segcirc,
                               V2* ff) {
  for (int i = 0; i < sx; ++i) ff[i] = Mk(0., 0.);
  if (nseg == 0) return;
  const double crv = PartK(xx, sx);
  for (int i = 0; i < sx; ++i) {
    const V2 x = xx[i];
    int best = -1;
    double dn = 1.7976931348623157e308;
    for (int l = 0; l < nseg; ++l) {
      const V2 dy = Sub(NearestSeg(x, sg[l]), x);
      const double d = Dot(dy, dy);
      if (d < dn) {
        dn = d;
        best = l;
      }
    }
    // the nearest segment's ends (zero ends when no distance was finite,
    // as the reference's initial pair)
    const V2 e0 = best < 0 ? Mk(0., 0.) : sg[best].x0;
    const V2 e1 = best < 0 ? Mk(0., 0.) : sg[best].x1;
    V2 xn = best < 0 ? Nearest(x, e0, e1) : NearestSeg(x, sg[best]);
    if (segcirc != 0.) {
      V2 nv = Sub(e1, e0);
      nv = Mk(nv.y, -nv.x);
      const double nn = Norm(nv);
      if (!(nn < 1e-10)) {
        nv = Mk(nv.x / nn, nv.y / nn);
        const V2 xc = Mul(Add(e0, e1), 0.5);
        const double dc = Norm(Sub(xn, xc));
        const double mdc = Norm(Sub(xc, e0));
        double s = SegCirc(crv, mdc, dc);
        s *= segcirc;
        xn = Add(xn, Mul(nv, s));
      }
    }
    ff[i] = Add(ff[i], Sub(xn, x));
  }
}

// PartStr::ApplyConstraints (partstr.h:395-646)
__device__ void ApplyConstraints(const V2* xx, int sx, double relax, int dn, V2* ff) {
  V2 xxn[kPsMaxNp], xa[kPsMaxNp], dd[kPsMaxNp];
  for (int i = 0; i < sx; ++i) ff[i] = Mul(ff[i], relax);
  for (int i = 0; i < sx; ++i) xxn[i] = xx[i];
  const int ic = (sx - 1) / 2;
  if (dn) {
    V2 dx = Mk(0., 0.);
    for (int i = 0; i < sx; ++i) dx = Add(dx, ff[i]);
    dx = Mk(dx.x / (double)sx, dx.y / (double)sx);
    dx.x = 0.;
    for (int i = 0; i < sx; ++i) {
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
    }
  } else {
    V2 dx = Mk(0., 0.);
    dx.y += ff[ic].y;
    for (int i = 0; i < sx; ++i) {
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
    }
  }
  {  // alpha: rotation of the string about its centre
    xa[ic] = Mk(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      xa[ic + q] = Add(xa[ic + q - 1], Rr(Sub(xxn[ic + q], xxn[ic + q - 1])));
      xa[ic - q] = Sub(xa[ic - q + 1], Rr(Sub(xxn[ic - q + 1], xxn[ic - q])));
    }
    double fa = 0., na = 0.;
    for (int i = 0; i < sx; ++i) {
      fa += Dot(ff[i], xa[i]);
      na += Dot(xa[i], xa[i]);
    }
    const double da = fa / na;
    double sda, cda;
    sincos(da, &sda, &cda);
    const V2 ea = Mk(cda, sda);
    dd[ic] = Mk(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = Sub(xxn[ic + q], xxn[ic + q - 1]);
      dd[ic - q] = Sub(xxn[ic - q + 1], xxn[ic - q]);
    }
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = Re(dd[ic + q], ea);
      dd[ic - q] = Re(dd[ic - q], ea);
    }
    for (int q = 1; q <= ic; ++q) {
      int i = ic + q;
      V2 dx = Sub(Add(xxn[i - 1], dd[i]), xxn[i]);
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
      i = ic - q;
      dx = Sub(Sub(xxn[i + 1], dd[i]), xxn[i]);
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
    }
  }
  {  // theta: bending, the angle between consecutive segments
    V2* xt = xa;
    xt[ic] = Mk(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      const double w = (double)q - 0.5;
      xt[ic + q] = Add(xt[ic + q - 1], Mul(Rr(Sub(xxn[ic + q], xxn[ic + q - 1])), w));
      xt[ic - q] = Add(xt[ic - q + 1], Mul(Rr(Sub(xxn[ic - q + 1], xxn[ic - q])), w));
    }
    double ft = 0., nt = 0.;
    for (int i = 0; i < sx; ++i) {
      ft += Dot(ff[i], xt[i]);
      nt += Dot(xt[i], xt[i]);
    }
    const double dt = ft / nt;
    double sdt, cdt;
    sincos(dt, &sdt, &cdt);
    const V2 eth = Mk(cdt, sdt);
    const V2 et = Re(eth, eth);
    dd[ic] = Mk(0., 0.);
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = Sub(xxn[ic + q], xxn[ic + q - 1]);
      dd[ic - q] = Sub(xxn[ic - q + 1], xxn[ic - q]);
    }
    V2 e = eth;
    for (int q = 1; q <= ic; ++q) {
      dd[ic + q] = Re(dd[ic + q], e);
      dd[ic - q] = Rem(dd[ic - q], e);
      e = Re(e, et);
    }
    for (int q = 1; q <= ic; ++q) {
      int i = ic + q;
      V2 dx = Sub(Add(xxn[i - 1], dd[i]), xxn[i]);
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
      i = ic - q;
      dx = Sub(Sub(xxn[i + 1], dd[i]), xxn[i]);
      xxn[i] = Add(xxn[i], dx);
      ff[i] = Sub(ff[i], dx);
    }
  }
  for (int i = 0; i < sx; ++i) ff[i] = Sub(xxn[i], xx[i]);
}

__device__ __forceinline__ bool Interfacial(double u) { return u > 0 && u < 1; }
__device__ __forceinline__ int Wrap(int q, int n) {
  if (q < 0) q += n;
  else if (q >= n) q -= n;
  if (q < 0 || q >= n) q = (q % n + n) % n;
  return q;
}

struct PartArgs {
  Dims d;
  double h;
  aphgpu_part_conf p;
};

// The PLIC polygon of each listed cell (GetCutPoly2, relative to the cell's
// centre) and the cell's position in the list: each polygon is cut once
// per call instead of once per string of every cell whose stencil holds it.
__global__ void KPartPolys(PartArgs A, const double* __restrict__ nrm,
                           const double* __restrict__ pa, const int* __restrict__ list,
                           const int* count, double* poly, int* pk, int* pos) {
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = list[t];
    const double nc[3] = {nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]};
    double xx[6][3];
    const int k = CutPoly2(nc, pa[c], A.h, xx);
    for (int q = 0; q < 6; ++q)
      for (int i = 0; i < 3; ++i) poly[(int64_t)t * 18 + 3 * q + i] = q < k ? xx[q][i] : 0.;
    pk[t] = k;
    pos[c] = t;
  }
}

// one string of a listed cell: t = position in the list * ns + string
__global__ void KPartStrings(PartArgs A, const double* __restrict__ u,
                             const double* __restrict__ nrm,
                             const double* __restrict__ kappa, int fill_only,
                             const int* __restrict__ list, const int* count,
                             const double* __restrict__ poly, const int* __restrict__ pk,
                             const int* __restrict__ pos, double* kpart) {
  const int ns = A.p.ns, np = A.p.np;
  const int64_t total = (int64_t)(*count) * ns;
  const Dims d = A.d;
  const double h = A.h, half = h * 0.5;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = t / ns;
    const int s = (int)(t - li * ns);
    const int64_t c = list[li];
    if (fill_only && kappa[c] == kappa[c]) continue;  // defined by the heights
    const int i = (int)(c % d.nx);
    const int j = (int)((c / d.nx) % d.ny);
    const int k = (int)(c / ((int64_t)d.nx * d.ny));
    const double xc[3] = {(0. + half) + (double)i * h, (0. + half) + (double)j * h,
                          (0. + half) + (double)k * h};
    const double an = (double)s * M_PI / (double)ns;
    const double nc[3] = {nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]};
    Basis B;
    PlaneBasis(xc, nc, pk[li], reinterpret_cast<const double(*)[3]>(poly + li * 18), an, B);
    double uz[3];
    Cross3(B.ux, B.uy, uz);
    // the interfacial cells of the 5x5x5 stencil in stencil order (dz, dy,
    // dx), listed first so that the polygon cuts below run once per listed
    // cell of each lane, not once per stencil cell some lane of the warp
    // needs
    unsigned char cand[kPsMaxSeg];
    int ncand = 0;
    for (int q = 0; q < 125; ++q) {
      const int dx = q % 5 - 2, dy = (q / 5) % 5 - 2, dz = q / 25 - 2;
      const int64_t cn = d.idx(Wrap(i + dx, d.nx), Wrap(j + dy, d.ny), Wrap(k + dz, d.nz));
      if (Interfacial(u[cn])) cand[ncand++] = (unsigned char)q;
    }
    Seg sg[kPsMaxSeg];
    int nseg = 0;
    for (int m = 0; m < ncand; ++m) {
      const int q = cand[m];
      const int dx = q % 5 - 2, dy = (q / 5) % 5 - 2, dz = q / 25 - 2;
      const int64_t cn = d.idx(Wrap(i + dx, d.nx), Wrap(j + dy, d.ny), Wrap(k + dz, d.nz));
      const double xn[3] = {(0. + half) + (double)(i + dx) * h,
                            (0. + half) + (double)(j + dy) * h,
                            (0. + half) + (double)(k + dz) * h};
      const double nn[3] = {nrm[3 * cn], nrm[3 * cn + 1], nrm[3 * cn + 2]};
      const int tn = pos[cn];
      V2 e[2];
      if (AppendInterface(B, uz, xn, pk[tn],
                          reinterpret_cast<const double(*)[3]>(poly + (int64_t)tn * 18), nn, e)) {
        Seg& g = sg[nseg++];
        g.x0 = e[0];
        g.x1 = e[1];
        g.l = Sub(e[1], e[0]);
        g.ll = Dot(g.l, g.l);
      }
    }
    // seed (PartStr::Add, partstr.h:82-92: centre 0, tangent (1, 0)) and
    // iterate (Run0 with Iter, partstr.h:110-157)
    V2 xx[kPsMaxNp], ff[kPsMaxNp];
    const double leq = A.p.leq * h / (double)(np - 1);
    for (int q = 0; q < np; ++q) {
      const double sq = ((double)q - (np - 1) * 0.5) * leq;
      xx[q] = Mk(0. + 1. * sq, 0. + 0. * sq);
    }
    for (int it = 0; it < A.p.itermax; ++it) {
      InterfaceForce(xx, np, sg, nseg, A.p.segcirc, ff);
      ApplyConstraints(xx, np, A.p.relax, A.p.dn, ff);
      double r = 0.;
      for (int q = 0; q < np; ++q) {
        xx[q] = Add(xx[q], ff[q]);
        const double ax = fabs(ff[q].x), ay = fabs(ff[q].y);
        r = r < ax ? ax : r;
        r = r < ay ? ay : r;
      }
      r /= h * A.p.relax;
      if (r < A.p.tol) break;
    }
    kpart[t] = PartK(xx, np);
  }
}

// mean over the strings of each listed cell, times 2 (dim 3)
__global__ void KPartAverage(int ns, const int* __restrict__ list, const int* count,
                             const double* __restrict__ kpart, int fill_only, double* kappa) {
  const int n = *count;
  for (int li = blockIdx.x * blockDim.x + threadIdx.x; li < n; li += gridDim.x * blockDim.x) {
    const int64_t c = list[li];
    if (fill_only && kappa[c] == kappa[c]) continue;
    double k = 0.;
    for (int s = 0; s < ns; ++s) k += kpart[(int64_t)li * ns + s];
    k /= (double)ns;
    k *= 2.;
    kappa[c] = k;
  }
}

}  // namespace

int CurvatureParticlesDevice(aphgpu_ctx* ctx, const aphgpu_part_conf& conf, bool hybrid) {
  if (conf.np < 3 || conf.np > kPsMaxNp || conf.np % 2 == 0 || conf.ns < 1 ||
      conf.itermax < 0 || !(conf.relax != 0))
    return SetError(ctx, APHGPU_ERR_ARG,
                    "particles: np odd in [3, %d], ns >= 1, itermax >= 0, relax != 0",
                    kPsMaxNp);
  const int* list = nullptr;
  const int* count = nullptr;
  if (hybrid) {
    APH_TRY(CurvatureDevice(ctx));  // heights; leaves the interface list
  }
  APH_TRY(InterfaceListDevice(ctx, &list, &count));
  int nif = 0;
  APH_CUDA(ctx, cudaMemcpyAsync(&nif, count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (!hybrid) APH_TRY(KFillNanDevice(ctx, ctx->kappa, ctx->N));
  if (nif == 0) return APHGPU_OK;
  const int64_t need = (int64_t)nif * conf.ns;
  if (need > ctx->kpart_cap) {
    if (ctx->kpart) {
      for (size_t i = 0; i < ctx->allocs.size(); ++i) {
        if (ctx->allocs[i] == ctx->kpart) {
          DeviceFree(ctx, ctx->kpart);
          ctx->allocs.erase(ctx->allocs.begin() + i);
          break;
        }
      }
      ctx->kpart = nullptr;
    }
    APH_TRY(Alloc(ctx, &ctx->kpart, need));
    ctx->kpart_cap = need;
  }
  // the polygons of the listed cells (18 doubles each), their vertex
  // counts, and the list position of each listed cell (N entries)
  if (nif > ctx->ppoly_cap) {
    for (void* q : {(void*)ctx->ppoly, (void*)ctx->ppk}) {
      if (!q) continue;
      for (size_t i = 0; i < ctx->allocs.size(); ++i)
        if (ctx->allocs[i] == q) {
          DeviceFree(ctx, q);
          ctx->allocs.erase(ctx->allocs.begin() + i);
          break;
        }
    }
    ctx->ppoly = nullptr;
    ctx->ppk = nullptr;
    APH_TRY(Alloc(ctx, &ctx->ppoly, (int64_t)nif * 18));
    APH_TRY(Alloc(ctx, &ctx->ppk, nif));
    ctx->ppoly_cap = nif;
  }
  if (!ctx->ppos) APH_TRY(Alloc(ctx, &ctx->ppos, ctx->N));
  PartArgs A{ctx->d, ctx->h, conf};
  KPartPolys<<<FlatBlocks(nif), kFlatThreads, 0, ctx->stream>>>(A, ctx->nrm, ctx->pa, list, count,
                                                              ctx->ppoly, ctx->ppk, ctx->ppos);
  APH_LAUNCHED(ctx);
  const int blocks = (int)std::min<int64_t>((need + 127) / 128, 16 * 1024);
  KPartStrings<<<blocks, 128, 0, ctx->stream>>>(A, ctx->u, ctx->nrm, ctx->kappa,
                                                hybrid ? 1 : 0, list, count, ctx->ppoly,
                                                ctx->ppk, ctx->ppos, ctx->kpart);
  APH_LAUNCHED(ctx);
  KPartAverage<<<FlatBlocks(nif), kFlatThreads, 0, ctx->stream>>>(
      conf.ns, list, count, ctx->kpart, hybrid ? 1 : 0, ctx->kappa);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

}  // namespace aphgpu

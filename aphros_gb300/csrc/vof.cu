// PLIC volume-of-fluid advection and height-function curvature on one
// GB300, FP64.
//
// This translation unit is compiled with -fmad=false: every floating-point
// expression keeps the association order of the reference
// (src/solver/reconst.h, vof.ipp, normal.ipp, curv.ipp, util/height.h) and is
// evaluated without fused multiply-adds, so the results agree with the
// reference built for x86-64 up to the last-bit differences of pow/acos/cos
// in the cubic branch of the plane-constant solve.
//
// Per step (Vof::MakeIteration, weymouth scheme, vof.ipp:498-583):
//   KListInterface       fcuu = u < 0.5 ? 0 : 1 (1 byte/cell), list of the
//                        interfacial cells (0 < u < 1)
//   3 x { KSweepFlux     fluid flux v*u(upwind) through the faces of one
//                        direction with a non-interfacial upwind cell
//         KSweepFluxList PLIC fluxes of the faces with a listed upwind cell
//         KSweepUpdate   u += fcuu*ds - dl, clipping; lists the new
//                        interfacial cells
//         KReconstructList } normals (Youngs + height) and plane constants
//                        of the listed cells
// Curvature (Heights::CalcCurvature, curv.ipp:358-414):
//   KHeights             13-cell columns rebuilt from the same two-step and
//                        four-step differences as CalcDiff2/CalcDiff4, then
//                        UHeight::Good, one height per direction
//   KCurvature           height-function curvature of interfacial cells
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace aphgpu {
namespace {

// ---------------------------------------------------------------------------
// PLIC geometry (reconst.h), device restatement
// ---------------------------------------------------------------------------

__device__ __forceinline__ double sqr(double a) { return a * a; }
__device__ __forceinline__ double cube(double a) { return a * a * a; }
// std::min / std::max argument semantics
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// reconst.h:38-49
__device__ double SolveCubic(double a, double b, double c, double d, int k) {
  double p = (3. * a * c - b * b) / (3. * a * a);
  p = smin(p, 0.);
  const double q =
      (2. * cube(b) - 9. * a * b * c + 27. * a * a * d) / (27. * cube(a));
  double r = 3. * q * sqrt(-3. / p) / (2. * p);
  r = smax(-1., smin(1., r));
  const double t =
      2. * sqrt(-p / 3.) * cos(1. / 3. * acos(r) - 2. * M_PI * k / 3.);
  return t - b / (3. * a);
}

__device__ __forceinline__ void Sort3(double v[3]) {
  double t;
  if (v[1] < v[0]) { t = v[0]; v[0] = v[1]; v[1] = t; }
  if (v[2] < v[1]) { t = v[1]; v[1] = v[2]; v[2] = t; }
  if (v[1] < v[0]) { t = v[0]; v[0] = v[1]; v[1] = t; }
}

// reconst.h:140-168.  Each branch forms its numerator and denominator and
// the one division follows the branches, so the lanes of a warp in
// different cases share it (each lane's operations are the reference's).
__device__ double LineU0(const double n[3], double a) {
  const double nx = n[0], ny = n[1], nz = n[2];
  const double f = a + 0.5 * (nx + ny + nz);
  if (f <= 0) return 0;
  double num, den;
  if (nx >= f) {
    num = cube(f);
    den = 6 * nx * ny * nz;
  } else if (ny >= f) {
    num = 3 * sqr(f) - 3 * f * nx + sqr(nx);
    den = 6 * ny * nz;
  } else if (nz >= f) {
    if (nx + ny >= f) {
      num = 3 * sqr(f) - 3 * f * nx + sqr(nx) - smin(1., (f - ny) / nx) * sqr(f - ny);
      den = 6 * ny * nz;
    } else {
      num = 2 * f - nx - ny;
      den = 2 * nz;
    }
  } else {
    num = cube(f) - cube(f - nx) - cube(f - ny) - cube(f - nz);
    den = 6 * nx * ny * nz;
  }
  return num / den;
}

// reconst.h:183-203, n already multiplied by h
__device__ double LineU1(const double n0[3], double a) {
  double n[3] = {fabs(n0[0]), fabs(n0[1]), fabs(n0[2])};
  Sort3(n);
  const double s = ((0 + n[0]) + n[1]) + n[2];
  a = smax(-0.5 * s, smin(0.5 * s, a));
  // one call site for both signs (the lanes of a warp share it)
  const bool neg = a < 0;
  const double r = LineU0(n, neg ? a : -a);
  return neg ? r : 1 - r;
}

__device__ __forceinline__ double LineU(const double n[3], double a, const double h[3]) {
  const double nh[3] = {n[0] * h[0], n[1] * h[1], n[2] * h[2]};
  return LineU1(nh, a);
}

// reconst.h:218-250.  The branches pick the case and, for the three cubic
// cases, the cubic's coefficients; SolveCubic then runs at one call site,
// so the lanes of a warp in different cubic cases share one evaluation (the
// operations of each lane are those of the reference's branch: a = 1 or 2
// as a value gives the same products as the constant).
__device__ double LineA0(const double n[3], double u) {
  const double nx = n[0], ny = n[1], nz = n[2];
  double f = 0;
  double ca = 1., cb = 0, cc = 0, cd = 0;
  bool cubic = false;
  if (6. * ny * nz * u < sqr(nx)) {
    f = pow(6. * nx * ny * nz * u, 1. / 3.);
  } else if (6. * ny * nz * u < 3. * sqr(ny) - 3 * nx * ny + sqr(nx)) {
    f = 0.5 * nx + sqrt(2. * ny * nz * u - sqr(nx) / 12.);
  } else if (nz > nx + ny) {
    if (2. * nz * u < nx + ny) {
      cubic = true;
      cb = -3. * (nx + ny);
      cc = 3. * (sqr(nx) + sqr(ny));
      cd = -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u;
    } else {
      f = nz * u + 0.5 * (nx + ny);
    }
  } else {
    cubic = true;
    if (6. * nx * ny * nz * u < -cube(nz) + 3. * sqr(nz) * (nx + ny) -
                                    3. * nz * (sqr(nx) + sqr(ny)) + cube(nx) +
                                    cube(ny)) {
      cb = -3. * (nx + ny);
      cc = 3. * (sqr(nx) + sqr(ny));
      cd = -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u;
    } else {
      ca = 2.;
      cb = -3. * (nx + ny + nz);
      cc = 3. * (sqr(nx) + sqr(ny) + sqr(nz));
      cd = -(cube(nx) + cube(ny) + cube(nz)) + 6. * nx * ny * nz * u;
    }
  }
  if (cubic) f = SolveCubic(ca, cb, cc, cd, 1);
  return f - 0.5 * (nx + ny + nz);
}

// reconst.h:264-285
__device__ double LineA(const double n0[3], double u, const double h[3]) {
  double n[3] = {fabs(n0[0] * h[0]), fabs(n0[1] * h[1]), fabs(n0[2] * h[2])};
  Sort3(n);
  u = smax(0., smin(1., u));
  // one call site for both halves (the lanes of a warp share it)
  const bool lo = u <= 0.5;
  const double r = LineA0(n, lo ? u : 1 - u);
  return lo ? r : -r;
}

// reconst.h:290-324 and 371-379
__device__ double LineFlux(const double n0[3], double a, const double h[3],
                           double q, double dt, int d) {
  const double s = ((h[0] * h[1]) * h[2]) / h[d];
  double dx = q / s * dt;
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
  const double uu = LineU(n, aa, hh);
  const double vv = (hh[0] * hh[1]) * hh[2];
  double r = uu * vv;
  r = smin(r, LineU(n, a, h) * ((h[0] * h[1]) * h[2]));
  if (q < 0.) r = -r;
  return r / dt;
}

// ---------------------------------------------------------------------------
// Interface normal (normal.ipp:71-133 then 283-312, force_overwrite=false)
// ---------------------------------------------------------------------------

__device__ void NormalCell(const double u3[27], double nout[3]) {
#define Q(dx, dy, dz) u3[((dx) + 1) + 3 * ((dy) + 1) + 9 * ((dz) + 1)]
  double nn[3] = {0, 0, 0};
  bool started[3] = {false, false, false};
#pragma unroll
  for (int dx = -1; dx <= 1; ++dx)
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
      for (int dz = -1; dz <= 1; ++dz) {
        const double q = Q(dx, dy, dz);
        const int o[3] = {dx, dy, dz};
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          if (o[e] == 0) continue;
          const int t1 = o[(e + 1) % 3], t2 = o[(e + 2) % 3];
          const double w = (double)(o[e] * (t1 == 0 ? 2 : 1) * (t2 == 0 ? 2 : 1));
          if (!started[e]) {
            nn[e] = w * q;
            started[e] = true;
          } else {
            nn[e] += w * q;
          }
        }
      }
  {
    const double ms = -(((0 + fabs(nn[0])) + fabs(nn[1])) + fabs(nn[2]));
    nn[0] /= ms;
    nn[1] /= ms;
    nn[2] /= ms;
  }
  double best[3] = {0, 0, 0};
  int bdz = 0;
#pragma unroll
  for (int dz = 0; dz < 3; ++dz) {
    const int dx = (dz + 1) % 3;
    const int dy = (dz + 2) % 3;
    int oz[3] = {0, 0, 0}, ox[3] = {0, 0, 0}, oy[3] = {0, 0, 0};
    oz[dz] = 1;
    ox[dx] = 1;
    oy[dy] = 1;
#define HH(s0, s1, s2)                                                   \
  ((Q((s0) - oz[0], (s1) - oz[1], (s2) - oz[2]) + Q((s0), (s1), (s2))) + \
   Q((s0) + oz[0], (s1) + oz[1], (s2) + oz[2]))
    double m[3];
    m[dx] = HH(ox[0], ox[1], ox[2]) - HH(-ox[0], -ox[1], -ox[2]);
    m[dy] = HH(oy[0], oy[1], oy[2]) - HH(-oy[0], -oy[1], -oy[2]);
    m[dz] = (Q(oz[0], oz[1], oz[2]) - Q(-oz[0], -oz[1], -oz[2]) > 0 ? 2 : -2);
#undef HH
    const double ms = -(((0 + fabs(m[0])) + fabs(m[1])) + fabs(m[2]));
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

__device__ __forceinline__ bool IsInterface(double u) { return u > 0 && u < 1; }

// Tests on the bit pattern of a double, exact and free of FP64 instructions
// (FP64 issue is the scarce resource on this GPU): positive doubles order
// like their bits as signed integers, negative ones have negative bits.
__device__ __forceinline__ long long Bits(double v) { return __double_as_longlong(v); }
constexpr long long kOneBits = 0x3FF0000000000000LL;
constexpr long long kHalfBits = 0x3FE0000000000000LL;
constexpr long long kInfBits = 0x7FF0000000000000LL;
// 0 < v < 1 (false for NaN)
__device__ __forceinline__ bool InterfaceBits(long long b) { return b > 0 && b < kOneBits; }
// v > 0 (false for NaN)
__device__ __forceinline__ bool PositiveBits(long long b) { return b > 0 && b <= kInfBits; }
__device__ __forceinline__ bool NanBits(long long b) {
  return (b & 0x7FFFFFFFFFFFFFFFLL) > kInfBits;
}
// biased exponent (0x7FF for inf and NaN)
__device__ __forceinline__ int ExpBits(long long b) { return (int)((b >> 52) & 0x7FF); }

#define VOF_CELL_LOOP(dims)                                      \
  const int i = blockIdx.x * kTileX + threadIdx.x;               \
  const int j = blockIdx.y * kTileY + threadIdx.y;               \
  const int kb = blockIdx.z * kTileZ;                            \
  const int ke = min(kb + kTileZ, (dims).nz);                    \
  if (i >= (dims).nx || j >= (dims).ny) return;                  \
  for (int k = kb; k < ke; ++k) {                                \
    const int64_t c = (dims).idx(i, j, k);

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Interface-cell lists.  Only cells with 0 < u < 1 need the plane
// reconstruction and the geometric fluxes; scattered over the grid they would
// leave most lanes of a warp idle in the long FP64 branches, so they are
// gathered into a list (warp-aggregated appends, order irrelevant: every
// list entry is processed independently) and processed densely by
// grid-stride kernels that read the list length on the device.

// Appends c to the list when `want`; every lane of the warp must call it.
__device__ __forceinline__ void ListAppend(bool want, int c, int* list, int* count) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = (threadIdx.x + blockDim.x * threadIdx.y) & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (want) list[base + __popc(m & ((1u << lane) - 1u))] = c;
}

__device__ __forceinline__ void CellIJK(const Dims& d, int64_t c, int& i, int& j, int& k) {
  i = (int)(c % d.nx);
  const int64_t r = c / d.nx;
  j = (int)(r % d.ny);
  k = (int)(r / d.ny);
}

// Lists the interfacial cells of u and, when fcuu != NULL, sets
// fcuu = u < 0.5 ? 0 : 1 (vof.ipp:516-519), 1 byte per cell.
__global__ void KListInterface(Dims d, const double* __restrict__ u, uint8_t* fcuu,
                               int* list, int* count) {
  const int i = blockIdx.x * kTileX + threadIdx.x;
  const int j = blockIdx.y * kTileY + threadIdx.y;
  const int kb = blockIdx.z * kTileZ;
  const int ke = min(kb + kTileZ, d.nz);
  const bool in = i < d.nx && j < d.ny;
  for (int k = kb; k < ke; ++k) {
    const int64_t c = in ? d.idx(i, j, k) : 0;
    const long long ub = in ? Bits(u[c]) : 0;
    // u < 0.5 <=> bits below those of 0.5, NaN excluded
    if (in && fcuu) fcuu[c] = (!NanBits(ub) && ub < kHalfBits) ? 0 : 1;
    ListAppend(in && InterfaceBits(ub), (int)c, list, count);
  }
}

// Init stage of Vof::MakeIteration with a volume source (vof.ipp:504-514):
// u = u + dt * src * (1 - u) in every cell and fcuu of that field, and the
// list of the interfacial cells of that field.  A listed cell that was not
// interfacial before has no plane from the previous reconstruction: its
// normal is zeroed, so its faces carry v*u (InterfaceFlux), as the
// reference's NaN normal does (vof.ipp:233-255); cells interfacial before
// keep their previous planes, as in the reference's first sweep.
__global__ void KSourceList(Dims d, double dt, const double* __restrict__ src, double* u,
                            uint8_t* fcuu, double* nrm, int* list, int* count) {
  const int i = blockIdx.x * kTileX + threadIdx.x;
  const int j = blockIdx.y * kTileY + threadIdx.y;
  const int kb = blockIdx.z * kTileZ;
  const int ke = min(kb + kTileZ, d.nz);
  const bool in = i < d.nx && j < d.ny;
  for (int k = kb; k < ke; ++k) {
    const int64_t c = in ? d.idx(i, j, k) : 0;
    bool want = false;
    if (in) {
      const double um = u[c];
      const double un = um + dt * src[c] * (1. - um);
      u[c] = un;
      const long long ub = Bits(un);
      fcuu[c] = (!NanBits(ub) && ub < kHalfBits) ? 0 : 1;
      want = InterfaceBits(ub);
      if (want && !InterfaceBits(Bits(um))) {
        nrm[3 * c] = 0.;
        nrm[3 * c + 1] = 0.;
        nrm[3 * c + 2] = 0.;
      }
    }
    ListAppend(want, (int)c, list, count);
  }
}

// Vof::ReconstPlanes (vof.ipp:70-90) on the listed interfacial cells;
// values of other cells are left untouched (they are never read).
__global__ void KReconstructList(Dims d, double hx, double hy, double hz,
                                 const double* __restrict__ u, double* nrm, double* pa,
                                 const int* __restrict__ list, const int* count) {
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = list[t];
    int i, j, k;
    CellIJK(d, c, i, j, k);
    const double uc = u[c];
    double u3[27];
#pragma unroll
    for (int dz = -1; dz <= 1; ++dz) {
      const int kk = wrapi(k + dz, d.nz);
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy) {
        const int jj = wrapi(j + dy, d.ny);
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          const int ii = wrapi(i + dx, d.nx);
          u3[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] = u[d.idx(ii, jj, kk)];
        }
      }
    }
    double nv[3];
    NormalCell(u3, nv);
    const double h[3] = {hx, hy, hz};
    nrm[3 * c + 0] = nv[0];
    nrm[3 * c + 1] = nv[1];
    nrm[3 * c + 2] = nv[2];
    pa[c] = LineA(nv, uc, h);
  }
}

// v * uu for a face whose upwind value uu is not interfacial; for finite v,
// v * (+0) is the zero with the sign of v and v * 1 is v (no FP64 multiply)
__device__ __forceinline__ double BulkFlux(double v, double uu) {
  const long long vb = Bits(v), ub = Bits(uu);
  const bool fin = ExpBits(vb) != 0x7FF;
  if (fin && ub == 0) return copysign(0.0, v);
  if (fin && ub == kOneBits) return v;
  return v * uu;
}

// Flux of a face with interfacial upwind cell (normal n, plane constant a,
// volume fraction uu): the PLIC flux when the normal is nonzero, else v*uu
__device__ __forceinline__ double InterfaceFlux(const double n[3], double a, double uu,
                                                const double h[3], double v, double dt,
                                                int dir) {
  const double sq = ((0 + sqr(n[0])) + sqr(n[1])) + sqr(n[2]);
  if (sq > 0) return LineFlux(n, a, h, v, dt, dir);
  return v * uu;
}

// The faces of direction dir whose upwind cell is a listed interfacial cell
// c: its lower face (index c) when the flux there is not positive, its upper
// face (index c + e_dir) when the flux there is positive.
__global__ void KSweepFluxList(Dims d, int dir, double hx, double hy, double hz,
                               const double* __restrict__ u,
                               const double* __restrict__ vflux,
                               const double* __restrict__ nrm,
                               const double* __restrict__ pa, double dt, double* ffvu,
                               const int* __restrict__ list, const int* count) {
  const double h[3] = {hx, hy, hz};
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = list[t];
    int i, j, k;
    CellIJK(d, c, i, j, k);
    const int64_t fp = dir == 0 ? d.idx(wrapp(i + 1, d.nx), j, k)
                     : dir == 1 ? d.idx(i, wrapp(j + 1, d.ny), k)
                                : d.idx(i, j, wrapp(k + 1, d.nz));
    const double nv[3] = {nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]};
    const double a = pa[c], uu = u[c];
    const double vl = vflux[c], vu = vflux[fp];
    // the lower face where its flux is not positive, the upper face where
    // its flux is positive; one call site for the first of them (most
    // cells have one), a second only for the cells that have both
    const bool lower = !(vl > 0), upper = vu > 0;
    if (lower || upper)
      ffvu[lower ? c : fp] = InterfaceFlux(nv, a, uu, h, lower ? vl : vu, dt, dir);
    if (lower && upper) ffvu[fp] = InterfaceFlux(nv, a, uu, h, vu, dt, dir);
  }
}

// Update of Vof::Sweep (vof.ipp:287-326), weymouth, with clipping:
//   u += fcuu * ds - dl,  ds = (v+ - v-) dt / vol,  dl = (f+ - f-) dt / vol
// (the reference divides each face flux by 1 + 1e-16, which is 1 in
// double).  The FP64 divisions (slow on this GPU) are skipped where IEEE
// arithmetic makes them unnecessary, with bit-identical results: a zero
// numerator gives a zero of the same sign; fcuu = 0 makes fcuu * ds a zero
// with the sign of ds (finite); fcuu = 1 with equal numerators makes
// ds - dl = +0.  That covers every cell away from the interface.  Where
// the cell volume is a power of two (ivol = 1 / vol, else 0), x * ivol is
// the correctly rounded x / vol itself (both round the same exact value),
// so the remaining divisions become multiplications.
// UpdateCell: one cell (fc = fcuu, uc = u, face fluxes v0 v1 and fluid
// fluxes f0 f1 of its lower and upper face); returns true for a bulk cell
// (u unchanged, w not set), else the new value in w.
__device__ __forceinline__ bool UpdateCell(int fc, double uc, double v0, double v1, double f0,
                                           double f1, double vol, double ivol, double big,
                                           double dt, double clipth, int emax, int full_ok,
                                           double& w) {
  const long long ub = Bits(uc);
  const long long a0 = Bits(v0), a1 = Bits(v1), b0 = Bits(f0), b1 = Bits(f1);
  // magnitudes below 2^(emax-1023): every difference times dt / vol below
  // is finite
  const bool fin =
      ExpBits(a0) < emax && ExpBits(a1) < emax && ExpBits(b0) < emax && ExpBits(b1) < emax;
  // bulk cells, no FP64 instruction: empty (u = +0, fcuu = 0, zero fluid
  // fluxes: u + (0*ds - dl) is +0 and stays +0 when clipped) and full (u =
  // 1, fcuu = 1, fluid fluxes equal to the face fluxes: ds - dl = +0, u
  // stays 1 for clipth <= 1); u is unchanged
  const bool bulk = fin && ((ub == 0 && fc == 0 && ((b0 | b1) << 1) == 0) ||
                            (full_ok && ub == kOneBits && fc == 1 && a0 == b0 && a1 == b1));
  if (bulk) return true;
  const double dsn = (v1 - v0) * dt;
  const double dln = (f1 - f0) * dt;
  const double dl = dln == 0 ? dln : ivol != 0 ? dln * ivol : dln / vol;
  double t;
  if (fc == 0 && fabs(dsn) <= big) {
    t = copysign(0.0, dsn) - dl;
  } else if (fc == 1 && fabs(dsn) <= big && Bits(dsn) == Bits(dln)) {
    t = 0.0;
  } else {
    t = (double)fc * (ivol != 0 ? dsn * ivol : dsn / vol) - dl;
  }
  w = uc;
  w += t;
  if (!(w >= clipth)) {
    w = 0;
  } else if (!(w <= 1 - clipth)) {
    w = 1;
  }
  return false;
}

// One cell of the fused pass: the fluid fluxes of its lower face (index c)
// and upper face (index fp) from the face fluxes v0 v1 and the old values
// um uc up (lower neighbour, cell, upper neighbour), then the update; returns
// the new value in w and whether the cell is interfacial after it.
__device__ __forceinline__ bool FusedCell(int64_t c, int64_t fp, double v0, double v1,
                                          double um, double uc, double up, int fc,
                                          const double* __restrict__ ffvu, double vol,
                                          double ivol, double big, double dt, double clipth,
                                          int emax, int full_ok, double& w) {
  // the cells of a pure region first: with the cell and both neighbours
  // exactly +0 and fcuu 0 (or exactly 1 and fcuu 1) and face fluxes of
  // magnitude below 2^(emax-1023), the fluid fluxes are the zeros (the face
  // fluxes) of BulkFlux and UpdateCell takes its bulk branch: u is unchanged
  // and the cell is not interfacial (fcuu is the step's first value, so it
  // is tested, not implied by u)
  {
    const long long bm = Bits(um), bc = Bits(uc), bp = Bits(up);
    const bool fin = ExpBits(Bits(v0)) < emax && ExpBits(Bits(v1)) < emax;
    if (fin && ((fc == 0 && (bm | bc | bp) == 0) ||
                (full_ok && fc == 1 && bm == kOneBits && bc == kOneBits && bp == kOneBits))) {
      w = uc;
      return false;
    }
  }
  // upwind values of the lower face (c) and the upper face (fp)
  const double u0 = PositiveBits(Bits(v0)) ? um : uc;
  const double u1 = PositiveBits(Bits(v1)) ? uc : up;
  const double f0 = InterfaceBits(Bits(u0)) ? ffvu[c] : BulkFlux(v0, u0);
  const double f1 = InterfaceBits(Bits(u1)) ? ffvu[fp] : BulkFlux(v1, u1);
  if (UpdateCell(fc, uc, v0, v1, f0, f1, vol, ivol, big, dt, clipth, emax, full_ok, w)) {
    w = uc;
    return false;
  }
  return InterfaceBits(Bits(w));
}

// Fluid fluxes and update of one direction of Vof::Sweep (vof.ipp:228-256,
// 287-326) in one pass, out of place.  The flux of a face whose upwind cell
// is not interfacial is v * u(upwind) of the old volume fraction uin
// (BulkFlux: the face flux v / 1. of the reference is v); the faces with an
// interfacial upwind cell are read from ffvu, written before by
// KSweepFluxList.  Every cell of uout is written (bulk cells with their old
// value); cells interfacial after the update are appended to the list.
// Per cell: uin and vflux read once (the neighbours' values come from
// cache), fcuu read, uout written (and, on the step's last sweep, the next
// step's fcuu byte).  DIR is the sweep direction; a thread
// walks the planes of a column with its lower and upper neighbours at fixed
// offsets (periodic wrap at the ends of the column's row, column or plane
// range), so a plane costs additions, not index products.
template <int DIR>
__global__ void __launch_bounds__(256, 5)
    KSweepFused(Dims d, double vol, double ivol, const double* __restrict__ uin,
                            double* __restrict__ uout, const double* __restrict__ vflux,
                            const double* __restrict__ ffvu,
                            const uint8_t* __restrict__ fcuu, double dt, double clipth,
                            int emax, int full_ok, int* list, int* count,
                            uint8_t* __restrict__ fcuu_out) {
  const int i = blockIdx.x * kTileX + threadIdx.x;
  const int j = blockIdx.y * kTileY + threadIdx.y;
  const int kb = blockIdx.z * kTileZ;
  const int ke = min(kb + kTileZ, d.nz);
  const bool in = i < d.nx && j < d.ny;
  const double big = vol * 1e300;
  const int64_t nxy = (int64_t)d.nx * d.ny;
  // offsets of the lower (dm) and upper (dp) neighbour; for DIR 2 they
  // change at the first and last plane only
  int64_t dm, dp;
  if (DIR == 0) {
    dm = i == 0 ? d.nx - 1 : -1;
    dp = i == d.nx - 1 ? -(int64_t)(d.nx - 1) : 1;
  } else if (DIR == 1) {
    dm = j == 0 ? (int64_t)(d.ny - 1) * d.nx : -(int64_t)d.nx;
    dp = j == d.ny - 1 ? -(int64_t)(d.ny - 1) * d.nx : (int64_t)d.nx;
  } else {
    dm = -nxy;
    dp = nxy;
  }
  auto offm = [&](int k) -> int64_t {
    return DIR == 2 && k == 0 ? (int64_t)(d.nz - 1) * nxy : dm;
  };
  auto offp = [&](int k) -> int64_t {
    return DIR == 2 && k == d.nz - 1 ? -(int64_t)(d.nz - 1) * nxy : dp;
  };
  // the loads of plane k+1 are issued before plane k is computed: two
  // planes of loads in flight per thread
  struct Plane {
    double v0, v1, um, uc, up;
    int fc;
  };
  auto load = [&](int64_t c, int k, Plane& q) {
    const int64_t fp = c + offp(k);
    q.v0 = vflux[c];
    q.v1 = vflux[fp];
    q.um = uin[c + offm(k)];
    q.uc = uin[c];
    q.up = uin[fp];
    q.fc = fcuu[c];
  };
  int64_t c = in ? d.idx(i, j, kb) : 0;
  Plane cur{}, nxt{};
  if (in && kb < ke) load(c, kb, cur);
  for (int k = kb; k < ke; ++k) {
    if (in && k + 1 < ke) load(c + nxy, k + 1, nxt);
    bool want = false;
    if (in) {
      double w;
      want = FusedCell(c, c + offp(k), cur.v0, cur.v1, cur.um, cur.uc, cur.up, cur.fc, ffvu,
                       vol, ivol, big, dt, clipth, emax, full_ok, w);
      uout[c] = w;
      if (fcuu_out) {
        // the next step's fcuu = u < 0.5 ? 0 : 1 of the new value, as
        // KListInterface sets it
        const long long wb = Bits(w);
        fcuu_out[c] = (!NanBits(wb) && wb < kHalfBits) ? 0 : 1;
      }
    }
    ListAppend(want, (int)c, list, count);
    cur = nxt;
    c += nxy;
  }
}

// UHeight::Good(uu) (util/height.h:69-124) on 13 values
__device__ double HeightGood(const double uu[13]) {
  const int si = 13, sih = 6;
  if (!IsInterface(uu[sih])) return nan("");
  int im = sih;
  while (im >= 0 && IsInterface(uu[im])) --im;
  if (im < 0) return nan("");
  int ip = sih;
  while (ip < si && IsInterface(uu[ip])) ++ip;
  if (ip >= si) return nan("");
  if (uu[ip] != uu[im]) {
    double s = 0.;
    for (int q = im; q <= ip; ++q) s += uu[q];
    s += (double)im * uu[im] + (double)(si - ip - 1) * uu[ip];
    if (uu[im] == 0) s = si - s;
    s -= si * 0.5;
    return s;
  }
  return nan("");
}

// Index q wrapped into [0, n) (periodic); one correction covers offsets
// smaller than n, the remainder the rest.
__device__ __forceinline__ int WrapAny(int q, int n) {
  if (q < 0) {
    q += n;
    if (q < 0) q = (q % n + n) % n;
  } else if (q >= n) {
    q -= n;
    if (q >= n) q %= n;
  }
  return q;
}

// Linear index of cell (i, j, k) shifted by o along axis A (periodic).
template <int A>
__device__ __forceinline__ int64_t ShiftIdx(const Dims& d, int i, int j, int k, int o) {
  if (A == 0) return d.idx(WrapAny(i + o, d.nx), j, k);
  if (A == 1) return d.idx(i, WrapAny(j + o, d.ny), k);
  return d.idx(i, j, WrapAny(k + o, d.nz));
}

// Height of an interfacial cell along axis A: CalcDiff2/CalcDiff4/
// CalcHeight (curv.ipp:100-254) fused; the 13-cell column is rebuilt
// exactly as CalcHeight does from the two-step differences du2(q) = u(q+2)
// - u(q-2) and the four-step differences du4(q) = du2(q+2) - du2(q-2).
template <int A>
__device__ __forceinline__ double HeightAlong(const Dims& d, double hA, int i, int j, int k,
                                              const double* __restrict__ u) {
  double uc[13];  // u at offsets -6..6 along A
#pragma unroll
  for (int s = -6; s <= 6; ++s) uc[s + 6] = u[ShiftIdx<A>(d, i, j, k, s)];
#define U(s) uc[(s) + 6]
#define DU2(s) ((0 + -1 * U((s)-2)) + 1 * U((s) + 2))
#define DU4(s) ((0 + -1 * DU2((s)-2)) + 1 * DU2((s) + 2))
  double uu[13];
  uu[6] = U(0);
  uu[5] = U(-1);
  uu[7] = U(1);
  uu[4] = U(-2);
  uu[8] = U(2);
  uu[3] = uu[7] - DU2(-1);
  uu[9] = uu[5] + DU2(1);
  uu[2] = uu[6] - DU2(-2);
  uu[10] = uu[6] + DU2(2);
  uu[1] = uu[9] - DU4(-1);
  uu[11] = uu[3] + DU4(1);
  uu[0] = uu[8] - DU4(-2);
  uu[12] = uu[4] + DU4(2);
#undef DU4
#undef DU2
#undef U
  const double off = HeightGood(uu);
  const int wA = A == 0 ? i : A == 1 ? j : k;
  const double center = (0. + hA * 0.5) + (double)wA * hA;
  return center + off * hA;
}

// Heights of the listed interfacial cells (the heights of the other cells
// are never read: the curvature reads the heights of interfacial cells).
__global__ void KHeightsList(Dims d, double hx, double hy, double hz,
                             const double* __restrict__ u, double* hgt,
                             const int* __restrict__ list, const int* count) {
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = list[t];
    int i, j, k;
    CellIJK(d, c, i, j, k);
    hgt[3 * c] = HeightAlong<0>(d, hx, i, j, k, u);
    hgt[3 * c + 1] = HeightAlong<1>(d, hy, i, j, k, u);
    hgt[3 * c + 2] = HeightAlong<2>(d, hz, i, j, k, u);
  }
}

// Height of column (sx, sy) of the 3x3 stencil around (i, j, k) in the
// plane across axis dn (dx = dn+1, dy = dn+2 mod 3): the height of the
// first interfacial cell among the shifts 0, 1, -1, 2, -2 along dn, NaN if
// none (CalcCurvHeight, curv.ipp:261-356).
__device__ __forceinline__ double ColumnHeight(const Dims& d, int i, int j, int k, int dn,
                                               int sx, int sy,
                                               const double* __restrict__ u,
                                               const double* __restrict__ hgt) {
  const int dx = dn == 2 ? 0 : dn + 1, dy = dn == 0 ? 2 : dn - 1;
  const int bi = i + (dx == 0 ? sx : 0) + (dy == 0 ? sy : 0);
  const int bj = j + (dx == 1 ? sx : 0) + (dy == 1 ? sy : 0);
  const int bk = k + (dx == 2 ? sx : 0) + (dy == 2 ? sy : 0);
  const int shifts[5] = {0, 1, -1, 2, -2};
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int o = shifts[t];
    const int64_t cn = d.idx(WrapAny(bi + (dn == 0 ? o : 0), d.nx),
                             WrapAny(bj + (dn == 1 ? o : 0), d.ny),
                             WrapAny(bk + (dn == 2 ? o : 0), d.nz));
    if (IsInterface(u[cn])) return hgt[3 * cn + dn];
  }
  return nan("");
}

// CalcCurvHeight (curv.ipp:261-356) on the listed interfacial cells (kappa
// of the other cells is set to NaN by KFillNan before).
__global__ void KCurvatureList(Dims d, double hx, double hy, double hz,
                               const double* __restrict__ u,
                               const double* __restrict__ nrm,
                               const double* __restrict__ hgt, double* kappa,
                               const int* __restrict__ list, const int* count) {
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = list[t];
    int i, j, k;
    CellIJK(d, c, i, j, k);
    const double n0 = nrm[3 * c], n1 = nrm[3 * c + 1], n2 = nrm[3 * c + 2];
    const double a0 = fabs(n0), a1 = fabs(n1), a2 = fabs(n2);
    int dn = 0;
    double amax = a0;
    if (a1 > amax) {
      dn = 1;
      amax = a1;
    }
    if (a2 > amax) dn = 2;
    const int dx = dn == 2 ? 0 : dn + 1, dy = dn == 0 ? 2 : dn - 1;
    const double lx = dx == 0 ? hx : dx == 1 ? hy : hz;
    const double ly = dy == 0 ? hx : dy == 1 ? hy : hz;
    const double hcc = ColumnHeight(d, i, j, k, dn, 0, 0, u, hgt);
    const double hmc = ColumnHeight(d, i, j, k, dn, -1, 0, u, hgt);
    const double hpc = ColumnHeight(d, i, j, k, dn, 1, 0, u, hgt);
    const double hcm = ColumnHeight(d, i, j, k, dn, 0, -1, u, hgt);
    const double hcp = ColumnHeight(d, i, j, k, dn, 0, 1, u, hgt);
    const double hmm = ColumnHeight(d, i, j, k, dn, -1, -1, u, hgt);
    const double hmp = ColumnHeight(d, i, j, k, dn, -1, 1, u, hgt);
    const double hpm = ColumnHeight(d, i, j, k, dn, 1, -1, u, hgt);
    const double hpp = ColumnHeight(d, i, j, k, dn, 1, 1, u, hgt);
    const double hxd = (hpc - hmc) / (2 * lx);
    const double hyd = (hcp - hcm) / (2 * ly);
    const double fl = 0.2;
    const double hxx = ((hpm - 2 * hcm + hmm) * fl + (hpc - 2 * hcc + hmc) +
                        (hpp - 2 * hcp + hmp) * fl) /
                       ((1 + 2 * fl) * lx * lx);
    const double hyy = ((hmp - 2 * hmc + hmm) * fl + (hcp - 2 * hcc + hcm) +
                        (hpp - 2 * hpc + hpm) * fl) /
                       ((1 + 2 * fl) * ly * ly);
    const double hxy = ((hpp - hmp) - (hpm - hmm)) / (4 * lx * ly);
    double kk = (2 * hxd * hyd * hxy - (sqr(hyd) + 1) * hxx - (sqr(hxd) + 1) * hyy) /
                pow(sqr(hxd) + sqr(hyd) + 1, 3. / 2.);
    const double ndn = dn == 0 ? n0 : dn == 1 ? n1 : n2;
    if (ndn < 0) kk *= -1;
    kappa[c] = kk;
  }
}

__global__ void KFillNan(int64_t n, double* v) {
  const double nanv = __longlong_as_double(0x7FF8000000000000LL);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    v[c] = nanv;
}

// AppendSurfaceTension (util/hydro.ipp:1289-1310) into zeroed face blocks
__global__ void KSurfaceTension(Dims d, double h, double sigma,
                                const double* __restrict__ u,
                                const double* __restrict__ kappa, double* febp) {
  const int64_t N = d.cells();
  VOF_CELL_LOOP(d)
  for (int q = 0; q < 3; ++q) {
    const int64_t cm = q == 0 ? d.idx(wrapm(i - 1, d.nx), j, k)
                     : q == 1 ? d.idx(i, wrapm(j - 1, d.ny), k)
                              : d.idx(i, j, wrapm(k - 1, d.nz));
    const double um = smax(0., smin(1., u[cm] / 1.));
    const double up = smax(0., smin(1., u[c] / 1.));
    const double ga = (up - um) / h;
    double f = 0;
    if (ga != 0.) {
      double kk = (fabs(um - 0.5) < fabs(up - 0.5) ? kappa[cm] : kappa[c]);
      kk = (isnan(kk) ? 0 : kk);
      f = 0 + ga * kk * sigma;
    }
    febp[q * N + c] = f;
  }
  }
}

}  // namespace

namespace {

// Scratch of a VOF step inside the context's u0 array: fcuu (1 byte per
// cell) in two slots, the interface list (4 bytes per cell, room for every
// cell) and its length.
struct VofScratch {
  uint8_t* fcuu;       // fcuu of the current volume fraction
  uint8_t* fcuu_next;  // fcuu of the next step's, written by its last sweep
  int* list;
  int* count;
};

// Two fcuu slots (ctx->fcuu_sel picks the current one), the list and its
// count, in the u0 array of N + 8 doubles: 16-byte aligned pieces of N, 4 N,
// 16 and N bytes.
VofScratch Scratch(aphgpu_ctx* ctx) {
  char* base = (char*)ctx->u0;
  const size_t n = (size_t)ctx->N;
  const size_t off = (n + 15) & ~(size_t)15;
  uint8_t* a = (uint8_t*)base;
  uint8_t* b = (uint8_t*)(base + off + 4 * n + 16);
  uint8_t* cur = ctx->fcuu_sel ? b : a;
  uint8_t* nxt = ctx->fcuu_sel ? a : b;
  return VofScratch{cur, nxt, (int*)(base + off), (int*)(base + off + 4 * n)};
}

// grid of the list kernels: 4 CTAs of 256 threads per SM, looping over the
// list
int ListGrid(aphgpu_ctx* ctx) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
      sms < 1) {
    cudaGetLastError();
    sms = 132;
  }
  return 4 * sms;
}

// interface list (and fcuu when `fcuu`) of the current volume fraction
int ListInterface(aphgpu_ctx* ctx, const VofScratch& sc, bool fcuu) {
  APH_CUDA(ctx, cudaMemsetAsync(sc.count, 0, sizeof(int), ctx->stream));
  KListInterface<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->u, fcuu ? sc.fcuu : nullptr, sc.list, sc.count);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int ReconstructListed(aphgpu_ctx* ctx, const VofScratch& sc) {
  const double h = ctx->h;
  KReconstructList<<<ListGrid(ctx), 256, 0, ctx->stream>>>(ctx->d, h, h, h, ctx->u, ctx->nrm,
                                                            ctx->pa, sc.list, sc.count);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

// fluid fluxes of the faces of direction dir with an interfacial upwind cell
int SweepFluxList(aphgpu_ctx* ctx, const VofScratch& sc, int dir, const double* vf,
                  double dt) {
  const double h = ctx->h;
  KSweepFluxList<<<ListGrid(ctx), 256, 0, ctx->stream>>>(ctx->d, dir, h, h, h, ctx->u, vf,
                                                          ctx->nrm, ctx->pa, dt, ctx->ffvu,
                                                          sc.list, sc.count);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

// the fused flux + update of direction dir from ctx->u into ctx->u_alt,
// then (swap) the two buffers exchanged: ctx->u is the new volume fraction
int SweepUpdate(aphgpu_ctx* ctx, const VofScratch& sc, int dir, const double* vf, double dt,
                bool swap, uint8_t* fcuu_out = nullptr) {
  const double h = ctx->h;
  APH_CUDA(ctx, cudaMemsetAsync(sc.count, 0, sizeof(int), ctx->stream));
  const double vol = (h * h) * h;
  // face values of magnitude below 2^(emax-1023) keep the differences
  // (below 2^(emax-1022)), their products with dt and the quotients by vol
  // below 2^1000: finite on the bulk path
  const double adt = std::fabs(dt);
  const double ratio = adt / vol;
  int emax = 0;
  if (std::isfinite(ratio) && std::isfinite(adt)) {
    double e = 2045.0;
    if (ratio > 0) e = std::min(e, std::floor(2021.0 - std::log2(ratio)));
    if (adt > 1) e = std::min(e, std::floor(2021.0 - std::log2(adt)));
    emax = (int)std::max(0.0, e);
  }
  // 1 / vol where vol is a power of two (and so is its reciprocal), else 0
  int ve = 0;
  const double vm = std::frexp(vol, &ve);
  const double ivol = (vm == 0.5 && std::isnormal(vol) && std::isnormal(std::ldexp(1.0, 1 - ve)))
                          ? std::ldexp(1.0, 1 - ve)
                          : 0.0;
  auto kern = dir == 0 ? KSweepFused<0> : dir == 1 ? KSweepFused<1> : KSweepFused<2>;
  kern<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, vol, ivol, ctx->u, ctx->u_alt, vf, ctx->ffvu, sc.fcuu, dt, ctx->clipth, emax,
      ctx->clipth <= 1 ? 1 : 0, sc.list, sc.count, fcuu_out);
  APH_LAUNCHED(ctx);
  if (swap) std::swap(ctx->u, ctx->u_alt);
  return APHGPU_OK;
}

}  // namespace

int VofReconstruct(aphgpu_ctx* ctx) {
  const VofScratch sc = Scratch(ctx);
  ctx->fcuu_ready = false;  // u was set from outside the steps
  APH_TRY(ListInterface(ctx, sc, false));
  ctx->vof_list_valid = true;
  return ReconstructListed(ctx, sc);
}

int VofStepDevice(aphgpu_ctx* ctx, const double* d_vflux, double dt) {
  const int64_t N = ctx->N;
  const VofScratch sc = Scratch(ctx);
  if (ctx->has_vof_src) {
    ctx->vof_list_valid = false;
    APH_CUDA(ctx, cudaMemsetAsync(sc.count, 0, sizeof(int), ctx->stream));
    KSourceList<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
        ctx->d, dt, ctx->vof_src, ctx->u, sc.fcuu, ctx->nrm, sc.list, sc.count);
    APH_LAUNCHED(ctx);
  } else if (!(ctx->fcuu_ready && ctx->vof_list_valid)) {
    // else the previous step's last sweep left both the list of the
    // interfacial cells and fcuu of the current volume fraction
    ctx->vof_list_valid = false;
    APH_TRY(ListInterface(ctx, sc, true));
  }
  ctx->vof_list_valid = false;
  ctx->fcuu_ready = false;
  int dd[3];
  const int cnt = ctx->vof_count % 3;  // vof.ipp:428-435
  if (cnt == 0) { dd[0] = 0; dd[1] = 1; dd[2] = 2; }
  else if (cnt == 1) { dd[0] = 1; dd[1] = 2; dd[2] = 0; }
  else { dd[0] = 2; dd[1] = 0; dd[2] = 1; }
  for (int id = 0; id < 3; ++id) {
    const int dir = dd[id];
    const double* vf = d_vflux + (int64_t)dir * N;
    APH_TRY(SweepFluxList(ctx, sc, dir, vf, dt));
    APH_TRY(SweepUpdate(ctx, sc, dir, vf, dt, true, id == 2 ? sc.fcuu_next : nullptr));
    APH_TRY(ReconstructListed(ctx, sc));
  }
  ctx->vof_count += 1;
  ctx->vof_dt = dt;
  // the last update listed the interfacial cells of the new u and wrote its
  // fcuu into the other slot
  ctx->vof_list_valid = true;
  ctx->fcuu_sel ^= 1;
  ctx->fcuu_ready = true;
  return APHGPU_OK;
}

namespace {
int HeightsListed(aphgpu_ctx* ctx, const VofScratch& sc) {
  const double h = ctx->h;
  KHeightsList<<<ListGrid(ctx), 256, 0, ctx->stream>>>(ctx->d, h, h, h, ctx->u, ctx->hgt,
                                                        sc.list, sc.count);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}
int CurvatureListed(aphgpu_ctx* ctx, const VofScratch& sc) {
  const double h = ctx->h;
  KFillNan<<<FlatBlocks(ctx->N), kFlatThreads, 0, ctx->stream>>>(ctx->N, ctx->kappa);
  APH_LAUNCHED(ctx);
  KCurvatureList<<<ListGrid(ctx), 256, 0, ctx->stream>>>(
      ctx->d, h, h, h, ctx->u, ctx->nrm, ctx->hgt, ctx->kappa, sc.list, sc.count);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}
}  // namespace

int InterfaceListDevice(aphgpu_ctx* ctx, const int** list, const int** count) {
  const VofScratch sc = Scratch(ctx);
  if (!ctx->vof_list_valid) {
    APH_TRY(ListInterface(ctx, sc, false));
    ctx->vof_list_valid = true;
  }
  *list = sc.list;
  *count = sc.count;
  return APHGPU_OK;
}

int KFillNanDevice(aphgpu_ctx* ctx, double* v, int64_t n) {
  KFillNan<<<FlatBlocks(n), kFlatThreads, 0, ctx->stream>>>(n, v);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

// Heights and curvature of the interfacial cells, from the interface list
// of the current volume fraction (rebuilt when the last VOF call did not
// leave it).
int CurvatureDevice(aphgpu_ctx* ctx) {
  const VofScratch sc = Scratch(ctx);
  if (!ctx->vof_list_valid) {
    APH_TRY(ListInterface(ctx, sc, false));
    ctx->vof_list_valid = true;
  }
  APH_TRY(HeightsListed(ctx, sc));
  return CurvatureListed(ctx, sc);
}

int TimeVofKernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms, double* bytes,
                  const double* d_vflux, double dt) {
  const double N = (double)ctx->N;
  cudaStream_t st = ctx->stream;
  const VofScratch sc = Scratch(ctx);
  // the interface list and fcuu of the current volume fraction (the
  // timed update leaves the list of its scratch output)
  APH_TRY(ListInterface(ctx, sc, true));
  ctx->vof_list_valid = kernel != APHGPU_K_VOF_UPDATE;
  ctx->fcuu_ready = false;
  int nif = 0;
  APH_CUDA(ctx, cudaMemcpyAsync(&nif, sc.count, sizeof(int), cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  double b = 0;
  switch (kernel) {
    // interfacial cells: index, normal, plane constant, u, two faces each way
    case APHGPU_K_VOF_FLUX: b = nif * (4.0 + 24 + 8 + 8 + 32); break;
    // u read and written, flux, fcuu, list entries
    case APHGPU_K_VOF_UPDATE: b = N * (8 + 8 + 8 + 1) + nif * 4.0; break;
    // listed cells: index, u, normal and plane constant written
    case APHGPU_K_RECONSTRUCT: b = nif * (4.0 + 8 + 24 + 8); break;
    // listed cells: index, 39 u values (mostly cached), 3 heights written
    case APHGPU_K_HEIGHTS: b = nif * (4.0 + 8 + 24); break;
    // NaN fill of kappa; listed cells: index, normal, u and heights of the
    // columns, kappa
    case APHGPU_K_CURVATURE: b = N * 8 + nif * (4.0 + 24 + 8 + 9 * 8 + 8); break;
    default: return SetError(ctx, APHGPU_ERR_ARG, "unknown kernel %d", kernel);
  }
  // flux and update of the x direction with the last step's time step (the
  // update writes the scratch copy of u: the state is left as it was, the
  // interface list as the update leaves it)
  auto launch = [&]() -> int {
    switch (kernel) {
      case APHGPU_K_VOF_FLUX: return SweepFluxList(ctx, sc, 0, d_vflux, dt);
      case APHGPU_K_VOF_UPDATE: return SweepUpdate(ctx, sc, 0, d_vflux, dt, false);
      case APHGPU_K_RECONSTRUCT: return ReconstructListed(ctx, sc);
      case APHGPU_K_HEIGHTS: return HeightsListed(ctx, sc);
      case APHGPU_K_CURVATURE: return CurvatureListed(ctx, sc);
    }
    APH_LAUNCHED(ctx);
    return APHGPU_OK;
  };
  APH_TRY(launch());
  APH_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  for (int r = 0; r < reps; ++r) APH_TRY(launch());
  APH_CUDA(ctx, cudaEventRecord(ctx->ev1, st));
  APH_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
  float t = 0;
  APH_CUDA(ctx, cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
  *ms = (double)t / reps;
  *bytes = b;
  return APHGPU_OK;
}

int SurfaceTensionDevice(aphgpu_ctx* ctx, double sigma, double* d_febp) {
  KSurfaceTension<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->h, sigma, ctx->u, ctx->kappa, d_febp);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

}  // namespace aphgpu

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
//   KFcuu                fcuu = u < 0.5 ? 0 : 1 (1 byte/cell)
//   3 x { KSweepFlux     fluid flux through the faces of one direction
//         KSweepUpdate   u += fcuu*ds - dl, clipping
//         KReconstruct } normals (Youngs + height) and plane constants of
//                        interfacial cells
// Curvature (Heights::CalcCurvature, curv.ipp:358-414):
//   KHeights             13-cell columns rebuilt from the same two-step and
//                        four-step differences as CalcDiff2/CalcDiff4, then
//                        UHeight::Good, one height per direction
//   KCurvature           height-function curvature of interfacial cells
#include <cuda_runtime.h>

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

// reconst.h:140-168
__device__ double LineU0(const double n[3], double a) {
  const double nx = n[0], ny = n[1], nz = n[2];
  const double f = a + 0.5 * (nx + ny + nz);
  if (f <= 0) return 0;
  if (nx >= f) return cube(f) / (6 * nx * ny * nz);
  if (ny >= f) return (3 * sqr(f) - 3 * f * nx + sqr(nx)) / (6 * ny * nz);
  if (nz >= f) {
    if (nx + ny >= f) {
      return (3 * sqr(f) - 3 * f * nx + sqr(nx) -
              smin(1., (f - ny) / nx) * sqr(f - ny)) /
             (6 * ny * nz);
    }
    return (2 * f - nx - ny) / (2 * nz);
  }
  return (cube(f) - cube(f - nx) - cube(f - ny) - cube(f - nz)) /
         (6 * nx * ny * nz);
}

// reconst.h:183-203, n already multiplied by h
__device__ double LineU1(const double n0[3], double a) {
  double n[3] = {fabs(n0[0]), fabs(n0[1]), fabs(n0[2])};
  Sort3(n);
  const double s = ((0 + n[0]) + n[1]) + n[2];
  a = smax(-0.5 * s, smin(0.5 * s, a));
  if (a < 0) return LineU0(n, a);
  return 1 - LineU0(n, -a);
}

__device__ __forceinline__ double LineU(const double n[3], double a, const double h[3]) {
  const double nh[3] = {n[0] * h[0], n[1] * h[1], n[2] * h[2]};
  return LineU1(nh, a);
}

// reconst.h:218-250
__device__ double LineA0(const double n[3], double u) {
  const double nx = n[0], ny = n[1], nz = n[2];
  double f;
  if (6. * ny * nz * u < sqr(nx)) {
    f = pow(6. * nx * ny * nz * u, 1. / 3.);
  } else if (6. * ny * nz * u < 3. * sqr(ny) - 3 * nx * ny + sqr(nx)) {
    f = 0.5 * nx + sqrt(2. * ny * nz * u - sqr(nx) / 12.);
  } else if (nz > nx + ny) {
    if (2. * nz * u < nx + ny) {
      f = SolveCubic(1., -3. * (nx + ny), 3. * (sqr(nx) + sqr(ny)),
                     -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u, 1);
    } else {
      f = nz * u + 0.5 * (nx + ny);
    }
  } else {
    if (6. * nx * ny * nz * u < -cube(nz) + 3. * sqr(nz) * (nx + ny) -
                                    3. * nz * (sqr(nx) + sqr(ny)) + cube(nx) +
                                    cube(ny)) {
      f = SolveCubic(1., -3. * (nx + ny), 3. * (sqr(nx) + sqr(ny)),
                     -(cube(nx) + cube(ny)) + 6. * nx * ny * nz * u, 1);
    } else {
      f = SolveCubic(2., -3. * (nx + ny + nz), 3. * (sqr(nx) + sqr(ny) + sqr(nz)),
                     -(cube(nx) + cube(ny) + cube(nz)) + 6. * nx * ny * nz * u, 1);
    }
  }
  return f - 0.5 * (nx + ny + nz);
}

// reconst.h:264-285
__device__ double LineA(const double n0[3], double u, const double h[3]) {
  double n[3] = {fabs(n0[0] * h[0]), fabs(n0[1] * h[1]), fabs(n0[2] * h[2])};
  Sort3(n);
  u = smax(0., smin(1., u));
  if (u <= 0.5) return LineA0(n, u);
  return -LineA0(n, 1 - u);
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

// Vof::ReconstPlanes (vof.ipp:70-90) on interfacial cells only; values of
// other cells are left untouched (they are never read).
__global__ void KReconstruct(Dims d, double hx, double hy, double hz,
                             const double* __restrict__ u, double* nrm,
                             double* pa) {
  VOF_CELL_LOOP(d)
  const double uc = u[c];
  if (!IsInterface(uc)) continue;
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
  double n[3];
  NormalCell(u3, n);
  const double h[3] = {hx, hy, hz};
  nrm[3 * c + 0] = n[0];
  nrm[3 * c + 1] = n[1];
  nrm[3 * c + 2] = n[2];
  pa[c] = LineA(n, uc, h);
  }
}

__global__ void KFcuu(int64_t n, const double* __restrict__ u, uint8_t* fcuu) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    fcuu[c] = u[c] < 0.5 ? 0 : 1;
}

// Fluxes of Vof::Sweep (vof.ipp:228-256) through the faces of direction dir
__global__ void KSweepFlux(Dims d, int dir, double hx, double hy, double hz,
                           const double* __restrict__ u,
                           const double* __restrict__ vflux,
                           const double* __restrict__ nrm,
                           const double* __restrict__ pa, double dt,
                           double* ffvu) {
  const double h[3] = {hx, hy, hz};
  VOF_CELL_LOOP(d)
  const int64_t cm = dir == 0 ? d.idx(wrapm(i - 1, d.nx), j, k)
                   : dir == 1 ? d.idx(i, wrapm(j - 1, d.ny), k)
                              : d.idx(i, j, wrapm(k - 1, d.nz));
  const double v = vflux[c];
  const double v0 = v / 1.;
  const int64_t up = v > 0 ? cm : c;
  const double uu = u[up];
  double f;
  if (uu > 0 && uu < 1) {
    const double n[3] = {nrm[3 * up], nrm[3 * up + 1], nrm[3 * up + 2]};
    const double sq = ((0 + sqr(n[0])) + sqr(n[1])) + sqr(n[2]);
    if (sq > 0) {
      f = LineFlux(n, pa[up], h, v0, dt, dir);
    } else {
      f = v0 * uu;
    }
  } else {
    f = v0 * uu;
  }
  ffvu[c] = f;
  }
}

// Update of Vof::Sweep (vof.ipp:287-326), weymouth, with clipping
__global__ void KSweepUpdate(Dims d, int dir, double vol, double* u,
                             const double* __restrict__ vflux,
                             const double* __restrict__ ffvu,
                             const uint8_t* __restrict__ fcuu, double dt,
                             double clipth) {
  VOF_CELL_LOOP(d)
  const int64_t fp = dir == 0 ? d.idx(wrapp(i + 1, d.nx), j, k)
                   : dir == 1 ? d.idx(i, wrapp(j + 1, d.ny), k)
                              : d.idx(i, j, wrapp(k + 1, d.nz));
  const double ds = (vflux[fp] / (1 + 1e-16) - vflux[c] / (1 + 1e-16)) * dt / vol;
  const double dl = (ffvu[fp] - ffvu[c]) * dt / vol;
  double w = u[c];
  w += (double)fcuu[c] * ds - dl;
  if (!(w >= clipth)) {
    w = 0;
  } else if (!(w <= 1 - clipth)) {
    w = 1;
  }
  u[c] = w;
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

// CalcDiff2/CalcDiff4/CalcHeight (curv.ipp:100-254) fused per interfacial
// cell: the column is rebuilt exactly as CalcHeight does from the
// two-step differences du2(q) = u(q+2) - u(q-2) and four-step differences
// du4(q) = du2(q+2) - du2(q-2).
__global__ void KHeights(Dims d, double hx, double hy, double hz,
                         const double* __restrict__ u, double* hgt) {
  const double h[3] = {hx, hy, hz};
  VOF_CELL_LOOP(d)
  if (!IsInterface(u[c])) continue;
  const int w[3] = {i, j, k};
  const int nd[3] = {d.nx, d.ny, d.nz};
#pragma unroll 1
  for (int dd = 0; dd < 3; ++dd) {
    double uc[13];  // u at offsets -6..6 along dd
#pragma unroll
    for (int s = -6; s <= 6; ++s) {
      int q[3] = {i, j, k};
      q[dd] = ((w[dd] + s) % nd[dd] + nd[dd]) % nd[dd];
      uc[s + 6] = u[d.idx(q[0], q[1], q[2])];
    }
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
    const double center = (0. + h[dd] * 0.5) + (double)w[dd] * h[dd];
    hgt[3 * c + dd] = center + off * h[dd];
  }
  }
}

// CalcCurvHeight (curv.ipp:261-356); NaN outside the interface
__global__ void KCurvature(Dims d, double hx, double hy, double hz,
                           const double* __restrict__ u,
                           const double* __restrict__ nrm,
                           const double* __restrict__ hgt, double* kappa) {
  const double h[3] = {hx, hy, hz};
  VOF_CELL_LOOP(d)
  if (!IsInterface(u[c])) {
    kappa[c] = nan("");
    continue;
  }
  const double n[3] = {nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]};
  const double an[3] = {fabs(n[0]), fabs(n[1]), fabs(n[2])};
  int dn = 0;
  if (an[1] > an[dn]) dn = 1;
  if (an[2] > an[dn]) dn = 2;
  const int dx = (dn + 1) % 3, dy = (dn + 2) % 3;
  const double lx = h[dx], ly = h[dy];
  const int nd[3] = {d.nx, d.ny, d.nz};
  const int w[3] = {i, j, k};
  double hv[3][3];
  for (int sy = -1; sy <= 1; ++sy)
    for (int sx = -1; sx <= 1; ++sx) {
      int b[3] = {w[0], w[1], w[2]};
      b[dx] += sx;
      b[dy] += sy;
      double r = nan("");
      const int shifts[5] = {0, 1, -1, 2, -2};
      for (int t = 0; t < 5; ++t) {
        int q[3] = {b[0], b[1], b[2]};
        q[dn] += shifts[t];
        for (int e = 0; e < 3; ++e) q[e] = ((q[e] % nd[e]) + nd[e]) % nd[e];
        const int64_t cn = d.idx(q[0], q[1], q[2]);
        if (IsInterface(u[cn])) {
          r = hgt[3 * cn + dn];
          break;
        }
      }
      hv[sy + 1][sx + 1] = r;
    }
  const double hcc = hv[1][1], hmc = hv[1][0], hpc = hv[1][2];
  const double hcm = hv[0][1], hcp = hv[2][1];
  const double hmm = hv[0][0], hmp = hv[2][0], hpm = hv[0][2], hpp = hv[2][2];
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
  if (n[dn] < 0) kk *= -1;
  kappa[c] = kk;
  }
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

int VofReconstruct(aphgpu_ctx* ctx) {
  const double h = ctx->h;
  KReconstruct<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, h, h, h, ctx->u, ctx->nrm, ctx->pa);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int VofStepDevice(aphgpu_ctx* ctx, const double* d_vflux, double dt) {
  const double h = ctx->h;
  const Dims d = ctx->d;
  const int64_t N = ctx->N;
  cudaStream_t st = ctx->stream;
  uint8_t* fcuu = (uint8_t*)ctx->u0;  // byte view of the scratch array
  KFcuu<<<FlatBlocks(N), kFlatThreads, 0, st>>>(N, ctx->u, fcuu);
  APH_LAUNCHED(ctx);
  int dd[3];
  const int cnt = ctx->vof_count % 3;  // vof.ipp:428-435
  if (cnt == 0) { dd[0] = 0; dd[1] = 1; dd[2] = 2; }
  else if (cnt == 1) { dd[0] = 1; dd[1] = 2; dd[2] = 0; }
  else { dd[0] = 2; dd[1] = 0; dd[2] = 1; }
  const double vol = (h * h) * h;
  for (int id = 0; id < 3; ++id) {
    const int dir = dd[id];
    const double* vf = d_vflux + (int64_t)dir * N;
    KSweepFlux<<<TileGrid(d), TileBlock(), 0, st>>>(d, dir, h, h, h, ctx->u, vf,
                                                    ctx->nrm, ctx->pa, dt, ctx->ffvu);
    APH_LAUNCHED(ctx);
    KSweepUpdate<<<TileGrid(d), TileBlock(), 0, st>>>(d, dir, vol, ctx->u, vf,
                                                      ctx->ffvu, fcuu, dt, ctx->clipth);
    APH_LAUNCHED(ctx);
    APH_TRY(VofReconstruct(ctx));
  }
  ctx->vof_count += 1;
  return APHGPU_OK;
}

int CurvatureDevice(aphgpu_ctx* ctx) {
  const double h = ctx->h;
  KHeights<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(ctx->d, h, h, h,
                                                               ctx->u, ctx->hgt);
  APH_LAUNCHED(ctx);
  KCurvature<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, h, h, h, ctx->u, ctx->nrm, ctx->hgt, ctx->kappa);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int TimeVofKernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms, double* bytes,
                  const double* d_vflux, double dt) {
  const double h = ctx->h;
  const Dims d = ctx->d;
  const double N = (double)ctx->N;
  cudaStream_t st = ctx->stream;
  uint8_t* fcuu = (uint8_t*)ctx->u0;
  double b = 0;
  auto launch = [&]() {
    switch (kernel) {
      case APHGPU_K_VOF_FLUX:
        KSweepFlux<<<TileGrid(d), TileBlock(), 0, st>>>(d, 0, h, h, h, ctx->u, d_vflux,
                                                        ctx->nrm, ctx->pa, dt, ctx->ffvu);
        break;
      case APHGPU_K_VOF_UPDATE:
        KSweepUpdate<<<TileGrid(d), TileBlock(), 0, st>>>(d, 0, h * h * h, ctx->u, d_vflux,
                                                          ctx->ffvu, fcuu, 0.0, ctx->clipth);
        break;
      case APHGPU_K_RECONSTRUCT:
        KReconstruct<<<TileGrid(d), TileBlock(), 0, st>>>(d, h, h, h, ctx->u, ctx->nrm, ctx->pa);
        break;
      case APHGPU_K_HEIGHTS:
        KHeights<<<TileGrid(d), TileBlock(), 0, st>>>(d, h, h, h, ctx->u, ctx->hgt);
        break;
      case APHGPU_K_CURVATURE:
        KCurvature<<<TileGrid(d), TileBlock(), 0, st>>>(d, h, h, h, ctx->u, ctx->nrm,
                                                        ctx->hgt, ctx->kappa);
        break;
    }
  };
  switch (kernel) {
    case APHGPU_K_VOF_FLUX: b = N * (8 + 8 + 8); break;          // u, flux, ffvu
    case APHGPU_K_VOF_UPDATE: b = N * (8 + 8 + 8 + 1 + 8); break;  // u r/w, flux, ffvu, fcuu
    case APHGPU_K_RECONSTRUCT: b = N * 8; break;                  // u (+ interface cells)
    case APHGPU_K_HEIGHTS: b = N * 8; break;
    case APHGPU_K_CURVATURE: b = N * (8 + 8); break;              // u, kappa
    default: return SetError(ctx, APHGPU_ERR_ARG, "unknown kernel %d", kernel);
  }
  launch();
  APH_LAUNCHED(ctx);
  APH_CUDA(ctx, cudaEventRecord(ctx->ev0, st));
  for (int r = 0; r < reps; ++r) launch();
  APH_LAUNCHED(ctx);
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

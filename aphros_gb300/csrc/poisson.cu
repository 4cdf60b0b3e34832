// Pressure Poisson solve of the projection step on one GB300.
//
// System storage (per cell, x-fastest, periodic):
//   w[d][c]  = e[1+2d] of aphros's Expr: coupling of cell c to its minus
//              neighbour in direction d.  The plus coupling e[2+2d] of c is
//              w[d][c+e_d] (symmetric systems only).
//   diag[c]  = e[0] when it differs from -(e1+...+e6); otherwise the
//              diagonal is recomputed on the fly in the same order as
//              GetFluxSum accumulates it (src/solver/proj.ipp:367-383).
//   b[c]     = -e[7].
// 24 B/cell of operator instead of the 64 B/cell AoS Expr.
//
// Solvers:
//   CG     the algorithm of linear::SolverConjugate (src/linear/linear.ipp:
//          24-129): three kernels per iteration, dot products reduced
//          deterministically in one grid-wide pass, the stopping test
//          evaluated on the device so that iterations run without host
//          round trips.
//   MGPCG  CG preconditioned by one geometric multigrid V-cycle (red-black
//          Gauss-Seidel, summed restriction, constant prolongation, coarse
//          operators from face-coefficient sums, FP64 CG on the coarsest
//          level), all FP64.
//   MIXED  FP64 defect correction: r = b - A x, the update and the outer
//          norms in FP64; the correction equation solved by FP32 MG-PCG;
//          the coarsest level solved in FP64.
#include <atomic>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <type_traits>

#include "common.cuh"
#include "stencil.cuh"
#include "dfloat.cuh"
#include "split.cuh"
#include "sweep.cuh"
#include "vec.cuh"

namespace aphgpu {

int FlatBlocks(int64_t n) {
  // SM count of device 0, read once (no runtime queries while a stream is
  // being captured into a graph)
  static const int sms = [] {
    int v = 152;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) {
      cudaGetLastError();
      v = 152;
    }
    return v;
  }();
  const int64_t want = (n + kFlatThreads - 1) / kFlatThreads;
  const int64_t cap = (int64_t)sms * 8;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

namespace {

// Explicitly rounded FP64 operations: the assembly and flux kernels must not
// be contracted into fused multiply-adds, so that they reproduce the
// reference's arithmetic bit for bit (the solver kernels may fuse).
__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }

// ---------------------------------------------------------------------------
// System set-up
// ---------------------------------------------------------------------------

// flags[0]: asymmetric cells, flags[1]: cells whose e0 != -(sum of e_q),
// flags[2]: cells whose row sum e0 + sum of e_q is more than rounding
// (a diagonal shift: the system is not singular), flags[3]: cells with a
// negative diagonal
__global__ void KExprToSystem(Dims d, const double* __restrict__ e8,
                              double* w0, double* w1, double* w2, double* diag,
                              double* b, unsigned int* flags) {
  unsigned int asym = 0, nonpure = 0, shifted = 0, negative = 0;
  TILE_LOOP_BEGIN(d)
  const double* e = e8 + 8 * c;
  w0[c] = e[1];
  w1[c] = e[3];
  w2[c] = e[5];
  diag[c] = e[0];
  b[c] = -e[7];
  const int ip = wrapp(i + 1, d.nx), jp = wrapp(j + 1, d.ny), kp = wrapp(k + 1, d.nz);
  if (e[2] != e8[8 * d.idx(ip, j, k) + 1]) ++asym;
  if (e[4] != e8[8 * d.idx(i, jp, k) + 3]) ++asym;
  if (e[6] != e8[8 * d.idx(i, j, kp) + 5]) ++asym;
  double s = 0, mag = fabs(e[0]);
  for (int q = 1; q <= 6; ++q) {
    s += e[q];
    mag += fabs(e[q]);
  }
  if (e[0] != -s) ++nonpure;
  if (!(fabs(e[0] + s) <= 1e-10 * mag)) ++shifted;
  if (e[0] < 0) ++negative;
  TILE_LOOP_END
  if (asym) atomicAdd(&flags[0], asym);
  if (nonpure) atomicAdd(&flags[1], nonpure);
  if (shifted) atomicAdd(&flags[2], shifted);
  if (negative) atomicAdd(&flags[3], negative);
}

// The system negated in place (couplings, diagonal, right-hand side): a
// negative definite system (aphros's own assembly without Proj's sign, as
// in its linear-solver test) becomes the positive definite one with the
// same solution and the same residual norms.
__global__ void KNegateSystem(int64_t n, double* w0, double* w1, double* w2, double* diag,
                              double* b) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    w0[c] = -w0[c];
    w1[c] = -w1[c];
    w2[c] = -w2[c];
    diag[c] = -diag[c];
    b[c] = -b[c];
  }
}

// Face coefficients and predicted fluxes (proj.ipp:343-360, 556-562):
// rho = rho1*(1-a)+rho2*a (hydro.ipp:1818-1821), face density harmonic
// (approx_eb.h:351-363), kk = -area/rho_f*dt, e0f = -(1/h)*kk; the Expr of
// the plus cell gets e[1+2d] = -e0f.
__global__ void KAssembleFaces(Dims d, const double* __restrict__ alpha,
                               double rho1, double rho2,
                               const double* __restrict__ vflux,
                               const double* __restrict__ febp, double dt,
                               double h, double* w0, double* w1, double* w2,
                               double* vstar) {
  const double area = h * h;
  const double ainv = 1 / h;
  const int64_t N = d.cells();
  TILE_LOOP_BEGIN(d)
  const double ac = alpha[c];
  const double rc = A(M(rho1, S(1, ac)), M(rho2, ac));
  const double invc = 1 / rc;
  double* ws[3] = {w0, w1, w2};
  for (int q = 0; q < 3; ++q) {
    const int64_t cm = q == 0 ? d.idx(wrapm(i - 1, d.nx), j, k)
                     : q == 1 ? d.idx(i, wrapm(j - 1, d.ny), k)
                              : d.idx(i, j, wrapm(k - 1, d.nz));
    const double am = alpha[cm];
    const double rm = A(M(rho1, S(1, am)), M(rho2, am));
    const double invm = 1 / rm;
    const double rf = 1 / M(A(invc, invm), 0.5);
    const double kk = M(-area / rf, dt);
    const double e0f = M(-ainv, kk);
    ws[q][c] = -e0f;
    double v = vflux[q * N + c];
    if (febp) v = A(v, M(M(febp[q * N + c] / rf, dt), area));
    vstar[q * N + c] = v;
  }
  TILE_LOOP_END
}

// e7 = sum over q of outward v* (AppendExpr order), b = -e7; reduces sum e7.
__global__ void KAssembleRhs(Dims d, const double* __restrict__ vstar,
                             double* b, RedBuf rb, double* out) {
  const int64_t N = d.cells();
  double v[1] = {0};
  const int op[1] = {0};
  TILE_LOOP_BEGIN(d)
  const int ip = wrapp(i + 1, d.nx), jp = wrapp(j + 1, d.ny), kp = wrapp(k + 1, d.nz);
  double s = 0;
  s = A(s, -vstar[c]);
  s = A(s, vstar[d.idx(ip, j, k)]);
  s = A(s, -vstar[N + c]);
  s = A(s, vstar[N + d.idx(i, jp, k)]);
  s = A(s, -vstar[2 * N + c]);
  s = A(s, vstar[2 * N + d.idx(i, j, kp)]);
  b[c] = -s;
  v[0] += s;
  TILE_LOOP_END
  GridReduce<1>(v, op, rb, out);
}

// b = -(e7 - mean) with e7 = -b
__global__ void KRemoveMean(int64_t n, double* b, const double* sum) {
  const double mean = sum[0] / (double)n;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double e7 = -b[c];
    b[c] = -S(e7, mean);
  }
}

// Expr of every cell from the compact storage (inverse of KExprToSystem):
// e0 as GetFluxSum accumulates it when no explicit diagonal is stored.
__global__ void KSystemToExpr(Op<double> Aop, const double* __restrict__ b,
                              double* e8, double sign) {
  TILE_LOOP_BEGIN(Aop.d)
  double e[6];
  Couplings(Aop, i, j, k, c, e);
  double* o = e8 + 8 * c;
  if (Aop.diag) {
    o[0] = sign * Aop.diag[c];
  } else {
    double s = 0;
    for (int q = 0; q < 6; ++q) s = A(s, -e[q]);
    o[0] = sign * s;
  }
  for (int q = 0; q < 6; ++q) o[1 + q] = sign * e[q];
  o[7] = -sign * b[c];
  TILE_LOOP_END
}

// diag = minus the sum of the six couplings (Diag without a stored diagonal)
__global__ void KFillDiag(Op<double> A, double* diag) {
  TILE_LOOP_BEGIN(A.d)
  double e[6];
  Couplings(A, i, j, k, c, e);
  diag[c] = Diag(A, c, e);
  TILE_LOOP_END
}

template <class T>
__global__ void KInvDiag(Op<T> A, T* invdiag) {
  TILE_LOOP_BEGIN(A.d)
  T e[6];
  Couplings(A, i, j, k, c, e);
  invdiag[c] = T(1) / Diag(A, c, e);
  TILE_LOOP_END
}

// ---------------------------------------------------------------------------
// Plain CG (linear.ipp:24-129)
// ---------------------------------------------------------------------------

// r = -(x*e0 + e7 + sum x_nb e_q), p = r   (stage init, linear.ipp:42-61)
__global__ void KCgInit(Op<double> A, const double* __restrict__ b,
                        const double* x, double* r, double* p, int zero_guess) {
  TILE_LOOP_BEGIN(A.d)
  double u;
  if (zero_guess) {
    u = -b[c];
  } else {
    double e[6];
    Couplings(A, i, j, k, c, e);
    const double e0 = Diag(A, c, e);
    const Dims& d = A.d;
    u = x[c] * e0 + (-b[c]);
    u += x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
    u += x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
    u += x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
    u += x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
    u += x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
    u += x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  }
  r[c] = -u;
  p[c] = -u;
  TILE_LOOP_END
}

// stage iter: lp = A p, dot_r_prev = r.r, dot_p_lp = p.lp
__global__ void KCgApply(Op<double> A, const double* __restrict__ r,
                         const double* __restrict__ p, double* ap,
                         SolveScalars* s, RedBuf rb) {
  if (s->done) return;
  double v[2] = {0, 0};
  const int op[2] = {0, 0};
  TILE_LOOP_BEGIN(A.d)
  const double y = Apply(A, p, i, j, k, c);
  ap[c] = y;
  v[0] += r[c] * r[c];
  v[1] += p[c] * y;
  TILE_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr_prev = out[0];
      s->pap = out[1];
      s->alpha = out[0] / (out[1] + 1e-100);
    }
  }
}

// stage iter2 + check: x += alpha p, r -= alpha lp, dot_r, max_r
__global__ void KCgUpdate(Dims d, double* x, double* r,
                          const double* __restrict__ p,
                          const double* __restrict__ ap, SolveScalars* s,
                          RedBuf rb) {
  if (s->done) return;
  const double alpha = s->alpha;
  double v[2] = {0, 0};
  const int op[2] = {0, 1};
  TILE_LOOP_BEGIN(d)
  x[c] += alpha * p[c];
  const double rn = r[c] - alpha * ap[c];
  r[c] = rn;
  v[0] += rn * rn;
  v[1] = fmax(v[1], fabs(rn));
  TILE_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      s->beta = out[0] / (s->rr_prev + 1e-100);
      const double res = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->residual = res * s->res_scale;
      if (s->hist && s->iter < s->hist_cap) s->hist[s->iter] = s->residual;
      s->iter += 1;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
}

// stage iter3: p = r + beta p
__global__ void KCgP(Dims d, const double* __restrict__ r, double* p,
                     const SolveScalars* s) {
  if (s->done) return;
  const double beta = s->beta;
  TILE_LOOP_BEGIN(d)
  p[c] = r[c] + beta * p[c];
  TILE_LOOP_END
}

// ---------------------------------------------------------------------------
// Preconditioned CG building blocks (templated on the vector precision)
// ---------------------------------------------------------------------------

// ap = A p, reduces p.ap -> alpha = rz / p.ap (and sum ap when projecting
// the constant mode)
template <class T>
__global__ void KPcgApply(Op<T> A, const T* __restrict__ p, T* ap,
                          SolveScalars* s, RedBuf rb) {
  if (s->done) return;
  double v[2] = {0, 0};
  const int op[2] = {0, 0};
  TILE_LOOP_BEGIN(A.d)
  const T y = Apply(A, p, i, j, k, c);
  ap[c] = y;
  v[0] += (double)p[c] * (double)y;
  v[1] += (double)y;
  TILE_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->pap = out[0];
      s->apsum = out[1];
      s->alpha = s->rz / (out[0] + 1e-300);
    }
  }
}

// x += alpha p, r -= alpha (ap - mean(ap) when projecting), reduces r.r and
// max|r|, then the stopping test
template <class T>
__global__ void KPcgUpdate(Dims d, T* x, T* r, const T* __restrict__ p,
                           const T* __restrict__ ap, SolveScalars* s,
                           RedBuf rb) {
  if (s->done) return;
  const T alpha = (T)s->alpha;
  const T apm = (s->flags & 1) ? (T)(s->apsum / (double)d.cells()) : T(0);
  double v[2] = {0, 0};
  const int op[2] = {0, 1};
  TILE_LOOP_BEGIN(d)
  x[c] += alpha * p[c];
  const T rn = r[c] - alpha * (ap[c] - apm);
  r[c] = rn;
  v[0] += (double)rn * (double)rn;
  v[1] = fmax(v[1], fabs((double)rn));
  TILE_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      const double res = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->residual = res * s->res_scale;
      if (s->hist && s->iter < s->hist_cap) s->hist[s->iter] = s->residual;
      s->iter += 1;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
}

// rz = r.z; first == 1: p = z (start), else beta = rz/rz_prev, or with the
// flexible variant (flags bit 1) beta = (r.z - r.z_old)/rz_prev
// (two passes: reduction kernel then update kernel)
template <class T>
__global__ void KDotRZ(Dims d, const T* __restrict__ r, const T* __restrict__ z,
                       const T* __restrict__ zold, SolveScalars* s, RedBuf rb,
                       int first) {
  if (s->done) return;
  const bool flex = (s->flags & 2) && !first && zold;
  double v[2] = {0, 0};
  const int op[2] = {0, 0};
  TILE_LOOP_BEGIN(d)
  v[0] += (double)r[c] * (double)z[c];
  if (flex) v[1] += (double)r[c] * (double)zold[c];
  TILE_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rz_prev = first ? 0.0 : s->rz;
      s->rz = out[0];
      s->rzold = out[1];
      const double num = flex ? out[0] - out[1] : out[0];
      s->beta = first ? 0.0 : num / (s->rz_prev + 1e-300);
    }
  }
}

template <class T>
__global__ void KPcgP(Dims d, const T* __restrict__ z, T* p,
                      const SolveScalars* s, int first) {
  if (s->done) return;
  const T beta = (T)s->beta;
  TILE_LOOP_BEGIN(d)
  p[c] = first ? z[c] : z[c] + beta * p[c];
  TILE_LOOP_END
}

// ---------------------------------------------------------------------------
// Multigrid kernels
// ---------------------------------------------------------------------------

// Red-black Gauss-Seidel half sweep on cells with (i+j+k)%2 == color:
// x_c = (b_c - sum_q e_q x_nb) / e0.  zero_init: the other colour is
// treated as zero (first half sweep from a zero guess).
template <class T>
__global__ void KSmooth(Op<T> A, const T* __restrict__ invdiag,
                        const T* __restrict__ b, T* x, int color,
                        int zero_init, const SolveScalars* s) {
  if (s && s->done) return;
  const Dims& d = A.d;
  TILE_LOOP_BEGIN(d)
  if (((i + j + k) & 1) != color) continue;
  if (zero_init) {
    x[c] = b[c] * invdiag[c];
    continue;
  }
  T e[6];
  Couplings(A, i, j, k, c, e);
  T acc = b[c];
  acc -= x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
  acc -= x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
  acc -= x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
  acc -= x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
  acc -= x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
  acc -= x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  x[c] = acc * invdiag[c];
  TILE_LOOP_END
}

// ---------------------------------------------------------------------------
// Vectorized FP32 kernels (nx % 4 == 0): each thread owns 4 consecutive
// cells in x (one float4), a CTA of 32x8 threads covers 128 x 8 cells of a
// plane and marches over kz planes in z (VecZ), keeping the z neighbours in
// registers.  x neighbours across float4 boundaries come from warp shuffles
// (global loads at warp and domain edges, periodic wrap).
// ---------------------------------------------------------------------------

// z planes per thread: 16 on large levels, halved until the grid has at
// least 4 CTAs per SM (small levels would otherwise leave SMs idle)
inline int VecZ(const Dims& d) {
  const int nq = d.nx / 4;
  const int64_t xy = (int64_t)((nq + 31) / 32) * ((d.ny + 7) / 8);
  int kz = 16;
  while (kz > 1 && xy * ((d.nz + kz - 1) / kz) < 4 * 152) kz /= 2;
  return kz;
}
inline dim3 VecGrid(const Dims& d) {
  const int nq = d.nx / 4;
  const int kz = VecZ(d);
  return dim3((nq + 31) / 32, (d.ny + 7) / 8, (d.nz + kz - 1) / kz);
}
inline bool VecOk(const Dims& d) { return (d.nx % 4) == 0 && d.nx >= 8; }
// the colour-split kernels (split.cuh): 4 positions of each half per
// thread, 32 x 8 threads per CTA, z planes per thread as VecZ
inline int SplitZ(const Dims& d) {
  const int nq = d.nx / 8;
  const int64_t xy = (int64_t)((nq + 31) / 32) * ((d.ny + 7) / 8);
  int kz = 16;
  while (kz > 1 && xy * ((d.nz + kz - 1) / kz) < 4 * 152) kz /= 2;
  return kz;
}
inline dim3 SplitGrid(const Dims& d) {
  const int kz = SplitZ(d);
  return dim3((d.nx / 8 + 31) / 32, (d.ny + 7) / 8, (d.nz + kz - 1) / kz);
}

// One red-black half sweep (FP32, vectorized); see KSmooth for the update.
// The diagonal is recomputed from the six couplings (read anyway) unless the
// operator stores one.
// (W = __half: FP16 couplings scaled by bscale)
template <class W>
__global__ void __launch_bounds__(256, 4) KSmooth4(Op<W> A, const float* __restrict__ b,
                                                float* x, int color, int zero_init,
                                                const SolveScalars* s, int kz, float bscale) {
  if (s && s->done) return;
  const int kb = blockIdx.z * kz;
  Smooth4Body(A, b, x, color, zero_init, blockIdx.x * 32 + threadIdx.x,
              blockIdx.y * 8 + threadIdx.y, kb, min(kb + kz, A.d.nz), 32, bscale);
}

// One red-black sweep, both colours fused, out of place (SweepRB4Tile):
// c0 the first colour, zero_init the zero initial guess of the first colour.
__global__ void __launch_bounds__(256, 3) KSweepRB4(Op<float> A, const float* __restrict__ b,
                                                   const float* xin, float* xout, int c0,
                                                   int zero_init, const SolveScalars* s, int kz) {
  if (s && s->done) return;
  __shared__ SweepPlanes sF;
  const int kb = blockIdx.z * kz;
  SweepRB4Tile(A, b, xin, xout, c0, zero_init, blockIdx.x, blockIdx.y, kb,
               min(kb + kz, A.d.nz), sF);
}

// levels the synchronous fused sweep handles
inline bool FusedOk(const Dims& d) { return VecOk(d); }

// The pipelined fused sweep (sweep.cuh): levels of at least kPipeMinCells
// cells in mode 1; every level with nx % 4 == 0, nx >= 16 and nz >= 8 in
// mode 2.
constexpr int64_t kPipeMinCells = int64_t(1) << 21;
inline bool PipeDims(const Dims& d) {
  return (d.nx % 4) == 0 && d.nx >= 16 && d.ny >= 2 && d.nz >= 8;
}
// The wavefront sweep (sweep.cuh): option value 5 on levels of at least
// kPipeMinCells cells, 6 on every level, where nx % 4 == 0, nz >= 4 and the
// tiles of 128 columns by bands of at most kWaveRows rows fit the SMs (one
// CTA per SM).
constexpr int kWaveMaxTiles = 4096;
// Planes per step of the wavefront sweep: three chunks of the level (the
// one prefetched, the one in its first colour, the one in its second) of x,
// b and the three couplings (20 bytes per cell) within about half of the
// 126 MB L2, and one chunk of a tile within 150 KB of L1 (a phase's items
// reread their neighbours' rows from there).
constexpr double kWaveL2Bytes = 60e6;
constexpr double kWaveL1Bytes = 150e3;
inline int WavePlanes(const aphgpu_ctx* ctx, const Dims& d, const WaveTiling& T) {
  if (ctx->wave_planes > 0) return std::min(ctx->wave_planes, d.nz);
  const double plane = 20.0 * (double)d.nx * (double)d.ny;
  const double tile = 20.0 * (double)T.w * (double)T.rows;
  const int k = (int)std::min(kWaveL2Bytes / (3.0 * plane), kWaveL1Bytes / tile);
  return std::max(1, std::min(k, d.nz));
}
inline WaveTiling WaveTiles(const Dims& d, int sms) {
  WaveTiling T;
  T.w = 128;
  T.xtiles = (d.nx + 127) / 128;
  const int bands_max = std::max(1, sms / T.xtiles);
  T.rows = (d.ny + bands_max - 1) / bands_max;
  T.bands = (d.ny + T.rows - 1) / T.rows;
  return T;
}
inline bool WaveDims(const Dims& d, int sms) {
  if (!((d.nx % 4) == 0 && d.nx >= 8 && d.nz >= 4)) return false;
  const WaveTiling T = WaveTiles(d, sms);
  return T.rows <= kWaveRows && T.xtiles * T.bands <= std::min(sms, kWaveMaxTiles);
}
inline bool PipeEligible(const aphgpu_ctx* ctx, const Dims& d) {
  if (!PipeDims(d)) return false;
  return ctx->fused_mode == 2 ||
         ((ctx->fused_mode == 1 || ctx->fused_mode == 4) && d.cells() >= kPipeMinCells);
}
// Tiles of the pipelined sweep: columns of at most kPipeCols (balanced),
// bands of at most `maxrows` rows (balanced), and z segments (at least 8
// planes each) so that the items fill the `slots` resident CTAs in as few
// waves as possible, the last one as full as possible.
inline PipeTiling PipeTiles(const Dims& d, int slots, int maxrows) {
  PipeTiling T;
  T.xtiles = (d.nx + kPipeCols - 1) / kPipeCols;
  T.w = 4 * ((d.nx / 4 + T.xtiles - 1) / T.xtiles);
  T.bands = (d.ny + maxrows - 1) / maxrows;
  T.rows = (d.ny + T.bands - 1) / T.bands;
  T.bands = (d.ny + T.rows - 1) / T.rows;
  const int tiles = T.xtiles * T.bands;
  T.zsegs = 1;
  double best = 0;
  for (int z = 1; z <= std::max(1, d.nz / 8); ++z) {
    const int64_t items = (int64_t)tiles * z;
    const int64_t waves = (items + slots - 1) / slots;
    // fill of the waves, with a small cost per segment (each restarts the
    // pipeline: about 3 extra planes of copies per segment)
    const double fill = (double)items / (double)(waves * slots);
    const double seg = (double)(d.nz / z) / (double)(d.nz / z + 3);
    if (fill * seg > best * 1.0001) {
      best = fill * seg;
      T.zsegs = z;
    }
  }
  return T;
}
inline int SmCount(aphgpu_ctx* ctx) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
      sms < 1) {
    cudaGetLastError();
    sms = 152;
  }
  return sms;
}
// one wavefront sweep in place (first colour c0; zero_init: the first
// colour starts from zero), cooperative launch
inline int LaunchWave(aphgpu_ctx* ctx, const Op<float>& A, const float* b, float* x, int c0,
                      int zero_init, const SolveScalars* s, cudaStream_t st) {
  const int sms = SmCount(ctx);
  const WaveTiling T = WaveTiles(A.d, sms);
  const int tiles = T.xtiles * T.bands;
  if (!ctx->wave_buf) APH_TRY(Alloc(ctx, &ctx->wave_buf, kWaveMaxTiles + 1));
  if (!ctx->wave_used) {
    APH_CUDA(ctx, cudaMemsetAsync(ctx->wave_buf + kWaveMaxTiles, 0, sizeof(int), st));
    ctx->wave_used = true;
  }
  APH_CUDA(ctx, cudaMemsetAsync(ctx->wave_buf, 0xff, sizeof(int) * tiles, st));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(tiles);
  cfg.blockDim = dim3(kWaveThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int* err = ctx->wave_buf + kWaveMaxTiles;
  const int K = WavePlanes(ctx, A.d, T);
  // all of the SM's shared storage as L1 (once per device; the attribute
  // is a preference, so a failure only clears the error)
  static std::atomic<uint64_t> carveout{0};
  const uint64_t bit = uint64_t(1) << (ctx->device & 63);
  if (!(carveout.load() & bit)) {
    cudaFuncSetAttribute(KSweepWave<0>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaFuncSetAttribute(KSweepWave<1>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    cudaGetLastError();
    carveout.fetch_or(bit);
  }
  if (zero_init)
    APH_CUDA(ctx, cudaLaunchKernelEx(&cfg, KSweepWave<1>, A, b, x, c0, s, T, K, ctx->wave_buf,
                                     err));
  else
    APH_CUDA(ctx, cudaLaunchKernelEx(&cfg, KSweepWave<0>, A, b, x, c0, s, T, K, ctx->wave_buf,
                                     err));
  return APHGPU_OK;
}
// the flag of a wavefront wait that gave up (after the solve's last sync)
int CheckWaveFlag(aphgpu_ctx* ctx) {
  if (!ctx->wave_used) return APHGPU_OK;
  int e = 0;
  APH_CUDA(ctx, cudaMemcpy(&e, ctx->wave_buf + kWaveMaxTiles, sizeof(int),
                           cudaMemcpyDeviceToHost));
  ctx->wave_used = false;
  if (e) {
    // cleared for the next solve, which sets it again only if it times out
    APH_CUDA(ctx, cudaMemset(ctx->wave_buf + kWaveMaxTiles, 0, sizeof(int)));
    return SetError(ctx, APHGPU_ERR_TIMEOUT, "wavefront sweep: a tile waited too long");
  }
  return APHGPU_OK;
}
// one pipelined sweep in -> out (first colour c0) with the kernel shape P
template <class P>
inline int LaunchPipeShape(aphgpu_ctx* ctx, const Op<float>& A, const float* b,
                           const float* in, float* out, int c0, int zero_init,
                           const SolveScalars* s, cudaStream_t st) {
  static bool attr_set[64] = {};
  const int dev = ctx->device;
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    APH_CUDA(ctx, cudaFuncSetAttribute(KSweepPipe<P, 0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       P::kSmemBytes));
    APH_CUDA(ctx, cudaFuncSetAttribute(KSweepPipe<P, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       P::kSmemBytes));
    attr_set[dev] = true;
  }
  const PipeTiling T = PipeTiles(A.d, P::kCtasPerSm * SmCount(ctx), P::kRows);
  const int items = T.xtiles * T.bands * T.zsegs;
  if (zero_init)
    KSweepPipe<P, 1><<<items, P::kThreads, P::kSmemBytes, st>>>(A, b, in, out, c0, s, T);
  else
    KSweepPipe<P, 0><<<items, P::kThreads, P::kSmemBytes, st>>>(A, b, in, out, c0, s, T);
  return APHGPU_OK;
}
inline int LaunchPipe(aphgpu_ctx* ctx, const Op<float>& A, const float* b, const float* in,
                      float* out, int c0, int zero_init, const SolveScalars* s,
                      cudaStream_t st) {
  if (ctx->fused_mode == 4)
    return LaunchPipeShape<PipeShort>(ctx, A, b, in, out, c0, zero_init, s, st);
  return LaunchPipeShape<PipeTall>(ctx, A, b, in, out, c0, zero_init, s, st);
}
inline dim3 SweepGrid(const Dims& d) {
  const int nq = d.nx / 4;
  const int kz = VecZ(d);
  return dim3((nq + 31) / 32, (d.ny + kSweepRows - 1) / kSweepRows, (d.nz + kz - 1) / kz);
}

// y = A p (FP32, vectorized) with the reductions p.y and sum y of KPcgApply
__global__ void __launch_bounds__(256, 4) KPcgApply4(Op<float> A, const float* __restrict__ p,
                                                  float* ap, SolveScalars* s, RedBuf rb, int kz) {
  if (s->done) return;
  const int kb = blockIdx.z * kz;
  // per-thread sums in FP32 (at most 4 * kz terms), CTA and grid sums in
  // FP64: FP64 arithmetic is scarce on GB300
  float fa0 = 0.f, fa1 = 0.f;
  Apply4Body(A, p, ap, blockIdx.x * 32 + threadIdx.x, blockIdx.y * 8 + threadIdx.y, kb,
             min(kb + kz, A.d.nz), fa0, fa1);
  double v[2] = {(double)fa0, (double)fa1};
  const int op[2] = {0, 0};
  __shared__ double out2[2];
  if (GridReduce<2>(v, op, rb, out2)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->pap = out2[0];
      s->apsum = out2[1];
      s->alpha = s->rz / (out2[0] + 1e-300);
    }
  }
}

// x_fine += x_coarse(parent), FP32 vectorized (one float4 = 2 coarse cells)
__global__ void KProlong4(Dims d, float* x, Dims dc, const float* __restrict__ xc,
                          const SolveScalars* s, int kz) {
  if (s && s->done) return;
  const int kb = blockIdx.z * kz;
  Prolong4Body(d, x, dc, xc, blockIdx.x * 32 + threadIdx.x, blockIdx.y * 8 + threadIdx.y, kb,
               min(kb + kz, d.nz));
}

// x_out = x + x_coarse(parent), the out-of-place KProlong4 (same addition)
__global__ void KProlong4To(Dims d, const float* __restrict__ x, float* xo, Dims dc,
                            const float* __restrict__ xc, const SolveScalars* s, int kz) {
  if (s && s->done) return;
  const int q = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * kz, ke = min(kb + kz, d.nz);
  if (q >= d.nx / 4 || j >= d.ny) return;
  for (int k = kb; k < ke; ++k) {
    const int64_t c = d.idx(4 * q, j, k);
    const float2 e = *reinterpret_cast<const float2*>(xc + dc.idx(2 * q, j >> 1, k >> 1));
    float4 v = *reinterpret_cast<const float4*>(x + c);
    v.x += e.x;
    v.y += e.x;
    v.z += e.y;
    v.w += e.y;
    *reinterpret_cast<float4*>(xo + c) = v;
  }
}

// x += alpha p, r -= alpha (ap - mean(ap)), reductions and stopping test of
// KPcgUpdate, FP32 vectorized over flat float4s (n % 4 == 0)
__global__ void __launch_bounds__(256) KPcgUpdate4(int64_t n4, float* x, float* r,
                                                   const float* __restrict__ p,
                                                   const float* __restrict__ ap,
                                                   SolveScalars* s, RedBuf rb, int64_t ncells) {
  if (s->done) return;
  const float alpha = (float)s->alpha;
  const float apm = (s->flags & 1) ? (float)(s->apsum / (double)ncells) : 0.f;
  float r2 = 0.f, rmax = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    float4 xv = Ld4(x + 4 * t), rv = Ld4(r + 4 * t);
    const float4 pv = Ld4(p + 4 * t), av = Ld4(ap + 4 * t);
    xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
    rv.x -= alpha * (av.x - apm); rv.y -= alpha * (av.y - apm);
    rv.z -= alpha * (av.z - apm); rv.w -= alpha * (av.w - apm);
    St4(x + 4 * t, xv);
    St4(r + 4 * t, rv);
    r2 += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
    rmax = fmaxf(rmax, fmaxf(fmaxf(fabsf(rv.x), fabsf(rv.y)), fmaxf(fabsf(rv.z), fabsf(rv.w))));
  }
  double v[2] = {(double)r2, (double)rmax};
  const int op[2] = {0, 1};
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      const double res = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->residual = res * s->res_scale;
      if (s->hist && s->iter < s->hist_cap) s->hist[s->iter] = s->residual;
      s->iter += 1;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
}

// r.z (and r.z_old for the flexible beta), FP32 vectorized; see KDotRZ
__global__ void __launch_bounds__(256) KDotRZ4(int64_t n4, const float* __restrict__ r,
                                               const float* __restrict__ z,
                                               const float* __restrict__ zold,
                                               SolveScalars* s, RedBuf rb, int first) {
  if (s->done) return;
  const bool flex = (s->flags & 2) && !first && zold;
  float a = 0.f, b = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float4 rv = Ld4(r + 4 * t), zv = Ld4(z + 4 * t);
    a += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
    if (flex) {
      const float4 ov = Ld4(zold + 4 * t);
      b += rv.x * ov.x + rv.y * ov.y + rv.z * ov.z + rv.w * ov.w;
    }
  }
  double v[2] = {(double)a, (double)b};
  const int op[2] = {0, 0};
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0) {
      s->rz_prev = first ? 0.0 : s->rz;
      s->rz = out[0];
      s->rzold = out[1];
      const double num = flex ? out[0] - out[1] : out[0];
      s->beta = first ? 0.0 : num / (s->rz_prev + 1e-300);
    }
  }
}

// p = z + beta p (p = z when first), FP32 vectorized
__global__ void KPcgP4(int64_t n4, const float* __restrict__ z, float* p,
                       const SolveScalars* s, int first) {
  if (s->done) return;
  const float beta = (float)s->beta;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float4 zv = Ld4(z + 4 * t);
    float4 pv = first ? zv : Ld4(p + 4 * t);
    if (!first) {
      pv.x = zv.x + beta * pv.x; pv.y = zv.y + beta * pv.y;
      pv.z = zv.z + beta * pv.z; pv.w = zv.w + beta * pv.w;
    }
    St4(p + 4 * t, pv);
  }
}

// Residual of a fine FP32 level summed over the 8 children into the coarse
// right-hand side, vectorized: a thread owns one fine float4 (2 coarse
// cells in x) of a coarse row and marches over coarse planes.
template <class W>
__global__ void __launch_bounds__(256, 4) KResidualRestrict4(Op<W> A, const float* __restrict__ b,
                                                          const float* __restrict__ x, Dims dc,
                                                          float* bc, const SolveScalars* s,
                                                          int kz, float rscale) {
  if (s && s->done) return;
  const int Kb = blockIdx.z * kz;
  ResidualRestrict4Body(A, b, x, dc, bc, blockIdx.x * 32 + threadIdx.x,
                        blockIdx.y * 8 + threadIdx.y, Kb, min(Kb + kz, dc.nz), 32, rscale);
}

// Residual of the fine level summed over the 8 children into the coarse
// right-hand side.  One thread per coarse cell.
template <class T, class TC>
__global__ void KResidualRestrict(Op<T> A, const T* __restrict__ b,
                                  const T* __restrict__ x, Dims dc, TC* bc,
                                  const SolveScalars* s) {
  if (s && s->done) return;
  const int I = blockIdx.x * kTileX + threadIdx.x;
  const int J = blockIdx.y * kTileY + threadIdx.y;
  const int kb = blockIdx.z * kTileZ;
  const int ke = min(kb + kTileZ, dc.nz);
  if (I >= dc.nx || J >= dc.ny) return;
  for (int K = kb; K < ke; ++K) {
    T sum = T(0);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
      const int64_t c = A.d.idx(i, j, k);
      sum += b[c] - Apply(A, x, i, j, k, c);
    }
    bc[dc.idx(I, J, K)] = (TC)sum;
  }
}

// x_fine += x_coarse(parent)
template <class T, class TC>
__global__ void KProlong(Dims d, T* x, Dims dc, const TC* __restrict__ xc,
                         const SolveScalars* s) {
  if (s && s->done) return;
  TILE_LOOP_BEGIN(d)
  x[c] += (T)xc[dc.idx(i >> 1, j >> 1, k >> 1)];
  TILE_LOOP_END
}

// Largest and smallest nonzero magnitude of three FP32 arrays, as float bits
// (non-negative floats order like unsigned integers): out[0] max, out[1]
// min (atomics on order-independent extrema, so deterministic).
__global__ void KAbsRange(int64_t n, const float* __restrict__ a, const float* __restrict__ b,
                          const float* __restrict__ c, unsigned int* out) {
  unsigned int mx = 0u, mn = 0x7f800000u;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned int v[3] = {__float_as_uint(fabsf(a[i])), __float_as_uint(fabsf(b[i])),
                               __float_as_uint(fabsf(c[i]))};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      mx = max(mx, v[q]);
      if (v[q] != 0u) mn = min(mn, v[q]);
    }
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  mn = __reduce_min_sync(0xffffffffu, mn);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], mx);
    atomicMin(&out[1], mn);
  }
}

// w16 = half(w * scale), scale a power of two (exact before the rounding)
__global__ void KToHalf(int64_t n, const float* __restrict__ w, __half* w16, float scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    w16[i] = __float2half_rn(w[i] * scale);
}

// Coupling of the minus face of coarse cell (I,J,K) along axis q, summed
// over the 4 fine lines that cross the face.  Per line, a blend of two
// estimates of the conductance between the two coarse centres:
//   Galerkin: 0.5 * e_bc, the Galerkin coupling of constant prolongation
//     scaled by one half (over-correction; exact for a constant
//     coefficient);
//   series: 1 / (0.5 / e_ab + 1 / e_bc + 0.5 / e_cd), the three fine
//     couplings on the line in series (e_bc the fine face on the coarse
//     face, e_ab and e_cd the fine faces inside the two coarse cells, each
//     crossed over half its length).
// Both equal e/2 where the three couplings are equal; across a density
// jump the series value follows the weak side, the Galerkin value the
// strong one.  `series` is the weight of the series value.  The series
// factor t = series / e_bc = a c / (0.5 c + a c + 0.5 a), a = e_ab / e_bc,
// c = e_cd / e_bc, is computed in FP32 (it only shapes the preconditioner;
// FP64 division is slow on this GPU); lines whose couplings are not all of
// one sign, or whose ratios do not fit FP32, keep the Galerkin value.
template <class T>
__device__ double CoarseFace(const Op<T>& A, int q, int I, int J, int K, double series) {
  const Dims& d = A.d;
  const T* w = q == 0 ? A.w0 : (q == 1 ? A.w1 : A.w2);
  double s = 0;
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const int u = m & 1, v = m >> 1;
    int i = 2 * I, j = 2 * J, k = 2 * K;
    int64_t cab, ccd;
    if (q == 0) {
      j += u;
      k += v;
      cab = d.idx(wrapm(i - 1, d.nx), j, k);
      ccd = d.idx(i + 1, j, k);
    } else if (q == 1) {
      i += u;
      k += v;
      cab = d.idx(i, wrapm(j - 1, d.ny), k);
      ccd = d.idx(i, j + 1, k);
    } else {
      i += u;
      j += v;
      cab = d.idx(i, j, wrapm(k - 1, d.nz));
      ccd = d.idx(i, j, k + 1);
    }
    const double bc = (double)w[d.idx(i, j, k)];
    double line = 0.5 * bc;
    if (series > 0.0) {
      const float rb = 1.0f / (float)bc;
      const float a = (float)w[cab] * rb, c = (float)w[ccd] * rb;
      if (a > 0.0f && c > 0.0f) {
        const float ac = a * c;
        const float t = ac / (0.5f * c + ac + 0.5f * a);
        if (t > 0.0f && t <= 1.0f) line = (1.0 - series) * line + series * (double)t * bc;
      }
    }
    s += line;
  }
  return s;
}

// Coarse operator of constant prolongation and summed restriction, pass 1:
// the three minus-face couplings of each coarse cell (CoarseFace) and, in
// `diag`, the summed diagonal shifts of its 8 children (shift = diagonal +
// sum of the couplings).  The shifts (mass terms of diffusion systems,
// given-pressure cells) take their Galerkin value, the sum: constant
// prolongation represents them exactly, unlike the couplings, whose
// Galerkin value is halved (CoarseFace).  Singular (flux-difference)
// systems have no shifts: with_shift = 0 keeps them exactly zero, so that
// the rounding of the coarse operators does not accumulate into them.
template <class T, class TC>
__global__ void KCoarsenFaces(Op<T> A, Dims dc, TC* w0, TC* w1, TC* w2, TC* diag,
                              double series, int with_shift) {
  const int I = blockIdx.x * kTileX + threadIdx.x;
  const int J = blockIdx.y * kTileY + threadIdx.y;
  const int kb = blockIdx.z * kTileZ;
  const int ke = min(kb + kTileZ, dc.nz);
  if (I >= dc.nx || J >= dc.ny) return;
  const Dims& d = A.d;
  for (int K = kb; K < ke; ++K) {
    // the children's summed row sums (diagonal shifts), for systems with one
    double shift = 0;
    for (int q = 0; with_shift && q < 8; ++q) {
      const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
      const int64_t c = d.idx(i, j, k);
      T e[6];
      Couplings(A, i, j, k, c, e);
      double row = (double)Diag(A, c, e);
      for (int m = 0; m < 6; ++m) row += (double)e[m];
      shift += row;
    }
    const int64_t C = dc.idx(I, J, K);
    w0[C] = (TC)CoarseFace(A, 0, I, J, K, series);
    w1[C] = (TC)CoarseFace(A, 1, I, J, K, series);
    w2[C] = (TC)CoarseFace(A, 2, I, J, K, series);
    diag[C] = with_shift ? (TC)shift : (TC)0;
  }
}

// Pass 2: diagonal = shift (from pass 1) minus the sum of the six
// stored coarse couplings (so the row sums of the stored operator are the
// shifts: the constant null space stays exact), and its inverse.
template <class TC>
__global__ void KCoarsenDiag(Op<TC> C, TC* diag, TC* invdiag) {
  TILE_LOOP_BEGIN(C.d)
  TC e[6];
  Couplings(C, i, j, k, c, e);
  double sum = 0;
  for (int m = 0; m < 6; ++m) sum += (double)e[m];
  const double dg = (double)diag[c] - sum;
  diag[c] = (TC)dg;
  invdiag[c] = (TC)(1.0 / dg);
  TILE_LOOP_END
}

// Coarse level `lc` from the fine operator A (both passes).
template <class T, class TC>
void CoarsenOp(cudaStream_t st, const Op<T>& A, Level<TC>& lc, double series, int with_shift) {
  KCoarsenFaces<T, TC><<<TileGrid(lc.d), TileBlock(), 0, st>>>(A, lc.d, lc.w[0], lc.w[1],
                                                                lc.w[2], lc.diag, series,
                                                                with_shift);
  const Op<TC> C{lc.d, lc.w[0], lc.w[1], lc.w[2], nullptr};
  KCoarsenDiag<TC><<<TileGrid(lc.d), TileBlock(), 0, st>>>(C, lc.diag, lc.invdiag);
}

template <class TS, class TD>
__global__ void KConvert(int64_t n, const TS* __restrict__ a, TD* out, double scale) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    out[c] = (TD)((double)a[c] * scale);
}

// Coarsest level: FP64 CG in a single CTA on <= 4096 cells, right-hand side
// mean removed (the periodic operator is singular), solved to a relative
// residual of 1e-13 (or 2000 iterations); the result overwrites xc.
template <class TC>
__global__ void __launch_bounds__(1024) KCoarsestCG(
    Op<TC> A, const TC* __restrict__ bc, TC* xc, double* r, double* p,
    double* ap, double* x, const SolveScalars* s, int singular) {
  if (s && s->done) return;
  const Dims& d = A.d;
  const int n = (int)d.cells();
  const int tid = threadIdx.x;
  __shared__ double red[32];
  __shared__ double bcast;
  auto bsum = [&](double v) -> double {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
      double w = tid < (int)(blockDim.x >> 5) ? red[tid] : 0.0;
      for (int o = 16; o > 0; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
      if (tid == 0) bcast = w;
    }
    __syncthreads();
    const double out = bcast;
    __syncthreads();
    return out;
  };
  double sb = 0;
  for (int c = tid; c < n; c += blockDim.x) sb += (double)bc[c];
  const double mean = singular ? bsum(sb) / n : 0.0;
  double rr = 0;
  for (int c = tid; c < n; c += blockDim.x) {
    const double v = (double)bc[c] - mean;
    r[c] = v;
    p[c] = v;
    x[c] = 0;
    rr += v * v;
  }
  rr = bsum(rr);
  const double stop = rr * 1e-26;
  for (int it = 0; it < 2000 && rr > stop && rr > 0; ++it) {
    double pap = 0;
    for (int c = tid; c < n; c += blockDim.x) {
      const int i = c % d.nx, j = (c / d.nx) % d.ny, k = c / (d.nx * d.ny);
      double e[6];
      {
        TC et[6];
        Couplings(A, i, j, k, c, et);
        for (int q = 0; q < 6; ++q) e[q] = (double)et[q];
      }
      const double e0 = A.diag ? (double)A.diag[c]
                               : -(e[0] + e[1] + e[2] + e[3] + e[4] + e[5]);
      double y = p[c] * e0;
      y += p[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
      y += p[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
      y += p[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
      y += p[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
      y += p[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
      y += p[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
      ap[c] = y;
      pap += p[c] * y;
    }
    pap = bsum(pap);
    if (!(pap > 0)) break;
    const double alpha = rr / pap;
    double rn = 0;
    for (int c = tid; c < n; c += blockDim.x) {
      x[c] += alpha * p[c];
      r[c] -= alpha * ap[c];
      rn += r[c] * r[c];
    }
    rn = bsum(rn);
    const double beta = rn / rr;
    rr = rn;
    for (int c = tid; c < n; c += blockDim.x) p[c] = r[c] + beta * p[c];
    __syncthreads();
  }
  for (int c = tid; c < n; c += blockDim.x) xc[c] = (TC)x[c];
}

// Coarsest level, direct: x = B^{-1} (b - mean(b)) with the precomputed
// dense inverse of B = A + 11^T c (c > 0), which equals the solution of the
// periodic (singular) A x = b - mean(b) with zero mean; for a non-singular
// A (diagonal shifts) B = A and x = A^{-1} b.  FP64 throughout.
template <class TC>
__global__ void __launch_bounds__(1024) KCoarsestDense(int n, const double* __restrict__ binv,
                                                       const TC* __restrict__ bc, TC* xc,
                                                       const SolveScalars* s, int singular) {
  if (s && s->done) return;
  __shared__ double sb[kDenseMax];
  __shared__ double red[32];
  const int tid = threadIdx.x;
  double part = 0;
  for (int c = tid; c < n; c += blockDim.x) {
    const double v = (double)bc[c];
    sb[c] = v;
    part += v;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) red[tid >> 5] = part;
  __syncthreads();
  if (tid == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[0] = singular ? t / n : 0.0;
  }
  __syncthreads();
  const double mean = red[0];
  for (int r = tid; r < n; r += blockDim.x) {
    const double* row = binv + (int64_t)r * n;
    double acc = 0;
    for (int c = 0; c < n; ++c) acc += row[c] * (sb[c] - mean);
    xc[r] = (TC)acc;
  }
}

// r = b - A x (FP64) with reductions r.r, max|r|, b.b; stopping test
// BB: also sum b.b (for aphgpu_residual_norms; the solves do not read it).
// The kernel is bound by FP64 issue on this GPU, so the running max|r| is
// taken on the bit patterns of |r| (integer instructions; for non-negative
// doubles the integer order is the numeric order, NaN skipped as fmax
// does) and the stored -u is u with its sign bit flipped: the same values.
template <bool BB>
__global__ void KResidual64(Op<double> A, const double* __restrict__ b,
                            const double* __restrict__ x, double* r,
                            SolveScalars* s, RedBuf rb, int count_iter,
                            int zero_guess = 0) {
  double v[3] = {0, 0, 0};
  const int op[3] = {0, 1, 0};
  long long amax = 0;  // bits of the largest |r| so far (+0)
  TILE_LOOP_BEGIN(A.d)
  // r = -(x*e0 + e7 + sum x_nb e_q) as linear.ipp:47-53, e7 = -b; with a
  // zero x, r = b (as KCgInit's zero guess: no stencil, no FP64 product)
  double u;
  if (zero_guess) {
    u = -b[c];
  } else {
    double e[6];
    Couplings(A, i, j, k, c, e);
    const double e0 = Diag(A, c, e);
    const Dims& d = A.d;
    u = x[c] * e0 + (-b[c]);
    u += x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
    u += x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
    u += x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
    u += x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
    u += x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
    u += x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  }
  const long long ub = __double_as_longlong(u);
  const double rv = __longlong_as_double(ub ^ (long long)0x8000000000000000ULL);
  if (r) r[c] = rv;
  v[0] += rv * rv;
  const long long ab = ub & 0x7FFFFFFFFFFFFFFFLL;
  if (ab <= 0x7FF0000000000000LL && ab > amax) amax = ab;
  if (BB) v[2] += b[c] * b[c];
  TILE_LOOP_END
  v[1] = __longlong_as_double(amax);
  __shared__ double out[3];
  if (GridReduce<3>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      s->tmp[0] = out[2];
      const double res = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->residual = res;
      if (count_iter) {
        if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
          s->done = 1;
          s->converged = s->residual < s->tol;
        }
      }
    }
  }
}

// x += scale * e
__global__ void KAddCorrection(int64_t n, double* x, const float* __restrict__ e,
                               const SolveScalars* s) {
  const double scale = s->tmp[1];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    x[c] += scale * (double)e[c];
}

// r32 = r / scale with scale = max|r| (s->maxr), stores scale in tmp[1]
__global__ void KScaleResidual(int64_t n, const double* __restrict__ r, float* r32,
                               SolveScalars* s) {
  const double m = s->maxr;
  const double scale = m > 0 ? m : 1.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) s->tmp[1] = scale;
  const double inv = 1.0 / scale;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    r32[c] = (float)(r[c] * inv);
}

__global__ void KZeroF(int64_t n, float* a) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    a[c] = 0.f;
}

// Corrected fluxes: v = p[cm]*k + p[cp]*(-k) + v*, k = -w (proj.ipp:399-403)
__global__ void KFluxCorrect(Dims d, const double* __restrict__ w0,
                             const double* __restrict__ w1,
                             const double* __restrict__ w2,
                             const double* __restrict__ p,
                             const double* __restrict__ vstar, double* out) {
  const int64_t N = d.cells();
  TILE_LOOP_BEGIN(d)
  const double* ws[3] = {w0, w1, w2};
  for (int q = 0; q < 3; ++q) {
    const int64_t cm = q == 0 ? d.idx(wrapm(i - 1, d.nx), j, k)
                     : q == 1 ? d.idx(i, wrapm(j - 1, d.ny), k)
                              : d.idx(i, j, wrapm(k - 1, d.nz));
    const double e0 = -ws[q][c];
    const double e1 = -e0;
    out[q * N + c] = A(A(M(p[cm], e0), M(p[c], e1)), vstar[q * N + c]);
  }
  TILE_LOOP_END
}

// Cell acceleration of Proj::GetAcceleration (proj.ipp:408-433)
__global__ void KAcceleration(Dims d, double h, const double* __restrict__ p,
                              const double* __restrict__ alpha, double rho1,
                              double rho2, const double* __restrict__ febp,
                              double* acc) {
  const int64_t N = d.cells();
  TILE_LOOP_BEGIN(d)
  double sacc[3] = {0, 0, 0};
  for (int q = 0; q < 6; ++q) {
    const int dd = q / 2;
    const int o[3] = {dd == 0, dd == 1, dd == 2};
    int64_t f, cm, cp;
    if (q % 2 == 0) {
      f = c;
      cm = d.idx(wrapm(i - o[0], d.nx), wrapm(j - o[1], d.ny), wrapm(k - o[2], d.nz));
      cp = c;
    } else {
      f = d.idx(wrapp(i + o[0], d.nx), wrapp(j + o[1], d.ny), wrapp(k + o[2], d.nz));
      cm = c;
      cp = f;
    }
    const double am = alpha[cm], ap = alpha[cp];
    const double invm = 1 / A(M(rho1, S(1, am)), M(rho2, am));
    const double invp = 1 / A(M(rho1, S(1, ap)), M(rho2, ap));
    const double rf = 1 / M(A(invp, invm), 0.5);
    const double gp = S(p[cp], p[cm]) / h;
    const double fb = febp ? febp[dd * N + f] : 0.;
    const double a = S(fb, gp) / rf;
    for (int e = 0; e < 3; ++e) sacc[e] = A(sacc[e], M(e == dd ? 1. : 0., M(a, 0.5)));
  }
  acc[3 * c + 0] = sacc[0];
  acc[3 * c + 1] = sacc[1];
  acc[3 * c + 2] = sacc[2];
  TILE_LOOP_END
}

// ---------------------------------------------------------------------------
// Host helpers
// ---------------------------------------------------------------------------


// The FP64 operator of the system.  Its diagonal is always the stored
// array: the explicit one, or minus the sum of the couplings computed once
// per system (KFillDiag, bit-identical to Diag's sum) so that the FP64
// kernels, bound by FP64 issue on this GPU, skip six additions per cell.
Op<double> FineOp(aphgpu_ctx* ctx) {
  return Op<double>{ctx->d, ctx->w[0], ctx->w[1], ctx->w[2],
                    ctx->diag_valid ? ctx->diag : nullptr};
}

int InitScalars(aphgpu_ctx* ctx, SolveScalars* s, const aphgpu_conf* conf,
                double res_scale, double* hist = nullptr, int flags = 0) {
  SolveScalars h{};
  h.hist = hist;
  h.hist_cap = hist ? kHistCap : 0;
  h.flags = flags;
  h.tol = conf->tol;
  h.cellvol = ctx->h * ctx->h * ctx->h;
  h.res_scale = res_scale;
  h.miniter = conf->miniter;
  h.maxiter = conf->maxiter;
  h.maxnorm = conf->maxnorm;
  APH_CUDA(ctx, cudaMemcpyAsync(s, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
  return APHGPU_OK;
}

int ReadScalars(aphgpu_ctx* ctx, const SolveScalars* s, SolveScalars* out) {
  APH_CUDA(ctx, cudaMemcpyAsync(ctx->hscal, s, sizeof(SolveScalars),
                                cudaMemcpyDeviceToHost, ctx->stream));
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = *ctx->hscal;
  return APHGPU_OK;
}

// Weight of the series coupling in the coarse operators (CoarseFace).
inline double CoarseSeries(const aphgpu_ctx* ctx) { return 0.01 * ctx->mg_series_pct; }

// Coarsening: halve while all dimensions are even and the level has more
// than `coarse_max` cells.
std::vector<Dims> LevelDims(Dims d, int coarse_max) {
  std::vector<Dims> v{d};
  while (true) {
    const Dims& c = v.back();
    if (c.cells() <= coarse_max) break;
    if ((c.nx & 1) || (c.ny & 1) || (c.nz & 1)) break;
    if (c.nx < 4 || c.ny < 4 || c.nz < 4) break;
    v.push_back(Dims{c.nx / 2, c.ny / 2, c.nz / 2});
  }
  return v;
}

template <class T>
int AllocLevel(aphgpu_ctx* ctx, Level<T>& L, bool op, bool vec) {
  const int64_t n = L.d.cells();
  if (op) {
    for (int q = 0; q < 3; ++q) APH_TRY(Alloc(ctx, &L.w[q], n));
    APH_TRY(Alloc(ctx, &L.diag, n));
    APH_TRY(Alloc(ctx, &L.invdiag, n));
  }
  if (vec) {
    APH_TRY(Alloc(ctx, &L.x, n));
    APH_TRY(Alloc(ctx, &L.b, n));
  }
  return APHGPU_OK;
}

int EnsureCoarsestScratch(aphgpu_ctx* ctx, int64_t n) {
  auto& mg = ctx->mg;
  if (mg.cr) return APHGPU_OK;
  const int64_t m = std::max<int64_t>(n, 4096);
  APH_TRY(Alloc(ctx, &mg.cr, m));
  APH_TRY(Alloc(ctx, &mg.cp, m));
  APH_TRY(Alloc(ctx, &mg.cap, m));
  APH_TRY(Alloc(ctx, &mg.cx, m));
  APH_TRY(Alloc(ctx, &mg.cb, m));
  return APHGPU_OK;
}

// Dense inverse of the coarsest operator B = A + 11^T c, c = mean(diag)/n,
// by Cholesky on the host (n <= kDenseMax cells; built once per system).
template <class T>
int BuildCoarsestInverse(aphgpu_ctx* ctx, const Level<T>& L, double** dinv, int* dn,
                         int singular) {
  const Dims d = L.d;
  const int n = (int)d.cells();
  if (n > kDenseMax) {
    *dn = 0;
    return APHGPU_OK;
  }
  std::vector<T> w0(n), w1(n), w2(n), dg(n);
  cudaStream_t st = ctx->stream;
  APH_CUDA(ctx, cudaMemcpyAsync(w0.data(), L.w[0], sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaMemcpyAsync(w1.data(), L.w[1], sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaMemcpyAsync(w2.data(), L.w[2], sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  if (L.has_diag)
    APH_CUDA(ctx, cudaMemcpyAsync(dg.data(), L.diag, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  std::vector<double> B((size_t)n * n, 0.0);
  auto at = [&](int r, int c) -> double& { return B[(size_t)r * n + c]; };
  double dsum = 0;
  for (int k = 0; k < d.nz; ++k)
    for (int j = 0; j < d.ny; ++j)
      for (int i = 0; i < d.nx; ++i) {
        const int c = (int)d.idx(i, j, k);
        const int xm = (int)d.idx((i + d.nx - 1) % d.nx, j, k);
        const int xp = (int)d.idx((i + 1) % d.nx, j, k);
        const int ym = (int)d.idx(i, (j + d.ny - 1) % d.ny, k);
        const int yp = (int)d.idx(i, (j + 1) % d.ny, k);
        const int zm = (int)d.idx(i, j, (k + d.nz - 1) % d.nz);
        const int zp = (int)d.idx(i, j, (k + 1) % d.nz);
        const double e[6] = {(double)w0[c], (double)w0[xp], (double)w1[c],
                             (double)w1[yp], (double)w2[c], (double)w2[zp]};
        const int nb[6] = {xm, xp, ym, yp, zm, zp};
        double diag = 0;
        for (int q = 0; q < 6; ++q) {
          at(c, nb[q]) += e[q];
          diag -= e[q];
        }
        if (L.has_diag) diag = (double)dg[c];
        at(c, c) += diag;
        dsum += diag;
      }
  // singular (periodic flux-difference operator, constant null space):
  // invert A + c 11^T instead
  const double cshift = singular ? dsum / n / n : 0.0;
  for (auto& v : B) v += cshift;
  // Cholesky B = L L^T, then B^{-1} column by column
  std::vector<double> Lm((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double sjj = at(j, j);
    for (int k = 0; k < j; ++k) sjj -= Lm[(size_t)j * n + k] * Lm[(size_t)j * n + k];
    if (!(sjj > 0))
      return SetError(ctx, APHGPU_ERR_UNSUPPORTED,
                      "coarsest operator is not positive semidefinite");
    const double ljj = std::sqrt(sjj);
    Lm[(size_t)j * n + j] = ljj;
    for (int i = j + 1; i < n; ++i) {
      double sij = at(i, j);
      for (int k = 0; k < j; ++k) sij -= Lm[(size_t)i * n + k] * Lm[(size_t)j * n + k];
      Lm[(size_t)i * n + j] = sij / ljj;
    }
  }
  std::vector<double> inv((size_t)n * n, 0.0), y(n);
  for (int col = 0; col < n; ++col) {
    for (int i = 0; i < n; ++i) {
      double v = (i == col) ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) v -= Lm[(size_t)i * n + k] * y[k];
      y[i] = v / Lm[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double v = y[i];
      for (int k = i + 1; k < n; ++k) v -= Lm[(size_t)k * n + i] * inv[(size_t)k * n + col];
      inv[(size_t)i * n + col] = v / Lm[(size_t)i * n + i];
    }
  }
  // sized for this level (a context keeps its grid, so n does not grow)
  if (!*dinv || *dn < n) APH_TRY(Alloc(ctx, dinv, (int64_t)n * n));
  APH_CUDA(ctx, cudaMemcpyAsync(*dinv, inv.data(), sizeof(double) * inv.size(),
                                cudaMemcpyHostToDevice, st));
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  *dn = n;
  return APHGPU_OK;
}

// Builds the FP64 (T=double) or FP32 hierarchy from the fine system.
template <class T>
int BuildHierarchy(aphgpu_ctx* ctx, std::vector<Level<T>>& lv, int coarse_max);

// FP16 copy of the finest FP32 couplings for the smoother and the
// restriction (the PCG operator keeps FP32), scaled by the power of two that
// puts the largest magnitude in [2^13, 2^14).  Left out (hscale = 0) for
// systems with an explicit diagonal, for levels the vectorized kernels do not
// handle, and when the smallest nonzero magnitude would leave the FP16
// normal range.
int BuildHalfCouplings(aphgpu_ctx* ctx, Level<float>& L) {
  L.hscale = 0.f;
  if (!ctx->use_half || L.has_diag || !VecOk(L.d)) return APHGPU_OK;
  const int64_t n = L.d.cells();
  cudaStream_t st = ctx->stream;
  const unsigned int init[2] = {0u, 0x7f800000u};
  APH_CUDA(ctx, cudaMemcpyAsync(ctx->flags + 2, init, sizeof(init), cudaMemcpyHostToDevice, st));
  KAbsRange<<<FlatBlocks(n), kFlatThreads, 0, st>>>(n, L.w[0], L.w[1], L.w[2], ctx->flags + 2);
  APH_LAUNCHED(ctx);
  unsigned int r[2] = {0u, 0u};
  APH_CUDA(ctx, cudaMemcpyAsync(r, ctx->flags + 2, sizeof(r), cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  float mx, mn;
  std::memcpy(&mx, &r[0], sizeof(float));
  std::memcpy(&mn, &r[1], sizeof(float));
  if (!(mx > 0.f) || !std::isfinite(mx)) return APHGPU_OK;
  int e = 0;
  std::frexp(mx, &e);
  const float scale = std::ldexp(1.f, 14 - e);
  if (mn * scale < 6.2e-5f) return APHGPU_OK;  // below the FP16 normal range
  for (int q = 0; q < 3; ++q) {
    if (!L.wh[q]) APH_TRY(Alloc(ctx, &L.wh[q], n));
    KToHalf<<<FlatBlocks(n), kFlatThreads, 0, st>>>(n, L.w[q], (__half*)L.wh[q], scale);
    APH_LAUNCHED(ctx);
  }
  L.hscale = scale;
  return APHGPU_OK;
}

template <>
int BuildHierarchy<double>(aphgpu_ctx* ctx, std::vector<Level<double>>& lv,
                           int coarse_max) {
  const auto dims = LevelDims(ctx->d, coarse_max);
  if (dims.back().cells() > 4096)
    return SetError(ctx, APHGPU_ERR_UNSUPPORTED,
                    "multigrid: coarsest level of %lld cells exceeds 4096 "
                    "(grid %dx%dx%d does not coarsen)",
                    (long long)dims.back().cells(), ctx->d.nx, ctx->d.ny, ctx->d.nz);
  if (lv.size() != dims.size()) {
    ctx->mg_epoch += 1;
    lv.assign(dims.size(), Level<double>{});
    for (size_t l = 0; l < dims.size(); ++l) {
      lv[l].d = dims[l];
      if (l > 0) APH_TRY(AllocLevel(ctx, lv[l], true, true));
      lv[l].has_diag = l > 0;
    }
  }
  Level<double>& f = lv[0];
  f.w[0] = ctx->w[0];
  f.w[1] = ctx->w[1];
  f.w[2] = ctx->w[2];
  f.diag = ctx->diag;
  f.has_diag = ctx->diag_valid;
  // the FP64 inverse diagonal, used by this hierarchy's smoother only: made
  // here, with the hierarchy, after every change of the system (the mixed
  // solver's FP32 levels have their own)
  KInvDiag<double><<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(FineOp(ctx), ctx->invdiag);
  APH_LAUNCHED(ctx);
  f.invdiag = ctx->invdiag;
  for (size_t l = 1; l < lv.size(); ++l) {
    const Op<double> A = MakeOp(lv[l - 1]);
    CoarsenOp<double, double>(ctx->stream, A, lv[l], CoarseSeries(ctx),
                              ctx->singular ? 0 : 1);
    ctx->launches += 1;  // two kernels
    APH_LAUNCHED(ctx);
  }
  APH_TRY(EnsureCoarsestScratch(ctx, lv.back().d.cells()));
  ctx->mg.csing64 = ctx->singular ? 1 : 0;
  APH_TRY(BuildCoarsestInverse(ctx, lv.back(), &ctx->mg.cinv64, &ctx->mg.cn64,
                               ctx->mg.csing64));
  return APHGPU_OK;
}

template <>
int BuildHierarchy<float>(aphgpu_ctx* ctx, std::vector<Level<float>>& lv,
                          int coarse_max) {
  const auto dims = LevelDims(ctx->d, coarse_max);
  if (dims.back().cells() > 4096)
    return SetError(ctx, APHGPU_ERR_UNSUPPORTED,
                    "multigrid: coarsest level of %lld cells exceeds 4096",
                    (long long)dims.back().cells());
  if (lv.size() != dims.size()) {
    ctx->mg_epoch += 1;
    lv.assign(dims.size(), Level<float>{});
    for (size_t l = 0; l < dims.size(); ++l) {
      lv[l].d = dims[l];
      APH_TRY(AllocLevel(ctx, lv[l], true, l > 0));
      lv[l].has_diag = true;
    }
  }
  // scratch of the out-of-place fused sweeps, also when the option was
  // switched on after the levels were first allocated
  for (size_t l = 0; l < dims.size(); ++l)
    if (!lv[l].r && (PipeEligible(ctx, dims[l]) || (ctx->fused_mode == 3 && FusedOk(dims[l]))))
      APH_TRY(Alloc(ctx, &lv[l].r, dims[l].cells()));
  // fine FP32 operator from the FP64 system: couplings rounded to FP32;
  // the diagonal is -(sum of the FP32 couplings) for flux-difference
  // systems (keeps the constant null space exact) or the rounded FP64
  // diagonal otherwise
  const int64_t N = ctx->N;
  const int fb = FlatBlocks(N);
  for (int q = 0; q < 3; ++q) {
    KConvert<double, float><<<fb, kFlatThreads, 0, ctx->stream>>>(N, ctx->w[q], lv[0].w[q], 1.0);
    APH_LAUNCHED(ctx);
  }
  if (!lv[0].diag) APH_TRY(Alloc(ctx, &lv[0].diag, N));
  if (!ctx->singular) {
    KConvert<double, float><<<fb, kFlatThreads, 0, ctx->stream>>>(N, ctx->diag, lv[0].diag, 1.0);
    APH_LAUNCHED(ctx);
    const Op<float> A{lv[0].d, lv[0].w[0], lv[0].w[1], lv[0].w[2], lv[0].diag};
    KInvDiag<float><<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(A, lv[0].invdiag);
    APH_LAUNCHED(ctx);
  } else {
    const Op<float> A{lv[0].d, lv[0].w[0], lv[0].w[1], lv[0].w[2], nullptr};
    KInvDiag<float><<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(A, lv[0].invdiag);
    APH_LAUNCHED(ctx);
  }
  lv[0].has_diag = !ctx->singular;
  ctx->mg.wlo_ready = false;
  APH_TRY(BuildHalfCouplings(ctx, lv[0]));
  for (size_t l = 1; l < lv.size(); ++l) {
    // coarse operators from the FP64 fine operator at level 1, FP32 below
    if (l == 1) {
      const Op<double> A = FineOp(ctx);
      CoarsenOp<double, float>(ctx->stream, A, lv[l], CoarseSeries(ctx),
                              ctx->singular ? 0 : 1);
    } else {
      const Op<float> A = MakeOp(lv[l - 1]);
      CoarsenOp<float, float>(ctx->stream, A, lv[l], CoarseSeries(ctx),
                              ctx->singular ? 0 : 1);
    }
    ctx->launches += 1;  // two kernels
    APH_LAUNCHED(ctx);
  }
  APH_TRY(EnsureCoarsestScratch(ctx, lv.back().d.cells()));
  ctx->mg.csing32 = ctx->singular ? 1 : 0;
  APH_TRY(BuildCoarsestInverse(ctx, lv.back(), &ctx->mg.cinv32, &ctx->mg.cn32,
                               ctx->mg.csing32));
  return CoarseOneSetup(ctx);
}

// Launch helpers: the vectorized FP32 kernels where the level allows them.
template <class T>
void LaunchSmooth(aphgpu_ctx* ctx, const Level<T>& f, const Op<T>& A, int color,
                  int zero_init, const SolveScalars* s) {
  KSmooth<T><<<TileGrid(f.d), TileBlock(), 0, ctx->stream>>>(A, f.invdiag, f.b, f.x,
                                                             color, zero_init, s);
}
template <>
void LaunchSmooth<float>(aphgpu_ctx* ctx, const Level<float>& f, const Op<float>& A,
                         int color, int zero_init, const SolveScalars* s) {
  if (f.split) {
    KSmoothSplit<<<SplitGrid(f.d), TileBlock(), 0, ctx->stream>>>(A, f.b, f.x, color, zero_init,
                                                                  s, SplitZ(f.d));
  } else if (VecOk(f.d) && f.wh[0] && f.hscale > 0.f) {
    const Op<__half> H{f.d, (const __half*)f.wh[0], (const __half*)f.wh[1],
                       (const __half*)f.wh[2], nullptr};
    KSmooth4<__half><<<VecGrid(f.d), TileBlock(), 0, ctx->stream>>>(
        H, f.b, f.x, color, zero_init, s, VecZ(f.d), f.hscale);
  } else if (VecOk(f.d)) {
    KSmooth4<float><<<VecGrid(f.d), TileBlock(), 0, ctx->stream>>>(A, f.b, f.x, color,
                                                                   zero_init, s, VecZ(f.d), 1.f);
  } else {
    KSmooth<float><<<TileGrid(f.d), TileBlock(), 0, ctx->stream>>>(A, f.invdiag, f.b, f.x,
                                                                   color, zero_init, s);
  }
}
// n red-black sweeps on level f (first colour c0; zero_first: the first
// sweep starts from a zero guess) with a fused out-of-place kernel,
// alternating between f.x and the level's scratch f.r so that the result
// ends in f.x; in_r: the current values are in f.r (the prolongation wrote
// them there), not in f.x.  Returns kNotFused (nothing launched) where the
// level or the context does not allow it, else APHGPU_OK or the launch
// error.
constexpr int kNotFused = -1;
template <class T>
bool PipeUse(const aphgpu_ctx*, const Level<T>&, const Op<T>&) {
  return false;
}
inline bool WaveUse(aphgpu_ctx* ctx, const Level<float>& f) {
  if (ctx->fused_mode != 5 && ctx->fused_mode != 6) return false;
  if (ctx->fused_mode == 5 && f.d.cells() < kPipeMinCells) return false;
  return WaveDims(f.d, SmCount(ctx));
}
template <>
bool PipeUse<float>(const aphgpu_ctx* ctx, const Level<float>& f, const Op<float>& A) {
  return f.r && !A.diag && PipeEligible(ctx, f.d);
}
template <class T>
int FusedSweeps(aphgpu_ctx*, Level<T>&, const Op<T>&, int, int, bool, const SolveScalars*,
                bool) {
  return kNotFused;
}
template <>
int FusedSweeps<float>(aphgpu_ctx* ctx, Level<float>& f, const Op<float>& A, int n, int c0,
                       bool zero_first, const SolveScalars* s, bool in_r) {
  if (WaveUse(ctx, f) && !in_r && n >= 1) {
    // in place: the result is in f.x after each sweep
    for (int k = 0; k < n; ++k)
      APH_TRY(LaunchWave(ctx, A, f.b, f.x, c0, (k == 0 && zero_first) ? 1 : 0, s,
                         ctx->stream));
    ctx->launches += n;
    return APHGPU_OK;
  }
  const bool pipe = PipeUse<float>(ctx, f, A);
  const bool sync = !pipe && ctx->fused_mode == 3 && f.r && FusedOk(f.d);
  if (n < 1 || !(pipe || sync)) return kNotFused;
  const dim3 g = SweepGrid(f.d);
  const int kz = VecZ(f.d);
  float* in = in_r ? f.r : f.x;
  // outputs: the last sweep writes f.x; a zero-guess first sweep reads
  // nothing, so it may write its input buffer too
  for (int k = 0; k < n; ++k) {
    const bool last_to_x = ((n - 1 - k) % 2) == 0;
    float* out = last_to_x ? f.x : f.r;
    if (out == in && !(k == 0 && zero_first)) out = (in == f.x) ? f.r : f.x;
    const int zero = (k == 0 && zero_first) ? 1 : 0;
    if (pipe) {
      APH_TRY(LaunchPipe(ctx, A, f.b, in, out, c0, zero, s, ctx->stream));
    } else {
      KSweepRB4<<<g, TileBlock(), 0, ctx->stream>>>(A, f.b, in, out, c0, zero, s, kz);
    }
    APH_LAUNCHED(ctx);
    in = out;
  }
  if (in != f.x)
    APH_CUDA(ctx, cudaMemcpyAsync(f.x, in, sizeof(float) * f.d.cells(),
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  return APHGPU_OK;
}

template <class T>
void LaunchProlong(aphgpu_ctx* ctx, const Level<T>& f, const Level<T>& c,
                   const SolveScalars* s) {
  KProlong<T, T><<<TileGrid(f.d), TileBlock(), 0, ctx->stream>>>(f.d, f.x, c.d, c.x, s);
}
// f.r = f.x + the coarse correction (vectorized levels only): the
// prolongation of KProlong4 written out of place, for an odd number of
// fused post-sweeps that then end in f.x without a copy
void LaunchProlongToR(aphgpu_ctx* ctx, const Level<float>& f, const Level<float>& c,
                      const SolveScalars* s) {
  KProlong4To<<<VecGrid(f.d), TileBlock(), 0, ctx->stream>>>(f.d, f.x, f.r, c.d, c.x, s,
                                                             VecZ(f.d));
}
template <>
void LaunchProlong<float>(aphgpu_ctx* ctx, const Level<float>& f, const Level<float>& c,
                          const SolveScalars* s) {
  if (f.split) {
    KProlongSplit<<<SplitGrid(f.d), TileBlock(), 0, ctx->stream>>>(f.d, f.x, c.d, c.x, s,
                                                                   SplitZ(f.d));
  } else if (VecOk(f.d)) {
    KProlong4<<<VecGrid(f.d), TileBlock(), 0, ctx->stream>>>(f.d, f.x, c.d, c.x, s, VecZ(f.d));
  } else {
    KProlong<float, float><<<TileGrid(f.d), TileBlock(), 0, ctx->stream>>>(f.d, f.x, c.d,
                                                                            c.x, s);
  }
}
template <class T>
void LaunchRestrict(aphgpu_ctx* ctx, const Level<T>& f, const Level<T>& c, const Op<T>& A,
                    const SolveScalars* s) {
  KResidualRestrict<T, T><<<TileGrid(c.d), TileBlock(), 0, ctx->stream>>>(A, f.b, f.x, c.d,
                                                                           c.b, s);
}
template <>
void LaunchRestrict<float>(aphgpu_ctx* ctx, const Level<float>& f, const Level<float>& c,
                           const Op<float>& A, const SolveScalars* s) {
  if (f.split) {
    const Dims& dc = c.d;
    int kz = 8;
    const int64_t xy = (int64_t)((f.d.nx / 8 + 31) / 32) * ((dc.ny + 7) / 8);
    while (kz > 1 && xy * ((dc.nz + kz - 1) / kz) < 4 * 152) kz /= 2;
    const dim3 g((f.d.nx / 8 + 31) / 32, (dc.ny + 7) / 8, (dc.nz + kz - 1) / kz);
    KResidualRestrictSplit<<<g, TileBlock(), 0, ctx->stream>>>(A, f.b, f.x, dc, c.b, s, kz);
  } else if (VecOk(f.d)) {
    const int64_t xy = (int64_t)((f.d.nx / 4 + 31) / 32) * ((c.d.ny + 7) / 8);
    int kz = 8;
    while (kz > 1 && xy * ((c.d.nz + kz - 1) / kz) < 4 * 152) kz /= 2;
    const dim3 g((f.d.nx / 4 + 31) / 32, (c.d.ny + 7) / 8, (c.d.nz + kz - 1) / kz);
    if (f.wh[0] && f.hscale > 0.f) {
      const Op<__half> H{f.d, (const __half*)f.wh[0], (const __half*)f.wh[1],
                         (const __half*)f.wh[2], nullptr};
      KResidualRestrict4<__half><<<g, TileBlock(), 0, ctx->stream>>>(H, f.b, f.x, c.d, c.b, s,
                                                                      kz, 1.f / f.hscale);
    } else {
      KResidualRestrict4<float><<<g, TileBlock(), 0, ctx->stream>>>(A, f.b, f.x, c.d, c.b, s,
                                                                     kz, 1.f);
    }
  } else {
    KResidualRestrict<float, float><<<TileGrid(c.d), TileBlock(), 0, ctx->stream>>>(
        A, f.b, f.x, c.d, c.b, s);
  }
}
template <class T>
void LaunchApply(aphgpu_ctx* ctx, const Op<T>& A, const T* p, T* ap, SolveScalars* s) {
  KPcgApply<T><<<TileGrid(A.d), TileBlock(), 0, ctx->stream>>>(A, p, ap, s, ctx->red);
}
template <>
void LaunchApply<float>(aphgpu_ctx* ctx, const Op<float>& A, const float* p, float* ap,
                        SolveScalars* s) {
  const auto& l32 = ctx->mg.l32;
  if (!l32.empty() && l32[0].split && A.w0 == l32[0].w[0]) {
    KPcgApplySplit<<<SplitGrid(A.d), TileBlock(), 0, ctx->stream>>>(A, p, ap, s, ctx->red,
                                                                    SplitZ(A.d));
  } else if (VecOk(A.d)) {
    KPcgApply4<<<VecGrid(A.d), TileBlock(), 0, ctx->stream>>>(A, p, ap, s, ctx->red, VecZ(A.d));
  } else {
    KPcgApply<float><<<TileGrid(A.d), TileBlock(), 0, ctx->stream>>>(A, p, ap, s, ctx->red);
  }
}

template <class T>
void LaunchUpdate(aphgpu_ctx* ctx, Dims d, T* x, T* r, const T* p, const T* ap,
                  SolveScalars* s) {
  KPcgUpdate<T><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, x, r, p, ap, s, ctx->red);
}
template <>
void LaunchUpdate<float>(aphgpu_ctx* ctx, Dims d, float* x, float* r, const float* p,
                         const float* ap, SolveScalars* s) {
  const int64_t n = d.cells();
  if (n % 4 == 0) {
    KPcgUpdate4<<<FlatBlocks(n / 4), kFlatThreads, 0, ctx->stream>>>(n / 4, x, r, p, ap, s,
                                                                     ctx->red, n);
  } else {
    KPcgUpdate<float><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, x, r, p, ap, s, ctx->red);
  }
}
template <class T>
void LaunchDotRZ(aphgpu_ctx* ctx, Dims d, const T* r, const T* z, const T* zold,
                 SolveScalars* s, int first) {
  KDotRZ<T><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, r, z, zold, s, ctx->red, first);
}
template <>
void LaunchDotRZ<float>(aphgpu_ctx* ctx, Dims d, const float* r, const float* z,
                        const float* zold, SolveScalars* s, int first) {
  const int64_t n = d.cells();
  if (n % 4 == 0) {
    KDotRZ4<<<FlatBlocks(n / 4), kFlatThreads, 0, ctx->stream>>>(n / 4, r, z, zold, s, ctx->red,
                                                                 first);
  } else {
    KDotRZ<float><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, r, z, zold, s, ctx->red, first);
  }
}
template <class T>
void LaunchP(aphgpu_ctx* ctx, Dims d, const T* z, T* p, const SolveScalars* s, int first) {
  KPcgP<T><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, z, p, s, first);
}
template <>
void LaunchP<float>(aphgpu_ctx* ctx, Dims d, const float* z, float* p, const SolveScalars* s,
                    int first) {
  const int64_t n = d.cells();
  if (n % 4 == 0) {
    KPcgP4<<<FlatBlocks(n / 4), kFlatThreads, 0, ctx->stream>>>(n / 4, z, p, s, first);
  } else {
    KPcgP<float><<<TileGrid(d), TileBlock(), 0, ctx->stream>>>(d, z, p, s, first);
  }
}

// Cycles of each level below the finest: the context's choice, or W (2)
// on grids of at least 256^3 cells, where the coarse visits are cheap next
// to the finest level, and V (1) below (launch latency dominates there).
inline int CycleGamma(const aphgpu_ctx* ctx) {
  if (ctx->mg_gamma == 1 || ctx->mg_gamma == 2) return ctx->mg_gamma;
  return ctx->N >= (int64_t)256 * 256 * 256 ? 2 : 1;
}

// Growth of the smoothing sweeps below the finest level: the context's
// choice (1 none, 2 linear, 3 doubling), or linear for V-cycles on grids of
// at least 256^3 cells and none otherwise (the extra coarse sweeps are
// cheap next to the finest level there; on small grids their launches cost
// more than the iterations they save, and W-cycles multiply them).
inline int SweepGrowth(const aphgpu_ctx* ctx) {
  if (ctx->mg_growth >= 1 && ctx->mg_growth <= 3) return ctx->mg_growth;
  return CycleGamma(ctx) == 1 && ctx->N >= (int64_t)256 * 256 * 256 ? 2 : 1;
}

// Smoothing sweeps on level l for a configured count n: n on the finest
// level; below it n (growth 1), n * (l + 1) (growth 2, a variable V-cycle
// in the sense of Bramble, Pasciak and Xu) or n * 2^l up to 16 (growth 3).
// More coarse sweeps make the coarse-grid correction more accurate.
inline int LevelSweeps(const aphgpu_ctx* ctx, int n, int l) {
  const int g = SweepGrowth(ctx);
  if (g == 2) return n * (l + 1);
  if (g == 3) return n > 0 ? std::min(n << std::min(l, 4), std::max(n, 16)) : 0;
  return n;
}

// Multigrid cycle from level l: pre-smoothing (from a zero guess on the
// level's first visit of the cycle, else from its current x), restriction
// of the residual, `gamma` cycles of level l+1 (1 from the finest level;
// ctx->mg_gamma below it: 1 V-cycle, 2 W-cycle), prolongation of the
// correction, post-smoothing.  The coarsest level is solved directly.
template <class T>
int CycleLevel(aphgpu_ctx* ctx, std::vector<Level<T>>& lv, int l, bool first, int pre,
               int post, const SolveScalars* s) {
  const int L = (int)lv.size();
  cudaStream_t st = ctx->stream;
  if constexpr (std::is_same<T, float>::value) {
    // the smallest levels in one CTA (no launch per pass)
    if (ctx->use_cta_coarse && l >= 1 && l == ctx->mg.clc && &lv == &ctx->mg.l32) {
      int np[kMgMaxLevels], nq[kMgMaxLevels];
      for (int q = 0; q < kMgMaxLevels; ++q) {
        np[q] = LevelSweeps(ctx, pre, q);
        nq[q] = LevelSweeps(ctx, post, q);
      }
      return CoarseOneLaunch(ctx, np, nq, CycleGamma(ctx), first, s);
    }
  }
  if (l == L - 1) {
    Level<T>& c = lv[L - 1];
    const Op<T> A = MakeOp(c);
    auto& mg = ctx->mg;
    const bool is64 = sizeof(T) == 8;
    const int dn = is64 ? mg.cn64 : mg.cn32;
    const double* dinv = is64 ? mg.cinv64 : mg.cinv32;
    const int sing = is64 ? mg.csing64 : mg.csing32;
    if (dn == (int)c.d.cells() && dinv) {
      KCoarsestDense<T><<<1, dn < 1024 ? ((dn + 31) / 32) * 32 : 1024, 0, st>>>(dn, dinv, c.b,
                                                                             c.x, s, sing);
    } else {
      KCoarsestCG<T><<<1, 1024, 0, st>>>(A, c.b, c.x, mg.cr, mg.cp, mg.cap, mg.cx, s,
                                         ctx->singular ? 1 : 0);
    }
    APH_LAUNCHED(ctx);
    return APHGPU_OK;
  }
  Level<T>& f = lv[l];
  const Op<T> A = MakeOp(f);
  const int np = LevelSweeps(ctx, pre, l), nq = LevelSweeps(ctx, post, l);
  const int fused = np > 0 ? FusedSweeps<T>(ctx, f, A, np, 0, first, s, false) : kNotFused;
  if (fused != kNotFused) APH_TRY(fused);
  for (int sw = 0; fused == kNotFused && sw < np; ++sw) {
    LaunchSmooth<T>(ctx, f, A, 0, first && sw == 0, s);
    APH_LAUNCHED(ctx);
    LaunchSmooth<T>(ctx, f, A, 1, 0, s);
    APH_LAUNCHED(ctx);
  }
  if (np == 0 && first) {
    LaunchSmooth<T>(ctx, f, A, 0, 1, s);
    APH_LAUNCHED(ctx);
    LaunchSmooth<T>(ctx, f, A, 1, 1, s);
    APH_LAUNCHED(ctx);
  }
  LaunchRestrict<T>(ctx, f, lv[l + 1], A, s);
  APH_LAUNCHED(ctx);
  // (a W-cycle's small levels visit theirs once: below 16^3 cells the
  // extra visits cost launches and one-CTA cycles, and buy no iterations)
  const int gamma = (l == 0 || f.d.cells() <= ctx->mg_wmin) ? 1 : CycleGamma(ctx);
  for (int g = 0; g < gamma; ++g) APH_TRY(CycleLevel<T>(ctx, lv, l + 1, g == 0, pre, post, s));
  // an odd number of pipelined post-sweeps starts from f.r, written by the
  // prolongation, and ends in f.x without a copy
  bool in_r = false;
  if constexpr (std::is_same<T, float>::value) {
    in_r = nq % 2 == 1 && PipeUse<float>(ctx, f, A);
    if (in_r) LaunchProlongToR(ctx, f, lv[l + 1], s);
  }
  if (!in_r) LaunchProlong<T>(ctx, f, lv[l + 1], s);
  APH_LAUNCHED(ctx);
  const int fused2 = nq > 0 ? FusedSweeps<T>(ctx, f, A, nq, 1, false, s, in_r) : kNotFused;
  if (fused2 != kNotFused) APH_TRY(fused2);
  for (int sw = 0; fused2 == kNotFused && sw < nq; ++sw) {
    LaunchSmooth<T>(ctx, f, A, 1, 0, s);
    APH_LAUNCHED(ctx);
    LaunchSmooth<T>(ctx, f, A, 0, 0, s);
    APH_LAUNCHED(ctx);
  }
  return APHGPU_OK;
}

// One cycle: lv[0].b -> lv[0].x (zero initial guess).
template <class T>
int VCycle(aphgpu_ctx* ctx, std::vector<Level<T>>& lv, int pre, int post,
           const SolveScalars* s) {
  return CycleLevel<T>(ctx, lv, 0, true, pre, post, s);
}

int SaveHistory(aphgpu_ctx* ctx, const double* d_hist, int n,
                std::vector<double>& out) {
  out.assign(std::min(n, kHistCap), 0.0);
  if (!d_hist || out.empty()) return APHGPU_OK;
  APH_CUDA(ctx, cudaMemcpyAsync(out.data(), d_hist, sizeof(double) * out.size(),
                                cudaMemcpyDeviceToHost, ctx->stream));
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return APHGPU_OK;
}

// Preconditioned CG with operator A and preconditioner `precond(r, z)`
// on vectors x (iterate), r (residual on entry), p, ap, z, zold (zold only
// for the flexible variant); scalars s (tolerances set by the caller).
inline uint64_t Mix(uint64_t h, uint64_t v) {
  h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
  return h;
}

// Preconditioned CG with operator A and preconditioner `precond(r, z)`
// on vectors x (iterate), r (residual on entry), p, ap, z, zold (zold only
// for the flexible variant); scalars s (tolerances set by the caller).
// Batches of `check_every` iterations (even) are captured once into a CUDA
// graph (slot `graph_slot` of the context, -1: no graph) and replayed; the
// host reads the device's stopping flag after each batch.
template <class T, class Precond>
int Pcg(aphgpu_ctx* ctx, const Op<T>& A, Precond precond, T* x, T* r, T* p,
        T* ap, T* z, T* zold, SolveScalars* s, const aphgpu_conf* conf,
        int check_every, int graph_slot = -1) {
  const Dims d = A.d;
  cudaStream_t st = ctx->stream;
  APH_TRY(precond(r, z));
  LaunchDotRZ<T>(ctx, d, r, z, (const T*)nullptr, s, 1);
  APH_LAUNCHED(ctx);
  LaunchP<T>(ctx, d, z, p, s, 1);
  APH_LAUNCHED(ctx);
  auto body = [&]() -> int {
    for (int it = 0; it < check_every; ++it) {
      LaunchApply<T>(ctx, A, p, ap, s);
      APH_LAUNCHED(ctx);
      LaunchUpdate<T>(ctx, d, x, r, p, ap, s);
      APH_LAUNCHED(ctx);
      if (zold) std::swap(z, zold);
      APH_TRY(precond(r, z));
      LaunchDotRZ<T>(ctx, d, r, z, zold, s, 0);
      APH_LAUNCHED(ctx);
      LaunchP<T>(ctx, d, z, p, s, 0);
      APH_LAUNCHED(ctx);
    }
    return APHGPU_OK;
  };
  cudaGraphExec_t exec = nullptr;
  int64_t graph_kernels = 0;
  if (graph_slot >= 0 && ctx->use_graphs && (check_every % 2 == 0 || !zold)) {
    auto& g = ctx->graphs[graph_slot];
    uint64_t key = 1469598103934665603ull;
    const void* ptrs[] = {x, r, p, ap, z, zold, s, A.w0, A.w1, A.w2, A.diag};
    for (const void* q : ptrs) key = Mix(key, (uint64_t)(uintptr_t)q);
    key = Mix(key, (uint64_t)ctx->mg_epoch);
    key = Mix(key, (uint64_t)(conf->mg_pre * 1000 + conf->mg_post));
    key = Mix(key, (uint64_t)check_every);
    key = Mix(key, (uint64_t)sizeof(T));
    key = Mix(key, (uint64_t)ctx->fused_mode);
    key = Mix(key, (uint64_t)ctx->wave_planes);
    key = Mix(key, (uint64_t)CycleGamma(ctx));
    key = Mix(key, (uint64_t)SweepGrowth(ctx));
    key = Mix(key, (uint64_t)ctx->mg_wmin);
    key = Mix(key, (uint64_t)(ctx->use_cta_coarse ? 1 + ctx->mg.clc : 0));
    key = Mix(key, (uint64_t)(!ctx->mg.l32.empty() && ctx->mg.l32[0].split));
    // the FP16 coupling scale is a kernel argument: part of the key
    float hs = ctx->mg.l32.empty() ? 0.f : ctx->mg.l32[0].hscale;
    uint32_t hb;
    std::memcpy(&hb, &hs, sizeof(hb));
    key = Mix(key, (uint64_t)hb);
    if (g.exec && g.key == key) {
      exec = g.exec;
      graph_kernels = g.kernels;
    } else {
      if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
      }
      const int64_t l0 = ctx->launches;
      cudaGraph_t graph = nullptr;
      T* z0 = z;
      T* zo0 = zold;
      bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      int rc = ok ? body() : APHGPU_OK;
      ok = (cudaStreamEndCapture(st, &graph) == cudaSuccess) && ok && rc == APHGPU_OK;
      z = z0;
      zold = zo0;
      ctx->launches = l0;  // captured launches are counted when replayed
      if (ok && cudaGraphInstantiate(&g.exec, graph, 0) == cudaSuccess) {
        g.key = key;
        g.kernels = 0;
        size_t nn = 0;
        if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess) g.kernels = (int64_t)nn;
        exec = g.exec;
        graph_kernels = g.kernels;
      } else {
        g.exec = nullptr;
      }
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
    }
  }
  // iterations are bounded on the device by maxiter (done flag); the host
  // loop gives up after maxiter + 2 batches in any case
  for (int batch = 0; batch <= conf->maxiter / check_every + 2; ++batch) {
    if (exec) {
      APH_CUDA(ctx, cudaGraphLaunch(exec, st));
      ctx->launches += graph_kernels;
    } else {
      APH_TRY(body());
    }
    SolveScalars hs;
    APH_TRY(ReadScalars(ctx, s, &hs));
    if (hs.done) break;
  }
  return APHGPU_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Entry points used by api.cpp
// ---------------------------------------------------------------------------

int EnsureSolverVectors(aphgpu_ctx* ctx) {
  if (ctx->r) return APHGPU_OK;
  const int64_t N = ctx->N;
  APH_TRY(Alloc(ctx, &ctx->r, N));
  APH_TRY(Alloc(ctx, &ctx->p, N));
  APH_TRY(Alloc(ctx, &ctx->ap, N));
  APH_TRY(Alloc(ctx, &ctx->z, N));
  APH_TRY(Alloc(ctx, &ctx->invdiag, N));
  return APHGPU_OK;
}

int SetSystemExprDevice(aphgpu_ctx* ctx, const double* d_expr8) {
  APH_TRY(EnsureSolverVectors(ctx));
  if (!ctx->diag) APH_TRY(Alloc(ctx, &ctx->diag, ctx->N));
  unsigned int* flags = ctx->flags;
  APH_CUDA(ctx, cudaMemsetAsync(flags, 0, 4 * sizeof(unsigned), ctx->stream));
  KExprToSystem<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, d_expr8, ctx->w[0], ctx->w[1], ctx->w[2], ctx->diag, ctx->b, flags);
  APH_LAUNCHED(ctx);
  unsigned int hf[4] = {0, 0, 0, 0};
  APH_CUDA(ctx, cudaMemcpyAsync(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream));
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (hf[0]) {
    ctx->has_system = false;
    return SetError(ctx, APHGPU_ERR_NOT_SYMMETRIC,
                    "system is not symmetric in %u couplings", hf[0]);
  }
  ctx->diag_explicit = hf[1] != 0;
  // singular: every row sum vanishes up to rounding (a flux-difference
  // system, e.g. aphros's projection system summed in its own order)
  ctx->singular = hf[2] == 0;
  // negative definite (every diagonal negative): solved as the negated,
  // positive definite system (the multigrid's smoothers and coarsest
  // solve assume positive diagonals); same solution, same residual norms
  ctx->negated = hf[3] == (unsigned)ctx->N;
  if (ctx->negated) {
    KNegateSystem<<<FlatBlocks(ctx->N), kFlatThreads, 0, ctx->stream>>>(
        ctx->N, ctx->w[0], ctx->w[1], ctx->w[2], ctx->diag, ctx->b);
    APH_LAUNCHED(ctx);
  }
  // diag holds e0: the explicit diagonal, or (flux-difference systems)
  // the value Diag computes from the couplings
  ctx->diag_valid = true;
  ctx->has_system = true;
  ctx->has_proj = false;
  ctx->mg.built64 = ctx->mg.built32 = false;
  return APHGPU_OK;
}

// Proj::ApplyCellCond (proj.ipp:326-338) for given-pressure cells:
// e[0] += 1 and e[7] -= pc, i.e. diag += 1 and b += pc (b = -e[7]), both
// times sign (-1 when the stored system is the negation of the one set);
// each listed cell at most once.
__global__ void KCellCond(int64_t count, const int64_t* __restrict__ cells,
                          const double* __restrict__ values, double* diag, double* b,
                          double sign) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = cells[t];
    diag[c] += sign;
    b[c] += sign * values[t];
  }
}

int ApplyCellCondDevice(aphgpu_ctx* ctx, int64_t count, const int64_t* d_cells,
                        const double* d_values) {
  if (count > 0) {
    KCellCond<<<FlatBlocks(count), kFlatThreads, 0, ctx->stream>>>(
        count, d_cells, d_values, ctx->diag, ctx->b, ctx->negated ? -1.0 : 1.0);
    APH_LAUNCHED(ctx);
  }
  // the diagonal is no longer minus the sum of the couplings: the system is
  // not singular any more, and the FP32 and coarse levels take the stored
  // diagonal
  ctx->diag_explicit = true;
  if (count > 0) ctx->singular = false;
  ctx->mg.built64 = ctx->mg.built32 = false;
  return APHGPU_OK;
}

int AssembleProjectionDevice(aphgpu_ctx* ctx, const double* d_alpha,
                             double rho1, double rho2, const double* d_vflux,
                             const double* d_febp, double dt, int remove_mean) {
  APH_TRY(EnsureSolverVectors(ctx));
  if (!ctx->vstar) APH_TRY(Alloc(ctx, &ctx->vstar, 3 * ctx->N));
  KAssembleFaces<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, d_alpha, rho1, rho2, d_vflux, d_febp, dt, ctx->h, ctx->w[0],
      ctx->w[1], ctx->w[2], ctx->vstar);
  APH_LAUNCHED(ctx);
  double* sum = &ctx->scal->tmp[2];
  KAssembleRhs<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->vstar, ctx->b, ctx->red, sum);
  APH_LAUNCHED(ctx);
  if (remove_mean) {
    KRemoveMean<<<FlatBlocks(ctx->N), kFlatThreads, 0, ctx->stream>>>(ctx->N, ctx->b, sum);
    APH_LAUNCHED(ctx);
  }
  ctx->diag_explicit = false;
  ctx->singular = true;
  ctx->negated = false;
  ctx->diag_valid = false;
  if (!ctx->diag) APH_TRY(Alloc(ctx, &ctx->diag, ctx->N));
  KFillDiag<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(FineOp(ctx), ctx->diag);
  APH_LAUNCHED(ctx);
  ctx->diag_valid = true;
  ctx->has_system = true;
  ctx->has_proj = true;
  ctx->mg.built64 = ctx->mg.built32 = false;
  return APHGPU_OK;
}

int SolveCG(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info) {
  const Op<double> A = FineOp(ctx);
  const Dims d = ctx->d;
  cudaStream_t st = ctx->stream;
  const dim3 tg = TileGrid(d), tb = TileBlock();
  APH_TRY(InitScalars(ctx, ctx->scal, conf, 1.0, ctx->hist));
  KCgInit<<<tg, tb, 0, st>>>(A, ctx->b, ctx->x, ctx->r, ctx->p, 0);
  APH_LAUNCHED(ctx);
  int batch = 4;
  SolveScalars hs{};
  int64_t launched = 0;
  for (;;) {
    for (int it = 0; it < batch; ++it) {
      KCgApply<<<tg, tb, 0, st>>>(A, ctx->r, ctx->p, ctx->ap, ctx->scal, ctx->red);
      APH_LAUNCHED(ctx);
      KCgUpdate<<<tg, tb, 0, st>>>(d, ctx->x, ctx->r, ctx->p, ctx->ap, ctx->scal, ctx->red);
      APH_LAUNCHED(ctx);
      KCgP<<<tg, tb, 0, st>>>(d, ctx->r, ctx->p, ctx->scal);
      APH_LAUNCHED(ctx);
    }
    APH_TRY(ReadScalars(ctx, ctx->scal, &hs));
    launched += batch;
    if (hs.done || launched > (int64_t)conf->maxiter + 2) break;
    batch = std::min(batch * 2, 256);
  }
  APH_TRY(SaveHistory(ctx, ctx->hist, hs.iter, ctx->hist_outer));
  info->residual = hs.residual;
  info->iter = hs.iter;
  info->inner_iter = 0;
  info->converged = hs.converged;
  return APHGPU_OK;
}

int EnsureMixedVectors(aphgpu_ctx* ctx) {
  if (ctx->r32) return APHGPU_OK;
  const int64_t N = ctx->N;
  APH_TRY(Alloc(ctx, &ctx->r32, N));
  APH_TRY(Alloc(ctx, &ctx->x32, N));
  APH_TRY(Alloc(ctx, &ctx->p32, N));
  APH_TRY(Alloc(ctx, &ctx->ap32, N));
  APH_TRY(Alloc(ctx, &ctx->z32, N));
  APH_TRY(Alloc(ctx, &ctx->zold32, N));
  return APHGPU_OK;
}

int EnsureMixedHierarchy(aphgpu_ctx* ctx, const aphgpu_conf* conf) {
  APH_TRY(EnsureMixedVectors(ctx));
  if (!ctx->mg.built32 || ctx->mg.cmax32 != conf->mg_coarse_max) {
    APH_TRY(BuildHierarchy<float>(ctx, ctx->mg.l32, conf->mg_coarse_max));
    ctx->mg.built32 = true;
    ctx->mg.cmax32 = conf->mg_coarse_max;
  }
  return APHGPU_OK;
}

int SolveMGPCG(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info) {
  auto& mg = ctx->mg;
  if (!mg.built64 || mg.cmax64 != conf->mg_coarse_max) {
    APH_TRY(BuildHierarchy<double>(ctx, mg.l64, conf->mg_coarse_max));
    mg.built64 = true;
    mg.cmax64 = conf->mg_coarse_max;
  }
  const Op<double> A = FineOp(ctx);
  cudaStream_t st = ctx->stream;
  APH_TRY(InitScalars(ctx, ctx->scal, conf, 1.0, ctx->hist));
  // r = b - A x0 (x holds the initial guess)
  KResidual64<false><<<TileGrid(ctx->d), TileBlock(), 0, st>>>(A, ctx->b, ctx->x, ctx->r,
                                                               ctx->scal, ctx->red, 0);
  APH_LAUNCHED(ctx);
  auto& lv = mg.l64;
  SolveScalars* s = ctx->scal;
  auto precond = [&](double* r, double* z) -> int {
    lv[0].b = r;
    lv[0].x = z;
    return VCycle(ctx, lv, conf->mg_pre, conf->mg_post, s);
  };
  APH_TRY(Pcg<double>(ctx, A, precond, ctx->x, ctx->r, ctx->p, ctx->ap, ctx->z,
                      (double*)nullptr, s, conf, 2, 0));
  SolveScalars hs;
  APH_TRY(ReadScalars(ctx, s, &hs));
  APH_TRY(SaveHistory(ctx, ctx->hist, hs.iter, ctx->hist_outer));
  info->residual = hs.residual;
  info->iter = hs.iter;
  info->inner_iter = 0;
  info->converged = hs.converged;
  return APHGPU_OK;
}

// FP64 CG with an FP32 V-cycle as preconditioner (z = V32(r) converted).
int SolveMGPCG32(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info) {
  auto& mg = ctx->mg;
  APH_TRY(EnsureMixedVectors(ctx));
  if (!mg.built32 || mg.cmax32 != conf->mg_coarse_max) {
    APH_TRY(BuildHierarchy<float>(ctx, mg.l32, conf->mg_coarse_max));
    mg.built32 = true;
    mg.cmax32 = conf->mg_coarse_max;
  }
  const Op<double> A = FineOp(ctx);
  cudaStream_t st = ctx->stream;
  const int64_t N = ctx->N;
  const int fb = FlatBlocks(N);
  APH_TRY(InitScalars(ctx, ctx->scal, conf, 1.0, ctx->hist));
  KResidual64<false><<<TileGrid(ctx->d), TileBlock(), 0, st>>>(A, ctx->b, ctx->x, ctx->r,
                                                               ctx->scal, ctx->red, 0);
  APH_LAUNCHED(ctx);
  auto& lv = mg.l32;
  lv[0].split = false;
  SolveScalars* s = ctx->scal;
  auto precond = [&](double* r, double* z) -> int {
    KConvert<double, float><<<fb, kFlatThreads, 0, st>>>(N, r, ctx->r32, 1.0);
    APH_LAUNCHED(ctx);
    lv[0].b = ctx->r32;
    lv[0].x = ctx->z32;
    APH_TRY(VCycle(ctx, lv, conf->mg_pre, conf->mg_post, s));
    KConvert<float, double><<<fb, kFlatThreads, 0, st>>>(N, ctx->z32, z, 1.0);
    APH_LAUNCHED(ctx);
    return APHGPU_OK;
  };
  APH_TRY(Pcg<double>(ctx, A, precond, ctx->x, ctx->r, ctx->p, ctx->ap, ctx->z,
                      (double*)nullptr, s, conf, 2, 1));
  SolveScalars hs;
  APH_TRY(ReadScalars(ctx, s, &hs));
  APH_TRY(SaveHistory(ctx, ctx->hist, hs.iter, ctx->hist_outer));
  info->residual = hs.residual;
  info->iter = hs.iter;
  info->inner_iter = 0;
  info->converged = hs.converged;
  return APHGPU_OK;
}

// Relative reduction asked of an inner FP32 solve when the outer residual
// is `residual`: inner_rtol, or only what is left to reach the tolerance
// (times a margin of 0.3 for the difference between the FP32 recursive
// residual and the recomputed FP64 one) when that is less.
inline double InnerReduction(const aphgpu_conf* conf, double residual) {
  double f = conf->inner_rtol;
  if (conf->tol > 0 && residual > 0) f = std::max(f, std::min(0.5, 0.3 * conf->tol / residual));
  return f;
}

int SolveMixed(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info) {
  auto& mg = ctx->mg;
  const int64_t N = ctx->N;
  APH_TRY(EnsureMixedVectors(ctx));
  if (!mg.built32 || mg.cmax32 != conf->mg_coarse_max) {
    APH_TRY(BuildHierarchy<float>(ctx, mg.l32, conf->mg_coarse_max));
    mg.built32 = true;
    mg.cmax32 = conf->mg_coarse_max;
  }
  const Op<double> A = FineOp(ctx);
  const Op<float> A32 = MakeOp(mg.l32[0]);
  cudaStream_t st = ctx->stream;
  const int fb = FlatBlocks(N);
  APH_TRY(InitScalars(ctx, ctx->scal, conf, 1.0));
  ctx->hist_outer.clear();
  ctx->hist_inner.clear();
  SolveScalars hs{};
  int outer = 0, inner_total = 0;
  aphgpu_conf ic = *conf;
  auto& lv = mg.l32;
  // the finest FP32 level in the colour-split order (split.cuh) when the
  // plain red-black smoother runs on it (no fused sweeps, no FP16
  // couplings) and the grid allows it
  const Dims d0 = lv[0].d;
  lv[0].split = (ctx->use_split == 1 || (ctx->use_split == 2 && N >= ((int64_t)1 << 22))) &&
                ctx->fused_mode == 0 && !(lv[0].wh[0] && lv[0].hscale > 0.f) &&
                d0.nx % 8 == 0 && d0.nx >= 16 && d0.ny % 2 == 0 && d0.nz % 2 == 0 &&
                lv.size() >= 2;
  const bool split = lv[0].split;
  const int rb = (int)std::min<int64_t>((int64_t)d0.ny * d0.nz, 32 * SmCount(ctx));
  // after the first outer iteration the residual is updated (r -= s A e)
  // in double-float arithmetic (dfloat.cuh) for flux-difference systems
  const bool df = ctx->singular &&
                  (ctx->use_df == 1 || (ctx->use_df == 2 && N >= ((int64_t)1 << 22)));
  if (df && !mg.wlo_ready) {
    for (int q = 0; q < 3; ++q) {
      if (!mg.wlo[q]) APH_TRY(Alloc(ctx, &mg.wlo[q], N));
      KCouplingLo<<<fb, kFlatThreads, 0, st>>>(N, ctx->w[q], lv[0].w[q], mg.wlo[q]);
      APH_LAUNCHED(ctx);
    }
    mg.wlo_ready = true;
  }
  const PairCouplings W{{lv[0].w[0], lv[0].w[1], lv[0].w[2]}, {mg.wlo[0], mg.wlo[1], mg.wlo[2]}};
  unsigned long long* rp = reinterpret_cast<unsigned long long*>(ctx->r);
  SolveScalars* s2 = ctx->scal2;
  auto precond = [&](float* r, float* z) -> int {
    lv[0].b = r;
    lv[0].x = z;
    return VCycle(ctx, lv, conf->mg_pre, conf->mg_post, s2);
  };
  for (;;) {
    // outer residual in FP64 and the stopping test (r = b for the zero
    // initial guess)
    // (from the second iteration on, the double-float update at the end of
    // the previous one has computed it)
    if (outer == 0 || !df) {
      KResidual64<false><<<TileGrid(ctx->d), TileBlock(), 0, st>>>(
          A, ctx->b, ctx->x, ctx->r, ctx->scal, ctx->red, 1, outer == 0 && ctx->x_zero ? 1 : 0);
      APH_LAUNCHED(ctx);
    }
    APH_TRY(ReadScalars(ctx, ctx->scal, &hs));
    ctx->hist_outer.push_back(hs.residual);
    if (hs.done || (outer >= conf->miniter && hs.residual < conf->tol)) {
      hs.converged = hs.residual < conf->tol;
      break;
    }
    if (outer > conf->maxiter) break;
    // inner FP32 MG-PCG on A e = r / max|r|
    const bool pairs = df && outer > 0;
    if (split && pairs)
      KScaleResidualDFSplit<<<rb, 256, 0, st>>>(d0, rp, ctx->r32, ctx->scal);
    else if (split)
      KScaleResidualSplit<<<rb, 256, 0, st>>>(d0, ctx->r, ctx->r32, ctx->scal);
    else if (pairs)
      KScaleResidualDF<<<fb, kFlatThreads, 0, st>>>(N, rp, ctx->r32, ctx->scal);
    else
      KScaleResidual<<<fb, kFlatThreads, 0, st>>>(N, ctx->r, ctx->r32, ctx->scal);
    APH_LAUNCHED(ctx);
    KZeroF<<<fb, kFlatThreads, 0, st>>>(N, ctx->x32);
    APH_LAUNCHED(ctx);
    const double scale = hs.maxr > 0 ? hs.maxr : 1.0;
    const double r0 = std::sqrt(hs.rr / (ctx->h * ctx->h * ctx->h)) / scale;
    ic.tol = InnerReduction(conf, hs.residual) * r0;
    ic.miniter = 1;
    ic.maxiter = conf->inner_maxiter;
    ic.maxnorm = 0;
    // the constant-mode projection is only valid for the singular
    // flux-difference operator (constant null space), not for systems with
    // an explicit diagonal shift
    const int flags = ctx->singular ? conf->inner_flags : (conf->inner_flags & ~1);
    APH_TRY(InitScalars(ctx, s2, &ic, 1.0, ctx->hist + kHistCap, flags));
    APH_TRY(Pcg<float>(ctx, A32, precond, ctx->x32, ctx->r32, ctx->p32, ctx->ap32,
                       ctx->z32, (conf->inner_flags & 2) ? ctx->zold32 : (float*)nullptr,
                       s2, &ic, 4, 2));
    SolveScalars is;
    APH_TRY(ReadScalars(ctx, s2, &is));
    inner_total += is.iter;
    std::vector<double> h;
    APH_TRY(SaveHistory(ctx, ctx->hist + kHistCap, is.iter, h));
    for (double v : h) ctx->hist_inner.push_back(v / r0);
    ctx->hist_inner.push_back(-1.0);  // separator between inner solves
    ++outer;
    const int it = outer;
    APH_CUDA(ctx, cudaMemcpyAsync(&ctx->scal->iter, &it, sizeof(int),
                                  cudaMemcpyHostToDevice, st));
    if (df) {
      // x += s e and the next residual with its stopping test
      // one CTA per resident slot (the rows are shared out grid-stride)
      auto launch = [&](auto kernel) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess)
          per_sm = 1;
        const int64_t grid = std::min<int64_t>((int64_t)d0.ny * d0.nz,
                                               (int64_t)std::max(per_sm, 1) * SmCount(ctx));
        kernel<<<(unsigned)grid, 256, 0, st>>>(d0, W, ctx->x32, ctx->x, rp, ctx->scal, ctx->red);
      };
      if (outer == 1 && split)
        launch(KCorrectDF<true, true>);
      else if (outer == 1)
        launch(KCorrectDF<true, false>);
      else if (split)
        launch(KCorrectDF<false, true>);
      else
        launch(KCorrectDF<false, false>);
    } else if (split) {
      KAddCorrectionSplit<<<rb, 256, 0, st>>>(d0, ctx->x, ctx->x32, ctx->scal);
    } else {
      KAddCorrection<<<fb, kFlatThreads, 0, st>>>(N, ctx->x, ctx->x32, ctx->scal);
    }
    APH_LAUNCHED(ctx);
    APH_CUDA(ctx, cudaStreamSynchronize(st));
  }
  info->residual = hs.residual;
  info->iter = outer;
  info->inner_iter = inner_total;
  info->converged = hs.converged;
  return APHGPU_OK;
}

int TimeSolverKernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms,
                     double* bytes) {
  cudaStream_t st = ctx->stream;
  const Dims d = ctx->d;
  const double N = (double)ctx->N;
  auto& mg = ctx->mg;
  std::function<void()> launch;
  double b = 0;
  switch (kernel) {
    case APHGPU_K_SMOOTH32: {
      if (!mg.built32 || !ctx->r32)
        return SetError(ctx, APHGPU_ERR_STATE, "run a mixed solve first");
      Level<float>& f = mg.l32[0];
      const Op<float> A = MakeOp(f);
      float* bb = ctx->r32;
      float* x = ctx->z32;
      Level<float> fl = f;
      fl.b = bb;
      fl.x = x;
      launch = [=]() { LaunchSmooth<float>(ctx, fl, A, 0, 0, nullptr); };
      // x read 4 + couplings 12 (6 as FP16) + half of (b 4, invdiag 4,
      // x write 4); colour-split: the other colour's x, the own b and x
      // (2 each) + couplings 12
      b = f.split ? N * 18.0 : N * (4 + (f.hscale > 0.f ? 6 : 12) + 0.5 * 12);
      break;
    }
    case APHGPU_K_SWEEP32: {
      const bool wave = mg.built32 && ctx->r32 && WaveUse(ctx, mg.l32[0]);
      if (!mg.built32 || !ctx->r32 || !(mg.l32[0].r || wave))
        return SetError(ctx, APHGPU_ERR_STATE, "run a mixed solve first (fused level)");
      Level<float>& f = mg.l32[0];
      const Op<float> A = MakeOp(f);
      const float* bb = ctx->r32;
      const float* x = ctx->z32;
      float* xo = f.r;
      const dim3 g = SweepGrid(d);
      const int kz = VecZ(d);
      if (wave) {
        // in place on the solver's scratch vector
        float* xw = ctx->z32;
        launch = [=]() { LaunchWave(ctx, A, bb, xw, 0, 0, nullptr, st); };
      } else if (PipeUse<float>(ctx, f, A)) {
        launch = [=]() { LaunchPipe(ctx, A, bb, x, xo, 0, 0, nullptr, st); };
      } else {
        launch = [=]() {
          KSweepRB4<<<g, TileBlock(), 0, st>>>(A, bb, x, xo, 0, 0, nullptr, kz);
        };
      }
      // couplings 12, b 4, x read 4, x written 4 (once each per full sweep)
      b = N * 24;
      break;
    }
    case APHGPU_K_SMOOTH64: {
      if (!mg.built64) return SetError(ctx, APHGPU_ERR_STATE, "run an MG-PCG solve first");
      Level<double>& f = mg.l64[0];
      const Op<double> A = MakeOp(f);
      const double* iv = ctx->invdiag;
      double* bb = ctx->r;
      double* x = ctx->z;
      launch = [=]() {
        KSmooth<double><<<TileGrid(d), TileBlock(), 0, st>>>(A, iv, bb, x, 0, 0, nullptr);
      };
      b = N * (8 + 24 + 0.5 * 24);
      break;
    }
    case APHGPU_K_APPLY64: {
      const Op<double> A = FineOp(ctx);
      SolveScalars* s = ctx->scal2;
      RedBuf rb = ctx->red;
      const double* p = ctx->p;
      double* ap = ctx->ap;
      APH_CUDA(ctx, cudaMemsetAsync(s, 0, sizeof(SolveScalars), st));
      launch = [=]() { KPcgApply<double><<<TileGrid(d), TileBlock(), 0, st>>>(A, p, ap, s, rb); };
      b = N * (8 + 24 + 8);
      break;
    }
    case APHGPU_K_APPLY32: {
      if (!mg.built32 || !ctx->r32)
        return SetError(ctx, APHGPU_ERR_STATE, "run a mixed solve first");
      const Op<float> A = MakeOp(mg.l32[0]);
      SolveScalars* s = ctx->scal2;
      const float* p = ctx->p32;
      float* ap = ctx->ap32;
      APH_CUDA(ctx, cudaMemsetAsync(s, 0, sizeof(SolveScalars), st));
      launch = [=]() { LaunchApply<float>(ctx, A, p, ap, s); };
      b = N * (4 + 12 + 4);
      break;
    }
    case APHGPU_K_RESTRICT32: {
      if (!mg.built32 || mg.l32.size() < 2 || !ctx->r32)
        return SetError(ctx, APHGPU_ERR_STATE, "run a mixed solve first");
      Level<float>& f = mg.l32[0];
      Level<float>& c = mg.l32[1];
      const Op<float> A = MakeOp(f);
      const float* bb = ctx->r32;
      const float* x = ctx->z32;
      Level<float> fl = f;
      fl.b = (float*)bb;
      fl.x = (float*)x;
      launch = [=]() { LaunchRestrict<float>(ctx, fl, c, A, nullptr); };
      b = N * (4 + 4 + 12) + N / 8 * 4;
      break;
    }
    default:
      return SetError(ctx, APHGPU_ERR_ARG, "unknown kernel %d", kernel);
  }
  launch();  // warm-up
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
  return CheckWave(ctx);
}

int SystemToExprDevice(aphgpu_ctx* ctx, double* d_e8) {
  KSystemToExpr<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      FineOp(ctx), ctx->b, d_e8, ctx->negated ? -1.0 : 1.0);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int ResidualNorms(aphgpu_ctx* ctx, double* rnorm, double* bnorm) {
  aphgpu_conf c;
  aphgpu_conf_default(&c);
  APH_TRY(InitScalars(ctx, ctx->scal2, &c, 1.0));
  KResidual64<true><<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      FineOp(ctx), ctx->b, ctx->x, nullptr, ctx->scal2, ctx->red, 0);
  APH_LAUNCHED(ctx);
  SolveScalars hs;
  APH_TRY(ReadScalars(ctx, ctx->scal2, &hs));
  if (rnorm) *rnorm = std::sqrt(hs.rr);
  if (bnorm) *bnorm = std::sqrt(hs.tmp[0]);
  return APHGPU_OK;
}

int FluxCorrect(aphgpu_ctx* ctx, double* d_out) {
  KFluxCorrect<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->w[0], ctx->w[1], ctx->w[2], ctx->x, ctx->vstar, d_out);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int Acceleration(aphgpu_ctx* ctx, double* d_acc, const double* d_alpha,
                 double rho1, double rho2) {
  KAcceleration<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->h, ctx->x, d_alpha, rho1, rho2,
      ctx->proj_force ? ctx->febp : nullptr, d_acc);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int CheckWave(aphgpu_ctx* ctx) { return CheckWaveFlag(ctx); }

int WaveWaitCheck(aphgpu_ctx* ctx) {
  if (!ctx->wave_buf) APH_TRY(Alloc(ctx, &ctx->wave_buf, kWaveMaxTiles + 1));
  APH_CUDA(ctx, cudaMemsetAsync(ctx->wave_buf, 0xff, sizeof(int), ctx->stream));
  APH_CUDA(ctx, cudaMemsetAsync(ctx->wave_buf + kWaveMaxTiles, 0, sizeof(int), ctx->stream));
  ctx->wave_used = true;
  KWaveWaitProbe<<<1, 32, 0, ctx->stream>>>(ctx->wave_buf, ctx->wave_buf + kWaveMaxTiles);
  APH_LAUNCHED(ctx);
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return CheckWaveFlag(ctx);
}

}  // namespace aphgpu

// The mixed solver's outer residual updated in double-float arithmetic.
//
// After an inner FP32 solve returns the correction e (in units of the
// scale s = max|r|), the defect correction sets x += s e and needs the new
// residual r' = b - A x'.  In exact arithmetic r' = r - s A e, and with A
// the flux-difference operator (every diagonal minus the sum of its row's
// couplings) A e = sum over the six faces of w (e_nb - e_c).  That update
// runs here on the FP32 pipe in double-float ("df64") arithmetic: a value
// is the unevaluated sum hi + lo of two floats (48 significant bits), the
// couplings are held as such pairs (hi: the FP32 couplings of the finest
// multigrid level, lo: the FP32 rounding of w - hi), e_nb - e_c is formed
// exactly by Knuth's TwoSum, products by Dekker's TwoProd with a fused
// multiply-add, sums by TwoSum with the low parts carried (the "sloppy"
// double-double addition of Hida, Li and Bailey, QD library paper, 2001).
// FP64 issues at a small fraction of the FP32 rate on this part: the FP64
// residual kernel is bound by it, this update by memory.
//
// Accuracy: every pair operation is accurate to a few units of 2^-44
// relative to its operands, so |r'(computed) - r'(exact)| is of order
// 2^-44 s |A| |e| <= 2^-44 |A| |e| max|r|, far below the 1e-10 relative
// stopping tolerances this solver serves; x itself is updated in FP64 as
// the plain defect correction does.  The first outer residual (from the
// initial guess) is computed in FP64.
//
// r is kept as (hi, lo) pairs in the FP64 residual array, each element
// read and written through one 64-bit integer pointer (low word hi, high
// word lo), so that no access goes through a second pointer type.
#pragma once

#include "common.cuh"
#include "stencil.cuh"

namespace aphgpu {

struct DF {
  float h, l;
};

// every operation with the _rn intrinsics: never contracted into an FMA
__device__ __forceinline__ DF TwoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ DF FastTwoSum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF DfAdd(DF a, DF b) {
  const DF s = TwoSum(a.h, b.h);
  return FastTwoSum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ DF DfMul(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return FastTwoSum(p, e);
}
__device__ __forceinline__ DF DfNeg(DF a) { return {-a.h, -a.l}; }

__device__ __forceinline__ unsigned long long PackDF(DF a) {
  return ((unsigned long long)__float_as_uint(a.l) << 32) | __float_as_uint(a.h);
}
__device__ __forceinline__ DF UnpackDF(unsigned long long v) {
  return {__uint_as_float((unsigned)(v & 0xffffffffu)), __uint_as_float((unsigned)(v >> 32))};
}
// an FP64 value as a pair (hi: its rounding, lo: the rounding of the rest)
__device__ __forceinline__ DF SplitDouble(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

// position of natural cell (i, j, k) in a vector of the finest FP32 level
// (natural, or colour-split: row halves by colour)
template <bool SPLIT>
__device__ __forceinline__ int64_t LevelIdx(const Dims& d, int i, int j, int k) {
  if (!SPLIT) return d.idx(i, j, k);
  return ((int64_t)k * d.ny + j) * d.nx + (int64_t)((i + j + k) & 1) * (d.nx >> 1) + (i >> 1);
}

struct PairCouplings {
  const float* h[3];
  const float* l[3];
};

// lo parts of the couplings: w - (double)hi rounded to FP32
__global__ void KCouplingLo(int64_t n, const double* __restrict__ w, const float* __restrict__ hi,
                            float* lo) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    lo[c] = __double2float_rn(w[c] - (double)hi[c]);
}

// A normal float widened to FP64 by rearranging its bits (IEEE 754 binary32
// to binary64: exponent rebiased by 1023 - 127, significand shifted by 29),
// exact, with integer instructions; zero, subnormals, infinities and NaN
// by the conversion instruction.
__device__ __forceinline__ double WidenFloat(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  if (ex == 0u || ex == 0xffu) return (double)f;
  const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// x += s e (FP64, as the plain defect correction) and r -= s A e (df64),
// with the norms of the new r and the stopping test of KResidual64
// (count_iter); FIRST: r read as FP64 (the residual of the initial guess).
// CTAs walk the rows grid-stride (the rows in flight at one time are
// consecutive, so their y and z neighbour rows are read by other CTAs at
// about the same time and come from L2), threads the cells of a row (two
// per iteration, their loads issued together); the grid is a few CTAs per
// SM, so the grid reduction is paid once per several hundred cells.
template <bool FIRST, bool SPLIT>
__global__ void __launch_bounds__(256) KCorrectDF(Dims d, PairCouplings W,
                                                  const float* __restrict__ e, double* x,
                                                  unsigned long long* rp, SolveScalars* s,
                                                  RedBuf rb) {
  const double scale = s->tmp[1];
  const DF sc = SplitDouble(scale);
  DF rr = {0.f, 0.f};
  unsigned amax = 0;  // bits of the largest |r| so far (+0)
  const int rows = d.ny * d.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % d.ny, k = row / d.ny;
    const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
    const int km = wrapm(k - 1, d.nz), kp = wrapp(k + 1, d.nz);
#pragma unroll 2
    for (int i = threadIdx.x; i < d.nx; i += blockDim.x) {
      const int64_t c = (int64_t)row * d.nx + i;
      const int im = wrapm(i - 1, d.nx), ip = wrapp(i + 1, d.nx);
      const float ec = e[LevelIdx<SPLIT>(d, i, j, k)];
      const float en[6] = {e[LevelIdx<SPLIT>(d, im, j, k)], e[LevelIdx<SPLIT>(d, ip, j, k)],
                           e[LevelIdx<SPLIT>(d, i, jm, k)], e[LevelIdx<SPLIT>(d, i, jp, k)],
                           e[LevelIdx<SPLIT>(d, i, j, km)], e[LevelIdx<SPLIT>(d, i, j, kp)]};
      const int64_t cw[6] = {c, d.idx(ip, j, k), c, d.idx(i, jp, k), c, d.idx(i, j, kp)};
      DF ae = {0.f, 0.f};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const DF w = {W.h[q >> 1][cw[q]], W.l[q >> 1][cw[q]]};
        ae = DfAdd(ae, DfMul(w, TwoSum(en[q], -ec)));
      }
      const unsigned long long rv = rp[c];
      const DF r0 = FIRST ? SplitDouble(__longlong_as_double((long long)rv)) : UnpackDF(rv);
      const DF r1 = DfAdd(r0, DfNeg(DfMul(sc, ae)));
      rp[c] = PackDF(r1);
      x[c] += scale * WidenFloat(ec);
      rr = DfAdd(rr, DfMul(r1, r1));
      const unsigned ab = __float_as_uint(r1.h) & 0x7fffffffu;
      if (ab <= 0x7f800000u && ab > amax) amax = ab;
    }
  }
  double v[3] = {(double)rr.h + (double)rr.l, (double)__uint_as_float(amax), 0.0};
  const int op[3] = {0, 1, 0};
  __shared__ double out[3];
  if (GridReduce<3>(v, op, rb, out)) {
    if (threadIdx.x == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      const double res = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->residual = res;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
}

// r32 = r / max|r| from the pairs (scale into s->tmp[1]); natural order
__global__ void KScaleResidualDF(int64_t n, const unsigned long long* __restrict__ rp, float* r32,
                                 SolveScalars* s) {
  const double m = s->maxr;
  const double scale = m > 0 ? m : 1.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) s->tmp[1] = scale;
  const float inv = __double2float_rn(1.0 / scale);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    r32[c] = __fmul_rn(UnpackDF(rp[c]).h, inv);
}

// the same into the colour-split order (rows walked by CTAs, a thread a
// natural pair of cells)
__global__ void KScaleResidualDFSplit(Dims d, const unsigned long long* __restrict__ rp,
                                      float* r32, SolveScalars* s) {
  const double m = s->maxr;
  const double scale = m > 0 ? m : 1.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) s->tmp[1] = scale;
  const float inv = __double2float_rn(1.0 / scale);
  const int nh = d.nx >> 1;
  const int rows = d.ny * d.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % d.ny, k = row / d.ny;
    const int h0 = (j + k) & 1;
    const int64_t base = (int64_t)row * d.nx;
    for (int t = threadIdx.x; t < nh; t += blockDim.x) {
      r32[base + (int64_t)h0 * nh + t] = __fmul_rn(UnpackDF(rp[base + 2 * t]).h, inv);
      r32[base + (int64_t)(1 - h0) * nh + t] = __fmul_rn(UnpackDF(rp[base + 2 * t + 1]).h, inv);
    }
  }
}

}  // namespace aphgpu

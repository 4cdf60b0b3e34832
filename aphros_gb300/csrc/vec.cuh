// Vectorized FP32 stencil bodies (nx % 4 == 0) shared by the single-domain
// kernels of poisson.cu and the batched kernels of batch.cu.
//
// Each thread owns 4 consecutive cells in x (one float4) at float4 column q
// and row j, and marches over the planes [kb, ke) in z, keeping the z
// neighbours in registers.  A warp holds 32 / tx row segments of tx
// consecutive columns (tx a power of two <= 32: rows narrower than 32
// float4s do not leave lanes idle); x neighbours across float4 boundaries
// come from warp shuffles within a segment (global loads at segment and
// domain edges, periodic wrap), so every lane of a warp must call a body,
// active or not (act = q < nq and the row is inside the level); a CTA is
// 32 x 8 threads.
#pragma once

#include <cuda_fp16.h>

#include <type_traits>

#include "stencil.cuh"

namespace aphgpu {

__device__ __forceinline__ float4 Ld4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ void St4(float* p, float4 v) {
  *reinterpret_cast<float4*>(p) = v;
}
__device__ __forceinline__ float El(const float4& v, int e) {
  return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}
__device__ __forceinline__ void SetEl(float4& v, int e, float a) {
  if (e == 0) v.x = a; else if (e == 1) v.y = a; else if (e == 2) v.z = a; else v.w = a;
}

// Couplings are FP32, or FP16 scaled by a power of two (the finest-level
// smoother and restriction, Level::wh): loaders to FP32.
__device__ __forceinline__ float ToF(float v) { return v; }
__device__ __forceinline__ float ToF(__half v) { return __half2float(v); }
template <class W>
__device__ __forceinline__ float4 LdW4(const W* p) {
  if constexpr (std::is_same<W, float>::value) {
    return Ld4(p);
  } else {
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
  }
}

// L2 prefetch (PTX prefetch.global.L2): starts the next plane's loads one
// plane early without holding registers; the plane loops are bound by the
// memory round trip per plane, not by bandwidth.
__device__ __forceinline__ void PrefetchL2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Left value (cell 4q-1) and right value (cell 4q+4) of a float4 row segment
// of tx lanes; every lane of the warp must call it (inactive lanes pass
// anything).
template <class W = float>
__device__ __forceinline__ void XHalo(const W* row, float4 v, int q, int nq,
                                      bool act, float& l, float& r, int tx = 32) {
  const int sl = threadIdx.x & (tx - 1);
  l = __shfl_up_sync(0xffffffffu, v.w, 1);
  r = __shfl_down_sync(0xffffffffu, v.x, 1);
  if (act) {
    if (sl == 0 || q == 0) l = ToF(row[q == 0 ? 4 * nq - 1 : 4 * q - 1]);
    if (sl == tx - 1 || q == nq - 1) r = ToF(row[q == nq - 1 ? 0 : 4 * q + 4]);
  }
}

// One red-black half sweep of colour `color` on planes [kb, ke): x = (b -
// sum of the couplings times the neighbours) / diagonal; zero_init: the
// neighbours are taken as zero.  The diagonal is recomputed from the six
// couplings (read anyway) unless the operator stores one.  FP16 couplings
// (W = __half) are scaled by bscale: the update is (bscale b - sum) / diag
// in the scaled units.
template <class W = float>
__device__ __forceinline__ void Smooth4Body(const Op<W>& A, const float* __restrict__ b,
                                            float* x, int color, int zero_init, int q, int j,
                                            int kb, int ke, int tx = 32, float bscale = 1.f) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const bool act = q < nq && j < d.ny;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int i0 = 4 * q;
  float4 xz0 = make_float4(0, 0, 0, 0), xz1 = xz0, xz2 = xz0, wz1 = xz0, wz2 = xz0;
  if (act && !zero_init) {
    xz0 = Ld4(x + d.idx(i0, j, wrapm(kb - 1, d.nz)));
    xz1 = Ld4(x + d.idx(i0, j, kb));
  }
  if (act) wz1 = LdW4(A.w2 + d.idx(i0, j, kb));
  for (int k = kb; k < ke; ++k) {
    const int kp = wrapp(k + 1, d.nz);
    const int64_t c = d.idx(i0, j, k);
    float4 w0v = xz0, w1v = xz0, w1n = xz0, bv = xz0, xjm = xz0, xjp = xz0;
    if (act && k + 1 < ke) {
      // what the next plane loads: couplings, b and the y neighbours of
      // plane k+1, w2 and x of plane k+2
      const int kq = wrapp(kp + 1, d.nz);
      const int64_t cn = d.idx(i0, j, kp);
      PrefetchL2(A.w0 + cn);
      PrefetchL2(A.w1 + cn);
      PrefetchL2(A.w1 + d.idx(i0, jp, kp));
      PrefetchL2(A.w2 + d.idx(i0, j, kq));
      PrefetchL2(b + cn);
      if (!zero_init) {
        PrefetchL2(x + d.idx(i0, j, kq));
        PrefetchL2(x + d.idx(i0, jm, kp));
        PrefetchL2(x + d.idx(i0, jp, kp));
      }
    }
    if (act) {
      wz2 = LdW4(A.w2 + d.idx(i0, j, kp));
      w0v = LdW4(A.w0 + c);
      w1v = LdW4(A.w1 + c);
      w1n = LdW4(A.w1 + d.idx(i0, jp, k));
      bv = Ld4(b + c);
      if (!zero_init) {
        xz2 = Ld4(x + d.idx(i0, j, kp));
        xjm = Ld4(x + d.idx(i0, jm, k));
        xjp = Ld4(x + d.idx(i0, jp, k));
      }
    }
    float xl, xr, wl, wr;
    XHalo(x + d.idx(0, act ? j : 0, k), xz1, q, nq, act && !zero_init, xl, xr, tx);
    XHalo(A.w0 + d.idx(0, act ? j : 0, k), w0v, q, nq, act, wl, wr, tx);
    (void)wl;
    if (act) {
      float4 out = xz1;
      const int e0 = (color + j + k) & 1;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if ((e & 1) != e0) continue;
        const float cxm = El(w0v, e);
        const float cxp = e == 3 ? wr : El(w0v, e + 1);
        const float cym = El(w1v, e), cyp = El(w1n, e);
        const float czm = El(wz1, e), czp = El(wz2, e);
        const float dg = A.diag ? ToF(A.diag[c + e])
                                : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
        float acc = El(bv, e);
        if constexpr (!std::is_same<W, float>::value) acc *= bscale;
        if (!zero_init) {
          const float vxm = e == 0 ? xl : El(xz1, e - 1);
          const float vxp = e == 3 ? xr : El(xz1, e + 1);
          acc -= cxm * vxm;
          acc -= cxp * vxp;
          acc -= cym * El(xjm, e);
          acc -= cyp * El(xjp, e);
          acc -= czm * El(xz0, e);
          acc -= czp * El(xz2, e);
        }
        SetEl(out, e, acc / dg);
      }
      St4(x + c, out);
    }
    xz0 = xz1;
    xz1 = xz2;
    wz1 = wz2;
  }
}

// y = A p on planes [kb, ke); per-thread FP32 sums of p.y (fa0) and of y
// (fa1) are added to the arguments.
__device__ __forceinline__ void Apply4Body(const Op<float>& A, const float* __restrict__ p,
                                           float* ap, int q, int j, int kb, int ke,
                                           float& fa0, float& fa1, int tx = 32) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const bool act = q < nq && j < d.ny;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int i0 = 4 * q;
  float4 z0 = make_float4(0, 0, 0, 0), z1 = z0, z2 = z0, wz1 = z0, wz2 = z0;
  if (act) {
    z0 = Ld4(p + d.idx(i0, j, wrapm(kb - 1, d.nz)));
    z1 = Ld4(p + d.idx(i0, j, kb));
    wz1 = Ld4(A.w2 + d.idx(i0, j, kb));
  }
  for (int k = kb; k < ke; ++k) {
    const int kp = wrapp(k + 1, d.nz);
    const int64_t c = d.idx(i0, j, k);
    float4 w0v = z0, w1v = z0, w1n = z0, pjm = z0, pjp = z0;
    if (act && k + 1 < ke) {
      const int kq = wrapp(kp + 1, d.nz);
      const int64_t cn = d.idx(i0, j, kp);
      PrefetchL2(A.w0 + cn);
      PrefetchL2(A.w1 + cn);
      PrefetchL2(A.w1 + d.idx(i0, jp, kp));
      PrefetchL2(A.w2 + d.idx(i0, j, kq));
      PrefetchL2(p + d.idx(i0, j, kq));
      PrefetchL2(p + d.idx(i0, jm, kp));
      PrefetchL2(p + d.idx(i0, jp, kp));
    }
    if (act) {
      z2 = Ld4(p + d.idx(i0, j, kp));
      wz2 = Ld4(A.w2 + d.idx(i0, j, kp));
      w0v = Ld4(A.w0 + c);
      w1v = Ld4(A.w1 + c);
      w1n = Ld4(A.w1 + d.idx(i0, jp, k));
      pjm = Ld4(p + d.idx(i0, jm, k));
      pjp = Ld4(p + d.idx(i0, jp, k));
    }
    float pl, pr, wl, wr;
    XHalo(p + d.idx(0, act ? j : 0, k), z1, q, nq, act, pl, pr, tx);
    XHalo(A.w0 + d.idx(0, act ? j : 0, k), w0v, q, nq, act, wl, wr, tx);
    (void)wl;
    if (act) {
      float4 out;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float cxm = El(w0v, e);
        const float cxp = e == 3 ? wr : El(w0v, e + 1);
        const float cym = El(w1v, e), cyp = El(w1n, e);
        const float czm = El(wz1, e), czp = El(wz2, e);
        const float dg = A.diag ? A.diag[c + e]
                                : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
        const float pc = El(z1, e);
        float y = pc * dg;
        y += (e == 0 ? pl : El(z1, e - 1)) * cxm;
        y += (e == 3 ? pr : El(z1, e + 1)) * cxp;
        y += El(pjm, e) * cym;
        y += El(pjp, e) * cyp;
        y += El(z0, e) * czm;
        y += El(z2, e) * czp;
        SetEl(out, e, y);
        fa0 += pc * y;
        fa1 += y;
      }
      St4(ap + c, out);
    }
    z0 = z1;
    z1 = z2;
    wz1 = wz2;
  }
}

// x_fine += x_coarse(parent) on fine planes [kb, ke) (one float4 = 2 coarse
// cells)
__device__ __forceinline__ void Prolong4Body(const Dims& d, float* x, const Dims& dc,
                                             const float* __restrict__ xc, int q, int j,
                                             int kb, int ke) {
  const int nq = d.nx >> 2;
  if (q >= nq || j >= d.ny) return;
  for (int k = kb; k < ke; ++k) {
    const int64_t c = d.idx(4 * q, j, k);
    const float2 e = *reinterpret_cast<const float2*>(xc + dc.idx(2 * q, j >> 1, k >> 1));
    float4 v = Ld4(x + c);
    v.x += e.x;
    v.y += e.x;
    v.z += e.y;
    v.w += e.y;
    St4(x + c, v);
  }
}

// Residual b - A x of the fine level summed over the 8 children into the
// coarse right-hand side bc: the thread owns one fine float4 (2 coarse cells
// in x) of coarse row J and marches over the coarse planes [Kb, Ke).
// (FP16 couplings, W = __half: A x is computed in the scaled units and
// multiplied by rscale, the inverse scale)
template <class W = float>
__device__ __forceinline__ void ResidualRestrict4Body(const Op<W>& A,
                                                      const float* __restrict__ b,
                                                      const float* __restrict__ x,
                                                      const Dims& dc, float* bc, int q, int J,
                                                      int Kb, int Ke, int tx = 32,
                                                      float rscale = 1.f) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const bool act = q < nq && J < dc.ny;
  const int i0 = 4 * q;
  for (int K = Kb; K < Ke; ++K) {
    float acc0 = 0.f, acc1 = 0.f;
#pragma unroll
    for (int sub = 0; sub < 4; ++sub) {
      const int j = 2 * J + (sub & 1);
      const int k = 2 * K + (sub >> 1);
      const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
      const int km = wrapm(k - 1, d.nz), kp = wrapp(k + 1, d.nz);
      const int64_t c = d.idx(i0, act ? j : 0, k);
      float4 xv = make_float4(0, 0, 0, 0), w0v = xv;
      if (act) {
        xv = Ld4(x + c);
        w0v = LdW4(A.w0 + c);
      }
      float xl, xr, wl, wr;
      XHalo(x + d.idx(0, act ? j : 0, k), xv, q, nq, act, xl, xr, tx);
      XHalo(A.w0 + d.idx(0, act ? j : 0, k), w0v, q, nq, act, wl, wr, tx);
      (void)wl;
      if (act) {
        const float4 w1v = LdW4(A.w1 + c), w1n = LdW4(A.w1 + d.idx(i0, jp, k));
        const float4 w2v = LdW4(A.w2 + c), w2n = LdW4(A.w2 + d.idx(i0, j, kp));
        const float4 xjm = Ld4(x + d.idx(i0, jm, k)), xjp = Ld4(x + d.idx(i0, jp, k));
        const float4 xkm = Ld4(x + d.idx(i0, j, km)), xkp = Ld4(x + d.idx(i0, j, kp));
        const float4 bv = Ld4(b + c);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float cxm = El(w0v, e);
          const float cxp = e == 3 ? wr : El(w0v, e + 1);
          const float cym = El(w1v, e), cyp = El(w1n, e);
          const float czm = El(w2v, e), czp = El(w2n, e);
          const float dg = A.diag ? ToF(A.diag[c + e])
                                  : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
          float y = El(xv, e) * dg;
          y += (e == 0 ? xl : El(xv, e - 1)) * cxm;
          y += (e == 3 ? xr : El(xv, e + 1)) * cxp;
          y += El(xjm, e) * cym;
          y += El(xjp, e) * cyp;
          y += El(xkm, e) * czm;
          y += El(xkp, e) * czp;
          if constexpr (!std::is_same<W, float>::value) y *= rscale;
          const float rv = El(bv, e) - y;
          if (e < 2) acc0 += rv; else acc1 += rv;
        }
      }
    }
    if (act) *reinterpret_cast<float2*>(bc + dc.idx(2 * q, J, K)) = make_float2(acc0, acc1);
  }
}

// ---------------------------------------------------------------------------
// Fused red-black Gauss-Seidel sweep, out of place: both colours in one pass
// over the level, so the couplings and the right-hand side are read once
// per sweep instead of once per half sweep.
//
// The CTA owns a tile of ncol <= 128 cells (32 float4 lanes) x nrow <= 29
// rows and marches over the planes [kb, ke); its 8 warps take the rows (and
// the two halo rows) in turn.  At plane step m it computes the first
// colour c0 of plane m+1 from x_in (old second-colour values) on its rows,
// on one halo row and one halo column on either side, into a ring of three
// planes in shared memory; then the second colour of plane m from the new
// first-colour values of planes m-1, m, m+1, and writes both colours of
// plane m to x_out.  Halo values are recomputed, not exchanged, and x_in is
// only read, so CTAs never race.  Every value is computed by the same
// operations as the two in-place half sweeps of Smooth4Body.
// Requires nx % 4 == 0, nx >= 8; x_out != x_in.
// ---------------------------------------------------------------------------

constexpr int kSweepRows = 29;  // interior rows of a tile (31 with the halos)
constexpr int kSweepCols = 128 + 2;
typedef float SweepPlanes[3][kSweepRows + 2][kSweepCols];

// Row-segment edges with the loads issued before the shuffles (no second
// round trip to memory): l / r take the neighbours of the float4 from the
// adjacent lanes, or at segment and domain edges from the row in memory.
__device__ __forceinline__ void XEdges(const float* row, int q, int nq, bool act, float& el,
                                       float& er) {
  const int sl = threadIdx.x & 31;
  el = 0.f;
  er = 0.f;
  if (act && (sl == 0 || q == 0)) el = row[q == 0 ? 4 * nq - 1 : 4 * q - 1];
  if (act && (sl == 31 || q == nq - 1)) er = row[q == nq - 1 ? 0 : 4 * q + 4];
}
__device__ __forceinline__ void XHaloPre(float4 v, int q, int nq, bool act, float el, float er,
                                         float& l, float& r) {
  const int sl = threadIdx.x & 31;
  l = __shfl_up_sync(0xffffffffu, v.w, 1);
  r = __shfl_down_sync(0xffffffffu, v.x, 1);
  if (act && (sl == 0 || q == 0)) l = el;
  if (act && (sl == 31 || q == nq - 1)) r = er;
}

// First colour of the float4 at column q, row j, plane p (other positions
// 0); every lane of the warp must call it.  All loads are issued first.
__device__ __forceinline__ float4 FirstColor4(const Op<float>& A, const float* __restrict__ b,
                                              const float* __restrict__ xin, int c0,
                                              int zero_init, int q, int j, int p, bool act) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const int i0 = 4 * q;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int pm = wrapm(p - 1, d.nz), pp = wrapp(p + 1, d.nz);
  const int64_t c = d.idx(i0, act ? j : 0, p);
  const float4 z4 = make_float4(0, 0, 0, 0);
  float4 xc = z4, w0v = z4, w1v = z4, w1n = z4, wz1 = z4, wz2 = z4, bv = z4;
  float4 xjm = z4, xjp = z4, xz0 = z4, xz2 = z4;
  float xel = 0.f, xer = 0.f, wel = 0.f, wer = 0.f;
  const int64_t row = d.idx(0, act ? j : 0, p);
  if (act) {
    w0v = Ld4(A.w0 + c);
    w1v = Ld4(A.w1 + c);
    w1n = Ld4(A.w1 + d.idx(i0, jp, p));
    wz1 = Ld4(A.w2 + c);
    wz2 = Ld4(A.w2 + d.idx(i0, j, pp));
    bv = Ld4(b + c);
    if (!zero_init) {
      xc = Ld4(xin + c);
      xjm = Ld4(xin + d.idx(i0, jm, p));
      xjp = Ld4(xin + d.idx(i0, jp, p));
      xz0 = Ld4(xin + d.idx(i0, j, pm));
      xz2 = Ld4(xin + d.idx(i0, j, pp));
    }
  }
  XEdges(A.w0 + row, q, nq, act, wel, wer);
  if (!zero_init) XEdges(xin + row, q, nq, act, xel, xer);
  float xl, xr, wl, wr;
  XHaloPre(xc, q, nq, act && !zero_init, xel, xer, xl, xr);
  XHaloPre(w0v, q, nq, act, wel, wer, wl, wr);
  (void)wl;
  float4 out = z4;
  if (act) {
    const int e0 = (c0 + j + p) & 1;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if ((e & 1) != e0) continue;
      const float cxm = El(w0v, e);
      const float cxp = e == 3 ? wr : El(w0v, e + 1);
      const float cym = El(w1v, e), cyp = El(w1n, e);
      const float czm = El(wz1, e), czp = El(wz2, e);
      const float dg = A.diag ? A.diag[c + e]
                              : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
      float acc = El(bv, e);
      if (!zero_init) {
        const float vxm = e == 0 ? xl : El(xc, e - 1);
        const float vxp = e == 3 ? xr : El(xc, e + 1);
        acc -= cxm * vxm;
        acc -= cxp * vxp;
        acc -= cym * El(xjm, e);
        acc -= cyp * El(xjp, e);
        acc -= czm * El(xz0, e);
        acc -= czp * El(xz2, e);
      }
      SetEl(out, e, acc / dg);
    }
  }
  return out;
}

// First colour of the single cell (i, j, p), 0 for the second colour.
__device__ __forceinline__ float FirstColor1(const Op<float>& A, const float* __restrict__ b,
                                             const float* __restrict__ xin, int c0,
                                             int zero_init, int i, int j, int p) {
  if (((i + j + p) & 1) != c0) return 0.f;
  const Dims d = A.d;
  const int im = wrapm(i - 1, d.nx), ip = wrapp(i + 1, d.nx);
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int pm = wrapm(p - 1, d.nz), pp = wrapp(p + 1, d.nz);
  const int64_t c = d.idx(i, j, p);
  const float cxm = A.w0[c], cxp = A.w0[d.idx(ip, j, p)];
  const float cym = A.w1[c], cyp = A.w1[d.idx(i, jp, p)];
  const float czm = A.w2[c], czp = A.w2[d.idx(i, j, pp)];
  const float dg = A.diag ? A.diag[c] : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
  float acc = b[c];
  if (!zero_init) {
    acc -= cxm * xin[d.idx(im, j, p)];
    acc -= cxp * xin[d.idx(ip, j, p)];
    acc -= cym * xin[d.idx(i, jm, p)];
    acc -= cyp * xin[d.idx(i, jp, p)];
    acc -= czm * xin[d.idx(i, j, pm)];
    acc -= czp * xin[d.idx(i, j, pp)];
  }
  return acc / dg;
}

// First colour of plane p (unwrapped, kb-1 <= p <= ke) of the tile into
// plane buffer P: rows -1..nrow and columns -1..ncol (shared index +1).
__device__ __forceinline__ void SweepFirstPlane(const Op<float>& A, const float* __restrict__ b,
                                                const float* __restrict__ xin, int c0,
                                                int zero_init, int bx, int j0, int nrow,
                                                int p, float (*P)[kSweepCols]) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const int pw = p < 0 ? p + d.nz : (p >= d.nz ? p - d.nz : p);
  const int lane = threadIdx.x;
  const int q = bx * 32 + lane;
  const bool act = q < nq;
  const int i0 = bx * 128;
  const int ncol = min(128, d.nx - i0);
  // halo columns of rows -1..nrow first: one scalar cell per thread, all
  // loads in flight together
  const int tid = lane + 32 * threadIdx.y;
  if (tid < 2 * (nrow + 2)) {
    const int t = tid >> 1, side = tid & 1;
    const int r = t - 1;
    const int j = r < 0 ? wrapm(j0 - 1, d.ny) : wrapp(j0 + r, d.ny);
    const int ih = side ? wrapp(i0 + ncol, d.nx) : wrapm(i0 - 1, d.nx);
    P[t][side ? ncol + 1 : 0] = FirstColor1(A, b, xin, c0, zero_init, ih, j, pw);
  }
  for (int t = threadIdx.y; t < nrow + 2; t += blockDim.y) {
    const int r = t - 1;
    const int j = r < 0 ? wrapm(j0 - 1, d.ny) : wrapp(j0 + r, d.ny);
    const float4 v = FirstColor4(A, b, xin, c0, zero_init, q, j, pw, act);
    if (act) {
      P[t][4 * lane + 1] = v.x;
      P[t][4 * lane + 2] = v.y;
      P[t][4 * lane + 3] = v.z;
      P[t][4 * lane + 4] = v.w;
    }
  }
}

// One fused sweep over the planes [kb, ke) of tile (bx, by); every thread of
// the 32 x 8 CTA must call it (barriers inside).
__device__ __forceinline__ void SweepRB4Tile(const Op<float>& A, const float* __restrict__ b,
                                             const float* __restrict__ xin, float* xout,
                                             int c0, int zero_init, int bx, int by, int kb,
                                             int ke, SweepPlanes& sF) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const int j0 = by * kSweepRows;
  const int nrow = min(kSweepRows, d.ny - j0);
  const int lane = threadIdx.x;
  const int q = bx * 32 + lane;
  const bool act = q < nq;
  SweepFirstPlane(A, b, xin, c0, zero_init, bx, j0, nrow, kb - 1, sF[0]);
  SweepFirstPlane(A, b, xin, c0, zero_init, bx, j0, nrow, kb, sF[1]);
  __syncthreads();
  for (int m = kb; m < ke; ++m) {
    const int sm = (m - kb) % 3, s0 = (m - kb + 1) % 3, sp = (m - kb + 2) % 3;
    SweepFirstPlane(A, b, xin, c0, zero_init, bx, j0, nrow, m + 1, sF[sp]);
    __syncthreads();
    // second colour of plane m from the new first-colour values
    const int pp = wrapp(m + 1, d.nz);
    for (int rr = threadIdx.y; rr < nrow; rr += blockDim.y) {
      const int j = j0 + rr;
      const int jp = wrapp(j + 1, d.ny);
      const int64_t c = d.idx(4 * q, j, m);
      const float4 z4 = make_float4(0, 0, 0, 0);
      float4 w0v = z4, w1v = z4, w1n = z4, wz1 = z4, wz2 = z4, bv = z4;
      if (act) {
        w0v = Ld4(A.w0 + c);
        w1v = Ld4(A.w1 + c);
        w1n = Ld4(A.w1 + d.idx(4 * q, jp, m));
        wz1 = Ld4(A.w2 + c);
        wz2 = Ld4(A.w2 + d.idx(4 * q, j, pp));
        bv = Ld4(b + c);
      }
      float wel, wer, wl, wr;
      XEdges(A.w0 + d.idx(0, j, m), q, nq, act, wel, wer);
      XHaloPre(w0v, q, nq, act, wel, wer, wl, wr);
      (void)wl;
      if (act) {
        float4 out;
        const int e0 = (c0 + j + m) & 1;  // first-colour positions
        const int r = rr + 1;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int lc = 4 * lane + e + 1;
          if ((e & 1) == e0) {
            SetEl(out, e, sF[s0][r][lc]);
            continue;
          }
          const float cxm = El(w0v, e);
          const float cxp = e == 3 ? wr : El(w0v, e + 1);
          const float cym = El(w1v, e), cyp = El(w1n, e);
          const float czm = El(wz1, e), czp = El(wz2, e);
          const float dg = A.diag ? A.diag[c + e]
                                  : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
          float acc = El(bv, e);
          acc -= cxm * sF[s0][r][lc - 1];
          acc -= cxp * sF[s0][r][lc + 1];
          acc -= cym * sF[s0][r - 1][lc];
          acc -= cyp * sF[s0][r + 1][lc];
          acc -= czm * sF[sm][r][lc];
          acc -= czp * sF[sp][r][lc];
          SetEl(out, e, acc / dg);
        }
        St4(xout + c, out);
      }
    }
    __syncthreads();
  }
}

}  // namespace aphgpu

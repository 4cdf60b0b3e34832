// Colour-split storage of the vectors of the mixed solver's finest FP32
// level (x, b and the inner PCG's vectors).
//
// Row r = j + ny k keeps its cells of colour 0 ((i + j + k) even) in its
// first half and those of colour 1 in its second, each half in increasing
// i: cell (i, j, k) sits at r nx + h nh + (i >> 1), h = (i + j + k) & 1,
// nh = nx / 2.  With nx, ny, nz even the colouring is consistent across the
// periodic boundaries, so every neighbour of a cell has the other colour:
// along y and z at the same position of the neighbouring row's other half,
// along x at the neighbouring positions of the row's own other half.  A
// red-black half sweep then reads the other colour's x and its own b and
// writes its own x, 2 + 2 + 2 bytes per cell beside the 12 of the three
// couplings (kept in the natural order: every face borders one cell of each
// colour, so a half sweep needs all of them): 18 B/cell instead of 24.
//
// Each thread owns 4 consecutive positions m0 .. m0+3 of a half, that is
// the 8 natural cells i0 = 2 m0 .. i0 + 7 of its row for both halves, and
// marches over planes as the natural kernels do.  Every cell is computed
// with the operations of the natural kernels in the same order (Smooth4Body,
// Apply4Body, ResidualRestrict4Body, Prolong4Body), so a half sweep, a
// restriction and a prolongation give the same values; only the FP32
// per-thread partial sums of the inner PCG's dot products group cells
// differently.
// Requires nx % 8 == 0, ny and nz even.
#pragma once

#include "common.cuh"
#include "stencil.cuh"
#include "vec.cuh"

namespace aphgpu {

__device__ __forceinline__ int64_t SplitRow(const Dims& d, int j, int k) {
  return ((int64_t)k * d.ny + j) * d.nx;
}

// element t (0..7) of the pair of float4 (a: elements 0-3, b: 4-7)
__device__ __forceinline__ float El8(const float4& a, const float4& b, int t) {
  return t < 4 ? El(a, t) : El(b, t - 4);
}

// The natural couplings of the 8 cells of a span (row j, plane k, natural
// x from i0) and of the faces above them in y and z, plus the x face after
// the span's last cell (wn: the next span's first, the periodic wrap for
// the row's last span).
struct SplitCoef {
  float4 w0a, w0b, w1a, w1b, w1na, w1nb, w2a, w2b, w2na, w2nb;
  float w0n;
};

// x neighbour values of the own cell e of a half whose cells have parity a
// (natural i = i0 + 2 e + a): the other half's positions m0 + e - 1 + a and
// m0 + e + a.  o: the other half's float4 at m0, ol / or: its values at
// m0 - 1 and m0 + 4.
__device__ __forceinline__ void SplitXNb(const float4& o, float ol, float orr, int a, int e,
                                         float& vxm, float& vxp) {
  if (a == 0) {
    vxm = e == 0 ? ol : El(o, e - 1);
    vxp = El(o, e);
  } else {
    vxm = El(o, e);
    vxp = e == 3 ? orr : El(o, e + 1);
  }
}

// the halo values of the other half's float4 o at positions m0 - 1 and
// m0 + 4 (shuffles within the warp, loads at the warp's and the row's ends,
// periodic); every lane calls it
__device__ __forceinline__ void SplitHalo(const float* half, const float4& o, int q, int nq,
                                          bool act, float& ol, float& orr) {
  const int sl = threadIdx.x & 31;
  ol = __shfl_up_sync(0xffffffffu, o.w, 1);
  orr = __shfl_down_sync(0xffffffffu, o.x, 1);
  if (act) {
    const int nh = 4 * nq;
    if (sl == 0 || q == 0) ol = half[q == 0 ? nh - 1 : 4 * q - 1];
    if (sl == 31 || q == nq - 1) orr = half[q == nq - 1 ? 0 : 4 * q + 4];
  }
}

// the span's couplings (every lane calls it: the shuffle of w0n)
__device__ __forceinline__ void SplitLoadCoef(const Op<float>& A, int q, int nq, int j, int k,
                                              bool act, SplitCoef& C) {
  const Dims d = A.d;
  const int i0 = 8 * q;
  const int jp = wrapp(j + 1, d.ny), kp = wrapp(k + 1, d.nz);
  const float4 z = make_float4(0, 0, 0, 0);
  const int sl = threadIdx.x & 31;
  C.w0a = C.w0b = C.w1a = C.w1b = C.w1na = C.w1nb = C.w2a = C.w2b = C.w2na = C.w2nb = z;
  // the x face after the span at the warp's and the row's ends, loaded with
  // the rest (not after the shuffle: no second round trip)
  float we = 0.f;
  if (act && (sl == 31 || q == nq - 1)) we = A.w0[d.idx(q == nq - 1 ? 0 : i0 + 8, j, k)];
  if (act) {
    const int64_t c = d.idx(i0, j, k);
    C.w0a = Ld4(A.w0 + c);
    C.w0b = Ld4(A.w0 + c + 4);
    C.w1a = Ld4(A.w1 + c);
    C.w1b = Ld4(A.w1 + c + 4);
    const int64_t cy = d.idx(i0, jp, k);
    C.w1na = Ld4(A.w1 + cy);
    C.w1nb = Ld4(A.w1 + cy + 4);
    C.w2a = Ld4(A.w2 + c);
    C.w2b = Ld4(A.w2 + c + 4);
    const int64_t cz = d.idx(i0, j, kp);
    C.w2na = Ld4(A.w2 + cz);
    C.w2nb = Ld4(A.w2 + cz + 4);
  }
  float wn = __shfl_down_sync(0xffffffffu, C.w0a.x, 1);
  if (act && (sl == 31 || q == nq - 1)) wn = we;
  C.w0n = wn;
}

// L2 prefetch of the couplings plane k + 1 of a span reads (w2 one plane
// further: its upper z faces)
__device__ __forceinline__ void SplitPrefetchCoef(const Op<float>& A, int q, int j, int kp,
                                                  int kq) {
  const Dims d = A.d;
  const int64_t cn = d.idx(8 * q, j, kp);
  PrefetchL2(A.w0 + cn);
  PrefetchL2(A.w1 + cn);
  PrefetchL2(A.w1 + d.idx(8 * q, wrapp(j + 1, d.ny), kp));
  PrefetchL2(A.w2 + d.idx(8 * q, j, kq));
}

// the couplings of natural cell t (0..7) of the span: cxm cxp cym cyp czm czp
__device__ __forceinline__ void SplitCoefs(const SplitCoef& C, int t, float& cxm, float& cxp,
                                           float& cym, float& cyp, float& czm, float& czp) {
  cxm = El8(C.w0a, C.w0b, t);
  cxp = t == 7 ? C.w0n : El8(C.w0a, C.w0b, t + 1);
  cym = El8(C.w1a, C.w1b, t);
  cyp = El8(C.w1na, C.w1nb, t);
  czm = El8(C.w2a, C.w2b, t);
  czp = El8(C.w2na, C.w2nb, t);
}

// One red-black half sweep of colour `color` (Smooth4Body's update) on the
// split level; zero_init: the other colour taken as zero.
__global__ void __launch_bounds__(256, 3) KSmoothSplit(Op<float> A, const float* __restrict__ b,
                                                    float* x, int color, int zero_init,
                                                    const SolveScalars* s, int kz) {
  if (s && s->done) return;
  const Dims d = A.d;
  const int nh = d.nx >> 1, nq = nh >> 2;
  const int q = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * kz, ke = min(kb + kz, d.nz);
  const bool act = q < nq && j < d.ny;
  const int jj = act ? j : 0;
  const int jm = wrapm(jj - 1, d.ny), jp = wrapp(jj + 1, d.ny);
  const int m0 = 4 * q;
  const int64_t oo = (int64_t)(1 - color) * nh + m0;  // the other half at m0
  const int64_t ow = (int64_t)color * nh + m0;        // the own half at m0
  const float4 z = make_float4(0, 0, 0, 0);
  float4 o0 = z, o1 = z, o2 = z;  // the other colour at planes k-1, k, k+1
  if (act && !zero_init) {
    o0 = Ld4(x + SplitRow(d, jj, wrapm(kb - 1, d.nz)) + oo);
    o1 = Ld4(x + SplitRow(d, jj, kb) + oo);
  }
  for (int k = kb; k < ke; ++k) {
    const int kp = wrapp(k + 1, d.nz);
    if (act && k + 1 < ke) {
      // what the next plane loads
      const int kq = wrapp(kp + 1, d.nz);
      SplitPrefetchCoef(A, q, jj, kp, kq);
      PrefetchL2(b + SplitRow(d, jj, kp) + ow);
      if (!zero_init) {
        PrefetchL2(x + SplitRow(d, jj, kq) + oo);
        PrefetchL2(x + SplitRow(d, jm, kp) + oo);
        PrefetchL2(x + SplitRow(d, jp, kp) + oo);
      }
    }
    float4 oym = z, oyp = z, bv = z;
    if (act) {
      bv = Ld4(b + SplitRow(d, jj, k) + ow);
      if (!zero_init) {
        o2 = Ld4(x + SplitRow(d, jj, kp) + oo);
        oym = Ld4(x + SplitRow(d, jm, k) + oo);
        oyp = Ld4(x + SplitRow(d, jp, k) + oo);
      }
    }
    SplitCoef C;
    SplitLoadCoef(A, q, nq, jj, k, act, C);
    float ol, orr;
    SplitHalo(x + SplitRow(d, jj, k) + (int64_t)(1 - color) * nh, o1, q, nq, act && !zero_init,
              ol, orr);
    if (act) {
      const int a = (color + j + k) & 1;
      const int64_t c0 = d.idx(8 * q, j, k);
      float4 out;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int t = 2 * e + a;
        float cxm, cxp, cym, cyp, czm, czp;
        SplitCoefs(C, t, cxm, cxp, cym, cyp, czm, czp);
        const float dg = A.diag ? A.diag[c0 + t]
                                : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
        float acc = El(bv, e);
        if (!zero_init) {
          float vxm, vxp;
          SplitXNb(o1, ol, orr, a, e, vxm, vxp);
          acc -= cxm * vxm;
          acc -= cxp * vxp;
          acc -= cym * El(oym, e);
          acc -= cyp * El(oyp, e);
          acc -= czm * El(o0, e);
          acc -= czp * El(o2, e);
        }
        SetEl(out, e, acc / dg);
      }
      St4(x + SplitRow(d, j, k) + ow, out);
    }
    o0 = o1;
    o1 = o2;
  }
}

// A p of both halves of the span (Apply4Body's operations per cell) with
// per-thread sums of p.(A p) and A p.
__device__ __forceinline__ void SplitApplySpan(const Op<float>& A, const float* p, int q,
                                               int nq, int j, int k, bool act,
                                               const float4 (&pz0)[2], const float4 (&pz1)[2],
                                               const float4 (&pz2)[2], float4 (&y)[2]) {
  const Dims d = A.d;
  const int nh = d.nx >> 1;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const float4 z = make_float4(0, 0, 0, 0);
  float4 pym[2] = {z, z}, pyp[2] = {z, z};
  if (act) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      pym[h] = Ld4(p + SplitRow(d, jm, k) + (int64_t)h * nh + 4 * q);
      pyp[h] = Ld4(p + SplitRow(d, jp, k) + (int64_t)h * nh + 4 * q);
    }
  }
  SplitCoef C;
  SplitLoadCoef(A, q, nq, j, k, act, C);
  float ol[2], orr[2];
#pragma unroll
  for (int h = 0; h < 2; ++h)
    SplitHalo(p + SplitRow(d, j, k) + (int64_t)h * nh, pz1[h], q, nq, act, ol[h], orr[h]);
  y[0] = y[1] = z;
  if (!act) return;
  const int64_t c0 = d.idx(8 * q, j, k);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int a = (h + j + k) & 1;
    const int oh = 1 - h;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int t = 2 * e + a;
      float cxm, cxp, cym, cyp, czm, czp;
      SplitCoefs(C, t, cxm, cxp, cym, cyp, czm, czp);
      const float dg = A.diag ? A.diag[c0 + t]
                              : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
      float vxm, vxp;
      SplitXNb(pz1[oh], ol[oh], orr[oh], a, e, vxm, vxp);
      const float pc = El(pz1[h], e);
      float v = pc * dg;
      v += vxm * cxm;
      v += vxp * cxp;
      v += El(pym[oh], e) * cym;
      v += El(pyp[oh], e) * cyp;
      v += El(pz0[oh], e) * czm;
      v += El(pz2[oh], e) * czp;
      SetEl(y[h], e, v);
    }
  }
}

// ap = A p on the split level, with the grid sums of p.Ap and Ap into s
// (KPcgApply4's results)
__global__ void __launch_bounds__(256, 2) KPcgApplySplit(Op<float> A, const float* __restrict__ p,
                                                      float* ap, SolveScalars* s, RedBuf rb,
                                                      int kz) {
  if (s->done) return;
  const Dims d = A.d;
  const int nh = d.nx >> 1, nq = nh >> 2;
  const int q = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * kz, ke = min(kb + kz, d.nz);
  const bool act = q < nq && j < d.ny;
  const int jj = act ? j : 0;
  const float4 z = make_float4(0, 0, 0, 0);
  float4 pz0[2] = {z, z}, pz1[2] = {z, z}, pz2[2] = {z, z};
  if (act) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      pz0[h] = Ld4(p + SplitRow(d, jj, wrapm(kb - 1, d.nz)) + (int64_t)h * nh + 4 * q);
      pz1[h] = Ld4(p + SplitRow(d, jj, kb) + (int64_t)h * nh + 4 * q);
    }
  }
  float fa0 = 0.f, fa1 = 0.f;
  const int jm = wrapm(jj - 1, d.ny), jp = wrapp(jj + 1, d.ny);
  for (int k = kb; k < ke; ++k) {
    const int kp = wrapp(k + 1, d.nz);
    if (act && k + 1 < ke) {
      const int kq = wrapp(kp + 1, d.nz);
      SplitPrefetchCoef(A, q, jj, kp, kq);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t off = (int64_t)h * nh + 4 * q;
        PrefetchL2(p + SplitRow(d, jj, kq) + off);
        PrefetchL2(p + SplitRow(d, jm, kp) + off);
        PrefetchL2(p + SplitRow(d, jp, kp) + off);
      }
    }
    if (act) {
#pragma unroll
      for (int h = 0; h < 2; ++h)
        pz2[h] = Ld4(p + SplitRow(d, jj, kp) + (int64_t)h * nh + 4 * q);
    }
    float4 y[2];
    SplitApplySpan(A, p, q, nq, jj, k, act, pz0, pz1, pz2, y);
    if (act) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        St4(ap + SplitRow(d, j, k) + (int64_t)h * nh + 4 * q, y[h]);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          fa0 += El(pz1[h], e) * El(y[h], e);
          fa1 += El(y[h], e);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      pz0[h] = pz1[h];
      pz1[h] = pz2[h];
    }
  }
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

// The residual b - A x of the split fine level summed over the 8 children
// of each coarse cell into the natural coarse right-hand side bc (the
// children's order of ResidualRestrict4Body: per fine row and plane of the
// coarse cell, x-first then x-second).  A thread owns the 4 coarse cells
// I = m0 .. m0+3 of coarse row J (the fine positions m0 .. m0+3 of both
// halves of the 4 fine rows) and marches over coarse planes.
__global__ void __launch_bounds__(256, 2) KResidualRestrictSplit(Op<float> A,
                                                              const float* __restrict__ b,
                                                              const float* __restrict__ x,
                                                              Dims dc, float* bc,
                                                              const SolveScalars* s, int kz) {
  if (s && s->done) return;
  const Dims d = A.d;
  const int nh = d.nx >> 1, nq = nh >> 2;
  const int q = blockIdx.x * 32 + threadIdx.x;
  const int J = blockIdx.y * 8 + threadIdx.y;
  const int Kb = blockIdx.z * kz, Ke = min(Kb + kz, dc.nz);
  const bool act = q < nq && J < dc.ny;
  const int JJ = act ? J : 0;
  const float4 z = make_float4(0, 0, 0, 0);
  for (int K = Kb; K < Ke; ++K) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int sub = 0; sub < 4; ++sub) {
      const int j = 2 * JJ + (sub & 1);
      const int k = 2 * K + (sub >> 1);
      const int km = wrapm(k - 1, d.nz), kp = wrapp(k + 1, d.nz);
      float4 xz0[2] = {z, z}, xz1[2] = {z, z}, xz2[2] = {z, z}, bv[2] = {z, z};
      if (act) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int64_t off = (int64_t)h * nh + 4 * q;
          xz0[h] = Ld4(x + SplitRow(d, j, km) + off);
          xz1[h] = Ld4(x + SplitRow(d, j, k) + off);
          xz2[h] = Ld4(x + SplitRow(d, j, kp) + off);
          bv[h] = Ld4(b + SplitRow(d, j, k) + off);
        }
      }
      float4 y[2];
      SplitApplySpan(A, x, q, nq, j, k, act, xz0, xz1, xz2, y);
      if (act) {
        // the natural cells 2I and 2I + 1 of coarse cell I = m0 + e: half
        // h0 = (j + k) & 1 holds 2I, the other half 2I + 1
        const int h0 = (j + k) & 1;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          acc[e] += El(bv[h0], e) - El(y[h0], e);
          acc[e] += El(bv[1 - h0], e) - El(y[1 - h0], e);
        }
      }
    }
    if (act)
      St4(bc + dc.idx(4 * q, J, K), make_float4(acc[0], acc[1], acc[2], acc[3]));
  }
}

// x_fine += x_coarse(parent) on the split fine level (Prolong4Body's
// additions): fine positions m0 .. m0+3 of both halves have the coarse
// parents I = m0 .. m0+3 of coarse row (j / 2, k / 2).
__global__ void KProlongSplit(Dims d, float* x, Dims dc, const float* __restrict__ xc,
                              const SolveScalars* s, int kz) {
  if (s && s->done) return;
  const int nh = d.nx >> 1, nq = nh >> 2;
  const int q = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int kb = blockIdx.z * kz, ke = min(kb + kz, d.nz);
  if (q >= nq || j >= d.ny) return;
  for (int k = kb; k < ke; ++k) {
    const float4 e = Ld4(xc + dc.idx(4 * q, j >> 1, k >> 1));
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float* p = x + SplitRow(d, j, k) + (int64_t)h * nh + 4 * q;
      float4 v = Ld4(p);
      v.x += e.x;
      v.y += e.y;
      v.z += e.z;
      v.w += e.w;
      St4(p, v);
    }
  }
}

// r32 (split) = r (natural) / scale with scale = max|r| (KScaleResidual's
// operations; scale into s->tmp[1]); a CTA walks rows, a thread a natural
// pair (2 t, 2 t + 1), whose cells sit at position t of the two halves
__global__ void KScaleResidualSplit(Dims d, const double* __restrict__ r, float* r32,
                                    SolveScalars* s) {
  const double m = s->maxr;
  const double scale = m > 0 ? m : 1.0;
  if (blockIdx.x == 0 && threadIdx.x == 0) s->tmp[1] = scale;
  const double inv = 1.0 / scale;
  const int nh = d.nx >> 1;
  const int rows = d.ny * d.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % d.ny, k = row / d.ny;
    const int h0 = (j + k) & 1;
    const int64_t base = (int64_t)row * d.nx;
    for (int t = threadIdx.x; t < nh; t += blockDim.x) {
      const double2 v = *reinterpret_cast<const double2*>(r + base + 2 * t);
      r32[base + (int64_t)h0 * nh + t] = (float)(v.x * inv);
      r32[base + (int64_t)(1 - h0) * nh + t] = (float)(v.y * inv);
    }
  }
}

// x (natural) += scale e (split) (KAddCorrection's operation)
__global__ void KAddCorrectionSplit(Dims d, double* x, const float* __restrict__ e,
                                    const SolveScalars* s) {
  const double scale = s->tmp[1];
  const int nh = d.nx >> 1;
  const int rows = d.ny * d.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % d.ny, k = row / d.ny;
    const int h0 = (j + k) & 1;
    const int64_t base = (int64_t)row * d.nx;
    for (int t = threadIdx.x; t < nh; t += blockDim.x) {
      double2 v = *reinterpret_cast<double2*>(x + base + 2 * t);
      v.x += scale * (double)e[base + (int64_t)h0 * nh + t];
      v.y += scale * (double)e[base + (int64_t)(1 - h0) * nh + t];
      *reinterpret_cast<double2*>(x + base + 2 * t) = v;
    }
  }
}

}  // namespace aphgpu

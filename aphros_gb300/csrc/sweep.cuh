// Fused red-black Gauss-Seidel sweep, out of place, fed by asynchronous bulk
// copies (TMA) into shared memory.
//
// One sweep updates the first colour c0 of every cell from the old values
// x_in of the other colour, then the second colour from the new first-colour
// values, and writes both colours to x_out (x_out != x_in).  Per full sweep
// every array is read once from HBM: x_in, the three couplings w0 w1 w2 and
// b (FP32), and x_out is written once: 24 bytes per cell.
//
// Work item: a tile of w <= 128 columns (x) by rows <= kPipeRows rows (y),
// marching over the planes [kb, ke) (z).  One CTA of 512 threads per SM; the
// host sizes the tiles so that all items run in one wave, so neighbouring
// tiles stream the same planes at the same time and the halo rows one tile
// reads again come from L2.
//
// Pipeline (time step t = kb-1 .. ke): F(t), the first colour of plane t on
// the tile's rows -1..rows and columns -1..w (halo recomputed, never
// exchanged), into a ring of three planes in shared memory; then S(t-1), the
// second colour of plane t-1, written with the first colour of that plane
// to x_out.  The data F(t) needs beyond earlier steps -- x_in of plane t+1,
// w0 w1 b of plane t, w2 of plane t+1 -- arrive as batch B(t): one row
// segment per array row, copied by cp.async.bulk from global to shared
// memory with completion on an mbarrier.  Batch B(t+2) is issued at the
// start of step t, so two planes of loads are in flight while a plane is
// computed.  Row segments span columns [i0-4, i0+w+4) (16-byte aligned);
// the periodic wrap in x splits a segment into two or three copies, the
// wrap in y and z only changes which row is copied.
//
// Every value is computed by the same operations, in the same order, as in
// the two in-place half sweeps (Smooth4Body), so results are bit-identical.
// Requires: nx % 4 == 0, nx >= 16, no stored diagonal (the diagonal is
// minus the sum of the couplings, as for the projection operator).
//
// Waits are bounded: a batch that does not complete within the limit sets
// *err, the CTA waits (bounded again) for the copies it issued and returns.
#pragma once

#include <cstdint>

#include "stencil.cuh"
#include "vec.cuh"

namespace aphgpu {

constexpr int kPipeCols = 128;                // columns of a tile at most
constexpr int kPipeRows = 14;                 // rows of a tile at most
constexpr int kPipeStride = kPipeCols + 8;    // floats per staged row
constexpr int kPipeThreads = 512;
constexpr int kPipeXs = 5, kPipeCs = 4, kPipeWs = 5, kPipeBars = 3;  // ring sizes
constexpr int kPipeXRows = kPipeRows + 4;     // x_in rows -2 .. rows+1
constexpr int kPipeW0Rows = kPipeRows + 2;    // w0 rows -1 .. rows
constexpr int kPipeW1Rows = kPipeRows + 3;    // w1 rows -1 .. rows+1
constexpr int kPipeBRows = kPipeRows + 2;     // b rows -1 .. rows
constexpr int kPipeCRows = kPipeW0Rows + kPipeW1Rows + kPipeBRows;
constexpr int kPipeW2Rows = kPipeRows + 2;    // w2 rows -1 .. rows
constexpr int kPipeFRows = kPipeRows + 2;     // first colour rows -1 .. rows
constexpr int kPipeSmemFloats =
    kPipeStride * (kPipeXs * kPipeXRows + kPipeCs * kPipeCRows + kPipeWs * kPipeW2Rows +
                   3 * kPipeFRows);
constexpr int kPipeSmemBytes = kPipeSmemFloats * 4 + kPipeBars * 8;
// iterations of mbarrier.try_wait (each may suspend the thread for a while)
// before a batch is given up
constexpr int kPipeWaitLimit = 1 << 22;

struct PipeTiling {
  int w;       // columns of a tile (multiple of 4, <= kPipeCols)
  int rows;    // rows of a band (<= kPipeRows)
  int xtiles, bands, zsegs;
};

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void MbarInit(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(SmemAddr(bar)), "r"(count));
}

__device__ __forceinline__ void MbarExpectTx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(SmemAddr(bar)),
               "r"(bytes)
               : "memory");
}

// true once the phase of `parity` has completed; false after the limit
__device__ __forceinline__ bool MbarWait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = SmemAddr(bar);
  for (int it = 0; it < kPipeWaitLimit; ++it) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 1-D bulk copy global -> shared, completion counted on `bar` (bytes: a
// multiple of 16, both addresses 16-byte aligned)
__device__ __forceinline__ void BulkG2S(void* dst, const void* src, uint32_t bytes,
                                        uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(SmemAddr(dst)), "l"(src), "r"(bytes), "r"(SmemAddr(bar))
      : "memory");
}

// Copies the periodic column range [i0-4, i0+w+4) of one row (row: the
// row's first element in global memory) to dst (the staged row, local
// column 0 = global column i0-4); one, two or three bulk copies.
__device__ __forceinline__ void CopyRowSegment(float* dst, const float* row, int nx, int i0,
                                               int w, uint64_t* bar) {
  int s = i0 - 4;
  int left = w + 8;
  int off = 0;
  if (s < 0) s += nx;
  while (left > 0) {
    const int n = min(left, nx - s);
    BulkG2S(dst + off, row + s, 4u * (uint32_t)n, bar);
    off += n;
    left -= n;
    s = 0;
  }
}

struct PipeSmem {
  float* xs;   // [kPipeXs][kPipeXRows][stride]
  float* cs;   // [kPipeCs][kPipeCRows][stride]: w0, w1, b
  float* ws;   // [kPipeWs][kPipeW2Rows][stride]
  float* fs;   // [3][kPipeFRows][stride]
  uint64_t* bars;
};

__device__ __forceinline__ int PosMod(int a, int m) {
  const int r = a % m;
  return r < 0 ? r + m : r;
}

// Rows of one batch: x_in planes px[0..nxp), the coefficient rows (w0, w1,
// b) of plane pc (pc_on), w2 planes pw[0..nwp).
struct PipeBatch {
  int px[3], nxp;
  int pc, pc_on;
  int pw[2], nwp;
};

// Issues a batch (by the 32 lanes of the calling warp) into the ring slots
// of its planes, completion on `bar`; lane 0 first registers the total
// bytes.
__device__ __forceinline__ void IssueBatch(const Op<float>& A, const float* __restrict__ b,
                                           const float* __restrict__ xin, const PipeSmem& S,
                                           int base, int i0, int w, int j0, int rows,
                                           const PipeBatch& B, uint64_t* bar) {
  const Dims d = A.d;
  const int lane = threadIdx.x & 31;
  const int nxr = rows + 4, nc0 = rows + 2, nc1 = rows + 3, nw = rows + 2;
  const int ncoef = B.pc_on ? nc0 + nc1 + nc0 : 0;
  const int total = B.nxp * nxr + ncoef + B.nwp * nw;
  const uint32_t rowb = 4u * (uint32_t)(w + 8);
  if (lane == 0) MbarExpectTx(bar, rowb * (uint32_t)total);
  __syncwarp();
  const int64_t plane = (int64_t)d.nx * d.ny;
  for (int q = lane; q < total; q += 32) {
    int t = q;
    const float* src;
    float* dst;
    int r, p;
    if (t < B.nxp * nxr) {
      p = B.px[t / nxr];
      r = t % nxr - 2;
      src = xin;
      dst = S.xs + ((size_t)PosMod(p - base, kPipeXs) * kPipeXRows + (r + 2)) * kPipeStride;
    } else if (t - B.nxp * nxr < ncoef) {
      t -= B.nxp * nxr;
      p = B.pc;
      float* slot = S.cs + (size_t)PosMod(p - base, kPipeCs) * kPipeCRows * kPipeStride;
      if (t < nc0) {
        r = t - 1;
        src = A.w0;
        dst = slot + (size_t)(r + 1) * kPipeStride;
      } else if (t < nc0 + nc1) {
        r = t - nc0 - 1;
        src = A.w1;
        dst = slot + (size_t)(kPipeW0Rows + r + 1) * kPipeStride;
      } else {
        r = t - nc0 - nc1 - 1;
        src = b;
        dst = slot + (size_t)(kPipeW0Rows + kPipeW1Rows + r + 1) * kPipeStride;
      }
    } else {
      t -= B.nxp * nxr + ncoef;
      p = B.pw[t / nw];
      r = t % nw - 1;
      src = A.w2;
      dst = S.ws + ((size_t)PosMod(p - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
    }
    const int jw = PosMod(j0 + r, d.ny);
    const int pz = PosMod(p, d.nz);
    CopyRowSegment(dst, src + pz * plane + (int64_t)jw * d.nx, d.nx, i0, w, bar);
  }
}

__device__ __forceinline__ float4 LdS4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

// First colour of row r (-1..rows) of plane p into its F slot: float4
// groups of the w columns, and (lanes 0 and 1) the halo columns -1 and w.
__device__ __forceinline__ void PipeFirst(const PipeSmem& S, int base, int c0, int zero_init,
                                          int i0, int w, int j0, int r, int p, int nyd,
                                          int nzd) {
  const int lane = threadIdx.x & 31;
  const float* X0 = S.xs + (size_t)PosMod(p - 1 - base, kPipeXs) * kPipeXRows * kPipeStride;
  const float* X1 = S.xs + (size_t)PosMod(p - base, kPipeXs) * kPipeXRows * kPipeStride;
  const float* X2 = S.xs + (size_t)PosMod(p + 1 - base, kPipeXs) * kPipeXRows * kPipeStride;
  const float* C = S.cs + (size_t)PosMod(p - base, kPipeCs) * kPipeCRows * kPipeStride;
  const float* W0 = C + (size_t)(r + 1) * kPipeStride;
  const float* W1 = C + (size_t)(kPipeW0Rows + r + 1) * kPipeStride;
  const float* W1n = W1 + kPipeStride;
  const float* B = C + (size_t)(kPipeW0Rows + kPipeW1Rows + r + 1) * kPipeStride;
  const float* Z1 =
      S.ws + ((size_t)PosMod(p - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
  const float* Z2 =
      S.ws + ((size_t)PosMod(p + 1 - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
  const float* Xc = X1 + (size_t)(r + 2) * kPipeStride;
  const float* Xm = Xc - kPipeStride;
  const float* Xp = Xc + kPipeStride;
  const float* Xz0 = X0 + (size_t)(r + 2) * kPipeStride;
  const float* Xz2 = X2 + (size_t)(r + 2) * kPipeStride;
  float* Fo = S.fs + ((size_t)PosMod(p - base, 3) * kPipeFRows + (r + 1)) * kPipeStride;
  // colour parity of the wrapped indices (i0 is a multiple of 4)
  const int j = PosMod(j0 + r, nyd);
  const int pz = PosMod(p, nzd);
  const int g = lane;
  if (4 * g < w) {
    const int l = 4 * g + 4;
    const float4 w0v = LdS4(W0 + l), w1v = LdS4(W1 + l), w1nv = LdS4(W1n + l);
    const float4 z1v = LdS4(Z1 + l), z2v = LdS4(Z2 + l), bv = LdS4(B + l);
    const float wr = W0[l + 4];
    float4 xc = make_float4(0, 0, 0, 0), xjm = xc, xjp = xc, xz0 = xc, xz2 = xc;
    float xl = 0.f, xr = 0.f;
    if (!zero_init) {
      xc = LdS4(Xc + l);
      xjm = LdS4(Xm + l);
      xjp = LdS4(Xp + l);
      xz0 = LdS4(Xz0 + l);
      xz2 = LdS4(Xz2 + l);
      xl = Xc[l - 1];
      xr = Xc[l + 4];
    }
    float4 out = make_float4(0, 0, 0, 0);
    const int e0 = (c0 + j + pz) & 1;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if ((e & 1) != e0) continue;
      const float cxm = El(w0v, e);
      const float cxp = e == 3 ? wr : El(w0v, e + 1);
      const float cym = El(w1v, e), cyp = El(w1nv, e);
      const float czm = El(z1v, e), czp = El(z2v, e);
      const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
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
    *reinterpret_cast<float4*>(Fo + l) = out;
  }
  // halo columns: lane 0 column -1, lane 1 column w (the parity of i0 - 1
  // and i0 + w equals that of their wrapped columns: nx is even)
  if (lane < 2) {
    const int col = lane == 0 ? -1 : w;
    const int l = col + 4;
    if (((col + j + pz) & 1) == c0) {
      const float cxm = W0[l], cxp = W0[l + 1];
      const float cym = W1[l], cyp = W1n[l];
      const float czm = Z1[l], czp = Z2[l];
      const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
      float acc = B[l];
      if (!zero_init) {
        acc -= cxm * Xc[l - 1];
        acc -= cxp * Xc[l + 1];
        acc -= cym * Xm[l];
        acc -= cyp * Xp[l];
        acc -= czm * Xz0[l];
        acc -= czp * Xz2[l];
      }
      Fo[l] = acc / dg;
    }
  }
}

// Second colour of row r (0..rows-1) of plane m from the first colour of
// planes m-1, m, m+1; both colours of the row's w columns to x_out.
__device__ __forceinline__ void PipeSecond(const PipeSmem& S, int base, int c0, int i0, int w,
                                           int j0, int r, int m, const Dims& d, float* xout) {
  const int lane = threadIdx.x & 31;
  const int g = lane;
  if (4 * g >= w) return;
  const int l = 4 * g + 4;
  const float* C = S.cs + (size_t)PosMod(m - base, kPipeCs) * kPipeCRows * kPipeStride;
  const float* W0 = C + (size_t)(r + 1) * kPipeStride;
  const float* W1 = C + (size_t)(kPipeW0Rows + r + 1) * kPipeStride;
  const float* W1n = W1 + kPipeStride;
  const float* B = C + (size_t)(kPipeW0Rows + kPipeW1Rows + r + 1) * kPipeStride;
  const float* Z1 =
      S.ws + ((size_t)PosMod(m - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
  const float* Z2 =
      S.ws + ((size_t)PosMod(m + 1 - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
  const float* Fm =
      S.fs + ((size_t)PosMod(m - 1 - base, 3) * kPipeFRows + (r + 1)) * kPipeStride;
  const float* F0 = S.fs + ((size_t)PosMod(m - base, 3) * kPipeFRows + (r + 1)) * kPipeStride;
  const float* Fp =
      S.fs + ((size_t)PosMod(m + 1 - base, 3) * kPipeFRows + (r + 1)) * kPipeStride;
  const float4 w0v = LdS4(W0 + l), w1v = LdS4(W1 + l), w1nv = LdS4(W1n + l);
  const float4 z1v = LdS4(Z1 + l), z2v = LdS4(Z2 + l), bv = LdS4(B + l);
  const float wr = W0[l + 4];
  const float4 f0 = LdS4(F0 + l);
  const float4 fym = LdS4(F0 - kPipeStride + l), fyp = LdS4(F0 + kPipeStride + l);
  const float4 fzm = LdS4(Fm + l), fzp = LdS4(Fp + l);
  const float fl = F0[l - 1], fr = F0[l + 4];
  const int j = j0 + r;
  const int pz = PosMod(m, d.nz);
  const int e0 = (c0 + j + pz) & 1;  // first-colour positions
  float4 out;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if ((e & 1) == e0) {
      SetEl(out, e, El(f0, e));
      continue;
    }
    const float cxm = El(w0v, e);
    const float cxp = e == 3 ? wr : El(w0v, e + 1);
    const float cym = El(w1v, e), cyp = El(w1nv, e);
    const float czm = El(z1v, e), czp = El(z2v, e);
    const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
    float acc = El(bv, e);
    acc -= cxm * (e == 0 ? fl : El(f0, e - 1));
    acc -= cxp * (e == 3 ? fr : El(f0, e + 1));
    acc -= cym * El(fym, e);
    acc -= cyp * El(fyp, e);
    acc -= czm * El(fzm, e);
    acc -= czp * El(fzp, e);
    SetEl(out, e, acc / dg);
  }
  *reinterpret_cast<float4*>(xout + d.idx(i0 + 4 * g, j, pz)) = out;
}

// One fused sweep of one work item (grid: one CTA of kPipeThreads per item,
// dynamic shared memory kPipeSmemBytes).  Item index: blockIdx.x =
// (zseg * bands + band) * xtiles + xtile.
__global__ void __launch_bounds__(kPipeThreads, 1)
    KSweepPipe(Op<float> A, const float* __restrict__ b, const float* __restrict__ xin,
               float* xout, int c0, int zero_init, const SolveScalars* s, PipeTiling T,
               int* err) {
  if (s && s->done) return;
  extern __shared__ __align__(128) float smem[];
  const Dims d = A.d;
  PipeSmem S;
  S.xs = smem;
  S.cs = S.xs + (size_t)kPipeXs * kPipeXRows * kPipeStride;
  S.ws = S.cs + (size_t)kPipeCs * kPipeCRows * kPipeStride;
  S.fs = S.ws + (size_t)kPipeWs * kPipeW2Rows * kPipeStride;
  S.bars = reinterpret_cast<uint64_t*>(S.fs + (size_t)3 * kPipeFRows * kPipeStride);
  const int item = blockIdx.x;
  const int xt = item % T.xtiles;
  const int band = (item / T.xtiles) % T.bands;
  const int zs = item / (T.xtiles * T.bands);
  const int i0 = xt * T.w;
  const int w = min(T.w, d.nx - i0);
  const int j0 = band * T.rows;
  const int rows = min(T.rows, d.ny - j0);
  const int kb = (int)((int64_t)d.nz * zs / T.zsegs);
  const int ke = (int)((int64_t)d.nz * (zs + 1) / T.zsegs);
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    for (int q = 0; q < kPipeBars; ++q) MbarInit(S.bars + q, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int base = kb - 2;  // ring position 0: plane kb-2
  const int t0 = kb - 1;    // first time step
  auto bar_of = [&](int t) { return S.bars + PosMod(t - t0, kPipeBars); };
  auto parity_of = [&](int t) { return (uint32_t)(((t - t0) / kPipeBars) & 1); };
  // batch B(t) for t > t0: x_in of plane t+1, coefficients of plane t, w2
  // of plane t+1; B(t0) also carries x_in of planes t0-1, t0 and w2 of t0
  auto batch = [&](int t) {
    PipeBatch B;
    B.nxp = 0;
    if (!zero_init) {
      B.px[B.nxp++] = t + 1;
      if (t == t0) {
        B.px[B.nxp++] = t - 1;
        B.px[B.nxp++] = t;
      }
    }
    B.pc = t;
    B.pc_on = 1;
    B.nwp = 0;
    B.pw[B.nwp++] = t + 1;
    if (t == t0) B.pw[B.nwp++] = t;
    return B;
  };
  if (warp == 0) {
    for (int t = t0; t <= min(t0 + 2, ke); ++t)
      IssueBatch(A, b, xin, S, base, i0, w, j0, rows, batch(t), bar_of(t));
  }
  bool ok = MbarWait(bar_of(t0), parity_of(t0));
  int failed = __syncthreads_or(!ok);
  int t_issued = min(t0 + 2, ke);  // last batch issued
  int t_wait = t0;                 // batch of the last wait
  for (int t = t0; t <= ke && !failed; ++t) {
    // B(t+2) into the slots of plane t-2, free since the end of step t-1
    if (warp == 0 && t + 2 <= ke && t > t0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      IssueBatch(A, b, xin, S, base, i0, w, j0, rows, batch(t + 2), bar_of(t + 2));
    }
    if (t + 2 <= ke) t_issued = t + 2;
    // F(t): warps 0 .. rows+1 take rows -1 .. rows
    if (warp < rows + 2) PipeFirst(S, base, c0, zero_init, i0, w, j0, warp - 1, t, d.ny, d.nz);
    __syncthreads();
    // S(t-1)
    if (t - 1 >= kb && warp < rows) PipeSecond(S, base, c0, i0, w, j0, warp, t - 1, d, xout);
    // data of the next step
    ok = true;
    if (t + 1 <= ke) {
      t_wait = t + 1;
      ok = MbarWait(bar_of(t + 1), parity_of(t + 1));
    }
    failed = __syncthreads_or(!ok);
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      // the batches issued but not seen complete (from the one whose wait
      // gave up): wait (bounded) for their copies before the shared memory
      // goes away
      for (int t = t_wait; t <= t_issued; ++t) MbarWait(bar_of(t), parity_of(t));
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The same sweep with the rows staged by per-thread asynchronous copies
// (cp.async, 16 bytes each) instead of bulk copies: every thread of the
// CTA copies its share of the batch's 16-byte chunks (a row segment
// [i0-4, i0+w+4) is (w+8)/4 chunks; the periodic wrap in x is per chunk,
// since nx and i0 are multiples of 4) and commits them as one group; a
// batch is complete once every thread has waited for its group
// (cp.async.wait_group) and the block has passed a barrier.  No mbarrier
// and no bounded wait is involved: each thread waits only for its own
// copies.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void CpAsync16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(SmemAddr(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void CpAsyncCommit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int kPending>
__device__ __forceinline__ void CpAsyncWait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory");
}

// Issues a batch by all threads of the CTA, then commits one group.
__device__ __forceinline__ void IssueBatchAsync(const Op<float>& A, const float* __restrict__ b,
                                                const float* __restrict__ xin,
                                                const PipeSmem& S, int base, int i0, int w,
                                                int j0, int rows, const PipeBatch& B) {
  const Dims d = A.d;
  const int nxr = rows + 4, nc0 = rows + 2, nc1 = rows + 3, nw = rows + 2;
  const int ncoef = B.pc_on ? nc0 + nc1 + nc0 : 0;
  const int total = B.nxp * nxr + ncoef + B.nwp * nw;  // rows
  const int cpr = (w + 8) / 4;                           // chunks per row
  const int64_t plane = (int64_t)d.nx * d.ny;
  for (int q = threadIdx.x; q < total * cpr; q += blockDim.x) {
    int t = q / cpr;
    const int ch = q - t * cpr;
    const float* src;
    float* dst;
    int r, p;
    if (t < B.nxp * nxr) {
      p = B.px[t / nxr];
      r = t % nxr - 2;
      src = xin;
      dst = S.xs + ((size_t)PosMod(p - base, kPipeXs) * kPipeXRows + (r + 2)) * kPipeStride;
    } else if (t - B.nxp * nxr < ncoef) {
      t -= B.nxp * nxr;
      p = B.pc;
      float* slot = S.cs + (size_t)PosMod(p - base, kPipeCs) * kPipeCRows * kPipeStride;
      if (t < nc0) {
        r = t - 1;
        src = A.w0;
        dst = slot + (size_t)(r + 1) * kPipeStride;
      } else if (t < nc0 + nc1) {
        r = t - nc0 - 1;
        src = A.w1;
        dst = slot + (size_t)(kPipeW0Rows + r + 1) * kPipeStride;
      } else {
        r = t - nc0 - nc1 - 1;
        src = b;
        dst = slot + (size_t)(kPipeW0Rows + kPipeW1Rows + r + 1) * kPipeStride;
      }
    } else {
      t -= B.nxp * nxr + ncoef;
      p = B.pw[t / nw];
      r = t % nw - 1;
      src = A.w2;
      dst = S.ws + ((size_t)PosMod(p - base, kPipeWs) * kPipeW2Rows + (r + 1)) * kPipeStride;
    }
    const int jw = PosMod(j0 + r, d.ny);
    const int pz = PosMod(p, d.nz);
    const int col = PosMod(i0 - 4 + 4 * ch, d.nx);
    CpAsync16(dst + 4 * ch, src + pz * plane + (int64_t)jw * d.nx + col);
  }
  CpAsyncCommit();
}

// KSweepPipe with cp.async staging (same tiling, rings and arithmetic).
__global__ void __launch_bounds__(kPipeThreads, 1)
    KSweepPipeAsync(Op<float> A, const float* __restrict__ b, const float* __restrict__ xin,
                    float* xout, int c0, int zero_init, const SolveScalars* s, PipeTiling T) {
  if (s && s->done) return;
  extern __shared__ __align__(128) float smem[];
  const Dims d = A.d;
  PipeSmem S;
  S.xs = smem;
  S.cs = S.xs + (size_t)kPipeXs * kPipeXRows * kPipeStride;
  S.ws = S.cs + (size_t)kPipeCs * kPipeCRows * kPipeStride;
  S.fs = S.ws + (size_t)kPipeWs * kPipeW2Rows * kPipeStride;
  S.bars = nullptr;
  const int item = blockIdx.x;
  const int xt = item % T.xtiles;
  const int band = (item / T.xtiles) % T.bands;
  const int zs = item / (T.xtiles * T.bands);
  const int i0 = xt * T.w;
  const int w = min(T.w, d.nx - i0);
  const int j0 = band * T.rows;
  const int rows = min(T.rows, d.ny - j0);
  const int kb = (int)((int64_t)d.nz * zs / T.zsegs);
  const int ke = (int)((int64_t)d.nz * (zs + 1) / T.zsegs);
  const int warp = threadIdx.x >> 5;
  const int base = kb - 2;
  const int t0 = kb - 1;
  auto batch = [&](int t) {
    PipeBatch B;
    B.nxp = 0;
    if (!zero_init) {
      B.px[B.nxp++] = t + 1;
      if (t == t0) {
        B.px[B.nxp++] = t - 1;
        B.px[B.nxp++] = t;
      }
    }
    B.pc = t;
    B.pc_on = 1;
    B.nwp = 0;
    B.pw[B.nwp++] = t + 1;
    if (t == t0) B.pw[B.nwp++] = t;
    return B;
  };
  // prologue: B(t0), B(t0+1), B(t0+2); a batch past ke is an empty group
  for (int t = t0; t <= t0 + 2; ++t) {
    if (t <= ke)
      IssueBatchAsync(A, b, xin, S, base, i0, w, j0, rows, batch(t));
    else
      CpAsyncCommit();
  }
  CpAsyncWait<2>();
  __syncthreads();
  for (int t = t0; t <= ke; ++t) {
    // F(t): warps 0 .. rows+1 take rows -1 .. rows
    if (warp < rows + 2) PipeFirst(S, base, c0, zero_init, i0, w, j0, warp - 1, t, d.ny, d.nz);
    __syncthreads();
    if (t - 1 >= kb && warp < rows) PipeSecond(S, base, c0, i0, w, j0, warp, t - 1, d, xout);
    // the slots of plane t-1 (coefficients, w2) and t-2 (x) are free once
    // every thread is past S(t-1): then B(t+3) may overwrite them
    __syncthreads();
    if (t + 3 <= ke)
      IssueBatchAsync(A, b, xin, S, base, i0, w, j0, rows, batch(t + 3));
    else
      CpAsyncCommit();
    // B(t+1) complete (B(t+2), B(t+3) may stay in flight)
    CpAsyncWait<2>();
    __syncthreads();
  }
  CpAsyncWait<0>();
}

}  // namespace aphgpu

// Fused red-black Gauss-Seidel sweep, out of place, with the planes staged
// in shared memory by asynchronous copies.
//
// One sweep updates the first colour c0 of every cell from the old values
// x_in of the other colour, then the second colour from the new first-colour
// values, and writes both colours to x_out (x_out != x_in).  Per full sweep
// every array is read once from HBM: x_in, the three couplings w0 w1 w2 and
// b (FP32), and x_out is written once: 24 bytes per cell.
//
// Work item: a tile of w <= 128 columns (x) by rows <= kPipeRows rows (y),
// marching over the planes [kb, ke) (z).  Two CTAs of 256 threads per SM
// (104 KB of shared memory each); the host sizes the tiles so that all
// items run in one wave, so neighbouring tiles stream the same planes at
// the same time and the halo rows a tile reads again come from L2.
//
// Pipeline (time step t = kb-1 .. ke): F(t), the first colour of plane t on
// the tile's rows -1..rows and columns -1..w (halo recomputed, never
// exchanged), into a ring of three planes; then S(t-1), the second colour
// of plane t-1, written with the first colour of that plane to x_out.  The
// data F(t) needs beyond earlier steps -- x_in of plane t+1, w0 w1 b of
// plane t, w2 of plane t+1 -- form batch B(t): for each array row the
// segment of columns [i0-4, i0+w+4), copied in 16-byte chunks by cp.async
// (the periodic wrap in x is per chunk, since nx and i0 are multiples of 4;
// the wraps in y and z only change which row is read).  Every thread copies
// its share of a batch and commits it as one group; B(t+2) is issued after
// S(t-1), so two planes of copies are in flight while a plane is computed,
// and a batch is complete once every thread has waited for its group
// (cp.async.wait_group) and the block has passed a barrier.  Each thread
// waits only for copies it issued itself.
//
// Every value is computed by the same operations, in the same order, as in
// the two in-place half sweeps (Smooth4Body), so results are bit-identical.
// Requires: nx % 4 == 0, nx >= 16, no stored diagonal (the diagonal is
// minus the sum of the couplings, as for the projection operator).
#pragma once

#include <cstdint>

#include "stencil.cuh"
#include "vec.cuh"

namespace aphgpu {

constexpr int kPipeCols = 128;                // columns of a tile at most
constexpr int kPipeRows = 7;                  // rows of a tile at most
constexpr int kPipeStride = kPipeCols + 8;    // floats per staged row
constexpr int kPipeThreads = 256;
constexpr int kPipeWarps = kPipeThreads / 32;
constexpr int kPipeXs = 4, kPipeCs = 3, kPipeWs = 4;  // ring sizes (planes)
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
constexpr int kPipeSmemBytes = kPipeSmemFloats * 4;
static_assert(2 * (kPipeSmemBytes + 1024) <= 228 * 1024, "two CTAs per SM");

struct PipeTiling {
  int w;       // columns of a tile (multiple of 4, <= kPipeCols)
  int rows;    // rows of a band (<= kPipeRows)
  int xtiles, bands, zsegs;
};

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

struct PipeSmem {
  float* xs;   // [kPipeXs][kPipeXRows][stride]
  float* cs;   // [kPipeCs][kPipeCRows][stride]: w0, w1, b
  float* ws;   // [kPipeWs][kPipeW2Rows][stride]
  float* fs;   // [3][kPipeFRows][stride]
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

// Chunks of a steady-state batch B(t) (x_in of plane t+1, w0 w1 b of plane
// t, w2 of plane t+1) owned by one thread: at most kPipeOwn chunks, each
// described once per work item by its array, its offset inside a plane of
// that array and its offset inside the ring slot; a step then only adds
// the planes' offsets.
constexpr int kPipeOwn = 8;
static_assert((5 * kPipeRows + 13) * ((kPipeCols + 8) / 4) <= kPipeOwn * kPipeThreads,
              "a steady batch has more chunks than the threads own");
struct PipeChunks {
  int n;
  int kind[kPipeOwn];     // 0 x, 1 w0, 2 w1, 3 b, 4 w2
  int goff[kPipeOwn];     // row * nx + column (wrapped) inside the plane
  int soff[kPipeOwn];     // offset inside the ring slot (floats)
};

__device__ __forceinline__ void PipeChunksInit(const Dims& d, int i0, int w, int j0, int rows,
                                               int zero_init, PipeChunks& C) {
  const int nxr = rows + 4, nc0 = rows + 2, nc1 = rows + 3, nw = rows + 2;
  const int nxp = zero_init ? 0 : 1;
  const int total = nxp * nxr + nc0 + nc1 + nc0 + nw;
  const int cpr = (w + 8) / 4;
  C.n = 0;
  for (int q = threadIdx.x; q < total * cpr && C.n < kPipeOwn; q += blockDim.x) {
    int t = q / cpr;
    const int ch = q - t * cpr;
    int kind, r, srow;
    if (t < nxp * nxr) {
      kind = 0;
      r = t - 2;
      srow = r + 2;
    } else if ((t -= nxp * nxr) < nc0) {
      kind = 1;
      r = t - 1;
      srow = r + 1;
    } else if ((t -= nc0) < nc1) {
      kind = 2;
      r = t - 1;
      srow = kPipeW0Rows + r + 1;
    } else if ((t -= nc1) < nc0) {
      kind = 3;
      r = t - 1;
      srow = kPipeW0Rows + kPipeW1Rows + r + 1;
    } else {
      t -= nc0;
      kind = 4;
      r = t - 1;
      srow = r + 1;
    }
    const int jw = PosMod(j0 + r, d.ny);
    const int col = PosMod(i0 - 4 + 4 * ch, d.nx);
    C.kind[C.n] = kind;
    C.goff[C.n] = jw * d.nx + col;
    C.soff[C.n] = srow * kPipeStride + 4 * ch;
    ++C.n;
  }
}

// Steady-state batch B(t) from the thread's precomputed chunks.
__device__ __forceinline__ void IssueSteadyAsync(const Op<float>& A, const float* __restrict__ b,
                                                 const float* __restrict__ xin,
                                                 const PipeSmem& S, int base, int t,
                                                 const PipeChunks& C) {
  const Dims d = A.d;
  const int64_t plane = (int64_t)d.nx * d.ny;
  const int64_t px = (int64_t)PosMod(t + 1, d.nz) * plane;  // x, w2
  const int64_t pc = (int64_t)PosMod(t, d.nz) * plane;      // w0, w1, b
  float* xs = S.xs + (size_t)PosMod(t + 1 - base, kPipeXs) * kPipeXRows * kPipeStride;
  float* cs = S.cs + (size_t)PosMod(t - base, kPipeCs) * kPipeCRows * kPipeStride;
  float* ws = S.ws + (size_t)PosMod(t + 1 - base, kPipeWs) * kPipeW2Rows * kPipeStride;
#pragma unroll
  for (int q = 0; q < kPipeOwn; ++q) {
    if (q >= C.n) break;
    const int k = C.kind[q];
    const float* src = k == 0 ? xin + px : k == 1 ? A.w0 + pc : k == 2 ? A.w1 + pc
                     : k == 3 ? b + pc : A.w2 + px;
    float* dst = k == 0 ? xs : k == 4 ? ws : cs;
    CpAsync16(dst + C.soff[q], src + C.goff[q]);
  }
  CpAsyncCommit();
}

// One fused sweep of one work item (grid: one CTA of kPipeThreads per item,
// dynamic shared memory kPipeSmemBytes).  Item index: blockIdx.x =
// (zseg * bands + band) * xtiles + xtile.
__global__ void __launch_bounds__(kPipeThreads, 2)
    KSweepPipe(Op<float> A, const float* __restrict__ b, const float* __restrict__ xin,
               float* xout, int c0, int zero_init, const SolveScalars* s, PipeTiling T) {
  if (s && s->done) return;
  extern __shared__ __align__(128) float smem[];
  const Dims d = A.d;
  PipeSmem S;
  S.xs = smem;
  S.cs = S.xs + (size_t)kPipeXs * kPipeXRows * kPipeStride;
  S.ws = S.cs + (size_t)kPipeCs * kPipeCRows * kPipeStride;
  S.fs = S.ws + (size_t)kPipeWs * kPipeW2Rows * kPipeStride;
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
  const int base = kb - 2;  // ring position 0: plane kb-2
  const int t0 = kb - 1;    // first time step
  // batch B(t0): x_in of planes t0-1 .. t0+1, coefficients of t0, w2 of
  // t0 and t0+1; later batches come from the precomputed chunks
  PipeBatch B0;
  B0.nxp = 0;
  if (!zero_init) {
    B0.px[B0.nxp++] = t0 + 1;
    B0.px[B0.nxp++] = t0 - 1;
    B0.px[B0.nxp++] = t0;
  }
  B0.pc = t0;
  B0.pc_on = 1;
  B0.nwp = 0;
  B0.pw[B0.nwp++] = t0 + 1;
  B0.pw[B0.nwp++] = t0;
  PipeChunks C;
  PipeChunksInit(d, i0, w, j0, rows, zero_init, C);
  IssueBatchAsync(A, b, xin, S, base, i0, w, j0, rows, B0);
  if (t0 + 1 <= ke)
    IssueSteadyAsync(A, b, xin, S, base, t0 + 1, C);
  else
    CpAsyncCommit();
  CpAsyncWait<1>();  // B(t0)
  __syncthreads();
  for (int t = t0; t <= ke; ++t) {
    // F(t): rows -1 .. rows over the warps
    for (int r = warp - 1; r <= rows; r += kPipeWarps)
      PipeFirst(S, base, c0, zero_init, i0, w, j0, r, t, d.ny, d.nz);
    __syncthreads();
    if (t - 1 >= kb && warp < rows) PipeSecond(S, base, c0, i0, w, j0, warp, t - 1, d, xout);
    // the slots of x_in plane t-1 and of the coefficients and w2 of plane
    // t-1 are free once every thread is past S(t-1): B(t+2) goes there
    __syncthreads();
    if (t + 2 <= ke)
      IssueSteadyAsync(A, b, xin, S, base, t + 2, C);
    else
      CpAsyncCommit();
    CpAsyncWait<1>();  // B(t+1) complete, B(t+2) may stay in flight
    __syncthreads();
  }
  CpAsyncWait<0>();
}

}  // namespace aphgpu

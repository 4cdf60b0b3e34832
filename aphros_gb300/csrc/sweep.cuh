// Fused red-black Gauss-Seidel sweep, out of place, with the planes staged
// in shared memory by asynchronous copies.
//
// One sweep updates the first colour c0 of every cell from the old values
// x_in of the other colour, then the second colour from the new first-colour
// values, and writes both colours to x_out (x_out != x_in).  Per full sweep
// every array is read once from HBM: x_in, the three couplings w0 w1 w2 and
// b (FP32), and x_out is written once: 24 bytes per cell.
//
// Work item: a tile of w <= 128 columns (x, one float4 per lane) by rows <=
// kPipeRows rows (y), marching over the planes [kb, ke) (z).  One CTA of
// kPipeRows + 2 warps per SM (the staged rings take 213 KB of shared
// memory); the host sizes the tiles so that all items run in one wave, so
// neighbouring tiles stream the same planes at the same time and the halo
// rows a tile reads again come from L2.
//
// Time step t (kb-1 .. ke):
//   F(t)  warp v updates the first colour of row v-1 (rows -1 .. rows) of
//         plane t, in place in the staged x_in plane: the first-colour
//         positions are written, the second-colour ones keep x_in, which is
//         what the later first-colour updates of planes t+-1 read there;
//   wait for batch B(t+1), barrier;
//   S(t-1) warps 0 .. rows-1 update the second colour of plane t-1 from the
//         first-colour values of planes t-2, t-1, t and write both colours
//         of the row to x_out; the two remaining warps update the first
//         colour of the halo columns -1 and w of plane t (read by S(t));
//   issue B(t+2) and an L2 prefetch of the planes two steps further.
// Batch B(t): x_in of plane t+1, w0 w1 b of plane t, w2 of plane t+1, each
// array row as the segment of columns [i0-4, i0+w+4) in 16-byte chunks
// copied by cp.async (the periodic wrap in x is per chunk, since nx and i0
// are multiples of 4; the wraps in y and z only change the row read).  The
// rings hold six x and w2 planes and four coefficient planes: a slot is
// refilled two steps after its last reader passed a barrier, so one barrier
// per step orders every read before the copy that overwrites it.  Each
// thread copies the same chunks of every plane (their offsets are computed
// once per item) and waits only for its own copies.
//
// Every value is computed by the same operations, in the same order, as in
// the two in-place half sweeps (Smooth4Body), so results are bit-identical.
// Requires: nx % 4 == 0, nx >= 16, ny >= 2, nz >= 8, no stored diagonal
// (the diagonal is minus the sum of the couplings, as for the projection
// operator).
#pragma once

#include <cstdint>

#include "stencil.cuh"
#include "vec.cuh"

namespace aphgpu {

constexpr int kPipeCols = 128;               // columns of a tile at most
constexpr int kPipeStride = kPipeCols + 8;   // floats per staged row
constexpr int kPipeAhead = 2;                // batches issued ahead
constexpr int kPipeXs = kPipeAhead + 4;      // x_in and w2 rings (planes)
constexpr int kPipeCs = 4;                   // w0 w1 b ring (planes)
constexpr int kPipePrefetch = 2;             // L2 prefetch: steps beyond the copies
static_assert(kPipeCs >= kPipeAhead + 2 && (kPipeCs & (kPipeCs - 1)) == 0,
              "coefficient ring: refilled two steps after its last read, power of two");
static_assert(kPipeXs >= kPipeAhead + 4, "x ring: refilled two steps after its last read");

// Shape of the kernel for bands of at most R rows: R + 2 warps (one per
// first-colour row), the staged rings, and the CTAs resident per SM.
template <int R>
struct PipeShape {
  static constexpr int kRows = R;
  static constexpr int kWarps = R + 2;
  static constexpr int kThreads = 32 * kWarps;
  static constexpr int kXRows = R + 4;    // x_in rows -2 .. rows+1
  static constexpr int kW0Rows = R + 2;   // w0 rows -1 .. rows
  static constexpr int kW1Rows = R + 3;   // w1 rows -1 .. rows+1
  static constexpr int kBRows = R + 2;    // b rows -1 .. rows
  static constexpr int kCRows = kW0Rows + kW1Rows + kBRows;
  static constexpr int kW2Rows = R + 2;   // w2 rows -1 .. rows
  static constexpr int kXSlot = kXRows * kPipeStride;  // floats
  static constexpr int kCSlot = kCRows * kPipeStride;
  static constexpr int kWSlot = kW2Rows * kPipeStride;
  static constexpr int kSmemBytes =
      4 * (kPipeXs * kXSlot + kPipeCs * kCSlot + kPipeXs * kWSlot);
  // CTAs per SM: 228 KB of shared memory per SM, 1 KB reserved per CTA
  static constexpr int kCtasPerSm = 233472 / (kSmemBytes + 1024) >= 2 ? 2 : 1;
  static_assert(kSmemBytes <= 227 * 1024, "shared memory of one CTA");
  static_assert(kXRows * (kPipeStride / 4) <= 2 * kThreads, "two chunks per thread and array");
  static_assert(2 * (R + 2) <= 64, "halo cells of a plane for the two spare warps");
  static_assert(5 * R + 13 <= kThreads, "one prefetched row per thread");
};
// the two shapes built: 14-row bands, one CTA of 16 warps per SM; 6-row
// bands, two CTAs of 8 warps per SM
using PipeTall = PipeShape<14>;
using PipeShort = PipeShape<6>;
static_assert(PipeTall::kCtasPerSm == 1 && PipeShort::kCtasPerSm == 2, "residency");

struct PipeTiling {
  int w;       // columns of a tile (multiple of 4, <= kPipeCols)
  int rows;    // rows of a band (<= kPipeRows)
  int xtiles, bands, zsegs;
};

__device__ __forceinline__ uint32_t SmemAddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ int PosMod(int a, int m) {
  const int r = a % m;
  return r < 0 ? r + m : r;
}

__device__ __forceinline__ float4 LdS4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

__device__ __forceinline__ void CpAsync16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void CpAsyncCommit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int kPending>
__device__ __forceinline__ void CpAsyncWait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory");
}
// L2 prefetch of a contiguous range (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void PrefetchBulkL2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// The chunks of one staged array that a thread copies: the array's rows
// r = 0 .. nrows-1 (array row j0 + r + roff, wrapped) land in slot rows
// srow0 + r; chunk q = threadIdx.x + i * kThreads (i = 0, 1) is column
// chunk q % cpr of row q / cpr.  g: offset inside a plane (floats); s:
// offset inside the slot (bytes), -1 if the thread has no such chunk.
struct PipeChunks {
  int g[2];
  int s[2];
};

template <int kThreads>
__device__ __forceinline__ PipeChunks PipeChunksOf(const Dims& d, int i0, int w, int j0,
                                                   int nrows, int roff, int srow0) {
  PipeChunks c;
  const int cpr = (w + 8) >> 2;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int q = threadIdx.x + i * kThreads;
    c.g[i] = 0;
    c.s[i] = -1;
    if (q < nrows * cpr) {
      const int r = q / cpr, ch = q - r * cpr;
      const int jw = PosMod(j0 + r + roff, d.ny);
      const int col = PosMod(i0 - 4 + 4 * ch, d.nx);
      c.g[i] = jw * d.nx + col;
      c.s[i] = 4 * ((srow0 + r) * kPipeStride + 4 * ch);
    }
  }
  return c;
}

__device__ __forceinline__ void PipeCopy(uint32_t slot, const float* plane, const PipeChunks& c) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
    if (c.s[i] >= 0) CpAsync16(slot + (uint32_t)c.s[i], plane + c.g[i]);
}

// First colour of the float4 group at slot column l of one row (elements E0
// and E0+2 carry the first colour), written in place into the row's staged
// x_in.  xc, xm, xp: x_in rows r, r-1, r+1 of plane t; xz0, xz2: row r of
// planes t-1, t+1; w0, w1, w1n (row r+1), bb: the coefficient rows; z1, z2:
// w2 row r of planes t, t+1.
template <int E0, int ZI>
__device__ __forceinline__ void PipeFirst(float* xc, const float* xm, const float* xp,
                                          const float* xz0, const float* xz2, const float* w0,
                                          const float* w1, const float* w1n, const float* bb,
                                          const float* z1, const float* z2, int l) {
  const float4 w0v = LdS4(w0 + l), w1v = LdS4(w1 + l), w1nv = LdS4(w1n + l);
  const float4 z1v = LdS4(z1 + l), z2v = LdS4(z2 + l), bv = LdS4(bb + l);
  const float wr = E0 == 1 ? w0[l + 4] : 0.f;
  float4 c = make_float4(0, 0, 0, 0), jm = c, jp = c, zm = c, zp = c;
  float xs = 0.f;  // the x neighbour outside the group
  if (!ZI) {
    c = LdS4(xc + l);
    jm = LdS4(xm + l);
    jp = LdS4(xp + l);
    zm = LdS4(xz0 + l);
    zp = LdS4(xz2 + l);
    xs = E0 == 0 ? xc[l - 1] : xc[l + 4];
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int e = E0 + 2 * h;
    const float cxm = El(w0v, e);
    const float cxp = e == 3 ? wr : El(w0v, e + 1);
    const float cym = El(w1v, e), cyp = El(w1nv, e);
    const float czm = El(z1v, e), czp = El(z2v, e);
    const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
    float acc = El(bv, e);
    if (!ZI) {
      const float vxm = e == 0 ? xs : El(c, e - 1);
      const float vxp = e == 3 ? xs : El(c, e + 1);
      acc -= cxm * vxm;
      acc -= cxp * vxp;
      acc -= cym * El(jm, e);
      acc -= cyp * El(jp, e);
      acc -= czm * El(zm, e);
      acc -= czp * El(zp, e);
    }
    xc[l + e] = acc / dg;
  }
}

// First colour of the single cell at slot column l (a halo column), same
// arguments as PipeFirst.
template <int ZI>
__device__ __forceinline__ void PipeFirstCell(float* xc, const float* xm, const float* xp,
                                              const float* xz0, const float* xz2,
                                              const float* w0, const float* w1,
                                              const float* w1n, const float* bb,
                                              const float* z1, const float* z2, int l) {
  const float cxm = w0[l], cxp = w0[l + 1];
  const float cym = w1[l], cyp = w1n[l];
  const float czm = z1[l], czp = z2[l];
  const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
  float acc = bb[l];
  if (!ZI) {
    acc -= cxm * xc[l - 1];
    acc -= cxp * xc[l + 1];
    acc -= cym * xm[l];
    acc -= cyp * xp[l];
    acc -= czm * xz0[l];
    acc -= czp * xz2[l];
  }
  xc[l] = acc / dg;
}

// Second colour of the group at slot column l of one row (elements 1-E0 and
// 3-E0, E0 the first colour's parity) from the first-colour values staged
// in the x_in slots: f0, fym, fyp rows r, r-1, r+1 of plane m; fzm, fzp row
// r of planes m-1, m+1; coefficient rows as in PipeFirst (z1, z2: w2 of
// planes m, m+1).  Both colours of the group go to out.
template <int E0>
__device__ __forceinline__ void PipeSecond(const float* f0, const float* fym, const float* fyp,
                                           const float* fzm, const float* fzp,
                                           const float* w0, const float* w1, const float* w1n,
                                           const float* bb, const float* z1, const float* z2,
                                           int l, float* out) {
  const float4 w0v = LdS4(w0 + l), w1v = LdS4(w1 + l), w1nv = LdS4(w1n + l);
  const float4 z1v = LdS4(z1 + l), z2v = LdS4(z2 + l), bv = LdS4(bb + l);
  const float wr = E0 == 0 ? w0[l + 4] : 0.f;
  const float4 fv = LdS4(f0 + l);
  const float4 jm = LdS4(fym + l), jp = LdS4(fyp + l), zm = LdS4(fzm + l), zp = LdS4(fzp + l);
  const float fs = E0 == 0 ? f0[l + 4] : f0[l - 1];
  float4 o = fv;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int e = 1 - E0 + 2 * h;
    const float cxm = El(w0v, e);
    const float cxp = e == 3 ? wr : El(w0v, e + 1);
    const float cym = El(w1v, e), cyp = El(w1nv, e);
    const float czm = El(z1v, e), czp = El(z2v, e);
    const float dg = -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
    float acc = El(bv, e);
    acc -= cxm * (e == 0 ? fs : El(fv, e - 1));
    acc -= cxp * (e == 3 ? fs : El(fv, e + 1));
    acc -= cym * El(jm, e);
    acc -= cyp * El(jp, e);
    acc -= czm * El(zm, e);
    acc -= czp * El(zp, e);
    SetEl(o, e, acc / dg);
  }
  St4(out, o);
}

// One fused sweep of one work item (grid: one CTA of P::kThreads per item,
// dynamic shared memory P::kSmemBytes).  Item index: blockIdx.x = (zseg *
// bands + band) * xtiles + xtile.  ZI: x_in is taken as zero (not read).
template <class P, int ZI>
__global__ void __launch_bounds__(P::kThreads, P::kCtasPerSm)
    KSweepPipe(Op<float> A, const float* __restrict__ b, const float* __restrict__ xin,
               float* __restrict__ xout, int c0, const SolveScalars* s, PipeTiling T) {
  constexpr int kPipeRows = P::kRows;
  constexpr int kPipeThreads = P::kThreads;
  constexpr int kPipeXSlot = P::kXSlot, kPipeCSlot = P::kCSlot, kPipeWSlot = P::kWSlot;
  constexpr int kPipeW0Rows = P::kW0Rows, kPipeW1Rows = P::kW1Rows;
  if (s && s->done) return;
  extern __shared__ __align__(128) float smem[];
  float* const XS = smem;
  float* const CS = XS + kPipeXs * kPipeXSlot;
  float* const WS = CS + kPipeCs * kPipeCSlot;
  const uint32_t xs_addr = SmemAddr(XS), cs_addr = SmemAddr(CS), ws_addr = SmemAddr(WS);
  const Dims d = A.d;
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
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t plane = (int64_t)d.nx * d.ny;
  const int base = kb - 2;  // ring position 0: plane kb-2
  const int t0 = kb - 1;    // first time step

  // the thread's chunks of every array
  const PipeChunks cx = PipeChunksOf<kPipeThreads>(d, i0, w, j0, ZI ? 0 : rows + 4, -2, 0);
  const PipeChunks c0w = PipeChunksOf<kPipeThreads>(d, i0, w, j0, rows + 2, -1, 0);
  const PipeChunks c1w = PipeChunksOf<kPipeThreads>(d, i0, w, j0, rows + 3, -1, kPipeW0Rows);
  const PipeChunks cbb = PipeChunksOf<kPipeThreads>(d, i0, w, j0, rows + 2, -1, kPipeW0Rows + kPipeW1Rows);
  const PipeChunks c2w = PipeChunksOf<kPipeThreads>(d, i0, w, j0, rows + 2, -1, 0);
  // the thread's L2 prefetch: one array row of a future batch (in-range
  // columns only; the 16-byte wrapped ends are left to the copies)
  const float* pf_src = nullptr;
  uint32_t pf_bytes = 0;
  int pf_coef = 0;
  {
    const int nr[5] = {ZI ? 0 : rows + 4, rows + 2, rows + 3, rows + 2, rows + 2};
    const float* arr[5] = {xin, A.w0, A.w1, b, A.w2};
    int q = threadIdx.x;
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      if (q >= 0 && q < nr[a]) {
        const int jw = PosMod(j0 + q + (a == 0 ? -2 : -1), d.ny);
        const int lo = max(i0 - 4, 0), hi = min(i0 + w + 4, d.nx);
        pf_src = arr[a] + (int64_t)jw * d.nx + lo;
        pf_bytes = 4u * (uint32_t)(hi - lo);
        pf_coef = a >= 1 && a <= 3;
      }
      q -= nr[a];
    }
  }
  // row of this warp's first-colour update (F) and second-colour update (S)
  const int rf = warp - 1, rs = warp;
  const int jf = PosMod(j0 + rf, d.ny), js = PosMod(j0 + rs, d.ny);
  // halo cell of the two spare warps: row rh, column -1 or w
  const int hh = (warp - kPipeRows) * 32 + lane;
  const int rh = (hh >> 1) - 1;
  const int colh = (hh & 1) ? w : -1;
  const int jh = PosMod(j0 + rh, d.ny);
  const bool f_on = rf <= rows && 4 * lane < w;
  const bool s_on = rs < rows && 4 * lane < w;
  const bool h_on = warp >= kPipeRows && rh <= rows;
  const int l = 4 * lane + 4;  // slot column of the lane's group

  // prologue: B(t0) (x_in of planes t0-1 .. t0+1, coefficients of t0, w2
  // of t0 and t0+1) and B(t0+1) .. B(t0+kPipeAhead-1)
  {
    const int pz = PosMod(t0, d.nz);
    const int pzm = PosMod(t0 - 1, d.nz), pzp = PosMod(t0 + 1, d.nz);
    if (!ZI) {
      PipeCopy(xs_addr + 4u * 0 * kPipeXSlot, xin + pzm * plane, cx);
      PipeCopy(xs_addr + 4u * 1 * kPipeXSlot, xin + pz * plane, cx);
      PipeCopy(xs_addr + 4u * 2 * kPipeXSlot, xin + pzp * plane, cx);
    }
    const uint32_t cslot = cs_addr + 4u * ((t0 - base) & (kPipeCs - 1)) * kPipeCSlot;
    PipeCopy(cslot, A.w0 + pz * plane, c0w);
    PipeCopy(cslot, A.w1 + pz * plane, c1w);
    PipeCopy(cslot, b + pz * plane, cbb);
    PipeCopy(ws_addr + 4u * 1 * kPipeWSlot, A.w2 + pz * plane, c2w);
    PipeCopy(ws_addr + 4u * 2 * kPipeWSlot, A.w2 + pzp * plane, c2w);
    CpAsyncCommit();
#pragma unroll
    for (int k = 1; k < kPipeAhead; ++k) {
      const int t = t0 + k;
      if (t <= ke) {
        const int64_t pc = (int64_t)PosMod(t, d.nz) * plane;
        const int64_t px = (int64_t)PosMod(t + 1, d.nz) * plane;
        const uint32_t xsl = 4u * ((t + 1 - base) % kPipeXs);
        if (!ZI) PipeCopy(xs_addr + xsl * kPipeXSlot, xin + px, cx);
        const uint32_t cslot2 = cs_addr + 4u * ((t - base) & (kPipeCs - 1)) * kPipeCSlot;
        PipeCopy(cslot2, A.w0 + pc, c0w);
        PipeCopy(cslot2, A.w1 + pc, c1w);
        PipeCopy(cslot2, b + pc, cbb);
        PipeCopy(ws_addr + xsl * kPipeWSlot, A.w2 + px, c2w);
      }
      CpAsyncCommit();
    }
    CpAsyncWait<kPipeAhead - 1>();
    __syncthreads();
  }

  int ph = t0 - base;         // (t - base) mod kPipeXs
  int pz = PosMod(t0, d.nz);  // t mod nz
  for (int t = t0; t <= ke; ++t) {
    auto xslot = [&](int k) {  // x_in / w2 ring slot of plane t + k (-2 <= k <= 3)
      const int v = ph + k;
      return v < 0 ? v + kPipeXs : (v >= kPipeXs ? v - kPipeXs : v);
    };
    const int cs0 = (t - base) & (kPipeCs - 1);
    float* const X0 = XS + xslot(0) * kPipeXSlot;
    float* const Xm1 = XS + xslot(-1) * kPipeXSlot;
    float* const Xp1 = XS + xslot(1) * kPipeXSlot;
    const float* const C0 = CS + cs0 * kPipeCSlot;
    const float* const W20 = WS + xslot(0) * kPipeWSlot;
    const float* const W2p = WS + xslot(1) * kPipeWSlot;
    // F(t)
    if (f_on) {
      float* xc = X0 + (rf + 2) * kPipeStride;
      const float* w0 = C0 + (rf + 1) * kPipeStride;
      const float* w1 = C0 + (kPipeW0Rows + rf + 1) * kPipeStride;
      const float* bb = C0 + (kPipeW0Rows + kPipeW1Rows + rf + 1) * kPipeStride;
      const float* xz0 = Xm1 + (rf + 2) * kPipeStride;
      const float* xz2 = Xp1 + (rf + 2) * kPipeStride;
      const float* z1 = W20 + (rf + 1) * kPipeStride;
      const float* z2 = W2p + (rf + 1) * kPipeStride;
      if ((c0 + jf + pz) & 1)
        PipeFirst<1, ZI>(xc, xc - kPipeStride, xc + kPipeStride, xz0, xz2, w0, w1,
                         w1 + kPipeStride, bb, z1, z2, l);
      else
        PipeFirst<0, ZI>(xc, xc - kPipeStride, xc + kPipeStride, xz0, xz2, w0, w1,
                         w1 + kPipeStride, bb, z1, z2, l);
    }
    CpAsyncWait<kPipeAhead - 2>();  // B(t+1)
    __syncthreads();
    // S(t-1)
    if (t - 1 >= kb && s_on) {
      const int m = t - 1;
      const int pzm = pz == 0 ? d.nz - 1 : pz - 1;
      const float* Fm = XS + xslot(-2) * kPipeXSlot;
      const float* C1 = CS + ((m - base) & (kPipeCs - 1)) * kPipeCSlot;
      const float* f0 = Xm1 + (rs + 2) * kPipeStride;
      const float* w0 = C1 + (rs + 1) * kPipeStride;
      const float* w1 = C1 + (kPipeW0Rows + rs + 1) * kPipeStride;
      const float* bb = C1 + (kPipeW0Rows + kPipeW1Rows + rs + 1) * kPipeStride;
      const float* z1 = WS + xslot(-1) * kPipeWSlot + (rs + 1) * kPipeStride;
      const float* z2 = W20 + (rs + 1) * kPipeStride;
      float* out = xout + pzm * plane + (int64_t)js * d.nx + i0 + 4 * lane;
      if ((c0 + js + pzm) & 1)
        PipeSecond<1>(f0, f0 - kPipeStride, f0 + kPipeStride, Fm + (rs + 2) * kPipeStride,
                      X0 + (rs + 2) * kPipeStride, w0, w1, w1 + kPipeStride, bb, z1, z2, l,
                      out);
      else
        PipeSecond<0>(f0, f0 - kPipeStride, f0 + kPipeStride, Fm + (rs + 2) * kPipeStride,
                      X0 + (rs + 2) * kPipeStride, w0, w1, w1 + kPipeStride, bb, z1, z2, l,
                      out);
    }
    // first colour of the halo columns of plane t (read by S(t))
    if (h_on && t >= kb && t < ke && ((colh + jh + pz + c0) & 1) == 0) {
      const int lh = colh + 4;
      float* xc = X0 + (rh + 2) * kPipeStride;
      const float* w1 = C0 + (kPipeW0Rows + rh + 1) * kPipeStride;
      PipeFirstCell<ZI>(xc, xc - kPipeStride, xc + kPipeStride, Xm1 + (rh + 2) * kPipeStride,
                        Xp1 + (rh + 2) * kPipeStride, C0 + (rh + 1) * kPipeStride, w1,
                        w1 + kPipeStride,
                        C0 + (kPipeW0Rows + kPipeW1Rows + rh + 1) * kPipeStride,
                        W20 + (rh + 1) * kPipeStride, W2p + (rh + 1) * kPipeStride, lh);
    }
    // B(t+kPipeAhead): x_in and w2 of plane t+kPipeAhead+1, coefficients of
    // t+kPipeAhead (their slots were last read before this step's barrier)
    if (t + kPipeAhead <= ke) {
      const int kc = kPipeAhead, kx = kPipeAhead + 1;
      const int pc = pz + kc >= d.nz ? pz + kc - d.nz : pz + kc;
      const int px = pz + kx >= d.nz ? pz + kx - d.nz : pz + kx;
      const uint32_t xsl = (uint32_t)xslot(kx - kPipeXs);
      if (!ZI) PipeCopy(xs_addr + 4u * xsl * kPipeXSlot, xin + px * plane, cx);
      const uint32_t cslot = cs_addr + 4u * ((t + kc - base) & (kPipeCs - 1)) * kPipeCSlot;
      PipeCopy(cslot, A.w0 + pc * plane, c0w);
      PipeCopy(cslot, A.w1 + pc * plane, c1w);
      PipeCopy(cslot, b + pc * plane, cbb);
      PipeCopy(ws_addr + 4u * xsl * kPipeWSlot, A.w2 + px * plane, c2w);
    }
    CpAsyncCommit();
    // L2 prefetch of the rows of B(t+kPipeAhead+kPipePrefetch)
    if (pf_bytes && t + kPipeAhead + kPipePrefetch <= ke) {
      const int k = kPipeAhead + kPipePrefetch + (pf_coef ? 0 : 1);
      const int pp = pz + k >= d.nz ? pz + k - d.nz : pz + k;
      PrefetchBulkL2(pf_src + pp * plane, pf_bytes);
    }
    ph = ph + 1 == kPipeXs ? 0 : ph + 1;
    pz = pz + 1 == d.nz ? 0 : pz + 1;
  }
  CpAsyncWait<0>();
}

}  // namespace aphgpu

namespace aphgpu {

// ---------------------------------------------------------------------------
// Wavefront red-black sweep, in place, one launch per full sweep.
//
// A CTA owns a tile of w <= 128 columns (one float4 per lane) by rows <=
// kWaveRows rows and walks the planes: at step s it updates the first
// colour c0 of plane s (the half sweep's operations, KSmooth4 / Smooth4Body,
// for that plane), publishes "first colour done up to plane s" in its
// progress counter, waits until the four neighbouring tiles have published
// at least s - kWaveLag, and updates the second colour of plane s -
// kWaveLag.  The second colour of plane 0 goes last (it reads the first
// colour of plane nz-1, and the first colour of plane nz-1 reads its old
// values).  Every value is read and written as in the two half sweeps: a
// first-colour update reads old second-colour values (a tile's own second
// colour of plane z changes only at step z + kWaveLag; a neighbour's only
// after this tile published z), a second-colour update reads final
// first-colour values (own planes up to s, the neighbours' after the wait),
// so whole solves are bit-identical to the half sweeps.  The neighbours
// lag each other by at most kWaveLag steps, so a plane's data is still in
// L2 when the second colour re-reads it: HBM traffic is one read of x, b,
// the couplings and one write of x per full sweep (24 B/cell).
//
// The CTAs wait on one another: the launch is cooperative (all CTAs
// resident), every wait is bounded, and a wait that gives up sets err[0]
// and goes on (the sweep's result is then wrong, and the solve reports
// APHGPU_ERR_TIMEOUT).  The minimum-progress tile never waits (its
// neighbours are at least at its own step), so the waits end.
constexpr int kWaveRows = 14;
constexpr int kWaveLag = 2;
constexpr int kWaveThreads = 32 * kWaveRows;

struct WaveTiling {
  int w;       // columns of a tile (multiple of 4, <= 128)
  int rows;    // rows of a band (<= kWaveRows)
  int xtiles, bands;
};

// The rolling z window of one front (first or second colour) of a thread:
// x of planes k-1 and k of its float4 and w2 of plane k.
struct WaveFront {
  float4 xz0, xz1, wz1;
};

// One plane k of one colour at the thread's float4 (column group q, row j),
// in place: the body of Smooth4Body for one plane.  Loads x of plane k+1
// into the window and rolls it.  Every lane of the warp calls it (XHalo).
template <int ZI>
__device__ __forceinline__ void WavePlane(const Op<float>& A, const float* __restrict__ b,
                                          float* x, int color, int q, int j, bool act, int k,
                                          WaveFront& F) {
  const Dims d = A.d;
  const int nq = d.nx >> 2;
  const int i0 = 4 * q;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int kp = wrapp(k + 1, d.nz);
  const int64_t c = d.idx(i0, j, k);
  float4 w0v = make_float4(0, 0, 0, 0), w1v = w0v, w1n = w0v, bv = w0v, xjm = w0v, xjp = w0v;
  float4 xz2 = w0v, wz2 = w0v;
  if (act) {
    wz2 = Ld4(A.w2 + d.idx(i0, j, kp));
    w0v = Ld4(A.w0 + c);
    w1v = Ld4(A.w1 + c);
    w1n = Ld4(A.w1 + d.idx(i0, jp, k));
    bv = Ld4(b + c);
    if (!ZI) {
      xz2 = Ld4(x + d.idx(i0, j, kp));
      xjm = Ld4(x + d.idx(i0, jm, k));
      xjp = Ld4(x + d.idx(i0, jp, k));
    }
  }
  float xl, xr, wl, wr;
  XHalo(x + d.idx(0, act ? j : 0, k), F.xz1, q, nq, act && !ZI, xl, xr);
  XHalo(A.w0 + d.idx(0, act ? j : 0, k), w0v, q, nq, act, wl, wr);
  (void)wl;
  if (act) {
    float4 out = F.xz1;
    const int e0 = (color + j + k) & 1;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      if ((e & 1) != e0) continue;
      const float cxm = El(w0v, e);
      const float cxp = e == 3 ? wr : El(w0v, e + 1);
      const float cym = El(w1v, e), cyp = El(w1n, e);
      const float czm = El(F.wz1, e), czp = El(wz2, e);
      const float dg = A.diag ? A.diag[c + e] : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
      float acc = El(bv, e);
      if (!ZI) {
        const float vxm = e == 0 ? xl : El(F.xz1, e - 1);
        const float vxp = e == 3 ? xr : El(F.xz1, e + 1);
        acc -= cxm * vxm;
        acc -= cxp * vxp;
        acc -= cym * El(xjm, e);
        acc -= cyp * El(xjp, e);
        acc -= czm * El(F.xz0, e);
        acc -= czp * El(xz2, e);
      }
      SetEl(out, e, acc / dg);
    }
    St4(x + c, out);
  }
  F.xz0 = F.xz1;
  F.xz1 = xz2;
  F.wz1 = wz2;
}

// the window of a front about to update plane k
template <int ZI>
__device__ __forceinline__ void WaveInit(const Op<float>& A, const float* x, int q, int j,
                                         bool act, int k, WaveFront& F) {
  const Dims d = A.d;
  const int i0 = 4 * q;
  F.xz0 = F.xz1 = F.wz1 = make_float4(0, 0, 0, 0);
  if (!act) return;
  F.wz1 = Ld4(A.w2 + d.idx(i0, j, k));
  if (!ZI) {
    F.xz0 = Ld4(x + d.idx(i0, j, wrapm(k - 1, d.nz)));
    F.xz1 = Ld4(x + d.idx(i0, j, k));
  }
}

// thread 0 of the CTA: waits (bounded, about 0.3 s) until the four
// neighbouring tiles have published at least z; err[0] = 1 when a wait
// gives up, after which no tile of the grid waits any more
__device__ __forceinline__ void WaveWait(const volatile int* prog, const int* nb, int z,
                                         int* err) {
  const volatile int* verr = err;
  for (int q = 0; q < 4; ++q) {
    int64_t it = 0;
    while (prog[nb[q]] < z && *verr == 0) {
      if (++it > (int64_t(1) << 22)) {
        atomicExch(err, 1);
        break;
      }
      __nanosleep(64);
    }
  }
  __threadfence();
}

// One full sweep (first colour c0; ZI: the first colour starts from zero).
// Grid: one CTA of kWaveThreads per tile (xtiles * bands), cooperative;
// prog: one counter per tile, -1 before the launch.
template <int ZI>
__global__ void __launch_bounds__(kWaveThreads, 1)
    KSweepWave(Op<float> A, const float* __restrict__ b, float* x, int c0,
               const SolveScalars* s, WaveTiling T, int* prog, int* err) {
  if (s && s->done) return;
  const Dims d = A.d;
  const int tile = blockIdx.x;
  const int xt = tile % T.xtiles, band = tile / T.xtiles;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int q = xt * (T.w >> 2) + lane;
  const int j0 = band * T.rows;
  const int rows = min(T.rows, d.ny - j0);
  const int j = j0 + min(wp, rows - 1);
  const bool act = wp < rows && 4 * lane < min(T.w, d.nx - xt * T.w);
  __shared__ int nb[4];
  if (threadIdx.x == 0) {
    nb[0] = band * T.xtiles + (xt == 0 ? T.xtiles - 1 : xt - 1);
    nb[1] = band * T.xtiles + (xt == T.xtiles - 1 ? 0 : xt + 1);
    nb[2] = (band == 0 ? T.bands - 1 : band - 1) * T.xtiles + xt;
    nb[3] = (band == T.bands - 1 ? 0 : band + 1) * T.xtiles + xt;
  }
  WaveFront f0, f1;
  WaveInit<ZI>(A, x, q, j, act, 0, f0);
  __syncthreads();
  const int c1 = 1 - c0;
  const int last = d.nz - 1 + kWaveLag;
  for (int st = 0; st <= last; ++st) {
    if (st < d.nz) {
      // plane st+2 into L2 for the first colour's next steps
      if (act && st + 2 < d.nz) {
        const int64_t cn = d.idx(4 * q, j, st + 2);
        PrefetchL2(A.w0 + cn);
        PrefetchL2(A.w1 + cn);
        PrefetchL2(A.w2 + cn);
        PrefetchL2(b + cn);
        PrefetchL2(x + cn);
      }
      WavePlane<ZI>(A, b, x, c0, q, j, act, st, f0);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        *(volatile int*)(prog + tile) = st;
      }
    }
    const int z = st - kWaveLag;
    if (z >= 1 && z <= d.nz - 1) {
      if (threadIdx.x == 0) WaveWait(prog, nb, z, err);
      __syncthreads();
      if (z == 1) WaveInit<0>(A, x, q, j, act, 1, f1);
      WavePlane<0>(A, b, x, c1, q, j, act, z, f1);
    }
  }
  // the second colour of plane 0, after every first colour of the
  // neighbours (it reads the first colour of plane nz-1)
  if (threadIdx.x == 0) WaveWait(prog, nb, d.nz - 1, err);
  __syncthreads();
  WaveInit<0>(A, x, q, j, act, 0, f1);
  WavePlane<0>(A, b, x, c1, q, j, act, 0, f1);
}

}  // namespace aphgpu

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
// A CTA owns a tile of w <= 128 columns (one float4 per lane) by `rows`
// rows and walks the planes in chunks of K: at step s it updates the first
// colour c0 of the chunk's planes [sK, sK+K) (the half sweep's operations,
// KSmooth4 / Smooth4Body, cell for cell), publishes in its progress counter
// the number of planes whose first colour is done, waits until the four
// neighbouring tiles have published at least the end of chunk s-1, and
// updates the second colour of the planes [(s-1)K - 1, sK - 1) (the first
// of them 1).  After the last chunk the remaining planes up to nz-1 follow,
// and the second colour of plane 0 goes last (it reads the first colour of
// plane nz-1, and the first colour of plane nz-1 reads its old values).
// Every value is read and written as in the two half sweeps: a first-colour
// update reads old second-colour values (a tile's own second colour of plane
// z changes only after its first colour of plane z+1; a neighbour's only
// after this tile published z+1), a second-colour update reads final
// first-colour values (own planes up to the chunk end, the neighbours' after
// the wait), so whole solves are bit-identical to the half sweeps.  Within a
// phase the (plane, row) items are independent and the 16 warps take them
// two at a time, both items' loads issued before either update: a phase is
// a few memory round trips however many planes it covers, and the
// synchronisation (a fence, a release, four polls in parallel, an acquire)
// is paid once per chunk.  The next chunk is prefetched into L2 at the start
// of a step (prefetch.global.L2 of each lane's float4 of the five arrays),
// and the host sizes K so that three chunks of the grid (prefetched, first
// colour, second colour) fit in L2 and a tile's chunk in L1, where the
// items of a phase find the rows their neighbours loaded: HBM traffic is
// one read of x, b and the couplings and one write of x per full sweep
// (24 B/cell).
//
// The CTAs wait on one another: the launch is cooperative (all CTAs
// resident), every wait is bounded, and a wait that gives up sets err[0]
// and goes on (the sweep's result is then wrong, and the solve reports
// APHGPU_ERR_TIMEOUT).  The tile at the smallest step never waits (every
// neighbour has published at least the chunk before), so the waits end.
constexpr int kWaveWarps = 16;
constexpr int kWaveThreads = 32 * kWaveWarps;
constexpr int kWaveRows = 64;

struct WaveTiling {
  int w;       // columns of a tile (multiple of 4, <= 128)
  int rows;    // rows of a band
  int xtiles, bands;
};

// Operands of one (plane k, row j) item of a colour at a thread's float4,
// loaded ahead of its update.  xl, xr, wr: the x and w0 values left and
// right of the float4 where a shuffle cannot supply them (tile edge lanes
// and the periodic wrap).
struct WaveLoads {
  float4 xc, xm, xp, xjm, xjp, wz, wzp, w0v, w1v, w1n, bv;
  float xl, xr, wr;
};

__device__ __forceinline__ float4 Ldcg4(const float* p) {
  return __ldcg(reinterpret_cast<const float4*>(p));
}

// Loads through L1, which is coherent with this CTA's own stores: a
// tile's own rows, and the neighbours' old second-colour values (which no
// one writes before this tile publishes).  SC (second colour): the rows and
// columns of the neighbouring tiles (first-colour values those tiles wrote
// after this SM may have cached the line) are read through L2 only, after
// the acquire of the wait.
template <int ZI, int SC>
__device__ __forceinline__ void WaveLoad(const Op<float>& A, const float* __restrict__ b,
                                         const float* x, int q, int j, int k, bool act,
                                         bool jfirst, bool jlast, WaveLoads& L) {
  const Dims d = A.d;
  const int nq = d.nx >> 2, i0 = 4 * q, sl = threadIdx.x & 31;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  L.xc = L.xm = L.xp = L.xjm = L.xjp = L.wz = L.wzp = L.w0v = L.w1v = L.w1n = L.bv = z4;
  L.xl = L.xr = L.wr = 0.f;
  if (!act) return;
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int km = wrapm(k - 1, d.nz), kp = wrapp(k + 1, d.nz);
  const int64_t c = d.idx(i0, j, k);
  const int64_t row = d.idx(0, j, k);
  const bool right = sl == 31 || q == nq - 1;
  L.wz = Ld4(A.w2 + c);
  L.wzp = Ld4(A.w2 + d.idx(i0, j, kp));
  L.w0v = Ld4(A.w0 + c);
  L.w1v = Ld4(A.w1 + c);
  L.w1n = Ld4(A.w1 + d.idx(i0, jp, k));
  L.bv = Ld4(b + c);
  if (right) L.wr = A.w0[row + (q == nq - 1 ? 0 : 4 * q + 4)];
  if (!ZI) {
    L.xc = Ld4(x + c);
    L.xm = Ld4(x + d.idx(i0, j, km));
    L.xp = Ld4(x + d.idx(i0, j, kp));
    const float* pjm = x + d.idx(i0, jm, k);
    const float* pjp = x + d.idx(i0, jp, k);
    L.xjm = SC && jfirst ? Ldcg4(pjm) : Ld4(pjm);
    L.xjp = SC && jlast ? Ldcg4(pjp) : Ld4(pjp);
    if (sl == 0 || q == 0) L.xl = __ldcg(x + row + (q == 0 ? 4 * nq - 1 : 4 * q - 1));
    if (right) L.xr = __ldcg(x + row + (q == nq - 1 ? 0 : 4 * q + 4));
  }
}

// The update of one item (every lane of the warp calls it: shuffles).
template <int ZI>
__device__ __forceinline__ void WaveUpdate(const Op<float>& A, float* x, int color, int q,
                                           int j, int k, bool act, const WaveLoads& L) {
  const Dims d = A.d;
  const int nq = d.nx >> 2, sl = threadIdx.x & 31;
  float xl = __shfl_up_sync(0xffffffffu, L.xc.w, 1);
  float xr = __shfl_down_sync(0xffffffffu, L.xc.x, 1);
  float wr = __shfl_down_sync(0xffffffffu, L.w0v.x, 1);
  if (!act) return;
  if (sl == 0 || q == 0) xl = L.xl;
  if (sl == 31 || q == nq - 1) {
    xr = L.xr;
    wr = L.wr;
  }
  const int64_t c = d.idx(4 * q, j, k);
  float4 out = L.xc;
  const int e0 = (color + j + k) & 1;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if ((e & 1) != e0) continue;
    const float cxm = El(L.w0v, e);
    const float cxp = e == 3 ? wr : El(L.w0v, e + 1);
    const float cym = El(L.w1v, e), cyp = El(L.w1n, e);
    const float czm = El(L.wz, e), czp = El(L.wzp, e);
    const float dg = A.diag ? A.diag[c + e] : -(((((cxm + cxp) + cym) + cyp) + czm) + czp);
    float acc = El(L.bv, e);
    if (!ZI) {
      const float vxm = e == 0 ? xl : El(L.xc, e - 1);
      const float vxp = e == 3 ? xr : El(L.xc, e + 1);
      acc -= cxm * vxm;
      acc -= cxp * vxp;
      acc -= cym * El(L.xjm, e);
      acc -= cyp * El(L.xjp, e);
      acc -= czm * El(L.xm, e);
      acc -= czp * El(L.xp, e);
    }
    SetEl(out, e, acc / dg);
  }
  St4(x + c, out);
}

// One colour on the planes [p0, p1) of the tile (rows j0 .. j0+rows-1):
// item i = (plane p0 + i / rows, row j0 + i % rows); warp v takes the items
// v, v + 16, v + 32, ... two at a time.
template <int ZI, int SC>
__device__ __forceinline__ void WavePhase(const Op<float>& A, const float* __restrict__ b,
                                          float* x, int color, int p0, int p1, int q,
                                          bool colok, int j0, int rows) {
  const int wp = threadIdx.x >> 5;
  const int n = (p1 - p0) * rows;
  for (int i = wp; i < n; i += 2 * kWaveWarps) {
    const int i2 = i + kWaveWarps;
    const bool two = i2 < n;  // uniform over the warp
    const int k1 = p0 + i / rows, j1 = j0 + i % rows;
    const int k2 = two ? p0 + i2 / rows : k1, j2 = two ? j0 + i2 % rows : j1;
    WaveLoads L1, L2;
    const int jl = j0 + rows - 1;
    WaveLoad<ZI, SC>(A, b, x, q, j1, k1, colok, j1 == j0, j1 == jl, L1);
    WaveLoad<ZI, SC>(A, b, x, q, j2, k2, colok && two, j2 == j0, j2 == jl, L2);
    WaveUpdate<ZI>(A, x, color, q, j1, k1, colok, L1);
    if (two) WaveUpdate<ZI>(A, x, color, q, j2, k2, colok, L2);
  }
}

// the tile's rows of x, b and the couplings on the planes [p0, p1) into L2:
// the items of a phase, each lane its float4 of the five arrays
__device__ __forceinline__ void WavePrefetch(const Op<float>& A, const float* b,
                                             const float* x, int p0, int p1, int q, bool colok,
                                             int j0, int rows) {
  const Dims d = A.d;
  const int wp = threadIdx.x >> 5;
  const int n = (p1 - p0) * rows;
  if (!colok) return;
  for (int i = wp; i < n; i += kWaveWarps) {
    const int64_t c = d.idx(4 * q, j0 + i % rows, p0 + i / rows);
    PrefetchL2(x + c);
    PrefetchL2(b + c);
    PrefetchL2(A.w0 + c);
    PrefetchL2(A.w1 + c);
    PrefetchL2(A.w2 + c);
  }
}

// one thread per neighbour: waits (bounded, at least 0.3 s) until the
// neighbouring tile t has published at least `need` planes; err[0] = 1 when
// a wait gives up, after which no tile of the grid waits any more
__device__ __forceinline__ void WaveWait(const volatile int* prog, int t, int need, int* err) {
  const volatile int* verr = err;
  int64_t it = 0;
  while (prog[t] < need && *verr == 0) {
    if (++it > (int64_t(1) << 22)) {
      atomicExch(err, 1);
      break;
    }
    __nanosleep(64);
  }
  __threadfence();
}

// One full sweep (first colour c0; ZI: the first colour starts from zero).
// Grid: one CTA of kWaveThreads per tile (xtiles * bands), cooperative;
// K: planes per chunk; prog: one counter per tile, -1 before the launch.
template <int ZI>
__global__ void __launch_bounds__(kWaveThreads, 1)
    KSweepWave(Op<float> A, const float* __restrict__ b, float* x, int c0,
               const SolveScalars* s, WaveTiling T, int K, int* prog, int* err) {
  if (s && s->done) return;
  const Dims d = A.d;
  const int tile = blockIdx.x;
  const int xt = tile % T.xtiles, band = tile / T.xtiles;
  const int lane = threadIdx.x & 31;
  const int q = xt * (T.w >> 2) + lane;
  const int i0 = xt * T.w;
  const int wcols = min(T.w, d.nx - i0);
  const bool colok = 4 * lane < wcols;
  const int j0 = band * T.rows;
  const int rows = min(T.rows, d.ny - j0);
  __shared__ int nb[4];
  if (threadIdx.x == 0) {
    nb[0] = band * T.xtiles + (xt == 0 ? T.xtiles - 1 : xt - 1);
    nb[1] = band * T.xtiles + (xt == T.xtiles - 1 ? 0 : xt + 1);
    nb[2] = (band == 0 ? T.bands - 1 : band - 1) * T.xtiles + xt;
    nb[3] = (band == T.bands - 1 ? 0 : band + 1) * T.xtiles + xt;
  }
  __syncthreads();
  const int c1 = 1 - c0;
  const int nch = (d.nz + K - 1) / K;
  WavePrefetch(A, b, x, 0, min(K, d.nz), q, colok, j0, rows);
  int blo = 1;
  for (int st = 0; st <= nch; ++st) {
    if (st < nch) {
      const int p0 = st * K, p1 = min(d.nz, p0 + K);
      if (st + 1 < nch) WavePrefetch(A, b, x, p1, min(d.nz, p1 + K), q, colok, j0, rows);
      WavePhase<ZI, 0>(A, b, x, c0, p0, p1, q, colok, j0, rows);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        *(volatile int*)(prog + tile) = p1;
      }
    }
    // planes whose second colour can go: up to the end of chunk st-1 minus
    // one (every plane after the last chunk)
    const int done = st < nch ? min(d.nz, st * K) : d.nz;
    const int bhi = st < nch ? done - 1 : d.nz;
    if (bhi > blo) {
      if (threadIdx.x < 4) WaveWait(prog, nb[threadIdx.x], done, err);
      __syncthreads();
      WavePhase<0, 1>(A, b, x, c1, blo, bhi, q, colok, j0, rows);
      blo = bhi;
    }
  }
  // the second colour of plane 0 (every neighbour has published nz above)
  __syncthreads();
  WavePhase<0, 1>(A, b, x, c1, 0, 1, q, colok, j0, rows);
}

// The sweep's wait run once on a progress counter that nothing sets
// (prog[0] = -1 before the launch): it gives up after its bound and sets
// err[0], the path a sweep takes when a neighbouring tile never publishes.
__global__ void KWaveWaitProbe(const int* prog, int* err) {
  if (threadIdx.x == 0) WaveWait(prog, 0, 1, err);
}

}  // namespace aphgpu

// Batched mixed-precision solve of many independent periodic domains of
// uneven size: every kernel launch covers all domains at one multigrid
// level.
//
// Each domain keeps its own context for set-up (assembly, FP32 hierarchy,
// dense coarsest inverse, solver vectors).  The batch builds, per domain, a
// descriptor of its level pointers and, per level, tile tables listing
// (domain, tile) pairs.  Kernels are persistent: a fixed grid loops over the
// current table, whose length is read on the device, so the tables can
// shrink to the domains still iterating without touching the captured CUDA
// graph.  Dot products reduce per domain (each domain's tiles share its
// reduction buffer and ticket), and every domain keeps its own stopping
// flags, so domains converge independently while the launches stay shared.
// Levels of a domain at or below `coarse_cells` cells are cycled by one CTA
// per domain in a single launch (pre-smoothing, restriction, dense coarsest
// solve, prolongation, post-smoothing with CTA barriers between them).
//
// Algorithm per domain: the mixed solver of poisson.cu (FP64 defect
// correction around FP32 MG-PCG, constant-mode projection, flexible beta,
// dense FP64 coarsest solve); the domains' hierarchies may differ in depth.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "stencil.cuh"
#include "vec.cuh"

namespace aphgpu {
namespace {

constexpr int kMaxLev = kMgMaxLevels;
constexpr int kCoarseThreads = 512;

struct BLevel {
  Op<float> A;
  float* x;
  float* b;
  const float* invdiag;
  int vec;  // float4 tiles (nx % 4 == 0, nx >= 8)
  int tx;   // float4 columns per row segment of a vectorized tile
};

struct BDom {
  int nlev;
  int lc;  // first level cycled by the per-domain coarse kernel
  BLevel lv[kMaxLev];
  Op<double> A64;
  const double* b64;
  double* x64;
  double* r64;
  float* x32;
  float* r32;
  float* p32;
  float* ap32;
  float* z32;
  SolveScalars* so;  // outer (FP64) scalars
  SolveScalars* si;  // inner (FP32 PCG) scalars
  RedBuf red;
  const double* cinv;
  int cn;
  int csing;  // singular coarsest operator: remove the mean of its b
  int flags;  // inner solver flags (bit 0 projection, bit 1 flexible beta)
};

// One tile of a batched launch: domain, tile coordinates (in float4 columns
// for vectorized levels), and its index among the tiles of the same domain
// in the table (for the per-domain reductions).
struct BTile {
  int dom;
  int bx, by, bz;
  int local, count;
};

// Persistent loop over a table whose length lives on the device.
#define BT_FOR(tab, ntab)                                                   \
  const int nt_ = *(ntab);                                                  \
  for (int ti_ = blockIdx.x; ti_ < nt_; ti_ += gridDim.x) {                 \
    const BTile t = (tab)[ti_];
#define BT_FOR_END }

// Thread coordinates in a tile of tx columns and 256 / tx rows: column
// t.bx * tx + (lane mod tx), row from the lane's row segment and warp.
__device__ __forceinline__ void TileCoords(const BTile& t, int tx, int& q, int& j) {
  q = t.bx * tx + (threadIdx.x & (tx - 1));
  j = t.by * ((kTileX * kTileY) / tx) + threadIdx.y * (kTileX / tx) + threadIdx.x / tx;
}

// Cells of a fine-level tile of domain D: w = 4 on vectorized tiles (tx
// float4 columns, 4 consecutive cells per thread) else 1 (tx = 32: 32 x 8).
#define BT_CELLS_BEGIN(dims, w, tx)                                         \
  {                                                                         \
    int q_, j;                                                              \
    TileCoords(t, (tx), q_, j);                                             \
    const int i0_ = q_ * (w);                                               \
    const int kb_ = t.bz * kz;                                              \
    const int ke_ = min(kb_ + kz, (dims).nz);                               \
    if (i0_ < (dims).nx && j < (dims).ny) {                                 \
      for (int k = kb_; k < ke_; ++k) {                                     \
        for (int e_ = 0; e_ < (w); ++e_) {                                  \
          const int i = i0_ + e_;                                           \
          const int64_t c = (dims).idx(i, j, k);
#define BT_CELLS_END \
        }            \
      }              \
    }                \
  }

// ---------------------------------------------------------------------------
// Outer (FP64) kernels on the outer fine table
// ---------------------------------------------------------------------------

// r = b - A x (FP64), per-domain reductions r.r, max|r|, b.b; on the first
// call the tolerance becomes max(tol, rtol ||b|| / sqrt(h^3)) (rtol in
// so->tmp[3]); then the stopping test of the outer iteration.
template <bool VEC>
__global__ void KBResidual64(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                             const int* ntab, int kz, int first) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.so;
  if (s->done) continue;
  const Op<double>& A = D.A64;
  const Dims& d = A.d;
  constexpr int w = VEC ? 4 : 1;
  double v[3] = {0, 0, 0};
  const int op[3] = {0, 1, 0};
  const double* x = D.x64;
  BT_CELLS_BEGIN(d, w, VEC ? D.lv[0].tx : kTileX)
  // the first outer residual is that of the zero initial guess: r = b
  double u = -D.b64[c];
  if (!first) {
    double e[6];
    Couplings(A, i, j, k, c, e);
    const double e0 = Diag(A, c, e);
    u = x[c] * e0 + (-D.b64[c]);
    u += x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
    u += x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
    u += x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
    u += x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
    u += x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
    u += x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  }
  const double rv = -u;
  D.r64[c] = rv;
  v[0] += rv * rv;
  v[1] = fmax(v[1], fabs(rv));
  v[2] += D.b64[c] * D.b64[c];
  BT_CELLS_END
  __shared__ double out[3];
  if (GroupReduce<3>(v, op, D.red, out, t.local, t.count)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      if (first) {
        s->tmp[0] = out[2];
        const double tr = s->tmp[3] * sqrt(out[2] / s->cellvol);
        if (tr > s->tol) s->tol = tr;
      }
      s->residual = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
  BT_FOR_END
}

// r32 = r64 / max|r|, x32 = 0 (scale kept in so->tmp[1])
template <bool VEC>
__global__ void KBScaleZero(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                            const int* ntab, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.so;
  if (s->done) continue;
  const double scale = s->maxr > 0 ? s->maxr : 1.0;
  if (t.local == 0 && threadIdx.x == 0 && threadIdx.y == 0) s->tmp[1] = scale;
  const double inv = 1.0 / scale;
  constexpr int w = VEC ? 4 : 1;
  BT_CELLS_BEGIN(D.A64.d, w, VEC ? D.lv[0].tx : kTileX)
  D.r32[c] = (float)(D.r64[c] * inv);
  D.x32[c] = 0.f;
  BT_CELLS_END
  BT_FOR_END
}

// x64 += scale * x32
template <bool VEC>
__global__ void KBAddCorrection(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                                const int* ntab, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  if (D.so->done) continue;
  const double scale = D.so->maxr > 0 ? D.so->maxr : 1.0;
  constexpr int w = VEC ? 4 : 1;
  BT_CELLS_BEGIN(D.A64.d, w, VEC ? D.lv[0].tx : kTileX)
  D.x64[c] += scale * (double)D.x32[c];
  BT_CELLS_END
  BT_FOR_END
}

// inner scalars of every domain from its outer state (one thread per domain)
__global__ void KBInnerInit(BDom* doms, int ndom, double inner_rtol, int inner_maxiter) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ndom) return;
  const BDom& D = doms[q];
  const SolveScalars* so = D.so;
  SolveScalars z{};
  const double scale = so->maxr > 0 ? so->maxr : 1.0;
  // inner_rtol, or only the reduction left to the outer tolerance (with a
  // margin of 0.3) when that is less
  double f = inner_rtol;
  if (so->tol > 0 && so->residual > 0) f = fmax(f, fmin(0.5, 0.3 * so->tol / so->residual));
  z.tol = f * sqrt(so->rr / so->cellvol) / scale;
  z.cellvol = so->cellvol;
  z.res_scale = 1.0;
  z.miniter = 1;
  z.maxiter = inner_maxiter;
  z.maxnorm = 0;
  z.flags = D.flags;
  z.done = so->done;
  *D.si = z;
}

// outer iteration count and accumulated inner iterations (so->tmp[2])
__global__ void KBOuterAdvance(BDom* doms, int ndom) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ndom) return;
  SolveScalars* so = doms[q].so;
  if (so->done) return;
  so->iter += 1;
  so->tmp[2] += (double)doms[q].si->iter;
}

// per-domain flag "still iterating" of the inner (which = 1) or outer (0)
// solve, and their count in flags[ndom]
__global__ void KBActive(const BDom* __restrict__ doms, int ndom, int which, int* flags) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  for (int q = threadIdx.x; q < ndom; q += blockDim.x) {
    const int a = (which ? doms[q].si->done : doms[q].so->done) ? 0 : 1;
    flags[q] = a;
    mine += a;
  }
  atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0) flags[ndom] = cnt;
}

// ---------------------------------------------------------------------------
// FP32 multigrid kernels on the batched levels (tile tables per level)
// ---------------------------------------------------------------------------

// Red-black half sweep on level l (the update of KSmooth / KSmooth4).
template <bool VEC>
__global__ void __launch_bounds__(256, 3) KBSmooth(const BDom* __restrict__ doms,
                                                   const BTile* __restrict__ tab,
                                                   const int* ntab, int l, int kz, int color,
                                                   int zero_init) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  if (D.si->done) continue;
  const BLevel& L = D.lv[l];
  const Dims& d = L.A.d;
  if constexpr (VEC) {
    const int kb = t.bz * kz;
    int q, j;
    TileCoords(t, L.tx, q, j);
    Smooth4Body(L.A, L.b, L.x, color, zero_init, q, j, kb, min(kb + kz, d.nz), L.tx);
    continue;
  }
  float* x = L.x;
  BT_CELLS_BEGIN(d, 1, kTileX)
  if (((i + j + k) & 1) != color) continue;
  if (zero_init) {
    x[c] = L.b[c] * L.invdiag[c];
    continue;
  }
  float e[6];
  Couplings(L.A, i, j, k, c, e);
  float acc = L.b[c];
  acc -= x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
  acc -= x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
  acc -= x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
  acc -= x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
  acc -= x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
  acc -= x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  x[c] = acc * L.invdiag[c];
  BT_CELLS_END
  BT_FOR_END
}

// Residual of level l summed over the children into b of level l+1; the
// table tiles level l+1 (vectorized: float4 columns of level l, i.e. two
// coarse cells per thread).
template <bool VEC>
__global__ void __launch_bounds__(256, 3) KBRestrict(const BDom* __restrict__ doms,
                                                     const BTile* __restrict__ tab,
                                                     const int* ntab, int l, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  if (D.si->done) continue;
  const BLevel& F = D.lv[l];
  const BLevel& C = D.lv[l + 1];
  const Dims& dc = C.A.d;
  const int Kb = t.bz * kz;
  const int Ke = min(Kb + kz, dc.nz);
  if constexpr (VEC) {
    int q, J;
    TileCoords(t, F.tx, q, J);
    ResidualRestrict4Body(F.A, F.b, F.x, dc, C.b, q, J, Kb, Ke, F.tx);
    continue;
  }
  const int I = t.bx * kTileX + threadIdx.x;
  const int J = t.by * kTileY + threadIdx.y;
  if (I >= dc.nx || J >= dc.ny) continue;
  for (int K = Kb; K < Ke; ++K) {
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
      const int64_t c = F.A.d.idx(i, j, k);
      sum += F.b[c] - Apply(F.A, F.x, i, j, k, c);
    }
    C.b[dc.idx(I, J, K)] = sum;
  }
  BT_FOR_END
}

// x of level l += x of level l+1 at the parent
template <bool VEC>
__global__ void __launch_bounds__(256, 4) KBProlong(const BDom* __restrict__ doms,
                                                    const BTile* __restrict__ tab,
                                                    const int* ntab, int l, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  if (D.si->done) continue;
  const BLevel& F = D.lv[l];
  const BLevel& C = D.lv[l + 1];
  const Dims& d = F.A.d;
  const Dims& dc = C.A.d;
  if constexpr (VEC) {
    const int kb = t.bz * kz;
    int q, j;
    TileCoords(t, F.tx, q, j);
    Prolong4Body(d, F.x, dc, C.x, q, j, kb, min(kb + kz, d.nz));
    continue;
  }
  BT_CELLS_BEGIN(d, 1, kTileX)
  F.x[c] += C.x[dc.idx(i >> 1, j >> 1, k >> 1)];
  BT_CELLS_END
  BT_FOR_END
}

// ---------------------------------------------------------------------------
// Per-domain cycle of the coarse levels (one CTA per domain)
// ---------------------------------------------------------------------------

// Coordinates (i, j, k) of the cells start, start + stride, ... of a level,
// advanced without integer divisions (the divisions per cell made the
// one-CTA passes issue-bound).
struct CellWalk {
  int i, j, k, si, sj, sk;
  __device__ CellWalk(const Dims& d, int start, int stride) {
    i = start % d.nx;
    const int r = start / d.nx;
    j = r % d.ny;
    k = r / d.ny;
    si = stride % d.nx;
    const int rs = stride / d.nx;
    sj = rs % d.ny;
    sk = rs / d.ny;
  }
  __device__ void Next(const Dims& d) {
    i += si;
    int cj = sj;
    if (i >= d.nx) {
      i -= d.nx;
      ++cj;
    }
    j += cj;
    int ck = sk;
    if (j >= d.ny) {
      j -= d.ny;
      ++ck;
    }
    k += ck;
  }
};

__device__ void CtaSmooth(const BLevel& L, int color, int zero_init) {
  const Dims& d = L.A.d;
  const int n = (int)d.cells();
  float* x = L.x;
  CellWalk w(d, threadIdx.x, blockDim.x);
  for (int c = threadIdx.x; c < n; c += blockDim.x, w.Next(d)) {
    const int i = w.i, j = w.j, k = w.k;
    if (((i + j + k) & 1) != color) continue;
    if (zero_init) {
      x[c] = L.b[c] * L.invdiag[c];
      continue;
    }
    float e[6];
    Couplings(L.A, i, j, k, c, e);
    float acc = L.b[c];
    acc -= x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
    acc -= x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
    acc -= x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
    acc -= x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
    acc -= x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
    acc -= x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
    x[c] = acc * L.invdiag[c];
  }
}

__device__ void CtaRestrict(const BLevel& F, const BLevel& C) {
  const Dims& dc = C.A.d;
  const int n = (int)dc.cells();
  CellWalk w(dc, threadIdx.x, blockDim.x);
  for (int cc = threadIdx.x; cc < n; cc += blockDim.x, w.Next(dc)) {
    const int I = w.i, J = w.j, K = w.k;
    float sum = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = 2 * I + (q & 1), j = 2 * J + ((q >> 1) & 1), k = 2 * K + (q >> 2);
      const int64_t c = F.A.d.idx(i, j, k);
      sum += F.b[c] - Apply(F.A, F.x, i, j, k, c);
    }
    C.b[cc] = sum;
  }
}

__device__ void CtaProlong(const BLevel& F, const BLevel& C) {
  const Dims& d = F.A.d;
  const Dims& dc = C.A.d;
  const int n = (int)d.cells();
  CellWalk w(d, threadIdx.x, blockDim.x);
  for (int c = threadIdx.x; c < n; c += blockDim.x, w.Next(d)) {
    F.x[c] += C.x[dc.idx(w.i >> 1, w.j >> 1, w.k >> 1)];
  }
}

// coarsest level: x = B^{-1} (b - mean b) with the dense inverse, the mean
// removed only for a singular operator (see KCoarsestDense)
__device__ void CtaDense(const BDom& D) {
  const BLevel& C = D.lv[D.nlev - 1];
  const int n = D.cn;
  __shared__ double sb[kDenseMax];
  __shared__ double red[kCoarseThreads / 32];
  const int tid = threadIdx.x;
  double part = 0;
  for (int c = tid; c < n; c += blockDim.x) {
    const double v = (double)C.b[c];
    sb[c] = v;
    part += v;
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) red[tid >> 5] = part;
  __syncthreads();
  if (tid == 0) {
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    red[0] = D.csing ? s / n : 0.0;
  }
  __syncthreads();
  const double mean = red[0];
  for (int r = tid; r < n; r += blockDim.x) {
    const double* row = D.cinv + (int64_t)r * n;
    double acc = 0;
    for (int c = 0; c < n; ++c) acc += row[c] * (sb[c] - mean);
    C.x[r] = (float)acc;
  }
}

// Levels lc .. nlev-1 of one domain: one multigrid cycle of those levels
// (pre-smoothing colours 0 then 1, post colours 1 then 0, as the launched
// levels), each level below lc visited `gamma` times per visit of the level
// above (1 V-cycle, 2 W-cycle; the exactly solved coarsest level once),
// CTA barriers between the passes; sweeps(l, 0) / sweeps(l, 1) are the
// pre / post sweeps of level l.  `first`: level lc starts from a zero
// guess (else from its current x, a repeated W-cycle visit).  The cycle is
// iterative: todo[l] counts the visits of level l+1 still to make from
// level l.
template <class Sweeps>
__device__ void CoarseCycleBody(const BDom& D, Sweeps sweeps, int gamma, bool first) {
  const int L = D.nlev;
  int todo[kMaxLev];
  int l = D.lc;
  for (;;) {
    if (l < L - 1) {
      // enter level l: pre-smoothing (zero guess on its first visit) and
      // restriction of its residual
      const BLevel& F = D.lv[l];
      const int pre = sweeps(l, 0);
      if (pre > 0) {
        for (int sw = 0; sw < pre; ++sw) {
          CtaSmooth(F, 0, first && sw == 0);
          __syncthreads();
          CtaSmooth(F, 1, 0);
          __syncthreads();
        }
      } else if (first) {
        CtaSmooth(F, 0, 1);
        __syncthreads();
        CtaSmooth(F, 1, 1);
        __syncthreads();
      }
      CtaRestrict(F, D.lv[l + 1]);
      __syncthreads();
      todo[l] = l + 1 == L - 1 ? 1 : gamma;
      ++l;
      first = true;
      continue;
    }
    CtaDense(D);
    __syncthreads();
    // leave levels upward until one still has a visit of its coarser level
    // to make
    for (;;) {
      --l;
      if (l < D.lc) return;
      if (--todo[l] > 0) {
        ++l;
        first = false;
        break;
      }
      const BLevel& F = D.lv[l];
      CtaProlong(F, D.lv[l + 1]);
      __syncthreads();
      const int post = sweeps(l, 1);
      for (int sw = 0; sw < post; ++sw) {
        CtaSmooth(F, 1, 0);
        __syncthreads();
        CtaSmooth(F, 0, 0);
        __syncthreads();
      }
    }
  }
}

// The coarse levels of every domain of a batch (one CTA per domain).
__global__ void __launch_bounds__(kCoarseThreads) KBCoarseCycle(const BDom* __restrict__ doms,
                                                                int pre, int post, int gamma) {
  const BDom& D = doms[blockIdx.x];
  if (D.si->done) return;
  CoarseCycleBody(D, [=](int, int which) { return which ? post : pre; }, gamma, true);
}

// The smallest levels of one single-domain hierarchy in one CTA (their
// launches would be latency-bound), with per-level sweep counts.
struct LevelSweepCounts {
  int pre[kMaxLev];
  int post[kMaxLev];
};

// Floats per cell of a level staged in shared memory: x, b, three
// couplings, diagonal, inverse diagonal.
constexpr int kStagedFloats = 7;

// The levels lc .. nlev-1 are staged in dynamic shared memory for the whole
// cycle (their couplings, diagonals and level lc's right-hand side and,
// on a repeated visit, its x are read once; level lc's x is written back
// at the end), and the cycle runs on the staged copies.
__global__ void __launch_bounds__(kCoarseThreads) KCoarseCycleOne(const BDom* __restrict__ dom,
                                                                  LevelSweepCounts sw, int gamma,
                                                                  int first,
                                                                  const SolveScalars* s) {
  if (s && s->done) return;
  extern __shared__ float staged[];
  __shared__ BDom S;
  const int tid = threadIdx.x;
  if (tid == 0) {
    S = *dom;
    int64_t off = 0;
    for (int l = S.lc; l < S.nlev; ++l) {
      BLevel& L = S.lv[l];
      const int64_t n = L.A.d.cells();
      float* base = staged + off;
      L.x = base;
      L.b = base + n;
      L.A.w0 = base + 2 * n;
      L.A.w1 = base + 3 * n;
      L.A.w2 = base + 4 * n;
      L.A.diag = L.A.diag ? base + 5 * n : nullptr;
      L.invdiag = base + 6 * n;
      off += kStagedFloats * n;
    }
  }
  __syncthreads();
  const BDom& G = *dom;
  for (int l = S.lc; l < S.nlev; ++l) {
    const BLevel& g = G.lv[l];
    const BLevel& t = S.lv[l];
    const int n = (int)g.A.d.cells();
    float* w0 = const_cast<float*>(t.A.w0);
    float* w1 = const_cast<float*>(t.A.w1);
    float* w2 = const_cast<float*>(t.A.w2);
    float* dg = const_cast<float*>(t.A.diag);
    float* idg = const_cast<float*>(t.invdiag);
    for (int c = tid; c < n; c += blockDim.x) {
      w0[c] = g.A.w0[c];
      w1[c] = g.A.w1[c];
      w2[c] = g.A.w2[c];
      if (dg) dg[c] = g.A.diag[c];
      idg[c] = g.invdiag[c];
      if (l == S.lc) {
        t.b[c] = g.b[c];
        if (!first) t.x[c] = g.x[c];
      }
    }
  }
  __syncthreads();
  CoarseCycleBody(S, [&](int l, int which) { return which ? sw.post[l] : sw.pre[l]; },
                  gamma, first != 0);
  __syncthreads();
  const int n = (int)G.lv[S.lc].A.d.cells();
  for (int c = tid; c < n; c += blockDim.x) G.lv[S.lc].x[c] = S.lv[S.lc].x[c];
}

// ---------------------------------------------------------------------------
// FP32 PCG kernels on the finest level (fine table)
// ---------------------------------------------------------------------------

// column q (float4 units) and row j of the thread in a fine tile
#define BT_VEC_COORDS                              \
  int q, j;                                        \
  TileCoords(t, D.lv[0].tx, q, j);                 \
  const int kb = t.bz * kz;                        \
  const int ke = min(kb + kz, d.nz);               \
  const bool act = 4 * q < d.nx && j < d.ny;

// ap = A p with the per-domain reductions p.Ap and sum Ap; alpha
template <bool VEC>
__global__ void __launch_bounds__(256, 3) KBApply(const BDom* __restrict__ doms,
                                                  const BTile* __restrict__ tab,
                                                  const int* ntab, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) continue;
  const Op<float>& A = D.lv[0].A;
  const Dims& d = A.d;
  float fa0 = 0.f, fa1 = 0.f;
  if constexpr (VEC) {
    const int kb = t.bz * kz;
    int q, j;
    TileCoords(t, D.lv[0].tx, q, j);
    Apply4Body(A, D.p32, D.ap32, q, j, kb, min(kb + kz, d.nz), fa0, fa1, D.lv[0].tx);
  } else {
    BT_CELLS_BEGIN(d, 1, kTileX)
    const float y = Apply(A, D.p32, i, j, k, c);
    D.ap32[c] = y;
    fa0 += D.p32[c] * y;
    fa1 += y;
    BT_CELLS_END
  }
  double v[2] = {(double)fa0, (double)fa1};
  const int op[2] = {0, 0};
  __shared__ double out[2];
  if (GroupReduce<2>(v, op, D.red, out, t.local, t.count)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->pap = out[0];
      s->apsum = out[1];
      s->alpha = s->rz / (out[0] + 1e-300);
    }
  }
  BT_FOR_END
}

// x += alpha p, r -= alpha (ap - mean ap); reductions r.r, max|r| and, for
// the flexible beta, r_new . z_old (z still holds the previous
// preconditioned residual until the next V-cycle); stopping test
template <bool VEC>
__global__ void __launch_bounds__(256, 4) KBUpdate(const BDom* __restrict__ doms,
                                                   const BTile* __restrict__ tab,
                                                   const int* ntab, int kz) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) continue;
  const Dims& d = D.lv[0].A.d;
  const float alpha = (float)s->alpha;
  const float apm = (s->flags & 1) ? (float)(s->apsum / (double)d.cells()) : 0.f;
  const bool flex = (s->flags & 2) != 0;
  float r2 = 0.f, rmax = 0.f, rzo = 0.f;
  if constexpr (VEC) {
    BT_VEC_COORDS
    if (act) {
      for (int k = kb; k < ke; ++k) {
        const int64_t c = d.idx(4 * q, j, k);
        float4 xv = Ld4(D.x32 + c), rv = Ld4(D.r32 + c);
        const float4 pv = Ld4(D.p32 + c), av = Ld4(D.ap32 + c);
        xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
        rv.x -= alpha * (av.x - apm); rv.y -= alpha * (av.y - apm);
        rv.z -= alpha * (av.z - apm); rv.w -= alpha * (av.w - apm);
        St4(D.x32 + c, xv);
        St4(D.r32 + c, rv);
        r2 += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
        rmax = fmaxf(rmax, fmaxf(fmaxf(fabsf(rv.x), fabsf(rv.y)),
                                 fmaxf(fabsf(rv.z), fabsf(rv.w))));
        if (flex) {
          const float4 zv = Ld4(D.z32 + c);
          rzo += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
        }
      }
    }
  } else {
    BT_CELLS_BEGIN(d, 1, kTileX)
    D.x32[c] += alpha * D.p32[c];
    const float rn = D.r32[c] - alpha * (D.ap32[c] - apm);
    D.r32[c] = rn;
    r2 += rn * rn;
    rmax = fmaxf(rmax, fabsf(rn));
    if (flex) rzo += rn * D.z32[c];
    BT_CELLS_END
  }
  double v[3] = {(double)r2, (double)rmax, (double)rzo};
  const int op[3] = {0, 1, 0};
  __shared__ double out[3];
  if (GroupReduce<3>(v, op, D.red, out, t.local, t.count)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      s->rzold = out[2];
      s->residual = sqrt(out[0] / s->cellvol);
      s->iter += 1;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
  BT_FOR_END
}

// rz = r.z; beta = rz / rz_prev, or (rz - r.z_old) / rz_prev when flexible
template <bool VEC>
__global__ void __launch_bounds__(256, 4) KBDotRZ(const BDom* __restrict__ doms,
                                                  const BTile* __restrict__ tab,
                                                  const int* ntab, int kz, int first) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) continue;
  const Dims& d = D.lv[0].A.d;
  float a = 0.f;
  if constexpr (VEC) {
    BT_VEC_COORDS
    if (act) {
      for (int k = kb; k < ke; ++k) {
        const int64_t c = d.idx(4 * q, j, k);
        const float4 rv = Ld4(D.r32 + c), zv = Ld4(D.z32 + c);
        a += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
      }
    }
  } else {
    BT_CELLS_BEGIN(d, 1, kTileX)
    a += D.r32[c] * D.z32[c];
    BT_CELLS_END
  }
  double v[1] = {(double)a};
  const int op[1] = {0};
  __shared__ double out[1];
  if (GroupReduce<1>(v, op, D.red, out, t.local, t.count)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rz_prev = first ? 0.0 : s->rz;
      s->rz = out[0];
      const double num = (s->flags & 2) ? out[0] - s->rzold : out[0];
      s->beta = first ? 0.0 : num / (s->rz_prev + 1e-300);
    }
  }
  BT_FOR_END
}

// p = z + beta p (p = z when first)
template <bool VEC>
__global__ void __launch_bounds__(256, 4) KBP(const BDom* __restrict__ doms,
                                              const BTile* __restrict__ tab, const int* ntab,
                                              int kz, int first) {
  BT_FOR(tab, ntab)
  const BDom& D = doms[t.dom];
  const SolveScalars* s = D.si;
  if (s->done) continue;
  const Dims& d = D.lv[0].A.d;
  const float beta = (float)s->beta;
  if constexpr (VEC) {
    BT_VEC_COORDS
    if (act) {
      for (int k = kb; k < ke; ++k) {
        const int64_t c = d.idx(4 * q, j, k);
        const float4 zv = Ld4(D.z32 + c);
        float4 pv = first ? zv : Ld4(D.p32 + c);
        if (!first) {
          pv.x = zv.x + beta * pv.x; pv.y = zv.y + beta * pv.y;
          pv.z = zv.z + beta * pv.z; pv.w = zv.w + beta * pv.w;
        }
        St4(D.p32 + c, pv);
      }
    }
  } else {
    BT_CELLS_BEGIN(d, 1, kTileX)
    D.p32[c] = first ? D.z32[c] : D.z32[c] + beta * D.p32[c];
    BT_CELLS_END
  }
  BT_FOR_END
}

}  // namespace
}  // namespace aphgpu

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

namespace aphgpu {
namespace {

// A tile table: each domain's tiles (host), the device table of the domains
// currently included, and the slot of its length in the device length array.
struct BTable {
  std::vector<std::vector<BTile>> by_dom;
  BTile* d_tab = nullptr;
  int cap = 0;   // tiles of all domains
  int n = 0;     // tiles currently in the device table
  int slot = 0;  // index in the length array
  size_t stage = 0;  // offset in the pinned staging buffer (tiles)
};

// The tiles of one kind of launch, split by tiling: k[1] vectorized levels,
// k[0] the others (each domain's tiles are in one of them); the kernels are
// instantiated for each.
struct BTableSet {
  BTable k[2];
};

}  // namespace
}  // namespace aphgpu

struct aphgpu_batch {
  std::vector<aphgpu_ctx*> ctxs;
  int ndom = 0;
  int nlev_max = 0;
  int kz = 4;                 // planes per thread of the batched tiles
  int coarse_cells = 4096;    // levels with at most this many cells: per-domain CTA
  int cycle = 1;              // visits of each per-domain coarse level (1 V, 2 W)
  int device = 0;
  int sms = 0;
  cudaStream_t st = nullptr;  // stream of the first context
  aphgpu::BDom* d_doms = nullptr;
  int* d_flags = nullptr;     // per-domain active flags + count
  int* h_flags = nullptr;     // pinned
  int* d_len = nullptr;       // table lengths
  int* h_len = nullptr;       // pinned
  aphgpu::BTile* h_stage = nullptr;  // pinned staging of the tables
  size_t stage_cap = 0;
  // tables: outer (fine level, domains of the outer iteration), fine (inner
  // iteration), per batched level (smoothing, prolongation) and per
  // restriction (tiles of the coarser level)
  aphgpu::BTableSet outer, fine;
  std::vector<aphgpu::BTableSet> lev, res;
  uint64_t layout_key = 0;
  std::vector<std::pair<const void*, int>> grids;  // persistent grid per kernel
  // captured batch of inner iterations
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_key = 0;
  int64_t graph_kernels = 0;
  int64_t launches = 0;
  double last_ms = 0;
  std::string err;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace aphgpu {
namespace {

int BErr(aphgpu_batch* B, int code, const char* what) {
  B->err = what;
  return code;
}

int BCuda(aphgpu_batch* B, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return APHGPU_OK;
  cudaGetLastError();
  B->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? APHGPU_ERR_NOMEM : APHGPU_ERR_CUDA;
}

#define B_CUDA(B, expr) APH_TRY(BCuda((B), (expr), #expr))
#define B_LAUNCHED(B)                                                       \
  do {                                                                      \
    ++(B)->launches;                                                        \
    const cudaError_t le_ = cudaGetLastError();                             \
    if (le_ != cudaSuccess) return BCuda((B), le_, "batched kernel launch"); \
  } while (0)

inline uint64_t BMix(uint64_t h, uint64_t v) {
  return h ^ (v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2));
}

// Persistent grid of a kernel: its resident CTAs per SM times the SMs,
// capped by the table capacity.
int BGrid(aphgpu_batch* B, const void* fn, int cap) {
  int per_sm = 0;
  for (auto& g : B->grids)
    if (g.first == fn) per_sm = g.second;
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kTileX * kTileY, 0) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 2;
    }
    B->grids.emplace_back(fn, per_sm);
  }
  return std::max(1, std::min(cap, per_sm * B->sms));
}

// float4 columns per row segment for a row of nq float4s: the power of two
// >= nq, at most a warp
inline int TxOf(int nq) {
  int tx = 1;
  while (tx < nq && tx < kTileX) tx *= 2;
  return tx;
}

// Tiles of level dims d for domain `dom`; vectorized (tx > 0): tx float4
// columns of a row of xcells cells (the level whose float4 columns the
// threads own) by 256 / tx rows; else 32 x 8 cells.
void DomTiles(std::vector<BTile>& out, int dom, const Dims& d, int tx, int xcells, int kz) {
  const int gx = tx ? ((xcells / 4) + tx - 1) / tx : (d.nx + kTileX - 1) / kTileX;
  const int rows = tx ? (kTileX * kTileY) / tx : kTileY;
  const int gy = (d.ny + rows - 1) / rows;
  const int gz = (d.nz + kz - 1) / kz;
  const int count = gx * gy * gz;
  int local = 0;
  out.clear();
  for (int bz = 0; bz < gz; ++bz)
    for (int by = 0; by < gy; ++by)
      for (int bx = 0; bx < gx; ++bx) out.push_back(BTile{dom, bx, by, bz, local++, count});
}

inline bool BVec(const Dims& d) { return (d.nx % 4) == 0 && d.nx >= 8; }

void FreeSet(BTableSet& S) {
  for (BTable& T : S.k) {
    if (T.d_tab) cudaFree(T.d_tab);
    T = BTable{};
  }
}

// every table of the batch (outer first when `outer`, then the inner ones)
std::vector<BTable*> Tables(aphgpu_batch* B, bool outer) {
  std::vector<BTable*> v;
  auto add = [&](BTableSet& S) {
    v.push_back(&S.k[0]);
    v.push_back(&S.k[1]);
  };
  if (outer) add(B->outer);
  add(B->fine);
  for (auto& S : B->lev) add(S);
  for (auto& S : B->res) add(S);
  return v;
}

// Descriptors and tile tables from the contexts' current hierarchies
// (rebuilt only when the hierarchies or the tiling change).
int BuildTables(aphgpu_batch* B, const aphgpu_conf* conf) {
  uint64_t key = 1469598103934665603ull;
  for (auto* c : B->ctxs) {
    int rc = EnsureSolverVectors(c);
    if (rc == APHGPU_OK) rc = EnsureMixedHierarchy(c, conf);
    if (rc != APHGPU_OK) return BErr(B, rc, aphgpu_last_error(c));
    key = BMix(key, (uint64_t)(uintptr_t)c);
    key = BMix(key, (uint64_t)c->mg_epoch);
    key = BMix(key, (uint64_t)(uintptr_t)c->mg.l32[0].w[0]);
    key = BMix(key, (uint64_t)(c->singular ? 1 : 0));
  }
  key = BMix(key, (uint64_t)B->kz);
  key = BMix(key, (uint64_t)B->coarse_cells);
  key = BMix(key, (uint64_t)conf->inner_flags);
  if (key == B->layout_key && B->d_doms) return APHGPU_OK;
  std::vector<BDom> doms(B->ndom);
  B->nlev_max = 0;
  for (int q = 0; q < B->ndom; ++q) {
    aphgpu_ctx* c = B->ctxs[q];
    auto& lv = c->mg.l32;
    const int nl = (int)lv.size();
    if (nl > kMaxLev) return BErr(B, APHGPU_ERR_UNSUPPORTED, "too many multigrid levels");
    if (!c->mg.cinv32 || c->mg.cn32 != (int)lv.back().d.cells())
      return BErr(B, APHGPU_ERR_UNSUPPORTED,
                  "coarsest level too large for the batch (dense solve of at most 1024 cells)");
    BDom& D = doms[q];
    std::memset(&D, 0, sizeof(D));
    D.nlev = nl;
    D.lc = nl - 1;
    for (int l = 0; l < nl; ++l)
      if (lv[l].d.cells() <= B->coarse_cells) {
        D.lc = l;
        break;
      }
    for (int l = 0; l < nl; ++l) {
      BLevel& L = D.lv[l];
      L.A = Op<float>{lv[l].d, lv[l].w[0], lv[l].w[1], lv[l].w[2],
                      lv[l].has_diag ? lv[l].diag : nullptr};
      L.invdiag = lv[l].invdiag;
      L.x = l == 0 ? c->z32 : lv[l].x;
      L.b = l == 0 ? c->r32 : lv[l].b;
      // vectorized where the single-domain solver is (not on CTA levels)
      L.vec = BVec(lv[l].d) && (l == 0 || l < D.lc) ? 1 : 0;
      L.tx = L.vec ? TxOf(lv[l].d.nx / 4) : kTileX;
    }
    D.A64 = Op<double>{c->d, c->w[0], c->w[1], c->w[2], c->diag_valid ? c->diag : nullptr};
    D.b64 = c->b;
    D.x64 = c->x;
    D.r64 = c->r;
    D.x32 = c->x32;
    D.r32 = c->r32;
    D.p32 = c->p32;
    D.ap32 = c->ap32;
    D.z32 = c->z32;
    D.so = c->scal;
    D.si = c->scal2;
    D.red = c->red;
    D.cinv = c->mg.cinv32;
    D.cn = c->mg.cn32;
    D.csing = c->mg.csing32;
    // the constant-mode projection holds only for the singular operator
    D.flags = c->singular ? conf->inner_flags : (conf->inner_flags & ~1);
    B->nlev_max = std::max(B->nlev_max, nl);
  }
  if (!B->d_doms) B_CUDA(B, cudaMalloc(&B->d_doms, sizeof(BDom) * B->ndom));
  B_CUDA(B, cudaMemcpy(B->d_doms, doms.data(), sizeof(BDom) * B->ndom, cudaMemcpyHostToDevice));
  // per-domain tiles of every table
  FreeSet(B->outer);
  FreeSet(B->fine);
  for (auto& S : B->lev) FreeSet(S);
  for (auto& S : B->res) FreeSet(S);
  const int nb = std::max(B->nlev_max - 1, 0);
  B->lev.assign(nb, BTableSet{});
  B->res.assign(nb, BTableSet{});
  std::vector<BTable*> all = Tables(B, true);
  for (BTable* T : all) T->by_dom.resize(B->ndom);
  for (int q = 0; q < B->ndom; ++q) {
    const BDom& D = doms[q];
    const Dims& d0 = D.lv[0].A.d;
    const int v0 = D.lv[0].vec;
    DomTiles(B->outer.k[v0].by_dom[q], q, d0, v0 ? D.lv[0].tx : 0, d0.nx, B->kz);
    B->fine.k[v0].by_dom[q] = B->outer.k[v0].by_dom[q];
    for (int l = 0; l < D.lc; ++l) {
      const Dims& d = D.lv[l].A.d;
      const int v = D.lv[l].vec;
      const int tx = v ? D.lv[l].tx : 0;
      DomTiles(B->lev[l].k[v].by_dom[q], q, d, tx, d.nx, B->kz);
      DomTiles(B->res[l].k[v].by_dom[q], q, D.lv[l + 1].A.d, tx, d.nx, B->kz);
    }
  }
  size_t total = 0;
  for (size_t s = 0; s < all.size(); ++s) {
    BTable& T = *all[s];
    T.cap = 0;
    for (auto& v : T.by_dom) T.cap += (int)v.size();
    for (auto& v : T.by_dom)
      for (auto& t : v)
        if (t.count > B->ctxs[t.dom]->red.max_blocks)
          return BErr(B, APHGPU_ERR_UNSUPPORTED, "reduction buffer too small for the tiles");
    T.slot = (int)s;
    T.stage = total;
    total += (size_t)T.cap;
    if (T.cap) B_CUDA(B, cudaMalloc(&T.d_tab, sizeof(BTile) * T.cap));
  }
  if (B->stage_cap < total) {
    if (B->h_stage) cudaFreeHost(B->h_stage);
    B->h_stage = nullptr;
    B_CUDA(B, cudaMallocHost(&B->h_stage, sizeof(BTile) * std::max<size_t>(total, 1)));
    B->stage_cap = total;
  }
  if (B->d_len) cudaFree(B->d_len);
  if (B->h_len) cudaFreeHost(B->h_len);
  B->d_len = nullptr;
  B->h_len = nullptr;
  B_CUDA(B, cudaMalloc(&B->d_len, sizeof(int) * all.size()));
  B_CUDA(B, cudaMallocHost(&B->h_len, sizeof(int) * all.size()));
  B_CUDA(B, cudaMemset(B->d_len, 0, sizeof(int) * all.size()));
  std::memset(B->h_len, 0, sizeof(int) * all.size());
  B->layout_key = key;
  return APHGPU_OK;
}

// Device tables hold the tiles of the domains with active[q] != 0: the inner
// tables always, the outer table too when `outer` is set.  Called with the
// stream idle (the staging buffer is reused).
int Activate(aphgpu_batch* B, const int* active, bool outer) {
  const std::vector<BTable*> ts = Tables(B, outer);
  const int nslots = (int)Tables(B, true).size();
  for (BTable* T : ts) {
    BTile* dst = B->h_stage + T->stage;
    int n = 0;
    for (int q = 0; q < B->ndom; ++q) {
      if (!active[q]) continue;
      const auto& v = T->by_dom[q];
      std::memcpy(dst + n, v.data(), sizeof(BTile) * v.size());
      n += (int)v.size();
    }
    T->n = n;
    B->h_len[T->slot] = n;
    if (n)
      B_CUDA(B, cudaMemcpyAsync(T->d_tab, dst, sizeof(BTile) * n, cudaMemcpyHostToDevice, B->st));
  }
  B_CUDA(B, cudaMemcpyAsync(B->d_len, B->h_len, sizeof(int) * nslots, cudaMemcpyHostToDevice,
                            B->st));
  return APHGPU_OK;
}

// Active flags of the inner (which = 1) or outer (0) solve into h_flags
// (count at h_flags[ndom]).
int BActive(aphgpu_batch* B, int which) {
  KBActive<<<1, 256, 0, B->st>>>(B->d_doms, B->ndom, which, B->d_flags);
  B_LAUNCHED(B);
  B_CUDA(B, cudaMemcpyAsync(B->h_flags, B->d_flags, sizeof(int) * (B->ndom + 1),
                            cudaMemcpyDeviceToHost, B->st));
  B_CUDA(B, cudaStreamSynchronize(B->st));
  return APHGPU_OK;
}

// launches kernel<false> on the scalar tiles and kernel<true> on the
// vectorized tiles of table set S (each only if it can hold tiles)
#define B_TABLE_LAUNCH(B, kernel, S, ...)                                            \
  do {                                                                               \
    if ((S).k[0].cap) {                                                              \
      kernel<false><<<BGrid((B), (const void*)kernel<false>, (S).k[0].cap), TileBlock(), 0, \
                      (B)->st>>>((B)->d_doms, (S).k[0].d_tab, (B)->d_len + (S).k[0].slot,  \
                                 __VA_ARGS__);                                       \
      B_LAUNCHED(B);                                                                 \
    }                                                                                \
    if ((S).k[1].cap) {                                                              \
      kernel<true><<<BGrid((B), (const void*)kernel<true>, (S).k[1].cap), TileBlock(), 0,   \
                     (B)->st>>>((B)->d_doms, (S).k[1].d_tab, (B)->d_len + (S).k[1].slot,   \
                                __VA_ARGS__);                                        \
      B_LAUNCHED(B);                                                                 \
    }                                                                                \
  } while (0)

int BVCycle(aphgpu_batch* B, int pre, int post) {
  const int kz = B->kz;
  const int nb = (int)B->lev.size();
  for (int l = 0; l < nb; ++l) {
    // pre == 0: both colours only take x = b / diag (zero initial guess)
    for (int sw = 0; sw < std::max(pre, 1); ++sw) {
      B_TABLE_LAUNCH(B, KBSmooth, B->lev[l], l, kz, 0, sw == 0 ? 1 : 0);
      B_TABLE_LAUNCH(B, KBSmooth, B->lev[l], l, kz, 1, pre == 0 ? 1 : 0);
    }
    B_TABLE_LAUNCH(B, KBRestrict, B->res[l], l, kz);
  }
  KBCoarseCycle<<<B->ndom, kCoarseThreads, 0, B->st>>>(B->d_doms, pre, post, B->cycle);
  B_LAUNCHED(B);
  for (int l = nb - 1; l >= 0; --l) {
    B_TABLE_LAUNCH(B, KBProlong, B->lev[l], l, kz);
    for (int sw = 0; sw < post; ++sw) {
      B_TABLE_LAUNCH(B, KBSmooth, B->lev[l], l, kz, 1, 0);
      B_TABLE_LAUNCH(B, KBSmooth, B->lev[l], l, kz, 0, 0);
    }
  }
  return APHGPU_OK;
}

// One batch of `every` inner iterations (captured once into a graph).
int BInnerBody(aphgpu_batch* B, const aphgpu_conf* conf, int every) {
  const int kz = B->kz;
  for (int it = 0; it < every; ++it) {
    B_TABLE_LAUNCH(B, KBApply, B->fine, kz);
    B_TABLE_LAUNCH(B, KBUpdate, B->fine, kz);
    APH_TRY(BVCycle(B, conf->mg_pre, conf->mg_post));
    B_TABLE_LAUNCH(B, KBDotRZ, B->fine, kz, 0);
    B_TABLE_LAUNCH(B, KBP, B->fine, kz, 0);
  }
  return APHGPU_OK;
}

int BEnsureGraph(aphgpu_batch* B, const aphgpu_conf* conf, int every) {
  uint64_t key = B->layout_key;
  key = BMix(key, (uint64_t)(conf->mg_pre * 1000 + conf->mg_post));
  key = BMix(key, (uint64_t)every);
  key = BMix(key, (uint64_t)B->cycle);
  if (B->graph && B->graph_key == key) return APHGPU_OK;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  B->graph = nullptr;
  const int64_t l0 = B->launches;
  cudaGraph_t g = nullptr;
  bool ok = cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  const int rc = ok ? BInnerBody(B, conf, every) : APHGPU_OK;
  ok = (cudaStreamEndCapture(B->st, &g) == cudaSuccess) && ok && rc == APHGPU_OK;
  B->launches = l0;  // captured launches are counted when replayed
  if (ok && cudaGraphInstantiate(&B->graph, g, 0) == cudaSuccess) {
    size_t nn = 0;
    if (cudaGraphGetNodes(g, nullptr, &nn) != cudaSuccess) nn = 0;
    B->graph_kernels = (int64_t)nn;
    B->graph_key = key;
  } else {
    B->graph = nullptr;  // launched directly instead
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  return APHGPU_OK;
}

int BSolve(aphgpu_batch* B, const aphgpu_conf* conf, aphgpu_info* infos) {
  cudaStream_t st = B->st;
  const int kz = B->kz;
  const int every = 4;
  // all contexts' pending work (assembly) is finished before the batch runs
  for (auto* c : B->ctxs) B_CUDA(B, cudaStreamSynchronize(c->stream));
  APH_TRY(BuildTables(B, conf));
  // outer scalars, zero initial guess
  for (auto* c : B->ctxs) {
    SolveScalars h{};
    h.tol = conf->tol;
    h.cellvol = c->h * c->h * c->h;
    h.res_scale = 1.0;
    h.miniter = conf->miniter;
    h.maxiter = conf->maxiter;
    h.maxnorm = conf->maxnorm;
    h.tmp[3] = conf->rtol;
    B_CUDA(B, cudaMemcpyAsync(c->scal, &h, sizeof(h), cudaMemcpyHostToDevice, st));
    B_CUDA(B, cudaMemsetAsync(c->x, 0, sizeof(double) * c->N, st));
  }
  B_CUDA(B, cudaStreamSynchronize(st));
  APH_TRY(BEnsureGraph(B, conf, every));
  std::vector<int> all(B->ndom, 1);
  APH_TRY(Activate(B, all.data(), true));
  B_CUDA(B, cudaEventRecord(B->ev0, st));
  B_TABLE_LAUNCH(B, KBResidual64, B->outer, kz, 1);
  for (int outer = 0; outer <= conf->maxiter + 1; ++outer) {
    APH_TRY(BActive(B, 0));
    if (!B->h_flags[B->ndom]) break;
    std::vector<int> act(B->h_flags, B->h_flags + B->ndom);
    APH_TRY(Activate(B, act.data(), true));
    B_TABLE_LAUNCH(B, KBScaleZero, B->outer, kz);
    KBInnerInit<<<(B->ndom + 127) / 128, 128, 0, st>>>(B->d_doms, B->ndom, conf->inner_rtol,
                                                       conf->inner_maxiter);
    B_LAUNCHED(B);
    APH_TRY(BVCycle(B, conf->mg_pre, conf->mg_post));
    B_TABLE_LAUNCH(B, KBDotRZ, B->fine, kz, 1);
    B_TABLE_LAUNCH(B, KBP, B->fine, kz, 1);
    for (int b = 0; b <= conf->inner_maxiter / every + 2; ++b) {
      if (B->graph) {
        B_CUDA(B, cudaGraphLaunch(B->graph, st));
        B->launches += B->graph_kernels;
      } else {
        APH_TRY(BInnerBody(B, conf, every));
      }
      APH_TRY(BActive(B, 1));
      if (!B->h_flags[B->ndom]) break;
      // shrink the inner tables to the domains still iterating once they
      // hold a quarter fewer tiles
      int tiles = 0;
      for (int q = 0; q < B->ndom; ++q)
        if (B->h_flags[q])
          tiles += (int)(B->fine.k[0].by_dom[q].size() + B->fine.k[1].by_dom[q].size());
      if (4 * tiles <= 3 * (B->fine.k[0].n + B->fine.k[1].n)) {
        std::vector<int> in(B->h_flags, B->h_flags + B->ndom);
        APH_TRY(Activate(B, in.data(), false));
      }
    }
    B_TABLE_LAUNCH(B, KBAddCorrection, B->outer, kz);
    KBOuterAdvance<<<(B->ndom + 127) / 128, 128, 0, st>>>(B->d_doms, B->ndom);
    B_LAUNCHED(B);
    B_TABLE_LAUNCH(B, KBResidual64, B->outer, kz, 0);
  }
  B_CUDA(B, cudaEventRecord(B->ev1, st));
  B_CUDA(B, cudaEventSynchronize(B->ev1));
  float ms = 0;
  B_CUDA(B, cudaEventElapsedTime(&ms, B->ev0, B->ev1));
  B->last_ms = ms;
  if (infos) {
    for (int q = 0; q < B->ndom; ++q) {
      SolveScalars h{};
      B_CUDA(B, cudaMemcpy(&h, B->ctxs[q]->scal, sizeof(h), cudaMemcpyDeviceToHost));
      infos[q].residual = h.residual;
      infos[q].iter = h.iter;
      infos[q].inner_iter = (int)h.tmp[2];
      infos[q].converged = h.converged;
    }
  }
  return APHGPU_OK;
}

}  // namespace
}  // namespace aphgpu

extern "C" {

int aphgpu_batch_create(aphgpu_batch** out, int count, aphgpu_ctx* const* ctxs) {
  using namespace aphgpu;
  if (!out || count < 1 || !ctxs) return APHGPU_ERR_ARG;
  for (int q = 0; q < count; ++q)
    if (!ctxs[q] || !ctxs[q]->stream || ctxs[q]->device != ctxs[0]->device)
      return APHGPU_ERR_ARG;
  aphgpu_batch* B = new (std::nothrow) aphgpu_batch();
  if (!B) return APHGPU_ERR_NOMEM;
  B->ctxs.assign(ctxs, ctxs + count);
  B->ndom = count;
  B->st = ctxs[0]->stream;
  B->device = ctxs[0]->device;
  if (cudaSetDevice(B->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, B->device) != cudaSuccess ||
      cudaEventCreate(&B->ev0) != cudaSuccess || cudaEventCreate(&B->ev1) != cudaSuccess ||
      cudaMalloc(&B->d_flags, sizeof(int) * (count + 1)) != cudaSuccess ||
      cudaMallocHost(&B->h_flags, sizeof(int) * (count + 1)) != cudaSuccess) {
    cudaGetLastError();
    aphgpu_batch_destroy(B);
    return APHGPU_ERR_CUDA;
  }
  // persistent grids are queried outside any stream capture
  BGrid(B, (const void*)KBResidual64<false>, 1);
  BGrid(B, (const void*)KBResidual64<true>, 1);
  BGrid(B, (const void*)KBScaleZero<false>, 1);
  BGrid(B, (const void*)KBScaleZero<true>, 1);
  BGrid(B, (const void*)KBAddCorrection<false>, 1);
  BGrid(B, (const void*)KBAddCorrection<true>, 1);
  BGrid(B, (const void*)KBSmooth<false>, 1);
  BGrid(B, (const void*)KBSmooth<true>, 1);
  BGrid(B, (const void*)KBRestrict<false>, 1);
  BGrid(B, (const void*)KBRestrict<true>, 1);
  BGrid(B, (const void*)KBProlong<false>, 1);
  BGrid(B, (const void*)KBProlong<true>, 1);
  BGrid(B, (const void*)KBApply<false>, 1);
  BGrid(B, (const void*)KBApply<true>, 1);
  BGrid(B, (const void*)KBUpdate<false>, 1);
  BGrid(B, (const void*)KBUpdate<true>, 1);
  BGrid(B, (const void*)KBDotRZ<false>, 1);
  BGrid(B, (const void*)KBDotRZ<true>, 1);
  BGrid(B, (const void*)KBP<false>, 1);
  BGrid(B, (const void*)KBP<true>, 1);
  *out = B;
  return APHGPU_OK;
}

void aphgpu_batch_destroy(aphgpu_batch* B) {
  if (!B) return;
  cudaSetDevice(B->device);
  if (B->st) cudaStreamSynchronize(B->st);
  if (B->graph) cudaGraphExecDestroy(B->graph);
  aphgpu::FreeSet(B->outer);
  aphgpu::FreeSet(B->fine);
  for (auto& S : B->lev) aphgpu::FreeSet(S);
  for (auto& S : B->res) aphgpu::FreeSet(S);
  if (B->d_doms) cudaFree(B->d_doms);
  if (B->d_flags) cudaFree(B->d_flags);
  if (B->h_flags) cudaFreeHost(B->h_flags);
  if (B->d_len) cudaFree(B->d_len);
  if (B->h_len) cudaFreeHost(B->h_len);
  if (B->h_stage) cudaFreeHost(B->h_stage);
  if (B->ev0) cudaEventDestroy(B->ev0);
  if (B->ev1) cudaEventDestroy(B->ev1);
  delete B;
}

const char* aphgpu_batch_last_error(const aphgpu_batch* B) {
  return B ? B->err.c_str() : "null batch";
}

int aphgpu_batch_solve(aphgpu_batch* B, const aphgpu_conf* conf, aphgpu_info* infos) {
  if (!B || !conf) return APHGPU_ERR_ARG;
  if (conf->mg_pre < 0 || conf->mg_post < 0 || conf->inner_maxiter < 1)
    return aphgpu::BErr(B, APHGPU_ERR_ARG, "invalid multigrid settings");
  for (auto* c : B->ctxs)
    if (!c->has_system) return aphgpu::BErr(B, APHGPU_ERR_STATE, "a context has no system");
  if (cudaSetDevice(B->device) != cudaSuccess) return APHGPU_ERR_CUDA;
  return aphgpu::BSolve(B, conf, infos);
}

int aphgpu_batch_set_tiles(aphgpu_batch* B, int planes, int coarse_cells) {
  if (!B || planes < 1 || planes > 64 || coarse_cells < 0) return APHGPU_ERR_ARG;
  B->kz = planes;
  B->coarse_cells = coarse_cells;
  return APHGPU_OK;
}

int aphgpu_batch_get_tiles(const aphgpu_batch* B, int* planes, int* coarse_cells) {
  if (!B) return APHGPU_ERR_ARG;
  if (planes) *planes = B->kz;
  if (coarse_cells) *coarse_cells = B->coarse_cells;
  return APHGPU_OK;
}

int aphgpu_batch_set_cycle(aphgpu_batch* B, int cycle) {
  if (!B || cycle < 1 || cycle > 2) return APHGPU_ERR_ARG;
  B->cycle = cycle;
  return APHGPU_OK;
}

int aphgpu_batch_get_cycle(const aphgpu_batch* B, int* cycle) {
  if (!B || !cycle) return APHGPU_ERR_ARG;
  *cycle = B->cycle;
  return APHGPU_OK;
}

int aphgpu_batch_tune(aphgpu_batch* B, aphgpu_conf* conf, double* best_ms) {
  if (!B || !conf) return APHGPU_ERR_ARG;
  // coordinate search: tile planes x coarse-level size x cycle at the given
  // sweeps, then the sweeps at the best of those
  const int kzs[] = {2, 4, 8};
  const int coarse[] = {512, 4096, 32768};
  const int cycles[] = {1, 2};
  const int sweeps[] = {1, 2, 3};
  double best = 1e300;
  int best_kz = B->kz, best_cc = B->coarse_cells, best_cy = B->cycle, best_sw = conf->mg_pre;
  aphgpu_conf c = *conf;
  c.mg_post = c.mg_pre;
  for (int kz : kzs) {
    for (int cc : coarse) {
      for (int cy : cycles) {
        B->kz = kz;
        B->coarse_cells = cc;
        B->cycle = cy;
        const int rc = aphgpu_batch_solve(B, &c, nullptr);
        if (rc != APHGPU_OK) return rc;
        if (B->last_ms < best) {
          best = B->last_ms;
          best_kz = kz;
          best_cc = cc;
          best_cy = cy;
        }
      }
    }
  }
  B->kz = best_kz;
  B->coarse_cells = best_cc;
  B->cycle = best_cy;
  for (int sw : sweeps) {
    if (sw == c.mg_pre) continue;
    aphgpu_conf t = c;
    t.mg_pre = t.mg_post = sw;
    const int rc = aphgpu_batch_solve(B, &t, nullptr);
    if (rc != APHGPU_OK) return rc;
    if (B->last_ms < best) {
      best = B->last_ms;
      best_sw = sw;
    }
  }
  conf->mg_pre = conf->mg_post = best_sw;
  if (best_ms) *best_ms = best;
  return APHGPU_OK;
}

int aphgpu_batch_last_ms(const aphgpu_batch* B, double* ms, int64_t* launches) {
  if (!B) return APHGPU_ERR_ARG;
  if (ms) *ms = B->last_ms;
  if (launches) *launches = B->launches;
  return APHGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Single-domain hierarchies: the smallest FP32 levels in one CTA
// ---------------------------------------------------------------------------

namespace aphgpu {

// Levels of at most this many cells (and below) are cycled by one CTA,
// staged in at most this much dynamic shared memory (the kernel's static
// shared memory, the coarsest right-hand side and the copy of the level
// description, stays within the 227 KB of a CTA).
constexpr int64_t kCoarseOneCells = 512;
constexpr size_t kCoarseOneSmem = 200 * 1024;

int CoarseOneSetup(aphgpu_ctx* ctx) {
  Multigrid& mg = ctx->mg;
  const std::vector<Level<float>>& lv = mg.l32;
  const int L = (int)lv.size();
  mg.clc = -1;
  if (L < 3 || L > kMaxLev || !mg.cinv32 || mg.cn32 != (int)lv.back().d.cells())
    return APHGPU_OK;
  int lc = L - 1;
  while (lc - 1 >= 1 && lv[lc - 1].d.cells() <= kCoarseOneCells) --lc;
  if (lc > L - 2) return APHGPU_OK;  // no level to smooth besides the coarsest
  BDom D{};
  D.nlev = L;
  D.lc = lc;
  for (int l = lc; l < L; ++l) {
    BLevel& b = D.lv[l];
    b.A = MakeOp(lv[l]);
    b.x = lv[l].x;
    b.b = lv[l].b;
    b.invdiag = lv[l].invdiag;
    b.vec = 0;
    b.tx = 0;
  }
  D.cinv = mg.cinv32;
  D.cn = mg.cn32;
  D.csing = mg.csing32;
  // the staged levels must fit the shared memory of one CTA
  int64_t staged = 0;
  for (int l = lc; l < L; ++l) staged += kStagedFloats * lv[l].d.cells();
  const size_t bytes = sizeof(float) * (size_t)staged;
  if (bytes > kCoarseOneSmem) return APHGPU_OK;
  APH_CUDA(ctx, cudaFuncSetAttribute(KCoarseCycleOne, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kCoarseOneSmem));
  mg.csmem = (int)bytes;
  if (!mg.cdom) {
    char* p = nullptr;
    APH_TRY(Alloc(ctx, &p, (int64_t)sizeof(BDom)));
    mg.cdom = p;
  }
  APH_CUDA(ctx, cudaMemcpyAsync(mg.cdom, &D, sizeof(BDom), cudaMemcpyHostToDevice, ctx->stream));
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  mg.clc = lc;
  return APHGPU_OK;
}

int CoarseOneLaunch(aphgpu_ctx* ctx, const int* pre, const int* post, int gamma, bool first,
                    const SolveScalars* s) {
  const Multigrid& mg = ctx->mg;
  LevelSweepCounts sw{};
  for (int l = 0; l < kMaxLev; ++l) {
    sw.pre[l] = pre[l];
    sw.post[l] = post[l];
  }
  KCoarseCycleOne<<<1, kCoarseThreads, mg.csmem, ctx->stream>>>((const BDom*)mg.cdom, sw,
                                                                 gamma, first ? 1 : 0, s);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

}  // namespace aphgpu

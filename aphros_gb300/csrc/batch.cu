// Batched mixed-precision solve of many independent periodic domains of
// uneven size: every kernel launch covers all domains at one multigrid
// level.
//
// Each domain keeps its own context for set-up (assembly, FP32 hierarchy,
// dense coarsest inverse, solver vectors).  The batch builds, per domain, a
// descriptor of its level pointers and, per level, a tile table listing
// (domain, tile) pairs; a CTA reads its entry and works on that domain's
// tile.  Dot products reduce per domain (each domain's CTAs share its
// reduction buffer and ticket), and every domain keeps its own stopping
// flags, so domains converge independently while the launches stay shared.
// Batches of inner iterations are captured into one CUDA graph.
//
// Algorithm per domain: the mixed solver of poisson.cu (FP64 defect
// correction around FP32 MG-PCG, constant-mode projection, dense FP64
// coarsest solve); the domains' hierarchies may have different depths.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "stencil.cuh"

namespace aphgpu {
namespace {

constexpr int kMaxLev = 12;

struct BLevel {
  Op<float> A;
  float* x;
  float* b;
  const float* invdiag;
};

struct BDom {
  int nlev;
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
  int flags;  // inner solver flags (bit 0 projection, bit 1 flexible beta)
  double cellvol;
};

// one CTA of a batched launch: domain, tile coordinates, and its index among
// the CTAs of the same domain in this launch
struct BTile {
  int dom;
  int bx, by, bz;
  int local, count;
};

#define BT_BEGIN(dims)                                           \
  const int i = t.bx * kTileX + threadIdx.x;                     \
  const int j = t.by * kTileY + threadIdx.y;                     \
  const int kb = t.bz * kz;                                      \
  const int ke = min(kb + kz, (dims).nz);                        \
  const bool inxy = i < (dims).nx && j < (dims).ny;              \
  for (int k = kb; k < ke; ++k) {                                \
    if (!inxy) continue;                                         \
    const int64_t c = (dims).idx(i, j, k);
#define BT_END }

// ---------------------------------------------------------------------------
// Outer (FP64) kernels
// ---------------------------------------------------------------------------

// r = b - A x (FP64), per-domain reductions r.r, max|r|, b.b; on the first
// call the tolerance becomes max(tol, rtol ||b||) (rtol in so->tmp[3]);
// then the stopping test of the outer iteration.
__global__ void KBResidual64(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                             int kz, int first) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.so;
  if (s->done) return;
  const Op<double>& A = D.A64;
  double v[3] = {0, 0, 0};
  const int op[3] = {0, 1, 0};
  BT_BEGIN(A.d)
  double e[6];
  Couplings(A, i, j, k, c, e);
  const double e0 = Diag(A, c, e);
  const Dims& d = A.d;
  const double* x = D.x64;
  double u = x[c] * e0 + (-D.b64[c]);
  u += x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
  u += x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
  u += x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
  u += x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
  u += x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
  u += x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  const double rv = -u;
  D.r64[c] = rv;
  v[0] += rv * rv;
  v[1] = fmax(v[1], fabs(rv));
  v[2] += D.b64[c] * D.b64[c];
  BT_END
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
}

// r32 = r64 / max|r|, x32 = 0 (scale kept in so->tmp[1])
__global__ void KBScaleZero(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                            int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.so;
  if (s->done) return;
  const double scale = s->maxr > 0 ? s->maxr : 1.0;
  if (t.local == 0 && threadIdx.x == 0 && threadIdx.y == 0) s->tmp[1] = scale;
  const double inv = 1.0 / scale;
  BT_BEGIN(D.A64.d)
  D.r32[c] = (float)(D.r64[c] * inv);
  D.x32[c] = 0.f;
  BT_END
}

// x64 += scale * x32
__global__ void KBAddCorrection(const BDom* __restrict__ doms, const BTile* __restrict__ tab,
                                int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  if (D.so->done) return;
  const double scale = D.so->maxr > 0 ? D.so->maxr : 1.0;
  BT_BEGIN(D.A64.d)
  D.x64[c] += scale * (double)D.x32[c];
  BT_END
}

// inner scalars of every domain from its outer state (one thread per domain)
__global__ void KBInnerInit(BDom* doms, int ndom, double inner_rtol, int inner_maxiter) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ndom) return;
  const BDom& D = doms[q];
  const SolveScalars* so = D.so;
  SolveScalars z{};
  const double scale = so->maxr > 0 ? so->maxr : 1.0;
  z.tol = inner_rtol * sqrt(so->rr / so->cellvol) / scale;
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

// number of domains whose inner (which = 1) or outer (0) solve still runs
__global__ void KBCountActive(const BDom* __restrict__ doms, int ndom, int which, int* out) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  int mine = 0;
  for (int q = threadIdx.x; q < ndom; q += blockDim.x)
    mine += (which ? doms[q].si->done : doms[q].so->done) ? 0 : 1;
  atomicAdd(&cnt, mine);
  __syncthreads();
  if (threadIdx.x == 0) *out = cnt;
}

// ---------------------------------------------------------------------------
// FP32 multigrid kernels (tile tables per level)
// ---------------------------------------------------------------------------

// red-black half sweep on level l (see KSmooth in poisson.cu)
__global__ void KBSmooth(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int l,
                         int kz, int color, int zero_init) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  if (D.si->done) return;
  const BLevel& L = D.lv[l];
  const Op<float>& A = L.A;
  const Dims& d = A.d;
  float* x = L.x;
  BT_BEGIN(d)
  if (((i + j + k) & 1) != color) continue;
  if (zero_init) {
    x[c] = L.b[c] * L.invdiag[c];
    continue;
  }
  float e[6];
  Couplings(A, i, j, k, c, e);
  float acc = L.b[c];
  acc -= x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[0];
  acc -= x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[1];
  acc -= x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[2];
  acc -= x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[3];
  acc -= x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[4];
  acc -= x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[5];
  x[c] = acc * L.invdiag[c];
  BT_END
}

// residual of level l summed over children into b of level l+1; the table
// tiles level l+1
__global__ void KBRestrict(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int l,
                           int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  if (D.si->done) return;
  const BLevel& F = D.lv[l];
  const BLevel& C = D.lv[l + 1];
  const Dims& dc = C.A.d;
  const int I = t.bx * kTileX + threadIdx.x;
  const int J = t.by * kTileY + threadIdx.y;
  const int Kb = t.bz * kz;
  const int Ke = min(Kb + kz, dc.nz);
  if (I >= dc.nx || J >= dc.ny) return;
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
}

// x of level l += x of level l+1 at the parent
__global__ void KBProlong(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int l,
                          int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  if (D.si->done) return;
  const BLevel& F = D.lv[l];
  const BLevel& C = D.lv[l + 1];
  const Dims& dc = C.A.d;
  BT_BEGIN(F.A.d)
  F.x[c] += C.x[dc.idx(i >> 1, j >> 1, k >> 1)];
  BT_END
}

// coarsest level of every domain: x = B^{-1} (b - mean b), one CTA per domain
__global__ void __launch_bounds__(256) KBCoarsest(const BDom* __restrict__ doms) {
  const BDom& D = doms[blockIdx.x];
  if (D.si->done) return;
  const BLevel& C = D.lv[D.nlev - 1];
  const int n = D.cn;
  __shared__ double sb[kDenseMax];
  __shared__ double red[8];
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
    red[0] = s / n;
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

// ---------------------------------------------------------------------------
// FP32 PCG kernels on the finest level (fine tile table)
// ---------------------------------------------------------------------------

__global__ void KBApply(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) return;
  const Op<float>& A = D.lv[0].A;
  float fa0 = 0.f, fa1 = 0.f;
  BT_BEGIN(A.d)
  const float y = Apply(A, D.p32, i, j, k, c);
  D.ap32[c] = y;
  fa0 += D.p32[c] * y;
  fa1 += y;
  BT_END
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
}

__global__ void KBUpdate(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int kz) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) return;
  const Dims& d = D.lv[0].A.d;
  const float alpha = (float)s->alpha;
  const float apm = (s->flags & 1) ? (float)(s->apsum / (double)d.cells()) : 0.f;
  const bool flex = (s->flags & 2) != 0;
  float r2 = 0.f, rmax = 0.f, rzo = 0.f;
  BT_BEGIN(d)
  D.x32[c] += alpha * D.p32[c];
  const float rn = D.r32[c] - alpha * (D.ap32[c] - apm);
  D.r32[c] = rn;
  r2 += rn * rn;
  rmax = fmaxf(rmax, fabsf(rn));
  // flexible variant: new residual against the previous preconditioned
  // residual, which z still holds until the next V-cycle overwrites it
  if (flex) rzo += rn * D.z32[c];
  BT_END
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
}

__global__ void KBDotRZ(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int kz,
                        int first) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  SolveScalars* s = D.si;
  if (s->done) return;
  float a = 0.f;
  BT_BEGIN(D.lv[0].A.d)
  a += D.r32[c] * D.z32[c];
  BT_END
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
}

__global__ void KBP(const BDom* __restrict__ doms, const BTile* __restrict__ tab, int kz,
                    int first) {
  const BTile t = tab[blockIdx.x];
  const BDom& D = doms[t.dom];
  const SolveScalars* s = D.si;
  if (s->done) return;
  const float beta = (float)s->beta;
  BT_BEGIN(D.lv[0].A.d)
  D.p32[c] = first ? D.z32[c] : D.z32[c] + beta * D.p32[c];
  BT_END
}

}  // namespace
}  // namespace aphgpu

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct aphgpu_batch {
  std::vector<aphgpu_ctx*> ctxs;
  int ndom = 0;
  int nlev_max = 0;
  int kz = 4;                     // planes per thread of the batched tiles
  cudaStream_t st = nullptr;      // stream of the first context
  aphgpu::BDom* d_doms = nullptr;
  int* d_count = nullptr;
  int* h_count = nullptr;         // pinned
  // tile tables: per level (smoothing, prolongation), per level for the
  // restriction (tiles of level l+1), and the finest level (PCG, outer)
  std::vector<aphgpu::BTile*> d_lev, d_res;
  std::vector<int> n_lev, n_res;
  aphgpu::BTile* d_fine = nullptr;
  int n_fine = 0;
  std::vector<void*> allocs;
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
  return APHGPU_ERR_CUDA;
}

#define B_CUDA(B, expr) APH_TRY(BCuda((B), (expr), #expr))
#define B_LAUNCHED(B)                                                   \
  do {                                                                  \
    ++(B)->launches;                                                    \
    const cudaError_t le_ = cudaGetLastError();                         \
    if (le_ != cudaSuccess) return BCuda((B), le_, "batched kernel launch"); \
  } while (0)

template <class T>
int BAlloc(aphgpu_batch* B, T** p, size_t count) {
  void* q = nullptr;
  if (cudaMalloc(&q, sizeof(T) * std::max<size_t>(count, 1)) != cudaSuccess) {
    cudaGetLastError();
    return BErr(B, APHGPU_ERR_NOMEM, "batch table allocation failed");
  }
  B->allocs.push_back(q);
  *p = (T*)q;
  return APHGPU_OK;
}

// tiles of dims d for domain `dom` appended to `out` (local indices follow)
void AddTiles(std::vector<BTile>& out, int dom, const Dims& d, int kz) {
  const int gx = (d.nx + kTileX - 1) / kTileX;
  const int gy = (d.ny + kTileY - 1) / kTileY;
  const int gz = (d.nz + kz - 1) / kz;
  const int count = gx * gy * gz;
  int local = 0;
  for (int bz = 0; bz < gz; ++bz)
    for (int by = 0; by < gy; ++by)
      for (int bx = 0; bx < gx; ++bx) out.push_back(BTile{dom, bx, by, bz, local++, count});
}

// Descriptors and tile tables from the contexts' current hierarchies.
int BuildTables(aphgpu_batch* B, const aphgpu_conf* conf) {
  std::vector<BDom> doms(B->ndom);
  B->nlev_max = 0;
  for (int q = 0; q < B->ndom; ++q) {
    aphgpu_ctx* c = B->ctxs[q];
    int rc = EnsureSolverVectors(c);
    if (rc == APHGPU_OK) rc = EnsureMixedHierarchy(c, conf);
    if (rc != APHGPU_OK) return BErr(B, rc, aphgpu_last_error(c));
    auto& lv = c->mg.l32;
    const int nl = (int)lv.size();
    if (nl > kMaxLev) return BErr(B, APHGPU_ERR_UNSUPPORTED, "too many multigrid levels");
    if (c->mg.cn32 != (int)lv.back().d.cells())
      return BErr(B, APHGPU_ERR_UNSUPPORTED, "coarsest level too large for the batch");
    BDom& D = doms[q];
    D.nlev = nl;
    for (int l = 0; l < nl; ++l) {
      BLevel& L = D.lv[l];
      L.A = Op<float>{lv[l].d, lv[l].w[0], lv[l].w[1], lv[l].w[2],
                      lv[l].has_diag ? lv[l].diag : nullptr};
      L.invdiag = lv[l].invdiag;
      L.x = l == 0 ? c->z32 : lv[l].x;
      L.b = l == 0 ? c->r32 : lv[l].b;
    }
    D.A64 = Op<double>{c->d, c->w[0], c->w[1], c->w[2], c->diag_explicit ? c->diag : nullptr};
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
    // the constant-mode projection holds only for the singular operator
    D.flags = c->diag_explicit ? (conf->inner_flags & ~1) : conf->inner_flags;
    D.cellvol = c->h * c->h * c->h;
    B->nlev_max = std::max(B->nlev_max, nl);
  }
  if (!B->d_doms) APH_TRY(BAlloc(B, &B->d_doms, B->ndom));
  B_CUDA(B, cudaMemcpy(B->d_doms, doms.data(), sizeof(BDom) * B->ndom, cudaMemcpyHostToDevice));
  // tables
  for (auto* p : B->d_lev) cudaFree(p);
  for (auto* p : B->d_res) cudaFree(p);
  if (B->d_fine) cudaFree(B->d_fine);
  B->d_lev.assign(B->nlev_max, nullptr);
  B->d_res.assign(B->nlev_max, nullptr);
  B->n_lev.assign(B->nlev_max, 0);
  B->n_res.assign(B->nlev_max, 0);
  auto upload = [&](const std::vector<BTile>& v, BTile** out) -> int {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(BTile) * std::max<size_t>(v.size(), 1)) != cudaSuccess) {
      cudaGetLastError();
      return BErr(B, APHGPU_ERR_NOMEM, "tile table allocation failed");
    }
    if (!v.empty() &&
        cudaMemcpy(q, v.data(), sizeof(BTile) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      return BErr(B, APHGPU_ERR_CUDA, "tile table upload failed");
    }
    *out = (BTile*)q;
    return APHGPU_OK;
  };
  for (int l = 0; l < B->nlev_max; ++l) {
    std::vector<BTile> lev, res;
    for (int q = 0; q < B->ndom; ++q) {
      if (l >= doms[q].nlev - 1) continue;  // coarsest or absent level
      AddTiles(lev, q, doms[q].lv[l].A.d, B->kz);
      AddTiles(res, q, doms[q].lv[l + 1].A.d, B->kz);
    }
    APH_TRY(upload(lev, &B->d_lev[l]));
    APH_TRY(upload(res, &B->d_res[l]));
    B->n_lev[l] = (int)lev.size();
    B->n_res[l] = (int)res.size();
  }
  std::vector<BTile> fine;
  for (int q = 0; q < B->ndom; ++q) AddTiles(fine, q, doms[q].lv[0].A.d, B->kz);
  for (auto& t : fine)
    if (t.count > B->ctxs[t.dom]->red.max_blocks)
      return BErr(B, APHGPU_ERR_UNSUPPORTED, "reduction buffer too small for the tiles");
  APH_TRY(upload(fine, &B->d_fine));
  B->n_fine = (int)fine.size();
  return APHGPU_OK;
}

int BVCycle(aphgpu_batch* B, int pre, int post) {
  const dim3 tb = TileBlock();
  cudaStream_t st = B->st;
  const int kz = B->kz;
  const int L = B->nlev_max;
  for (int l = 0; l < L - 1; ++l) {
    if (!B->n_lev[l]) continue;
    // pre == 0: both colours only take x = b / diag (zero initial guess)
    for (int sw = 0; sw < std::max(pre, 1); ++sw) {
      KBSmooth<<<B->n_lev[l], tb, 0, st>>>(B->d_doms, B->d_lev[l], l, kz, 0, sw == 0);
      B_LAUNCHED(B);
      KBSmooth<<<B->n_lev[l], tb, 0, st>>>(B->d_doms, B->d_lev[l], l, kz, 1, pre == 0);
      B_LAUNCHED(B);
    }
    KBRestrict<<<B->n_res[l], tb, 0, st>>>(B->d_doms, B->d_res[l], l, kz);
    B_LAUNCHED(B);
  }
  KBCoarsest<<<B->ndom, 256, 0, st>>>(B->d_doms);
  B_LAUNCHED(B);
  for (int l = L - 2; l >= 0; --l) {
    if (!B->n_lev[l]) continue;
    KBProlong<<<B->n_lev[l], tb, 0, st>>>(B->d_doms, B->d_lev[l], l, kz);
    B_LAUNCHED(B);
    for (int sw = 0; sw < post; ++sw) {
      KBSmooth<<<B->n_lev[l], tb, 0, st>>>(B->d_doms, B->d_lev[l], l, kz, 1, 0);
      B_LAUNCHED(B);
      KBSmooth<<<B->n_lev[l], tb, 0, st>>>(B->d_doms, B->d_lev[l], l, kz, 0, 0);
      B_LAUNCHED(B);
    }
  }
  return APHGPU_OK;
}

int BCount(aphgpu_batch* B, int which, int* active) {
  KBCountActive<<<1, 256, 0, B->st>>>(B->d_doms, B->ndom, which, B->d_count);
  B_LAUNCHED(B);
  B_CUDA(B, cudaMemcpyAsync(B->h_count, B->d_count, sizeof(int), cudaMemcpyDeviceToHost, B->st));
  B_CUDA(B, cudaStreamSynchronize(B->st));
  *active = *B->h_count;
  return APHGPU_OK;
}

inline uint64_t BMix(uint64_t h, uint64_t v) {
  return h ^ (v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2));
}

// One batch of `every` inner iterations for all domains (captured once).
int BInnerBody(aphgpu_batch* B, const aphgpu_conf* conf, int every) {
  const dim3 tb = TileBlock();
  for (int it = 0; it < every; ++it) {
    KBApply<<<B->n_fine, tb, 0, B->st>>>(B->d_doms, B->d_fine, B->kz);
    B_LAUNCHED(B);
    KBUpdate<<<B->n_fine, tb, 0, B->st>>>(B->d_doms, B->d_fine, B->kz);
    B_LAUNCHED(B);
    APH_TRY(BVCycle(B, conf->mg_pre, conf->mg_post));
    KBDotRZ<<<B->n_fine, tb, 0, B->st>>>(B->d_doms, B->d_fine, B->kz, 0);
    B_LAUNCHED(B);
    KBP<<<B->n_fine, tb, 0, B->st>>>(B->d_doms, B->d_fine, B->kz, 0);
    B_LAUNCHED(B);
  }
  return APHGPU_OK;
}

int BSolve(aphgpu_batch* B, const aphgpu_conf* conf, aphgpu_info* infos) {
  const dim3 tb = TileBlock();
  cudaStream_t st = B->st;
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
  // graph of one batch of inner iterations, keyed by the tables and settings
  uint64_t key = 1469598103934665603ull;
  key = BMix(key, (uint64_t)(uintptr_t)B->d_fine);
  for (auto* p : B->d_lev) key = BMix(key, (uint64_t)(uintptr_t)p);
  key = BMix(key, (uint64_t)(conf->mg_pre * 1000 + conf->mg_post));
  key = BMix(key, (uint64_t)B->kz);
  key = BMix(key, (uint64_t)B->n_fine);
  for (int n : B->n_lev) key = BMix(key, (uint64_t)n);
  for (int n : B->n_res) key = BMix(key, (uint64_t)n);
  if (!B->graph || B->graph_key != key) {
    if (B->graph) cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
    const int64_t l0 = B->launches;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    const int rc = ok ? BInnerBody(B, conf, every) : APHGPU_OK;
    ok = (cudaStreamEndCapture(st, &g) == cudaSuccess) && ok && rc == APHGPU_OK;
    B->launches = l0;
    if (ok && cudaGraphInstantiate(&B->graph, g, 0) == cudaSuccess) {
      size_t nn = 0;
      cudaGraphGetNodes(g, nullptr, &nn);
      B->graph_kernels = (int64_t)nn;
      B->graph_key = key;
    } else {
      B->graph = nullptr;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
  }
  B_CUDA(B, cudaEventRecord(B->ev0, st));
  KBResidual64<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz, 1);
  B_LAUNCHED(B);
  for (int outer = 0; outer <= conf->maxiter + 1; ++outer) {
    int active = 0;
    APH_TRY(BCount(B, 0, &active));
    if (!active) break;
    KBScaleZero<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz);
    B_LAUNCHED(B);
    KBInnerInit<<<(B->ndom + 127) / 128, 128, 0, st>>>(B->d_doms, B->ndom, conf->inner_rtol,
                                                       conf->inner_maxiter);
    B_LAUNCHED(B);
    APH_TRY(BVCycle(B, conf->mg_pre, conf->mg_post));
    KBDotRZ<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz, 1);
    B_LAUNCHED(B);
    KBP<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz, 1);
    B_LAUNCHED(B);
    for (int b = 0; b <= conf->inner_maxiter / every + 2; ++b) {
      if (B->graph) {
        B_CUDA(B, cudaGraphLaunch(B->graph, st));
        B->launches += B->graph_kernels;
      } else {
        APH_TRY(BInnerBody(B, conf, every));
      }
      APH_TRY(BCount(B, 1, &active));
      if (!active) break;
    }
    KBAddCorrection<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz);
    B_LAUNCHED(B);
    KBOuterAdvance<<<(B->ndom + 127) / 128, 128, 0, st>>>(B->d_doms, B->ndom);
    B_LAUNCHED(B);
    KBResidual64<<<B->n_fine, tb, 0, st>>>(B->d_doms, B->d_fine, B->kz, 0);
    B_LAUNCHED(B);
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
  if (cudaSetDevice(ctxs[0]->device) != cudaSuccess ||
      cudaEventCreate(&B->ev0) != cudaSuccess || cudaEventCreate(&B->ev1) != cudaSuccess ||
      cudaMalloc(&B->d_count, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&B->h_count, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    aphgpu_batch_destroy(B);
    return APHGPU_ERR_CUDA;
  }
  *out = B;
  return APHGPU_OK;
}

void aphgpu_batch_destroy(aphgpu_batch* B) {
  if (!B) return;
  if (B->st) cudaStreamSynchronize(B->st);
  if (B->graph) cudaGraphExecDestroy(B->graph);
  for (auto* p : B->d_lev) if (p) cudaFree(p);
  for (auto* p : B->d_res) if (p) cudaFree(p);
  if (B->d_fine) cudaFree(B->d_fine);
  for (void* p : B->allocs) cudaFree(p);
  if (B->d_count) cudaFree(B->d_count);
  if (B->h_count) cudaFreeHost(B->h_count);
  if (B->ev0) cudaEventDestroy(B->ev0);
  if (B->ev1) cudaEventDestroy(B->ev1);
  delete B;
}

const char* aphgpu_batch_last_error(const aphgpu_batch* B) {
  return B ? B->err.c_str() : "null batch";
}

int aphgpu_batch_solve(aphgpu_batch* B, const aphgpu_conf* conf, aphgpu_info* infos) {
  if (!B || !conf) return APHGPU_ERR_ARG;
  for (auto* c : B->ctxs)
    if (!c->has_system) return aphgpu::BErr(B, APHGPU_ERR_STATE, "a context has no system");
  if (cudaSetDevice(B->ctxs[0]->device) != cudaSuccess) return APHGPU_ERR_CUDA;
  return aphgpu::BSolve(B, conf, infos);
}

int aphgpu_batch_tune(aphgpu_batch* B, aphgpu_conf* conf, double* best_ms) {
  using namespace aphgpu;
  if (!B || !conf) return APHGPU_ERR_ARG;
  // candidates: planes per thread of the batched tiles, smoothing sweeps
  const int kzs[] = {2, 4, 8};
  const int sweeps[] = {1, 2, 3};
  double best = 1e300;
  int best_kz = B->kz, best_sw = conf->mg_pre;
  aphgpu_conf c = *conf;
  for (int kz : kzs) {
    for (int sw : sweeps) {
      B->kz = kz;
      c.mg_pre = c.mg_post = sw;
      const int rc = aphgpu_batch_solve(B, &c, nullptr);
      if (rc != APHGPU_OK) return rc;
      if (B->last_ms < best) {
        best = B->last_ms;
        best_kz = kz;
        best_sw = sw;
      }
    }
  }
  B->kz = best_kz;
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

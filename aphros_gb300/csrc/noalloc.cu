// aphgpu_cg_solve_noalloc: the plain FP64 CG solve without any device
// allocation, for callers that cannot call cudaMalloc.
//
// Who needs it: a solver plug-in loaded into a host application that owns
// the GPU's memory (it reserves the device memory up front for its own pool
// allocator, so a cudaMalloc from the plug-in fails or fragments that
// pool), and step loops with a fixed time budget, where cudaMalloc and
// cudaFree would synchronize the device and stall the loop for an unbounded
// time.  Such a caller owns its input and output arrays already; the
// solver's own work vectors live in a fixed device array in this file
// instead of on the heap.
//
// The call blocks: every few iterations it synchronizes the given stream
// and copies the solver's convergence flag to the host, and it returns once
// the solve has finished.
//
// Scratch: one file-scope __device__ array `g_noalloc_scratch` of
// kScratchDoubles doubles (about 1.6 MB).  Every GPU that loads the library
// holds it until the process exits.  It holds the residual r, the search
// direction p and A p (kMaxCells each), the per-CTA partial sums of the
// grid reductions and the solver scalars.
//
// All calls share this one array and it keeps the contents of the last
// call; the solve resets everything it reads before use.  Two calls whose
// work overlaps on the GPU (different streams or host threads at the same
// time) race on the array and give wrong results: serialize them.
//
// Set-up: the device address of the array is looked up once per device with
// cudaGetSymbolAddress, by the first call made while that device is
// current.  Make that first call before any stream capture starts.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"

namespace aphgpu {
namespace {

constexpr int64_t kMaxCells = 65536;   // largest grid: 2^16 cells
constexpr int kMaxCtas = 4096;         // largest tile grid of a reduction
constexpr int kScalarDoubles = 32;     // room for SolveScalars + ticket
constexpr int64_t kScratchDoubles =
    3 * kMaxCells + 2 * (int64_t)kMaxCtas + kScalarDoubles;

static_assert(sizeof(SolveScalars) + 8 <= kScalarDoubles * 8,
              "scalar area too small");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_base[kMaxDevices] = {};

struct Scratch {
  double* r;
  double* p;
  double* ap;
  RedBuf red;
  SolveScalars* s;
};

Scratch Carve(double* base) {
  Scratch sc;
  sc.r = base;
  sc.p = base + kMaxCells;
  sc.ap = base + 2 * kMaxCells;
  sc.red.part = base + 3 * kMaxCells;
  sc.red.max_blocks = kMaxCtas;
  double* tail = base + 3 * kMaxCells + 2 * (int64_t)kMaxCtas;
  sc.s = (SolveScalars*)tail;
  sc.red.ticket = (unsigned int*)(tail + (kScalarDoubles - 1));
  return sc;
}

// Expr access: e[0]*x[c] + sum_q e[1+q]*x[nb_q] (+ e[7]), q = xm,xp,ym,yp,zm,zp
__device__ __forceinline__ double ApplyExpr(const Dims& d, const double* e,
                                            const double* x, int i, int j, int k,
                                            int64_t c) {
  double u = x[c] * e[0];
  u += x[d.idx(wrapm(i - 1, d.nx), j, k)] * e[1];
  u += x[d.idx(wrapp(i + 1, d.nx), j, k)] * e[2];
  u += x[d.idx(i, wrapm(j - 1, d.ny), k)] * e[3];
  u += x[d.idx(i, wrapp(j + 1, d.ny), k)] * e[4];
  u += x[d.idx(i, j, wrapm(k - 1, d.nz))] * e[5];
  u += x[d.idx(i, j, wrapp(k + 1, d.nz))] * e[6];
  return u;
}

#define NA_LOOP_BEGIN(dims)                                      \
  const int i = blockIdx.x * kTileX + threadIdx.x;               \
  const int j = blockIdx.y * kTileY + threadIdx.y;               \
  const int kb = blockIdx.z * kTileZ;                            \
  const int ke = min(kb + kTileZ, (dims).nz);                    \
  const bool inxy = i < (dims).nx && j < (dims).ny;              \
  for (int k = kb; k < ke; ++k) {                                \
    if (!inxy) continue;                                         \
    const int64_t c = (dims).idx(i, j, k);
#define NA_LOOP_END }

// scalars and the reduction ticket start from zero on every call
__global__ void KNaSetup(SolveScalars* s, unsigned int* ticket, double tol,
                         double cellvol, int miniter, int maxiter, int maxnorm) {
  SolveScalars z{};
  z.tol = tol;
  z.cellvol = cellvol;
  z.res_scale = 1.0;
  z.miniter = miniter;
  z.maxiter = maxiter;
  z.maxnorm = maxnorm;
  *s = z;
  *ticket = 0;
}

// stage init of linear.ipp:42-61: r = -(A x0 + e7) (x0 = 0 when absent),
// p = r; x itself is set afterwards by KNaCopyGuess
__global__ void KNaInit(Dims d, const double* __restrict__ e8,
                        const double* x0, double* r, double* p) {
  NA_LOOP_BEGIN(d)
  const double* e = e8 + 8 * c;
  double u;
  if (x0) {
    u = x0[c] * e[0] + e[7];
    u += x0[d.idx(wrapm(i - 1, d.nx), j, k)] * e[1];
    u += x0[d.idx(wrapp(i + 1, d.nx), j, k)] * e[2];
    u += x0[d.idx(i, wrapm(j - 1, d.ny), k)] * e[3];
    u += x0[d.idx(i, wrapp(j + 1, d.ny), k)] * e[4];
    u += x0[d.idx(i, j, wrapm(k - 1, d.nz))] * e[5];
    u += x0[d.idx(i, j, wrapp(k + 1, d.nz))] * e[6];
  } else {
    u = 0. * e[0] + e[7];
  }
  r[c] = -u;
  p[c] = -u;
  NA_LOOP_END
}

// x = x0 (or 0), after KNaInit has read x0; x0 may alias x, the copy is
// then a no-op (each thread reads and writes only its own cell)
__global__ void KNaCopyGuess(int64_t n, const double* x0, double* x) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    x[c] = x0 ? x0[c] : 0.0;
}

// stage iter: ap = A p; r.r and p.ap
__global__ void KNaApply(Dims d, const double* __restrict__ e8,
                         const double* __restrict__ r,
                         const double* __restrict__ p, double* ap,
                         SolveScalars* s, RedBuf rb) {
  if (s->done) return;
  double v[2] = {0, 0};
  const int op[2] = {0, 0};
  NA_LOOP_BEGIN(d)
  const double y = ApplyExpr(d, e8 + 8 * c, p, i, j, k, c);
  ap[c] = y;
  v[0] += r[c] * r[c];
  v[1] += p[c] * y;
  NA_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr_prev = out[0];
      s->pap = out[1];
      s->alpha = out[0] / (out[1] + 1e-100);
    }
  }
}

// stage iter2 + check
__global__ void KNaUpdate(Dims d, double* x, double* r,
                          const double* __restrict__ p,
                          const double* __restrict__ ap, SolveScalars* s,
                          RedBuf rb) {
  if (s->done) return;
  const double alpha = s->alpha;
  double v[2] = {0, 0};
  const int op[2] = {0, 1};
  NA_LOOP_BEGIN(d)
  x[c] += alpha * p[c];
  const double rn = r[c] - alpha * ap[c];
  r[c] = rn;
  v[0] += rn * rn;
  v[1] = fmax(v[1], fabs(rn));
  NA_LOOP_END
  __shared__ double out[2];
  if (GridReduce<2>(v, op, rb, out)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      s->rr = out[0];
      s->maxr = out[1];
      s->beta = out[0] / (s->rr_prev + 1e-100);
      s->residual = s->maxnorm ? out[1] / s->cellvol : sqrt(out[0] / s->cellvol);
      s->iter += 1;
      if (s->iter >= s->miniter && (s->iter > s->maxiter || s->residual < s->tol)) {
        s->done = 1;
        s->converged = s->residual < s->tol;
      }
    }
  }
}

// stage iter3: p = r + beta p
__global__ void KNaP(Dims d, const double* __restrict__ r, double* p,
                     const SolveScalars* s) {
  if (s->done) return;
  const double beta = s->beta;
  NA_LOOP_BEGIN(d)
  p[c] = r[c] + beta * p[c];
  NA_LOOP_END
}

// Device address of the scratch array for the current device (looked up
// once per device).
int ScratchBase(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return APHGPU_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_base[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      cudaGetLastError();
      return APHGPU_ERR_CUDA;
    }
    g_base[dev] = (double*)ptr;
  }
  *out = g_base[dev];
  return APHGPU_OK;
}

}  // namespace
}  // namespace aphgpu

extern "C" int aphgpu_cg_solve_noalloc(int nx, int ny, int nz, double cellvol,
                                       const double* d_expr8, const double* d_x0,
                                       double* d_x, double tol, int miniter,
                                       int maxiter, int maxnorm, void* stream,
                                       aphgpu_info* info) {
  using namespace aphgpu;
  if (!d_expr8 || !d_x || !info || nx < 3 || ny < 3 || nz < 3 || !(cellvol > 0) ||
      maxiter < 0)
    return APHGPU_ERR_ARG;
  const Dims d{nx, ny, nz};
  const int64_t n = d.cells();
  if (n > kMaxCells || TileCount(d) > kMaxCtas) return APHGPU_ERR_ARG;
  double* base = nullptr;
  const int rc = ScratchBase(&base);
  if (rc != APHGPU_OK) return rc;
  const Scratch sc = Carve(base);
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 tg = TileGrid(d), tb = TileBlock();
  KNaSetup<<<1, 1, 0, st>>>(sc.s, sc.red.ticket, tol, cellvol, miniter, maxiter, maxnorm);
  KNaInit<<<tg, tb, 0, st>>>(d, d_expr8, d_x0, sc.r, sc.p);
  KNaCopyGuess<<<FlatBlocks(n), kFlatThreads, 0, st>>>(n, d_x0, d_x);
  if (cudaGetLastError() != cudaSuccess) return APHGPU_ERR_CUDA;
  SolveScalars hs{};
  int batch = 4;
  int64_t launched = 0;
  for (;;) {
    for (int it = 0; it < batch; ++it) {
      KNaApply<<<tg, tb, 0, st>>>(d, d_expr8, sc.r, sc.p, sc.ap, sc.s, sc.red);
      KNaUpdate<<<tg, tb, 0, st>>>(d, d_x, sc.r, sc.p, sc.ap, sc.s, sc.red);
      KNaP<<<tg, tb, 0, st>>>(d, sc.r, sc.p, sc.s);
    }
    if (cudaGetLastError() != cudaSuccess) return APHGPU_ERR_CUDA;
    // a plain copy into this stack variable: no pinned staging allocated
    if (cudaMemcpyAsync(&hs, sc.s, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      return APHGPU_ERR_CUDA;
    }
    launched += batch;
    if (hs.done || launched > (int64_t)maxiter + 2) break;
    batch = batch * 2 < 256 ? batch * 2 : 256;
  }
  info->residual = hs.residual;
  info->iter = hs.iter;
  info->inner_iter = 0;
  info->converged = hs.converged;
  return APHGPU_OK;
}

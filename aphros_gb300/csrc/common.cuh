// Internal definitions shared by the aphgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "aphgpu.h"

namespace aphgpu {

// ---------------------------------------------------------------------------
// Grid geometry
// ---------------------------------------------------------------------------

struct Dims {
  int nx, ny, nz;
  __host__ __device__ int64_t cells() const {
    return (int64_t)nx * ny * nz;
  }
  __host__ __device__ int64_t idx(int i, int j, int k) const {
    return (int64_t)i + (int64_t)nx * ((int64_t)j + (int64_t)ny * k);
  }
};

__device__ __forceinline__ int wrapm(int i, int n) {
  return i < 0 ? i + n : i;
}
__device__ __forceinline__ int wrapp(int i, int n) {
  return i >= n ? i - n : i;
}
__device__ __forceinline__ int wrapi(int i, int n) {
  return i < 0 ? i + n : (i >= n ? i - n : i);
}

// Stencil tiles: a CTA of kTileX*kTileY threads owns an x-y tile and
// marches over kTileZ planes in z.
constexpr int kTileX = 32;
constexpr int kTileY = 8;
constexpr int kTileZ = 8;

inline dim3 TileGrid(const Dims& d) {
  return dim3((d.nx + kTileX - 1) / kTileX, (d.ny + kTileY - 1) / kTileY,
              (d.nz + kTileZ - 1) / kTileZ);
}
inline dim3 TileBlock() {
  return dim3(kTileX, kTileY, 1);
}
inline int64_t TileCount(const Dims& d) {
  const dim3 g = TileGrid(d);
  return (int64_t)g.x * g.y * g.z;
}

// Flat kernels: fixed-size grid (a multiple of the SM count) with a
// grid-stride loop.
constexpr int kFlatThreads = 256;
int FlatBlocks(int64_t n);

// ---------------------------------------------------------------------------
// Deterministic grid-wide reductions.
//
// Each CTA reduces its values (warp shuffles, then shared memory), writes
// one partial per value, and the last CTA to arrive (atomic ticket) sums the
// partials in a fixed order.  The result does not depend on CTA scheduling,
// so repeated solves are bit-identical.
// ---------------------------------------------------------------------------

struct RedBuf {
  double* part;        // [kMaxRedVals][max_blocks]
  unsigned int* ticket;
  int max_blocks;
};
constexpr int kMaxRedVals = 4;
constexpr int kHistCap = 4096;

// op: 0 = sum, 1 = max
template <int NV>
__device__ __forceinline__ void WarpReduce(double (&v)[NV], const int (&op)[NV]) {
#pragma unroll
  for (int q = 0; q < NV; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_down_sync(0xffffffffu, v[q], o);
      v[q] = op[q] ? fmax(v[q], w) : v[q] + w;
    }
  }
}

// Returns true in all threads of the last CTA; `out[q]` then holds the
// result over the `nblocks` CTAs sharing `rb` (visible to that CTA after
// the call).  bid: index of this CTA among them.  nthreads: threads per
// CTA (multiple of 32, <= 1024).
template <int NV>
__device__ bool GroupReduce(double (&v)[NV], const int (&op)[NV], RedBuf rb,
                            double* out, int bid, int nblocks) {
  __shared__ double sm[32][NV];
  __shared__ bool last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  WarpReduce<NV>(v, op);
  const int lane = tid & 31, warp = tid >> 5;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) sm[warp][q] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = nthreads >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = lane < nw ? sm[lane][q] : (op[q] ? -1e308 : 0.0);
    WarpReduce<NV>(v, op);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NV; ++q) rb.part[q * rb.max_blocks + bid] = v[q];
      __threadfence();
      const unsigned t = atomicAdd(rb.ticket, 1u);
      last = (t == (unsigned)nblocks - 1);
    }
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // last CTA: ordered reduction of the partials
  double a[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) a[q] = op[q] ? -1e308 : 0.0;
  for (int b = tid; b < nblocks; b += nthreads) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const double w = ((volatile double*)rb.part)[q * rb.max_blocks + b];
      a[q] = op[q] ? fmax(a[q], w) : a[q] + w;
    }
  }
  WarpReduce<NV>(a, op);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) sm[warp][q] = a[q];
  }
  __syncthreads();
  if (tid == 0) {
    const int nw = nthreads >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double s = sm[0][q];
      for (int w = 1; w < nw; ++w) s = op[q] ? fmax(s, sm[w][q]) : s + sm[w][q];
      out[q] = s;
    }
    *rb.ticket = 0;
    __threadfence();
  }
  __syncthreads();
  return true;
}

// GroupReduce over the whole grid (CTA index linearised over a 3-D grid).
template <int NV>
__device__ __forceinline__ bool GridReduce(double (&v)[NV], const int (&op)[NV],
                                           RedBuf rb, double* out) {
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const int nblocks = gridDim.x * gridDim.y * gridDim.z;
  return GroupReduce<NV>(v, op, rb, out, bid, nblocks);
}

}  // namespace aphgpu

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------

namespace aphgpu {

// Scalars of an iterative solve, resident on the device so that the
// iteration loop never waits for the host.
struct SolveScalars {
  double rr;        // r.r after the last update
  double rr_prev;   // r.r before it
  double pap;       // p.Ap
  double rz;        // r.z (preconditioned)
  double rz_prev;
  double maxr;      // max |r|
  double alpha, beta;
  double residual;  // reported residual (norm of linear.ipp:102-114)
  double tol;
  double cellvol;
  double res_scale; // multiplies the residual (inner solves)
  double tmp[4];
  double apsum;     // sum of A p (constant-mode projection)
  double rzold;     // r_new . z_old (flexible beta)
  double* hist;     // residual after each iteration (may be NULL)
  int hist_cap;
  int iter;
  int miniter, maxiter, maxnorm;
  int done;
  int converged;
  int flags;        // bit 0 project constant mode, bit 1 flexible beta
  int pad;
};

template <class T>
struct Level {
  Dims d;
  T* w[3];       // coupling to the minus neighbour in x, y, z (e[1], e[3], e[5])
  T* invdiag;    // 1 / diagonal
  T* diag;       // diagonal array (may be unused, see has_diag)
  bool has_diag; // false: diagonal = -(sum of the six couplings)
  T* x;          // iterate / correction
  T* b;          // right-hand side
  T* r;          // residual scratch
  // FP16 copy of the couplings scaled by hscale (a power of two), used by
  // the smoother and the restriction of the finest FP32 level when set
  uint16_t* wh[3];
  float hscale;
  // x, b (and the inner PCG's vectors on the finest level) in the
  // colour-split order of split.cuh (the mixed solver's finest level)
  bool split;
};

struct Multigrid {
  int nlevels = 0;
  std::vector<Level<double>> l64;  // level 0 aliases the fine system
  std::vector<Level<float>> l32;
  bool built64 = false, built32 = false;
  int cmax64 = 0, cmax32 = 0;  // the coarse_max each hierarchy was built with
  // coarsest-level CG scratch (FP64)
  double* cr = nullptr;
  double* cp = nullptr;
  double* cap = nullptr;
  double* cx = nullptr;
  double* cb = nullptr;
  // dense inverse of the coarsest operator (A + 11^T mean(diag)/n),
  // FP64, one per hierarchy (n x n, n <= kDenseMax)
  double* cinv64 = nullptr;
  double* cinv32 = nullptr;
  int cn64 = 0, cn32 = 0;
  // the coarsest operator is singular (row sums zero: periodic
  // flux-difference systems): its dense inverse is that of A + c 11^T and
  // the coarsest solves remove the mean of the right-hand side
  int csing64 = 1, csing32 = 1;
  // one-CTA cycle of the smallest FP32 levels: device description of the
  // levels and the first level it covers (-1: not used)
  void* cdom = nullptr;
  int clc = -1;
  int csmem = 0;  // dynamic shared memory of that cycle (bytes)
  // FP32 low parts of the fine couplings (w - (double)l32[0].w), for the
  // mixed solver's double-float residual update; made at its first use
  // after each build of the FP32 hierarchy
  float* wlo[3] = {nullptr, nullptr, nullptr};
  bool wlo_ready = false;
};
constexpr int kDenseMax = 1024;

}  // namespace aphgpu

struct aphgpu_ctx {
  int device = 0;
  aphgpu::Dims d{0, 0, 0};
  int64_t N = 0;
  double h = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t bytes = 0;
  std::vector<void*> allocs;

  // fine FP64 system: e1,e3,e5 of each cell, explicit diagonal when the
  // system is not a pure flux-difference operator, b = -e7
  double* w[3] = {nullptr, nullptr, nullptr};
  double* diag = nullptr;      // NULL: diagonal = -(e1+...+e6) in order
  bool diag_explicit = false;
  // every row sum vanishes (periodic flux-difference system: the constant
  // null space); false with diagonal shifts (diffusion, given pressures)
  bool singular = true;
  // the stored system is the negation of the one set (negative definite
  // input): readbacks negate it again
  bool negated = false;
  bool diag_valid = false;  // `diag` holds the FP64 diagonal (explicit or computed)
  bool x_zero = false;      // x was zeroed for the solve being run
  double* invdiag = nullptr;   // 1/diagonal (multigrid smoother)
  double* b = nullptr;
  bool has_system = false;
  double* e8 = nullptr;        // staging of aphgpu_set_system_expr (8N)

  // projection: predicted fluxes with force (face blocks), resident force
  double* vstar = nullptr;     // 3N
  double* febp = nullptr;      // 3N
  bool has_proj = false;
  bool force_resident = false;
  bool proj_force = false;     // the last assembly included a face force
  double proj_rho[2] = {1, 1}; // rho1, rho2 of the last assembly
  double* alpha_proj = nullptr;  // volume fraction of the last assembly

  // solver vectors
  double* x = nullptr;
  double* r = nullptr;
  double* p = nullptr;
  double* ap = nullptr;
  double* z = nullptr;
  float* r32 = nullptr;
  float* x32 = nullptr;        // inner correction
  float* p32 = nullptr;
  float* ap32 = nullptr;
  float* z32 = nullptr;
  float* zold32 = nullptr;     // previous preconditioned residual (flexible CG)
  aphgpu::SolveScalars* scal = nullptr;   // outer
  aphgpu::SolveScalars* scal2 = nullptr;  // inner
  aphgpu::SolveScalars* hscal = nullptr;  // pinned host copy
  double* hist = nullptr;      // device residual history, 2 x kHistCap
  std::vector<double> hist_outer, hist_inner;
  aphgpu::RedBuf red{nullptr, nullptr, 0};
  unsigned int* flags = nullptr;  // 5 counters: validation kernels, FP16 range
  aphgpu::Multigrid mg;

  // VOF state
  double* u = nullptr;
  double* u_alt = nullptr;     // N, written by each directional update, then
                               // exchanged with u
  bool vof_list_valid = false; // the scratch list holds the interfacial
                               // cells of u
  double* kpart = nullptr;     // curvature of each particle string
  int64_t kpart_cap = 0;
  double* ppoly = nullptr;     // PLIC polygon of each listed cell (particle strings)
  int* ppk = nullptr;          // its vertex count
  int64_t ppoly_cap = 0;
  int* ppos = nullptr;         // list position of each listed cell (N entries)
  // the wavefront sweep: progress counters (one per tile) and, after them,
  // the flag of a wait that gave up; set when a solve launched it
  int* wave_buf = nullptr;
  bool wave_used = false;
  double* u0 = nullptr;
  double* nrm = nullptr;       // 3N AoS
  double* pa = nullptr;        // plane constant
  double* ffvu = nullptr;      // N, fluid flux of one direction
  double* vflux_res = nullptr; // 3N resident corrected fluxes
  bool has_vflux_res = false;
  double* kappa = nullptr;
  double* hgt = nullptr;       // 3N AoS
  // given-pressure cells of the last aphgpu_apply_cell_cond: values, then
  // cell indices (int64), room for cc_cap cells
  double* cc_buf = nullptr;
  int64_t cc_cap = 0;
  // projection fluid step (fluid.cu): time layer (velocity, fluxes),
  // iteration layer, work arrays, cell viscosity, pressures
  struct {
    double* vel = nullptr;    // 3N, blocks per component
    double* vi = nullptr;     // 3N
    double* flux = nullptr;   // 3N face blocks
    double* ffv = nullptr;    // 3N
    double* ffu = nullptr;    // 3N
    double* acc = nullptr;    // 3N AoS
    double* guess = nullptr;  // 3N
    double* mu = nullptr;
    double* p = nullptr;
    double* ppred = nullptr;
    double* e8 = nullptr;     // 8N diffusion system
    double rho1 = 1, rho2 = 1;
    int steps = 0;
    int unconverged = 0;
    bool follow_vof = false;  // density from the resident volume fraction
    bool ready = false;
  } fluid;
  double* vof_src = nullptr;   // N, volume source of the VOF step
  bool has_vof_src = false;
  double clipth = 1e-10;
  int vof_count = 0;
  int fcuu_sel = 0;         // which of the two fcuu slots of the VOF scratch is current
  bool fcuu_ready = false;  // the current slot holds fcuu of u (left by the last step)
  double vof_dt = 0;  // time step of the last VOF step (kernel timing)
  bool vof_ready = false;

  // device scratch of the field dumps (dump.cu)
  void* dump_scratch = nullptr;
  // connected-component colours of the volume fraction (label.cu; -1 none)
  double* cl = nullptr;
  struct {
    int* par = nullptr;     // union-find parent, then root (gas cells only)
    int* gas = nullptr;     // the gas cells (u > 0.5), listed
    int* slot = nullptr;    // component slot of each root
    int* croot = nullptr;   // root of each slot
    unsigned long long* first = nullptr;  // first halo-order position per slot
    double* stable = nullptr;  // previous colour at that position
    double* color = nullptr;   // new colour per slot
    double* pre = nullptr;     // colours before the propagation pass
    int* ctl = nullptr;        // component count, error flag, gas and candidate counts
    unsigned char* flag = nullptr;  // the propagation's candidate cells (1 byte each)
  } lab;
  // host staging (pinned)
  void* pinned = nullptr;
  size_t pinned_bytes = 0;

  // CUDA graphs of PCG iteration batches (one per solver role), keyed by
  // the pointers and settings they were captured with
  struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    uint64_t key = 0;
    int64_t kernels = 0;
  } graphs[4];
  int64_t mg_epoch = 0;        // bumped whenever a hierarchy is (re)allocated
  bool use_graphs = true;
  // fused out-of-place red-black sweeps on the FP32 levels: 0 off (two
  // in-place half sweeps, default), 1 the pipelined kernel (asynchronous
  // copies into shared memory) on levels of at least kPipeMinCells cells, 2 the
  // pipelined kernel on every level it supports, 3 the synchronous fused
  // kernel on every level it supports
  int fused_mode = 0;
  int wave_planes = 0;  // planes per step of the wavefront sweep (0: sized to L2)
  int use_split = 2;  // colour-split finest level (mixed solver): 0 off, 1 on, 2 from 2^22 cells
  int use_df = 2;  // double-float outer residual update: 0 off, 1 on, 2 from 2^22 cells
  bool use_half = false;   // FP16 couplings for the finest-level smoother
  int mg_gamma = 0;        // cycles of each level below the finest (1 V, 2 W, 0 auto)
  int64_t mg_wmin = 4096; // W-cycles: levels of at most so many cells visit their child once
  int mg_series_pct = 60;  // weight (%) of the series couplings in the coarse operators
  int mg_growth = 0;       // sweeps below the finest level (1 same, 2 linear, 3 doubling, 0 auto)
  bool use_cta_coarse = true;  // smallest FP32 levels cycled by one CTA

  // timing
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t ev_slot[2] = {nullptr, nullptr};
  cudaEvent_t marks[8] = {nullptr, nullptr, nullptr, nullptr,
                          nullptr, nullptr, nullptr, nullptr};
  double last_ms = 0;
  int64_t last_launches = 0;
  int64_t launches = 0;
};

namespace aphgpu {

int SetError(aphgpu_ctx* ctx, int code, const char* fmt, ...);
int CheckCuda(aphgpu_ctx* ctx, cudaError_t e, const char* what);
// Device memory of the contexts comes from one stream-ordered pool per
// device that keeps freed memory for reuse: destroying a context (an
// eviction of the serving loop) does not synchronize the device, and the
// next context reuses the memory without asking the driver.
int DeviceAlloc(aphgpu_ctx* ctx, void** p, size_t bytes);
void DeviceFree(aphgpu_ctx* ctx, void* p);
// Pinned host buffers, recycled across contexts.
void* PinnedTake(size_t bytes, size_t* got);
void PinnedGive(void* p, size_t bytes);

template <class T>
int Alloc(aphgpu_ctx* ctx, T** p, int64_t count) {
  void* q = nullptr;
  const size_t bytes = sizeof(T) * (size_t)(count > 0 ? count : 1);
  const int rc = DeviceAlloc(ctx, &q, bytes);
  if (rc != APHGPU_OK) return rc;
  ctx->allocs.push_back(q);
  ctx->bytes += (int64_t)bytes;
  *p = (T*)q;
  return APHGPU_OK;
}
// Pinned host staging buffer of at least `bytes`.
int Staging(aphgpu_ctx* ctx, size_t bytes, void** out);

#define APH_TRY(expr)          \
  do {                         \
    const int rc_ = (expr);    \
    if (rc_ != APHGPU_OK) return rc_; \
  } while (0)
#define APH_CUDA(ctx, expr) APH_TRY(::aphgpu::CheckCuda((ctx), (expr), #expr))
#define APH_LAUNCHED(ctx)                                                \
  do {                                                                   \
    ++(ctx)->launches;                                                   \
    const cudaError_t le_ = cudaGetLastError();                          \
    if (le_ != cudaSuccess) return ::aphgpu::CheckCuda((ctx), le_, "kernel launch"); \
  } while (0)

// poisson.cu
int EnsureSolverVectors(aphgpu_ctx* ctx);
int SolveCG(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info);
int SolveMGPCG(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info);
int SolveMixed(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info);
int SolveMGPCG32(aphgpu_ctx* ctx, const aphgpu_conf* conf, aphgpu_info* info);
int EnsureMixedVectors(aphgpu_ctx* ctx);
int EnsureMixedHierarchy(aphgpu_ctx* ctx, const aphgpu_conf* conf);
// One-CTA cycle of the smallest FP32 levels of a single-domain hierarchy
// (batch.cu): set up after the hierarchy is built; launched from the cycle
// with the pre / post sweeps of every level (kMgMaxLevels entries).
constexpr int kMgMaxLevels = 12;
int CoarseOneSetup(aphgpu_ctx* ctx);
int CoarseOneLaunch(aphgpu_ctx* ctx, const int* pre, const int* post, int gamma, bool first,
                    const SolveScalars* s);
int SetSystemExprDevice(aphgpu_ctx* ctx, const double* d_expr8);
int ApplyCellCondDevice(aphgpu_ctx* ctx, int64_t count, const int64_t* d_cells,
                        const double* d_values);
int AssembleProjectionDevice(aphgpu_ctx* ctx, const double* d_alpha,
                             double rho1, double rho2, const double* d_vflux,
                             const double* d_febp, double dt, int remove_mean);
int ResidualNorms(aphgpu_ctx* ctx, double* rnorm, double* bnorm);
int SystemToExprDevice(aphgpu_ctx* ctx, double* d_e8);
int FluxCorrect(aphgpu_ctx* ctx, double* d_out);
int Acceleration(aphgpu_ctx* ctx, double* d_acc, const double* d_alpha,
                 double rho1, double rho2);
// fluid.cu
int FluidInitDevice(aphgpu_ctx* ctx, double rho1, double rho2, double mu1, double mu2);
int FluidStepDevice(aphgpu_ctx* ctx, double dt, const aphgpu_conf* conf, aphgpu_info* info,
                    double* d_res);
int BcgFacesDevice(aphgpu_ctx* ctx, const double* u, const double* vflux, const double* src,
                   double dt, double* out);
// vof.cu
int VofReconstruct(aphgpu_ctx* ctx);
int ColorInit(aphgpu_ctx* ctx);
int Recolor(aphgpu_ctx* ctx);
int VofStepDevice(aphgpu_ctx* ctx, const double* d_vflux, double dt);
int CurvatureDevice(aphgpu_ctx* ctx);
// the interface list (cells with 0 < u < 1) of the current u, rebuilt if
// the last VOF call did not leave it: device pointers to the cell indices
// and their count
int InterfaceListDevice(aphgpu_ctx* ctx, const int** list, const int** count);
int KFillNanDevice(aphgpu_ctx* ctx, double* v, int64_t n);
// partstr.cu
int CurvatureParticlesDevice(aphgpu_ctx* ctx, const aphgpu_part_conf& conf, bool hybrid);
int SurfaceTensionDevice(aphgpu_ctx* ctx, double sigma, double* d_febp);
int TimeVofKernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms, double* bytes,
                  const double* d_vflux, double dt);
int TimeSolverKernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms, double* bytes);
// the error flag of the wavefront sweeps launched since the last check
int CheckWave(aphgpu_ctx* ctx);
// the wavefront sweep's bounded wait on a counter nothing sets
int WaveWaitCheck(aphgpu_ctx* ctx);

}  // namespace aphgpu

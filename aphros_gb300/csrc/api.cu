// C ABI of libaphgpu (include/aphgpu.h): context management, host<->device
// staging through pinned buffers, and dispatch to the solver and VOF code.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>

#include "common.cuh"

using aphgpu::Alloc;

namespace aphgpu {

int SetError(aphgpu_ctx* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) ctx->err = buf;
  return code;
}

int CheckCuda(aphgpu_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return APHGPU_OK;
  cudaGetLastError();
  return SetError(ctx, e == cudaErrorMemoryAllocation ? APHGPU_ERR_NOMEM : APHGPU_ERR_CUDA,
                  "%s: %s", what, cudaGetErrorString(e));
}

namespace {

std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
bool g_pool_failed[64] = {};

// the device's pool, created on first use; nullptr if pools are unsupported
cudaMemPool_t DevicePool(int device) {
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  if (g_pools[device] || g_pool_failed[device]) return g_pools[device];
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    cudaGetLastError();
    g_pool_failed[device] = true;
    return nullptr;
  }
  uint64_t keep = UINT64_MAX;  // freed memory stays in the pool
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  g_pools[device] = pool;
  return pool;
}

// pinned host buffers returned by destroyed contexts, at most kPinnedKeep
// bytes in all
constexpr size_t kPinnedKeep = size_t(8) << 30;
std::mutex g_pin_mu;
std::vector<std::pair<void*, size_t>> g_pinned;
size_t g_pinned_bytes = 0;

}  // namespace

int DeviceAlloc(aphgpu_ctx* ctx, void** p, size_t bytes) {
  cudaMemPool_t pool = DevicePool(ctx->device);
  cudaError_t e = pool ? cudaMallocFromPoolAsync(p, bytes, pool, ctx->stream)
                       : cudaMalloc(p, bytes);
  if (e != cudaSuccess && pool) {
    // memory kept by the pool but free: release it and try once more
    cudaGetLastError();
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(p, bytes, pool, ctx->stream);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SetError(ctx, APHGPU_ERR_NOMEM, "device allocation of %zu bytes failed: %s", bytes,
                    cudaGetErrorString(e));
  }
  return APHGPU_OK;
}

void DeviceFree(aphgpu_ctx* ctx, void* p) {
  if (!p) return;
  if (DevicePool(ctx->device))
    cudaFreeAsync(p, ctx->stream);
  else
    cudaFree(p);
}

void* PinnedTake(size_t bytes, size_t* got) {
  {
    std::lock_guard<std::mutex> lock(g_pin_mu);
    // the smallest kept buffer that is large enough (and not much larger)
    size_t best = g_pinned.size();
    for (size_t i = 0; i < g_pinned.size(); ++i) {
      const size_t sz = g_pinned[i].second;
      if (sz >= bytes && sz <= 4 * bytes + 4096 &&
          (best == g_pinned.size() || sz < g_pinned[best].second))
        best = i;
    }
    if (best < g_pinned.size()) {
      void* p = g_pinned[best].first;
      *got = g_pinned[best].second;
      g_pinned_bytes -= *got;
      g_pinned.erase(g_pinned.begin() + best);
      return p;
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  *got = bytes;
  return p;
}

void PinnedGive(void* p, size_t bytes) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lock(g_pin_mu);
    if (g_pinned_bytes + bytes <= kPinnedKeep) {
      g_pinned.emplace_back(p, bytes);
      g_pinned_bytes += bytes;
      return;
    }
  }
  cudaFreeHost(p);
}

int Staging(aphgpu_ctx* ctx, size_t bytes, void** out) {
  if (ctx->pinned_bytes < bytes) {
    PinnedGive(ctx->pinned, ctx->pinned_bytes);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
    size_t got = 0;
    void* p = PinnedTake(bytes, &got);
    if (!p) return SetError(ctx, APHGPU_ERR_NOMEM, "pinned host allocation of %zu bytes", bytes);
    ctx->pinned = p;
    ctx->pinned_bytes = got;
  }
  *out = ctx->pinned;
  return APHGPU_OK;
}

}  // namespace aphgpu

namespace {

using namespace aphgpu;

// Host -> device copy that accepts pageable caller memory: chunks go
// through two pinned staging slots, each reused only after its previous copy
// completed.  Returns after the data is on the device.
int H2D(aphgpu_ctx* ctx, double* dst, const void* src, size_t bytes) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, src) == cudaSuccess &&
      (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice ||
       at.type == cudaMemoryTypeManaged)) {
    APH_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
    APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return APHGPU_OK;
  }
  cudaGetLastError();
  const size_t chunk = std::min<size_t>(64ull << 20, bytes);
  void* stage = nullptr;
  APH_TRY(Staging(ctx, 2 * chunk, &stage));
  cudaEvent_t ev[2] = {ctx->ev_slot[0], ctx->ev_slot[1]};
  bool used[2] = {false, false};
  size_t off = 0;
  int slot = 0;
  while (off < bytes) {
    const size_t n = std::min(chunk, bytes - off);
    if (used[slot]) APH_CUDA(ctx, cudaEventSynchronize(ev[slot]));
    char* s = (char*)stage + slot * chunk;
    std::memcpy(s, (const char*)src + off, n);
    APH_CUDA(ctx, cudaMemcpyAsync((char*)dst + off, s, n, cudaMemcpyHostToDevice, ctx->stream));
    APH_CUDA(ctx, cudaEventRecord(ev[slot], ctx->stream));
    used[slot] = true;
    off += n;
    slot ^= 1;
  }
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return APHGPU_OK;
}

int D2H(aphgpu_ctx* ctx, void* dst, const void* src, size_t bytes) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, dst) == cudaSuccess &&
      (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice ||
       at.type == cudaMemoryTypeManaged)) {
    APH_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream));
    APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return APHGPU_OK;
  }
  cudaGetLastError();
  const size_t chunk = 64ull << 20;
  void* stage = nullptr;
  APH_TRY(Staging(ctx, std::min(bytes, chunk), &stage));
  const size_t cap = std::min(chunk, ctx->pinned_bytes);
  size_t off = 0;
  while (off < bytes) {
    const size_t n = std::min(cap, bytes - off);
    APH_CUDA(ctx, cudaMemcpyAsync(stage, (const char*)src + off, n, cudaMemcpyDeviceToHost, ctx->stream));
    APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy((char*)dst + off, stage, n);
    off += n;
  }
  return APHGPU_OK;
}

bool Valid(aphgpu_ctx* ctx) { return ctx != nullptr && ctx->stream != nullptr; }

int SetDevice(aphgpu_ctx* ctx) {
  APH_CUDA(ctx, cudaSetDevice(ctx->device));
  return APHGPU_OK;
}

struct Timer {
  aphgpu_ctx* ctx;
  int64_t l0;
  explicit Timer(aphgpu_ctx* c) : ctx(c), l0(c->launches) {
    cudaEventRecord(ctx->ev0, ctx->stream);
  }
  void Stop() {
    cudaEventRecord(ctx->ev1, ctx->stream);
    cudaEventSynchronize(ctx->ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->last_ms = ms;
    ctx->last_launches = ctx->launches - l0;
  }
};

int EnsureVof(aphgpu_ctx* ctx) {
  if (ctx->u) return APHGPU_OK;
  const int64_t N = ctx->N;
  // the interface-cell lists of the advection hold 32-bit cell indices
  if (N >= INT32_MAX)
    return SetError(ctx, APHGPU_ERR_UNSUPPORTED, "VOF needs fewer than 2^31 cells");
  APH_TRY(Alloc(ctx, &ctx->u, N));
  APH_TRY(Alloc(ctx, &ctx->u_alt, N));
  APH_TRY(Alloc(ctx, &ctx->u0, N + 8));  // the VOF scratch (two fcuu slots, the list)
  APH_TRY(Alloc(ctx, &ctx->nrm, 3 * N));
  APH_TRY(Alloc(ctx, &ctx->pa, N));
  APH_TRY(Alloc(ctx, &ctx->ffvu, N));
  APH_TRY(Alloc(ctx, &ctx->kappa, N));
  APH_TRY(Alloc(ctx, &ctx->hgt, 3 * N));
  // all-ones bytes are NaN: curvature and heights read before any
  // aphgpu_curvature call are NaN, as the reference initialises them
  APH_CUDA(ctx, cudaMemsetAsync(ctx->kappa, 0xff, sizeof(double) * N, ctx->stream));
  APH_CUDA(ctx, cudaMemsetAsync(ctx->hgt, 0xff, sizeof(double) * 3 * N, ctx->stream));
  return APHGPU_OK;
}

// scratch device array of 3N doubles used to stage face inputs
int FaceScratch(aphgpu_ctx* ctx, double** out) {
  if (!ctx->vflux_res) APH_TRY(Alloc(ctx, &ctx->vflux_res, 3 * ctx->N));
  *out = ctx->vflux_res;
  return APHGPU_OK;
}

}  // namespace

extern "C" {

void aphgpu_conf_default(aphgpu_conf* c) {
  if (!c) return;
  c->solver = APHGPU_SOLVER_MGPCG;
  c->tol = 0;
  c->miniter = 1;
  c->maxiter = 1000;
  c->maxnorm = 0;
  c->mg_pre = 2;
  c->mg_post = 2;
  c->mg_coarse_max = 64;
  c->inner_rtol = 3e-4;
  c->inner_maxiter = 200;
  c->inner_flags = 3;
  c->rtol = 0;
}

int aphgpu_create(aphgpu_ctx** out, int nx, int ny, int nz, double h, int device) {
  if (!out) return APHGPU_ERR_ARG;
  *out = nullptr;
  if (nx < 3 || ny < 3 || nz < 3 || !(h > 0)) return APHGPU_ERR_ARG;
  aphgpu_ctx* ctx = new (std::nothrow) aphgpu_ctx();
  if (!ctx) return APHGPU_ERR_NOMEM;
  ctx->device = device;
  ctx->d = Dims{nx, ny, nz};
  ctx->N = (int64_t)nx * ny * nz;
  ctx->h = h;
  int rc = APHGPU_OK;
  auto fail = [&](int code) {
    aphgpu_destroy(ctx);
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return APHGPU_ERR_CUDA;
  }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return APHGPU_ERR_CUDA;
  }
  cudaEventCreate(&ctx->ev0);
  cudaEventCreate(&ctx->ev1);
  cudaEventCreateWithFlags(&ctx->ev_slot[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&ctx->ev_slot[1], cudaEventDisableTiming);
  const int64_t N = ctx->N;
  for (int q = 0; q < 3; ++q)
    if ((rc = Alloc(ctx, &ctx->w[q], N))) return fail(rc);
  if ((rc = Alloc(ctx, &ctx->b, N))) return fail(rc);
  if ((rc = Alloc(ctx, &ctx->x, N))) return fail(rc);
  if ((rc = Alloc(ctx, &ctx->scal, 1))) return fail(rc);
  if ((rc = Alloc(ctx, &ctx->scal2, 1))) return fail(rc);
  if ((rc = Alloc(ctx, &ctx->flags, 5))) return fail(rc);
  if (cudaMemsetAsync(ctx->flags, 0, 5 * sizeof(unsigned int), ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(APHGPU_ERR_CUDA);
  }
  if ((rc = Alloc(ctx, &ctx->hist, 2 * (int64_t)kHistCap))) return fail(rc);
  ctx->red.max_blocks = (int)std::max<int64_t>(TileCount(ctx->d), 4096);
  if ((rc = Alloc(ctx, &ctx->red.part, (int64_t)kMaxRedVals * ctx->red.max_blocks)))
    return fail(rc);
  if ((rc = Alloc(ctx, &ctx->red.ticket, 1))) return fail(rc);
  {
    size_t got = 0;
    ctx->hscal = (SolveScalars*)PinnedTake(sizeof(SolveScalars), &got);
    if (!ctx->hscal) return fail(APHGPU_ERR_NOMEM);
  }
  cudaMemsetAsync(ctx->red.ticket, 0, sizeof(unsigned), ctx->stream);
  cudaMemsetAsync(ctx->x, 0, sizeof(double) * N, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(APHGPU_ERR_CUDA);
  }
  *out = ctx;
  return APHGPU_OK;
}

void aphgpu_destroy(aphgpu_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& g : ctx->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  for (void* p : ctx->allocs) DeviceFree(ctx, p);
  ctx->allocs.clear();
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  // pinned buffers are kept for the next contexts
  PinnedGive(ctx->hscal, sizeof(SolveScalars));
  PinnedGive(ctx->pinned, ctx->pinned_bytes);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (int q = 0; q < 8; ++q)
    if (ctx->marks[q]) cudaEventDestroy(ctx->marks[q]);
  for (int q = 0; q < 2; ++q)
    if (ctx->ev_slot[q]) cudaEventDestroy(ctx->ev_slot[q]);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* aphgpu_last_error(const aphgpu_ctx* ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

int64_t aphgpu_device_bytes(const aphgpu_ctx* ctx) {
  return ctx ? ctx->bytes : 0;
}

int aphgpu_sync(aphgpu_ctx* ctx) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return APHGPU_OK;
}

int aphgpu_set_system_expr(aphgpu_ctx* ctx, const double* expr8) {
  if (!Valid(ctx) || !expr8) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  // the AoS expressions are staged in a device buffer kept for later calls
  // (8 doubles per cell; the drop-in is called once per solve)
  if (!ctx->e8) APH_TRY(Alloc(ctx, &ctx->e8, 8 * ctx->N));
  APH_TRY(H2D(ctx, ctx->e8, expr8, sizeof(double) * 8 * ctx->N));
  return SetSystemExprDevice(ctx, ctx->e8);
}

int aphgpu_apply_cell_cond(aphgpu_ctx* ctx, int64_t count, const int64_t* cells,
                           const double* values) {
  if (!Valid(ctx) || count < 0 || (count > 0 && (!cells || !values))) return APHGPU_ERR_ARG;
  if (!ctx->has_system) return SetError(ctx, APHGPU_ERR_STATE, "no system set");
  std::vector<int64_t> sorted(cells, cells + count);
  std::sort(sorted.begin(), sorted.end());
  for (int64_t t = 0; t < count; ++t) {
    if (sorted[t] < 0 || sorted[t] >= ctx->N)
      return SetError(ctx, APHGPU_ERR_ARG, "cell %lld outside the domain",
                      (long long)sorted[t]);
    if (t > 0 && sorted[t] == sorted[t - 1])
      return SetError(ctx, APHGPU_ERR_ARG, "cell %lld given twice", (long long)sorted[t]);
  }
  APH_TRY(SetDevice(ctx));
  if (count > ctx->cc_cap) {
    if (ctx->cc_buf) {
      for (size_t i = 0; i < ctx->allocs.size(); ++i) {
        if (ctx->allocs[i] == ctx->cc_buf) {
          APH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
          DeviceFree(ctx, ctx->cc_buf);
          ctx->allocs.erase(ctx->allocs.begin() + i);
          ctx->bytes -= (int64_t)sizeof(double) * 2 * ctx->cc_cap;
          break;
        }
      }
      ctx->cc_buf = nullptr;
      ctx->cc_cap = 0;
    }
    APH_TRY(Alloc(ctx, &ctx->cc_buf, 2 * count));
    ctx->cc_cap = count;
  }
  if (count > 0) {
    APH_TRY(H2D(ctx, ctx->cc_buf, values, sizeof(double) * count));
    APH_TRY(H2D(ctx, ctx->cc_buf + ctx->cc_cap, cells, sizeof(int64_t) * count));
  }
  return ApplyCellCondDevice(ctx, count, (const int64_t*)(ctx->cc_buf + ctx->cc_cap),
                             ctx->cc_buf);
}

int aphgpu_get_system_expr(aphgpu_ctx* ctx, double* expr8) {
  if (!Valid(ctx) || !expr8) return APHGPU_ERR_ARG;
  if (!ctx->has_system) return SetError(ctx, APHGPU_ERR_STATE, "no system set");
  APH_TRY(SetDevice(ctx));
  double* d_e8 = nullptr;
  APH_TRY(Alloc(ctx, &d_e8, 8 * ctx->N));
  int rc = SystemToExprDevice(ctx, d_e8);
  if (rc == APHGPU_OK) rc = D2H(ctx, expr8, d_e8, sizeof(double) * 8 * ctx->N);
  cudaStreamSynchronize(ctx->stream);
  for (size_t i = 0; i < ctx->allocs.size(); ++i) {
    if (ctx->allocs[i] == d_e8) {
      DeviceFree(ctx, d_e8);
      ctx->allocs.erase(ctx->allocs.begin() + i);
      ctx->bytes -= (int64_t)sizeof(double) * 8 * ctx->N;
      break;
    }
  }
  return rc;
}

int aphgpu_assemble_projection(aphgpu_ctx* ctx, const double* alpha, double rho1,
                               double rho2, const double* vflux, const double* febp,
                               double dt, int remove_mean) {
  if (!Valid(ctx) || !vflux) return APHGPU_ERR_ARG;
  if (!alpha && !ctx->vof_ready)
    return SetError(ctx, APHGPU_ERR_STATE, "alpha is NULL and no resident volume fraction");
  APH_TRY(SetDevice(ctx));
  APH_TRY(EnsureSolverVectors(ctx));
  APH_TRY(EnsureVof(ctx));
  const int64_t N = ctx->N;
  // alpha staged in its own array (kept for aphgpu_acceleration), fluxes in
  // the face scratch, force in the resident force array
  if (!ctx->alpha_proj) APH_TRY(Alloc(ctx, &ctx->alpha_proj, N));
  double* d_alpha = ctx->alpha_proj;
  double* d_vf = nullptr;
  APH_TRY(FaceScratch(ctx, &d_vf));
  if (alpha) {
    APH_TRY(H2D(ctx, d_alpha, alpha, sizeof(double) * N));
  } else {
    APH_CUDA(ctx, cudaMemcpyAsync(d_alpha, ctx->u, sizeof(double) * N,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  }
  APH_TRY(H2D(ctx, d_vf, vflux, sizeof(double) * 3 * N));
  const double* d_febp = nullptr;
  if (febp) {
    if (!ctx->febp) APH_TRY(Alloc(ctx, &ctx->febp, 3 * N));
    APH_TRY(H2D(ctx, ctx->febp, febp, sizeof(double) * 3 * N));
    d_febp = ctx->febp;
  } else if (ctx->force_resident && ctx->febp) {
    d_febp = ctx->febp;
  }
  Timer t(ctx);
  APH_TRY(AssembleProjectionDevice(ctx, d_alpha, rho1, rho2, d_vf, d_febp, dt, remove_mean));
  t.Stop();
  ctx->has_vflux_res = false;
  ctx->proj_rho[0] = rho1;
  ctx->proj_rho[1] = rho2;
  ctx->proj_force = d_febp != nullptr;
  return APHGPU_OK;
}

int aphgpu_solve_resident(aphgpu_ctx* ctx, const aphgpu_conf* conf, int zero_guess,
                          aphgpu_info* info) {
  if (!Valid(ctx) || !conf || !info) return APHGPU_ERR_ARG;
  if (!ctx->has_system) return SetError(ctx, APHGPU_ERR_STATE, "no system set");
  APH_TRY(SetDevice(ctx));
  APH_TRY(EnsureSolverVectors(ctx));
  if (zero_guess) APH_CUDA(ctx, cudaMemsetAsync(ctx->x, 0, sizeof(double) * ctx->N, ctx->stream));
  aphgpu_conf cf = *conf;
  if (conf->rtol > 0) {
    double rn = 0, bn = 0;
    APH_TRY(ResidualNorms(ctx, &rn, &bn));
    const double t = conf->rtol * bn / std::sqrt(ctx->h * ctx->h * ctx->h);
    cf.tol = std::max(cf.tol, t);
  }
  conf = &cf;
  Timer t(ctx);
  int rc;
  ctx->x_zero = zero_guess != 0;
  switch (conf->solver) {
    case APHGPU_SOLVER_CG: rc = SolveCG(ctx, conf, info); break;
    case APHGPU_SOLVER_MGPCG: rc = SolveMGPCG(ctx, conf, info); break;
    case APHGPU_SOLVER_MIXED: rc = SolveMixed(ctx, conf, info); break;
    case APHGPU_SOLVER_MGPCG32: rc = SolveMGPCG32(ctx, conf, info); break;
    default: ctx->x_zero = false; return SetError(ctx, APHGPU_ERR_ARG, "unknown solver %d", conf->solver);
  }
  ctx->x_zero = false;
  t.Stop();
  if (rc == APHGPU_OK) rc = CheckWave(ctx);
  return rc;
}

int aphgpu_solve(aphgpu_ctx* ctx, const aphgpu_conf* conf, const double* x0, double* x,
                 aphgpu_info* info) {
  if (!Valid(ctx) || !conf || !info) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  if (x0) APH_TRY(H2D(ctx, ctx->x, x0, sizeof(double) * ctx->N));
  APH_TRY(aphgpu_solve_resident(ctx, conf, x0 ? 0 : 1, info));
  if (x) APH_TRY(D2H(ctx, x, ctx->x, sizeof(double) * ctx->N));
  return APHGPU_OK;
}

int aphgpu_residual_history(aphgpu_ctx* ctx, int which, double* out, int cap,
                            int* count) {
  if (!Valid(ctx) || (which != 0 && which != 1) || cap < 0) return APHGPU_ERR_ARG;
  const std::vector<double>& h = which == 0 ? ctx->hist_outer : ctx->hist_inner;
  if (count) *count = (int)h.size();
  if (out) {
    for (int i = 0; i < cap && i < (int)h.size(); ++i) out[i] = h[i];
  }
  return APHGPU_OK;
}

int aphgpu_set_solution(aphgpu_ctx* ctx, const double* x) {
  if (!Valid(ctx) || !x) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  return H2D(ctx, ctx->x, x, sizeof(double) * ctx->N);
}

int aphgpu_get_solution(aphgpu_ctx* ctx, double* x) {
  if (!Valid(ctx) || !x) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  return D2H(ctx, x, ctx->x, sizeof(double) * ctx->N);
}

int aphgpu_residual_norms(aphgpu_ctx* ctx, double* rnorm, double* bnorm) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->has_system) return SetError(ctx, APHGPU_ERR_STATE, "no system set");
  APH_TRY(SetDevice(ctx));
  return ResidualNorms(ctx, rnorm, bnorm);
}

int aphgpu_flux_correct(aphgpu_ctx* ctx, double* vflux_out) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->has_proj) return SetError(ctx, APHGPU_ERR_STATE, "no projection system assembled");
  APH_TRY(SetDevice(ctx));
  double* d_out = nullptr;
  APH_TRY(FaceScratch(ctx, &d_out));
  APH_TRY(FluxCorrect(ctx, d_out));
  ctx->has_vflux_res = true;
  if (vflux_out) APH_TRY(D2H(ctx, vflux_out, d_out, sizeof(double) * 3 * ctx->N));
  return APHGPU_OK;
}

int aphgpu_acceleration(aphgpu_ctx* ctx, double* acc) {
  if (!Valid(ctx) || !acc) return APHGPU_ERR_ARG;
  if (!ctx->has_proj) return SetError(ctx, APHGPU_ERR_STATE, "no projection system assembled");
  APH_TRY(SetDevice(ctx));
  double* d_acc = nullptr;
  APH_TRY(Alloc(ctx, &d_acc, 3 * ctx->N));
  int rc = Acceleration(ctx, d_acc, ctx->alpha_proj, ctx->proj_rho[0], ctx->proj_rho[1]);
  if (rc == APHGPU_OK) rc = D2H(ctx, acc, d_acc, sizeof(double) * 3 * ctx->N);
  cudaStreamSynchronize(ctx->stream);
  for (size_t i = 0; i < ctx->allocs.size(); ++i) {
    if (ctx->allocs[i] == d_acc) {
      DeviceFree(ctx, d_acc);
      ctx->allocs.erase(ctx->allocs.begin() + i);
      ctx->bytes -= (int64_t)sizeof(double) * 3 * ctx->N;
      break;
    }
  }
  return rc;
}

int aphgpu_vof_init(aphgpu_ctx* ctx, const double* alpha, double clipth) {
  if (!Valid(ctx) || !alpha) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  APH_TRY(EnsureVof(ctx));
  APH_TRY(H2D(ctx, ctx->u, alpha, sizeof(double) * ctx->N));
  ctx->clipth = clipth;
  ctx->vof_count = 0;
  Timer t(ctx);
  APH_TRY(VofReconstruct(ctx));
  APH_TRY(ColorInit(ctx));
  t.Stop();
  ctx->vof_ready = true;
  return APHGPU_OK;
}

int aphgpu_vof_recolor(aphgpu_ctx* ctx) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  Timer t(ctx);
  APH_TRY(Recolor(ctx));
  t.Stop();
  return APHGPU_OK;
}

int aphgpu_vof_colors(aphgpu_ctx* ctx, double* cl) {
  if (!Valid(ctx) || !cl) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  return D2H(ctx, cl, ctx->cl, sizeof(double) * ctx->N);
}

int aphgpu_vof_step(aphgpu_ctx* ctx, const double* vflux, double dt) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  double* d_vf = nullptr;
  APH_TRY(FaceScratch(ctx, &d_vf));
  if (vflux) {
    APH_TRY(H2D(ctx, d_vf, vflux, sizeof(double) * 3 * ctx->N));
    ctx->has_vflux_res = false;
  } else if (!ctx->has_vflux_res) {
    return SetError(ctx, APHGPU_ERR_STATE, "no resident corrected fluxes");
  }
  Timer t(ctx);
  APH_TRY(VofStepDevice(ctx, d_vf, dt));
  t.Stop();
  return APHGPU_OK;
}

int aphgpu_fluid_init(aphgpu_ctx* ctx, const double* alpha, double rho1, double rho2,
                      double mu1, double mu2, const double* vel) {
  if (!Valid(ctx) || !vel) return APHGPU_ERR_ARG;
  if (!alpha && !ctx->vof_ready)
    return SetError(ctx, APHGPU_ERR_STATE, "alpha is NULL and no resident volume fraction");
  APH_TRY(SetDevice(ctx));
  APH_TRY(EnsureSolverVectors(ctx));
  APH_TRY(EnsureVof(ctx));
  const int64_t N = ctx->N;
  auto& F = ctx->fluid;
  if (!F.vel) {
    for (double** p : {&F.vel, &F.vi, &F.flux, &F.ffv, &F.ffu, &F.acc, &F.guess})
      APH_TRY(Alloc(ctx, p, 3 * N));
    for (double** p : {&F.mu, &F.p, &F.ppred}) APH_TRY(Alloc(ctx, p, N));
    APH_TRY(Alloc(ctx, &F.e8, 8 * N));
  }
  if (!ctx->alpha_proj) APH_TRY(Alloc(ctx, &ctx->alpha_proj, N));
  if (alpha) {
    APH_TRY(H2D(ctx, ctx->alpha_proj, alpha, sizeof(double) * N));
  } else {
    APH_CUDA(ctx, cudaMemcpyAsync(ctx->alpha_proj, ctx->u, sizeof(double) * N,
                                  cudaMemcpyDeviceToDevice, ctx->stream));
  }
  F.follow_vof = alpha == nullptr;
  APH_TRY(H2D(ctx, F.vel, vel, sizeof(double) * 3 * N));
  APH_TRY(FluidInitDevice(ctx, rho1, rho2, mu1, mu2));
  ctx->proj_rho[0] = rho1;
  ctx->proj_rho[1] = rho2;
  F.ready = true;
  return aphgpu_sync(ctx);
}

int aphgpu_fluid_step(aphgpu_ctx* ctx, double dt, const aphgpu_conf* conf, aphgpu_info* info) {
  if (!Valid(ctx) || !conf || !info || !(dt > 0)) return APHGPU_ERR_ARG;
  if (!ctx->fluid.ready) return SetError(ctx, APHGPU_ERR_STATE, "fluid not initialised");
  if (ctx->fluid.follow_vof && !ctx->vof_ready)
    return SetError(ctx, APHGPU_ERR_STATE, "no resident volume fraction");
  APH_TRY(SetDevice(ctx));
  double* d_res = nullptr;
  APH_TRY(FaceScratch(ctx, &d_res));
  Timer t(ctx);
  const int rc = FluidStepDevice(ctx, dt, conf, info, d_res);
  t.Stop();
  return rc;
}

int aphgpu_fluid_get(aphgpu_ctx* ctx, double* vel, double* p, double* flux) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->fluid.ready) return SetError(ctx, APHGPU_ERR_STATE, "fluid not initialised");
  APH_TRY(SetDevice(ctx));
  const int64_t N = ctx->N;
  if (vel) APH_TRY(D2H(ctx, vel, ctx->fluid.vel, sizeof(double) * 3 * N));
  if (p) APH_TRY(D2H(ctx, p, ctx->fluid.p, sizeof(double) * N));
  if (flux) APH_TRY(D2H(ctx, flux, ctx->fluid.flux, sizeof(double) * 3 * N));
  return APHGPU_OK;
}

int aphgpu_bcg_faces(aphgpu_ctx* ctx, const double* u, const double* vflux, const double* src,
                     double dt, double* out) {
  if (!Valid(ctx) || !u || !vflux || !src || !out) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  const int64_t N = ctx->N;
  // inputs and output staged in one temporary block of 8N doubles
  double* d = nullptr;
  APH_TRY(Alloc(ctx, &d, 8 * N));
  int rc = H2D(ctx, d, u, sizeof(double) * N);
  if (rc == APHGPU_OK) rc = H2D(ctx, d + N, vflux, sizeof(double) * 3 * N);
  if (rc == APHGPU_OK) rc = H2D(ctx, d + 4 * N, src, sizeof(double) * N);
  if (rc == APHGPU_OK) rc = BcgFacesDevice(ctx, d, d + N, d + 4 * N, dt, d + 5 * N);
  if (rc == APHGPU_OK) rc = D2H(ctx, out, d + 5 * N, sizeof(double) * 3 * N);
  cudaStreamSynchronize(ctx->stream);
  for (size_t i = 0; i < ctx->allocs.size(); ++i) {
    if (ctx->allocs[i] == d) {
      DeviceFree(ctx, d);
      ctx->allocs.erase(ctx->allocs.begin() + i);
      ctx->bytes -= (int64_t)sizeof(double) * 8 * N;
      break;
    }
  }
  return rc;
}

int aphgpu_vof_set_source(aphgpu_ctx* ctx, const double* src) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  if (!src) {
    ctx->has_vof_src = false;
    return APHGPU_OK;
  }
  if (!ctx->vof_src) APH_TRY(Alloc(ctx, &ctx->vof_src, ctx->N));
  APH_TRY(H2D(ctx, ctx->vof_src, src, sizeof(double) * ctx->N));
  ctx->has_vof_src = true;
  return APHGPU_OK;
}

int aphgpu_vof_get(aphgpu_ctx* ctx, double* alpha, double* normals, double* plane,
                   uint8_t* mask) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  const int64_t N = ctx->N;
  std::vector<double> ua;
  double* u = alpha;
  if (!u && (normals || plane || mask)) {
    ua.resize(N);
    u = ua.data();
  }
  if (u) APH_TRY(D2H(ctx, u, ctx->u, sizeof(double) * N));
  if (normals) APH_TRY(D2H(ctx, normals, ctx->nrm, sizeof(double) * 3 * N));
  if (plane) APH_TRY(D2H(ctx, plane, ctx->pa, sizeof(double) * N));
  // values of non-interfacial cells are never computed on the device: the
  // reference stores NaN there (vof.ipp:70-81, normal.ipp:359)
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int64_t c = 0; c < N && u; ++c) {
    const bool m = u[c] > 0 && u[c] < 1;
    if (mask) mask[c] = m ? 1 : 0;
    if (!m) {
      if (normals) normals[3 * c] = normals[3 * c + 1] = normals[3 * c + 2] = nan;
      if (plane) plane[c] = nan;
    }
  }
  return APHGPU_OK;
}

int aphgpu_curvature(aphgpu_ctx* ctx, double* kappa, double* heights) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  Timer t(ctx);
  APH_TRY(CurvatureDevice(ctx));
  t.Stop();
  const int64_t N = ctx->N;
  if (kappa) APH_TRY(D2H(ctx, kappa, ctx->kappa, sizeof(double) * N));
  if (heights) {
    APH_TRY(D2H(ctx, heights, ctx->hgt, sizeof(double) * 3 * N));
    std::vector<double> u(N);
    APH_TRY(D2H(ctx, u.data(), ctx->u, sizeof(double) * N));
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int64_t c = 0; c < N; ++c)
      if (!(u[c] > 0 && u[c] < 1)) heights[3 * c] = heights[3 * c + 1] = heights[3 * c + 2] = nan;
  }
  return APHGPU_OK;
}

void aphgpu_part_conf_default(aphgpu_part_conf* conf) {
  if (!conf) return;
  conf->np = 7;
  conf->ns = 3;
  conf->leq = 4;
  conf->relax = 0.5;
  conf->tol = 1e-5;
  conf->itermax = 20;
  conf->segcirc = 0;
  conf->dn = 0;
}

int aphgpu_curvature_estimator(aphgpu_ctx* ctx, int estimator, const aphgpu_part_conf* conf,
                               double* kappa) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  if (estimator < APHGPU_CURV_HEIGHTS || estimator > APHGPU_CURV_HYBRID)
    return SetError(ctx, APHGPU_ERR_ARG, "unknown curvature estimator %d", estimator);
  APH_TRY(SetDevice(ctx));
  aphgpu_part_conf pc;
  aphgpu_part_conf_default(&pc);
  if (conf) pc = *conf;
  Timer t(ctx);
  if (estimator == APHGPU_CURV_HEIGHTS) {
    APH_TRY(CurvatureDevice(ctx));
  } else {
    APH_TRY(CurvatureParticlesDevice(ctx, pc, estimator == APHGPU_CURV_HYBRID));
  }
  t.Stop();
  if (kappa) APH_TRY(D2H(ctx, kappa, ctx->kappa, sizeof(double) * ctx->N));
  return APHGPU_OK;
}

int aphgpu_surface_tension(aphgpu_ctx* ctx, double sigma, double* febp) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
  APH_TRY(SetDevice(ctx));
  if (!ctx->febp) APH_TRY(Alloc(ctx, &ctx->febp, 3 * ctx->N));
  APH_TRY(SurfaceTensionDevice(ctx, sigma, ctx->febp));
  if (febp) APH_TRY(D2H(ctx, febp, ctx->febp, sizeof(double) * 3 * ctx->N));
  return APHGPU_OK;
}

int aphgpu_set_force_resident(aphgpu_ctx* ctx, int on) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  ctx->force_resident = on != 0;
  return APHGPU_OK;
}

int aphgpu_set_option(aphgpu_ctx* ctx, int option, int value) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  switch (option) {
    case APHGPU_OPT_GRAPHS: ctx->use_graphs = value != 0; return APHGPU_OK;
    case APHGPU_OPT_FUSED_SWEEPS:
      if (value < 0 || value > 6) return SetError(ctx, APHGPU_ERR_ARG, "fused sweeps %d", value);
      if (value != ctx->fused_mode) ctx->mg.built32 = false;  // scratch of the levels
      ctx->fused_mode = value;
      return APHGPU_OK;
    case APHGPU_OPT_CYCLE:
      if (value < 0 || value > 2) return SetError(ctx, APHGPU_ERR_ARG, "cycle must be 0, 1 or 2");
      ctx->mg_gamma = value;
      return APHGPU_OK;
    case APHGPU_OPT_CTA_COARSE: ctx->use_cta_coarse = value != 0; return APHGPU_OK;
    case APHGPU_OPT_COLOR_SPLIT:
      if (value < 0 || value > 2) return SetError(ctx, APHGPU_ERR_ARG, "colour split must be 0..2");
      ctx->use_split = value;
      return APHGPU_OK;
    case APHGPU_OPT_W_MIN_CELLS:
      if (value < 0) return SetError(ctx, APHGPU_ERR_ARG, "W-cycle floor must be >= 0");
      ctx->mg_wmin = value;
      return APHGPU_OK;
    case APHGPU_OPT_DF_RESIDUAL:
      if (value < 0 || value > 2) return SetError(ctx, APHGPU_ERR_ARG, "df residual must be 0..2");
      ctx->use_df = value;
      return APHGPU_OK;
    case APHGPU_OPT_WAVE_PLANES:
      if (value < 0 || value > 4096)
        return SetError(ctx, APHGPU_ERR_ARG, "wave planes must be 0..4096");
      ctx->wave_planes = value;
      return APHGPU_OK;
    case APHGPU_OPT_SWEEP_GROWTH:
      if (value < 0 || value > 3) return SetError(ctx, APHGPU_ERR_ARG, "sweep growth must be 0..3");
      ctx->mg_growth = value;
      return APHGPU_OK;
    case APHGPU_OPT_COARSE_SERIES:
      if (value < 0 || value > 100)
        return SetError(ctx, APHGPU_ERR_ARG, "coarse series weight must be 0..100");
      if (value != ctx->mg_series_pct) {
        ctx->mg_series_pct = value;
        ctx->mg.built64 = ctx->mg.built32 = false;  // rebuilt at the next solve
      }
      return APHGPU_OK;
    case APHGPU_OPT_HALF_COUPLINGS:
      ctx->use_half = value != 0;
      ctx->mg.built32 = false;  // rebuilt with or without them at the next solve
      return APHGPU_OK;
    default: return SetError(ctx, APHGPU_ERR_ARG, "unknown option %d", option);
  }
}

int aphgpu_mark(aphgpu_ctx* ctx, int slot) {
  if (!Valid(ctx) || slot < 0 || slot >= 8) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  if (!ctx->marks[slot]) APH_CUDA(ctx, cudaEventCreate(&ctx->marks[slot]));
  APH_CUDA(ctx, cudaEventRecord(ctx->marks[slot], ctx->stream));
  return APHGPU_OK;
}

int aphgpu_elapsed(aphgpu_ctx* ctx, int s0, int s1, double* ms) {
  if (!Valid(ctx) || !ms || s0 < 0 || s0 >= 8 || s1 < 0 || s1 >= 8) return APHGPU_ERR_ARG;
  if (!ctx->marks[s0] || !ctx->marks[s1]) return SetError(ctx, APHGPU_ERR_STATE, "slot not recorded");
  APH_CUDA(ctx, cudaEventSynchronize(ctx->marks[s1]));
  float t = 0;
  APH_CUDA(ctx, cudaEventElapsedTime(&t, ctx->marks[s0], ctx->marks[s1]));
  *ms = t;
  return APHGPU_OK;
}

int aphgpu_time_kernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms, double* bytes) {
  if (!Valid(ctx) || !ms || !bytes || reps < 1) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  if (kernel >= APHGPU_K_VOF_FLUX && kernel <= APHGPU_K_CURVATURE) {
    if (!ctx->vof_ready) return SetError(ctx, APHGPU_ERR_STATE, "vof not initialised");
    double* d_vf = nullptr;
    APH_TRY(FaceScratch(ctx, &d_vf));
    return TimeVofKernel(ctx, kernel, reps, ms, bytes, d_vf, ctx->vof_dt);
  }
  return TimeSolverKernel(ctx, kernel, reps, ms, bytes);
}

int aphgpu_wave_wait_check(aphgpu_ctx* ctx) {
  if (!Valid(ctx)) return APHGPU_ERR_ARG;
  APH_TRY(SetDevice(ctx));
  return WaveWaitCheck(ctx);
}

int aphgpu_last_timing(const aphgpu_ctx* ctx, double* ms, int64_t* launches) {
  if (!ctx) return APHGPU_ERR_ARG;
  if (ms) *ms = ctx->last_ms;
  if (launches) *launches = ctx->last_launches;
  return APHGPU_OK;
}

}  // extern "C"

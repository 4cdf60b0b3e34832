// Serving loop: time-step requests for many resident simulations, run with
// continuous batching on one GPU.
//
// Each simulation owns a context (aphgpu_ctx, its own CUDA stream) holding
// its volume fraction, pressure and surface-tension force between steps.  A
// request is one full step:
//   projection (assembly from the resident volume fraction, the request's
//   predicted fluxes and the resident surface-tension force; solve warm-
//   started from the resident pressure; corrected fluxes) ->
//   PLIC advection with the corrected fluxes -> height curvature ->
//   surface-tension force for the next step.
// `slots` worker threads take requests as they arrive; requests of
// different simulations run concurrently on their own streams, so their
// kernels overlap on the device, and a new request is started as soon as a
// slot and the memory for its simulation are free.  Steps of one
// simulation run in submission order.
//
// Admission: the device bytes of resident simulations stay within the
// budget.  To admit a simulation the server evicts the least recently used
// idle simulations: their state (volume fraction, pressure, force) is copied
// to host memory and their context destroyed; on re-admission it is restored
// and the interface reconstructed from the same volume fraction, so a step
// after a restore is identical to a step without one.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

// device bytes per cell of a resident simulation (FP64 system, solver and
// VOF state, FP32 hierarchy), used before its first step measures it
constexpr double kBytesPerCellEstimate = 448.0;

struct Sim {
  int id = 0;
  int n[3] = {0, 0, 0};
  double h = 0;
  double rho1 = 1, rho2 = 1, sigma = 0;
  aphgpu_ctx* ctx = nullptr;  // NULL when not resident
  bool busy = false;
  bool has_force = false;
  bool has_pressure = false;
  int64_t bytes = 0;          // device bytes while resident (estimate first)
  int64_t last_use = 0;
  int steps = 0;
  // host copies while evicted
  std::vector<double> alpha, pressure;
  int evictions = 0;
};

struct Request {
  int64_t ticket;
  int sim;
  double dt;
  std::vector<double> vflux;
  Clock::time_point submitted;
};

}  // namespace

struct aphgpu_server {
  int device = 0;
  int64_t budget = 0;
  int slots = 1;
  aphgpu_conf conf{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::map<int, std::unique_ptr<Sim>> sims;
  std::map<int64_t, aphgpu_step_result> done;
  int64_t next_ticket = 1;
  int next_sim = 0;
  int64_t resident_bytes = 0;
  int64_t use_clock = 0;
  int64_t completed = 0, evictions = 0, admissions = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::string err;
};

namespace {

int64_t Cells(const Sim& s) { return (int64_t)s.n[0] * s.n[1] * s.n[2]; }

// Copies a simulation's state to the host and destroys its context.  Runs
// without the lock on a victim that SelectVictims reserved (busy, bytes
// already taken off the resident total); counters are updated by the caller.
int Evict(Sim& s) {
  const int64_t N = Cells(s);
  s.alpha.resize(N);
  int rc = aphgpu_vof_get(s.ctx, s.alpha.data(), nullptr, nullptr, nullptr);
  if (rc == APHGPU_OK && s.has_pressure) {
    s.pressure.resize(N);
    rc = aphgpu_get_solution(s.ctx, s.pressure.data());
  }
  // the surface-tension force is not copied: it is a function of the
  // volume fraction and is recomputed on re-admission
  if (rc != APHGPU_OK) return rc;
  // the sweep order of the next step follows the steps the context took
  s.steps = s.ctx->vof_count;
  aphgpu_destroy(s.ctx);
  s.ctx = nullptr;
  return APHGPU_OK;
}

// Creates the context of a simulation and restores its state.
int Admit(aphgpu_server* S, Sim& s) {
  int rc = aphgpu_create(&s.ctx, s.n[0], s.n[1], s.n[2], s.h, S->device);
  if (rc != APHGPU_OK) return rc;
  rc = aphgpu_vof_init(s.ctx, s.alpha.data(), 1e-10);
  // the split order of the sweeps follows the number of steps taken
  if (rc == APHGPU_OK) s.ctx->vof_count = s.steps;
  if (rc == APHGPU_OK && s.has_force) {
    // restore the resident force by recomputing it: curvature and force are
    // functions of the restored volume fraction and interface
    rc = aphgpu_curvature(s.ctx, nullptr, nullptr);
    if (rc == APHGPU_OK) rc = aphgpu_surface_tension(s.ctx, s.sigma, nullptr);
  }
  if (rc == APHGPU_OK && s.has_pressure) {
    // the pressure is the warm start of the next solve
    rc = aphgpu_set_solution(s.ctx, s.pressure.data());
  }
  if (rc != APHGPU_OK) {
    aphgpu_destroy(s.ctx);
    s.ctx = nullptr;
    return rc;
  }
  s.alpha.clear();
  s.alpha.shrink_to_fit();
  s.pressure.clear();
  s.pressure.shrink_to_fit();
  S->admissions += 1;
  return APHGPU_OK;
}

// Completes the oldest queued request of simulation `sim` with error `rc`.
// Called with the lock held.
void FailOldest(aphgpu_server* S, int sim, int rc, const char* why) {
  S->err = why;
  for (auto q = S->queue.begin(); q != S->queue.end(); ++q) {
    if (q->sim != sim) continue;
    aphgpu_step_result res{};
    res.ticket = q->ticket;
    res.sim = sim;
    res.status = rc;
    S->done[q->ticket] = res;
    S->queue.erase(q);
    S->cv_done.notify_all();
    return;
  }
}

// Picks idle resident simulations, least recently used first, whose
// eviction makes room for `need` bytes, reserves them (busy) and takes their
// bytes off the resident total.  Called with the lock held; the evictions
// themselves run without it (EvictReserved).  Returns false, reserving
// nothing, if not enough idle simulations exist now.
bool SelectVictims(aphgpu_server* S, int64_t need, int except, std::vector<Sim*>* out) {
  out->clear();
  int64_t freed = 0;
  while (S->resident_bytes - freed + need > S->budget) {
    Sim* victim = nullptr;
    for (auto& kv : S->sims) {
      Sim& s = *kv.second;
      if (s.id == except || !s.ctx || s.busy) continue;
      if (std::find(out->begin(), out->end(), &s) != out->end()) continue;
      if (!victim || s.last_use < victim->last_use) victim = &s;
    }
    if (!victim) {
      out->clear();
      return false;
    }
    out->push_back(victim);
    freed += victim->bytes;
  }
  for (Sim* v : *out) {
    v->busy = true;
    S->resident_bytes -= v->bytes;
  }
  return true;
}

// Evicts the reserved victims; called without the lock, which it takes to
// release them.  A victim whose copy failed stays resident.  Returns false
// if any eviction failed.
bool EvictReserved(aphgpu_server* S, const std::vector<Sim*>& victims,
                   std::unique_lock<std::mutex>& lock) {
  std::vector<int> rcs;
  for (Sim* v : victims) rcs.push_back(Evict(*v));
  lock.lock();
  bool ok = true;
  for (size_t i = 0; i < victims.size(); ++i) {
    Sim* v = victims[i];
    v->busy = false;
    if (rcs[i] == APHGPU_OK) {
      v->evictions += 1;
      S->evictions += 1;
    } else {
      S->resident_bytes += v->bytes;
      ok = false;
    }
  }
  return ok;
}

// One step of a simulation (see the file comment).  Runs without the lock.
int RunStep(aphgpu_server* S, Sim& s, const Request& r, aphgpu_step_result* out) {
  aphgpu_ctx* ctx = s.ctx;
  int rc = aphgpu_set_force_resident(ctx, s.has_force ? 1 : 0);
  if (rc) return rc;
  rc = aphgpu_assemble_projection(ctx, nullptr, s.rho1, s.rho2, r.vflux.data(), nullptr,
                                  r.dt, 1);
  if (rc) return rc;
  aphgpu_info info{};
  rc = aphgpu_solve_resident(ctx, &S->conf, s.has_pressure ? 0 : 1, &info);
  if (rc) return rc;
  double ms_solve = 0;
  aphgpu_last_timing(ctx, &ms_solve, nullptr);
  rc = aphgpu_flux_correct(ctx, nullptr);
  if (rc) return rc;
  rc = aphgpu_vof_step(ctx, nullptr, r.dt);
  if (rc) return rc;
  double ms_vof = 0;
  aphgpu_last_timing(ctx, &ms_vof, nullptr);
  rc = aphgpu_curvature(ctx, nullptr, nullptr);
  if (rc) return rc;
  double ms_curv = 0;
  aphgpu_last_timing(ctx, &ms_curv, nullptr);
  rc = aphgpu_surface_tension(ctx, s.sigma, nullptr);
  if (rc) return rc;
  s.has_force = true;
  s.has_pressure = true;
  out->iters = info.iter;
  out->inner_iters = info.inner_iter;
  out->residual = info.residual;
  out->converged = info.converged;
  out->device_ms = ms_solve + ms_vof + ms_curv;
  return APHGPU_OK;
}

void Worker(aphgpu_server* S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lock(S->mu);
  for (;;) {
    // first queued request whose simulation is idle and is (or can be made)
    // resident; requests of one simulation keep their order because the
    // first one found for an idle simulation is its oldest
    auto it = S->queue.end();
    bool rescan = false;
    std::vector<int> seen;
    for (auto q = S->queue.begin(); q != S->queue.end(); ++q) {
      Sim& s = *S->sims[q->sim];
      if (std::find(seen.begin(), seen.end(), q->sim) != seen.end()) continue;
      seen.push_back(q->sim);
      if (s.busy) continue;
      if (!s.ctx) {
        const int64_t need = s.bytes;
        if (need > S->budget) {
          // its measured footprint outgrew the budget: it can never be
          // re-admitted, so its oldest request fails instead of waiting
          FailOldest(S, s.id, APHGPU_ERR_NOMEM, "simulation larger than the budget");
          rescan = true;
          break;
        }
        std::vector<Sim*> victims;
        if (!SelectVictims(S, need, s.id, &victims)) continue;
        s.busy = true;  // reserve while evicting and admitting without the lock
        S->resident_bytes += need;
        lock.unlock();
        if (!victims.empty()) {
          // EvictReserved returns with the lock held
          if (!EvictReserved(S, victims, lock)) {
            // a copy failed and its victim stayed resident: release the
            // reservation and fail the request that needed the room
            s.busy = false;
            S->resident_bytes -= need;
            FailOldest(S, s.id, APHGPU_ERR_CUDA, "eviction failed");
            rescan = true;
            break;
          }
          lock.unlock();
        }
        const int rc = Admit(S, s);
        lock.lock();
        if (rc != APHGPU_OK) {
          // the simulation's oldest request fails with the admission error
          s.busy = false;
          S->resident_bytes -= need;
          FailOldest(S, s.id, rc, "admission failed");
          rescan = true;
          break;
        }
        // run the admitted simulation's oldest request now, still reserved:
        // released idle, another worker making room would evict it again
        // before its step (admission/eviction thrash)
        for (auto q2 = S->queue.begin(); q2 != S->queue.end(); ++q2)
          if (q2->sim == s.id) {
            it = q2;
            break;
          }
        if (it == S->queue.end()) {
          s.busy = false;
          rescan = true;
        }
        break;
      }
      it = q;
      break;
    }
    if (rescan) continue;
    if (it == S->queue.end()) {
      if (S->stop) return;
      S->cv_work.wait(lock);
      continue;
    }
    Request r = std::move(*it);
    S->queue.erase(it);
    Sim& s = *S->sims[r.sim];
    s.busy = true;
    s.last_use = ++S->use_clock;
    const auto t_start = Clock::now();
    lock.unlock();
    aphgpu_step_result res{};
    res.ticket = r.ticket;
    res.sim = r.sim;
    res.status = RunStep(S, s, r, &res);
    const auto t_end = Clock::now();
    lock.lock();
    // measured footprint replaces the estimate
    const int64_t measured = aphgpu_device_bytes(s.ctx);
    S->resident_bytes += measured - s.bytes;
    s.bytes = measured;
    if (res.status == APHGPU_OK) s.steps += 1;
    s.busy = false;
    res.queue_ms = std::chrono::duration<double, std::milli>(t_start - r.submitted).count();
    res.latency_ms = std::chrono::duration<double, std::milli>(t_end - r.submitted).count();
    S->done[r.ticket] = res;
    S->completed += 1;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int aphgpu_server_create(aphgpu_server** out, int device, double budget_bytes, int slots,
                         const aphgpu_conf* conf) {
  if (!out || slots < 1 || slots > 256 || !(budget_bytes > 0)) return APHGPU_ERR_ARG;
  aphgpu_server* S = new (std::nothrow) aphgpu_server();
  if (!S) return APHGPU_ERR_NOMEM;
  S->device = device;
  S->budget = (int64_t)budget_bytes;
  S->slots = slots;
  if (conf) {
    S->conf = *conf;
  } else {
    aphgpu_conf_default(&S->conf);
    S->conf.solver = APHGPU_SOLVER_MIXED;
    S->conf.rtol = 1e-10;
  }
  for (int i = 0; i < slots; ++i) S->workers.emplace_back(Worker, S);
  *out = S;
  return APHGPU_OK;
}

void aphgpu_server_destroy(aphgpu_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  for (auto& kv : S->sims)
    if (kv.second->ctx) aphgpu_destroy(kv.second->ctx);
  delete S;
}

int aphgpu_server_add_sim(aphgpu_server* S, int nx, int ny, int nz, double h,
                          const double* alpha, double rho1, double rho2, double sigma,
                          int* sim) {
  if (!S || !alpha || !sim || nx < 3 || ny < 3 || nz < 3 || !(h > 0)) return APHGPU_ERR_ARG;
  auto s = std::make_unique<Sim>();
  s->n[0] = nx;
  s->n[1] = ny;
  s->n[2] = nz;
  s->h = h;
  s->rho1 = rho1;
  s->rho2 = rho2;
  s->sigma = sigma;
  const int64_t N = (int64_t)nx * ny * nz;
  s->alpha.assign(alpha, alpha + N);  // admitted lazily, at its first step
  s->bytes = (int64_t)(kBytesPerCellEstimate * N) + (1 << 20);
  std::lock_guard<std::mutex> lock(S->mu);
  if (s->bytes > S->budget) return APHGPU_ERR_NOMEM;  // could never be admitted
  s->id = S->next_sim++;
  *sim = s->id;
  S->sims[s->id] = std::move(s);
  return APHGPU_OK;
}

int aphgpu_server_submit(aphgpu_server* S, int sim, const double* vflux, double dt,
                         int64_t* ticket) {
  if (!S || !vflux || !ticket) return APHGPU_ERR_ARG;
  Request r;
  r.sim = sim;
  r.dt = dt;
  r.submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lock(S->mu);
    auto it = S->sims.find(sim);
    if (it == S->sims.end()) return APHGPU_ERR_ARG;
    const int64_t N = Cells(*it->second);
    r.vflux.assign(vflux, vflux + 3 * N);
    r.ticket = S->next_ticket++;
    *ticket = r.ticket;
    S->queue.push_back(std::move(r));
  }
  S->cv_work.notify_one();
  return APHGPU_OK;
}

int aphgpu_server_wait(aphgpu_server* S, int64_t ticket, aphgpu_step_result* out) {
  return aphgpu_server_wait_timeout(S, ticket, -1.0, out);
}

int aphgpu_server_wait_timeout(aphgpu_server* S, int64_t ticket, double timeout_ms,
                               aphgpu_step_result* out) {
  if (!S || !out) return APHGPU_ERR_ARG;
  std::unique_lock<std::mutex> lock(S->mu);
  if (ticket <= 0 || ticket >= S->next_ticket) return APHGPU_ERR_ARG;
  auto ready = [&] { return S->done.count(ticket) > 0; };
  if (timeout_ms < 0) {
    S->cv_done.wait(lock, ready);
  } else if (!S->cv_done.wait_for(lock, std::chrono::duration<double, std::milli>(timeout_ms),
                                  ready)) {
    return APHGPU_ERR_TIMEOUT;  // still pending: may be waited for again
  }
  *out = S->done[ticket];
  S->done.erase(ticket);
  return APHGPU_OK;
}

int aphgpu_server_get_state(aphgpu_server* S, int sim, double* alpha, double* pressure) {
  if (!S) return APHGPU_ERR_ARG;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->sims.find(sim);
  if (it == S->sims.end()) return APHGPU_ERR_ARG;
  Sim& s = *it->second;
  S->cv_done.wait(lock, [&] { return !s.busy; });
  const int64_t N = Cells(s);
  if (!s.ctx) {
    if (alpha) std::memcpy(alpha, s.alpha.data(), sizeof(double) * N);
    if (pressure) {
      if (s.has_pressure) std::memcpy(pressure, s.pressure.data(), sizeof(double) * N);
      else std::fill(pressure, pressure + N, 0.0);
    }
    return APHGPU_OK;
  }
  int rc = APHGPU_OK;
  if (alpha) rc = aphgpu_vof_get(s.ctx, alpha, nullptr, nullptr, nullptr);
  if (rc == APHGPU_OK && pressure) rc = aphgpu_get_solution(s.ctx, pressure);
  return rc;
}

int aphgpu_server_get_stats(aphgpu_server* S, aphgpu_server_stats* st) {
  if (!S || !st) return APHGPU_ERR_ARG;
  std::lock_guard<std::mutex> lock(S->mu);
  st->sims = (int)S->sims.size();
  int resident = 0;
  for (auto& kv : S->sims) resident += kv.second->ctx ? 1 : 0;
  st->resident = resident;
  st->resident_bytes = S->resident_bytes;
  st->budget_bytes = S->budget;
  st->completed = S->completed;
  st->queued = (int64_t)S->queue.size();
  st->evictions = S->evictions;
  st->admissions = S->admissions;
  return APHGPU_OK;
}

}  // extern "C"

/*
 * aphgpu: GB300-native (sm_103a) projection-step hot path of the aphros
 * multiphase flow solver, behind a plain C ABI.
 *
 * One context (`aphgpu_ctx`) owns one periodic Cartesian domain of
 * nx*ny*nz cells of size h resident on one GPU, with its own CUDA stream.
 * Host arrays are x-fastest over the domain's cells (no halo cells), i.e.
 * FieldCell values in the order of aphros's GIndex (geom/block.h:149-158).
 * Face arrays hold three consecutive blocks (x, y, z faces) of nx*ny*nz
 * values; entry c of block d is the face between cell c-e_d and cell c.
 * Vector cell fields (normals) are AoS, 3 doubles per cell (FieldCell<Vect>).
 *
 * Every entry point returns APHGPU_OK (0) or an error code; the message of
 * the last error of a context is returned by aphgpu_last_error().  No C++
 * exception crosses this boundary.  All calls on one context must come from
 * one host thread at a time.  Unless stated otherwise a call returns after
 * its results are complete (host output arrays filled).
 */
#ifndef APHGPU_H_
#define APHGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct aphgpu_ctx aphgpu_ctx;

enum {
  APHGPU_OK = 0,
  APHGPU_ERR_ARG = 1,          /* invalid argument */
  APHGPU_ERR_CUDA = 2,         /* CUDA runtime error */
  APHGPU_ERR_NOMEM = 3,        /* device allocation failed */
  APHGPU_ERR_NOT_SYMMETRIC = 4,/* system handed to a symmetric solver is not */
  APHGPU_ERR_STATE = 5,        /* call order violated (e.g. no system set) */
  APHGPU_ERR_UNSUPPORTED = 6,  /* grid shape not supported by the solver */
  APHGPU_ERR_TIMEOUT = 7       /* bounded wait ended before completion */
};

/* Solver kinds (the `linsolver_symm` values `gpu_cg`, `gpu`, `gpu_mixed`). */
enum {
  APHGPU_SOLVER_CG = 0,    /* plain FP64 CG, the algorithm of SolverConjugate */
  APHGPU_SOLVER_MGPCG = 1, /* FP64 CG preconditioned by an FP64 MG V-cycle */
  APHGPU_SOLVER_MIXED = 2, /* FP64 defect correction around FP32 MG-PCG */
  APHGPU_SOLVER_MGPCG32 = 3 /* FP64 CG preconditioned by an FP32 V-cycle */
};

/* Stopping rule and limits; mirrors linear::Solver::Conf
 * (src/linear/linear.h:21-25) plus the norm choice of
 * SolverConjugate::Extra (linear.h:85-87). */
typedef struct {
  int solver;        /* APHGPU_SOLVER_* */
  double tol;        /* absolute tolerance on the residual norm below */
  int miniter;       /* minimum iterations (reference default 1) */
  int maxiter;       /* maximum iterations */
  int maxnorm;       /* 0: sqrt(sum r^2 / h^3), 1: max|r| / h^3 */
  /* multigrid (ignored by APHGPU_SOLVER_CG) */
  int mg_pre;        /* red-black Gauss-Seidel sweeps before restriction */
  int mg_post;       /* sweeps after prolongation */
  int mg_coarse_max; /* largest coarsest-level cell count (<= 4096) */
  /* mixed precision: relative reduction asked of each inner FP32 solve
   * (less when less is left to reach the tolerance: the reduction left
   * times 0.3) */
  double inner_rtol;
  int inner_maxiter;
  /* inner FP32 PCG options: bit 0 keeps the residual free of the constant
   * (null-space) component that FP32 rounding adds to A p; bit 1 uses the
   * flexible (Polak-Ribiere) beta, robust to the FP32 preconditioner's
   * rounding */
  int inner_flags;
  /* relative tolerance: when > 0 the solve stops at
   * max(tol, rtol * sqrt(sum b^2 / h^3)), i.e. ||r||/||b|| <= rtol from a
   * zero guess */
  double rtol;
} aphgpu_conf;

/* Result; mirrors linear::Solver::Info (linear.h:27-30).  `iter` counts
 * outer iterations; for APHGPU_SOLVER_MIXED `inner_iter` is the total
 * number of FP32 PCG iterations. */
typedef struct {
  double residual;
  int iter;
  int inner_iter;
  int converged;
} aphgpu_info;

/* Fills `conf` with defaults: MG-PCG, tol 0, miniter 1, maxiter 1000,
 * L2 norm, 2+2 sweeps, coarsest <= 64 cells, inner_rtol 3e-4,
 * inner_maxiter 200, inner_flags 3 (projection and flexible beta). */
void aphgpu_conf_default(aphgpu_conf* conf);

/* ---- context ---- */

/* Creates a context for a periodic nx*ny*nz domain of cubic cells of edge h
 * on CUDA device `device`.  Replaces the per-mesh device state that
 * SolverConjugateCL keeps in its Shared struct
 * (src/linear/conjugate_cl.ipp:155-187). */
int aphgpu_create(aphgpu_ctx** ctx, int nx, int ny, int nz, double h,
                  int device);
void aphgpu_destroy(aphgpu_ctx* ctx);
const char* aphgpu_last_error(const aphgpu_ctx* ctx);
/* Bytes of device memory held by the context. */
int64_t aphgpu_device_bytes(const aphgpu_ctx* ctx);
/* Waits for all work of the context. */
int aphgpu_sync(aphgpu_ctx* ctx);

/* ---- Poisson / projection ---- */

/* Sets the linear system from aphros's per-cell expressions
 * e[0]*x[c] + sum_q e[1+q]*x[nb_q] + e[7] = 0, q = xm,xp,ym,yp,zm,zp,
 * 8 doubles per cell (FieldCell<Expr>, src/geom/mesh.h:481-485), the input
 * of linear::Solver::Solve (src/linear/linear.h:44-46).  The system must be
 * symmetric (e[2] of c equals e[1] of c+x, etc.), as CG requires. */
int aphgpu_set_system_expr(aphgpu_ctx* ctx, const double* expr8);

/* Given-pressure cells: Proj::ApplyCellCond (src/solver/proj.ipp:326-338)
 * on the current system (after aphgpu_assemble_projection or
 * aphgpu_set_system_expr), e[0] += 1 and e[7] -= values[t] in cell
 * cells[t] (x-fastest index), as aphros does for each CondCellVal of its
 * cell-condition map.  Each cell at most once (else APHGPU_ERR_ARG).  The
 * system then has an explicit diagonal and is no longer singular. */
int aphgpu_apply_cell_cond(aphgpu_ctx* ctx, int64_t count, const int64_t* cells,
                           const double* values);

/* Copies the current system back as per-cell expressions (8 doubles per
 * cell, the layout of aphgpu_set_system_expr), e.g. to inspect the system
 * assembled by aphgpu_assemble_projection. */
int aphgpu_get_system_expr(aphgpu_ctx* ctx, double* expr8);

/* Assembles the projection system on the device from the gas volume
 * fraction and the predicted face fluxes, fusing
 *   Hydro::CalcMixture density (src/kernel/hydro.ipp:1815-1822),
 *   UEmbed::InterpolateHarmonic face density (src/solver/approx_eb.h:351-363),
 *   the surface-tension face force term (src/solver/proj.ipp:556-562),
 *   Proj::GetFlux and Proj::GetFluxSum (src/solver/proj.ipp:343-383).
 * alpha: nx*ny*nz, or NULL to use the resident VOF volume fraction;
 * vflux: 3 face blocks (u*.S); febp: face force per unit volume (NULL: none,
 * or the resident surface-tension force after aphgpu_set_force_resident);
 * dt: time step; remove_mean: subtract the mean of the constant term
 * (src/solver/pois.h:41-47).  The fluxes stay resident for
 * aphgpu_flux_correct(). */
int aphgpu_assemble_projection(aphgpu_ctx* ctx, const double* alpha,
                               double rho1, double rho2, const double* vflux,
                               const double* febp, double dt, int remove_mean);

/* Solves the current system: the drop-in for linear::Solver::Solve
 * (src/linear/linear.h:44-46) as used by Proj::Project
 * (src/solver/proj.ipp:396-398).  x0: initial guess (NULL: zero, may equal
 * x); x: solution (NULL: keep it resident only).  Non-convergence is not an
 * error: info->converged = 0 and info->iter > maxiter, like CG. */
int aphgpu_solve(aphgpu_ctx* ctx, const aphgpu_conf* conf, const double* x0,
                 double* x, aphgpu_info* info);

/* Solves with the resident solution as initial guess (zero_guess = 0) or
 * from zero, leaving the solution resident. */
int aphgpu_solve_resident(aphgpu_ctx* ctx, const aphgpu_conf* conf,
                          int zero_guess, aphgpu_info* info);

/* Residual history of the last solve: which = 0 the (outer) iterations,
 * which = 1 the inner FP32 iterations of a mixed solve (all inner solves
 * concatenated).  Copies at most cap values; *count receives the number
 * available. */
int aphgpu_residual_history(aphgpu_ctx* ctx, int which, double* out, int cap,
                            int* count);

/* Sets the resident solution (initial guess of aphgpu_solve_resident with
 * zero_guess = 0), e.g. to restore a checkpointed pressure. */
int aphgpu_set_solution(aphgpu_ctx* ctx, const double* x);

/* Copies the resident solution (pressure) to the host. */
int aphgpu_get_solution(aphgpu_ctx* ctx, double* x);

/* Residual norm sqrt(sum r^2) and sqrt(sum b^2) of the resident solution,
 * r = b - A x, b = -e[7] (FP64). */
int aphgpu_residual_norms(aphgpu_ctx* ctx, double* rnorm, double* bnorm);

/* Corrected face fluxes v = k*(p[cm] - p[cp]) + v* of Proj::Project
 * (src/solver/proj.ipp:399-403, UEmbed::Eval src/solver/approx_eb.h:338-343)
 * for the last assembled projection system and the resident pressure.
 * vflux_out: 3 face blocks, host (NULL: keep resident as the advection
 * flux of the next aphgpu_vof_step with vflux == NULL). */
int aphgpu_flux_correct(aphgpu_ctx* ctx, double* vflux_out);

/* Cell acceleration (febp - grad p)/rho_f averaged to cells, Proj
 * GetAcceleration (src/solver/proj.ipp:408-433) without cell force, for the
 * last assembled projection (its density and force) and the resident
 * pressure; acc: 3 doubles per cell (AoS). */
int aphgpu_acceleration(aphgpu_ctx* ctx, double* acc);

/* ---- PLIC volume of fluid ---- */

/* Sets the volume fraction and reconstructs the interface: the state of
 * Vof after StartStep at t=0 (src/solver/vof.ipp:177-195, 70-90). */
int aphgpu_vof_init(aphgpu_ctx* ctx, const double* alpha, double clipth);

/* One advection step: Vof::MakeIteration (src/solver/vof.ipp:498-583),
 * scheme weymouth, three directionally split sweeps (Vof::Sweep,
 * vof.ipp:212-327) in the order selected by the step count, each followed
 * by interface reconstruction; then FinishStep.  vflux: mixture face fluxes
 * (host, 3 face blocks) or NULL to use the resident corrected fluxes of
 * aphgpu_flux_correct().  Colour labelling is not part of this path; the
 * volume source, if any, is the one of aphgpu_vof_set_source. */
int aphgpu_vof_step(aphgpu_ctx* ctx, const double* vflux, double dt);

/* Sets the volume source of the following aphgpu_vof_step calls (host, one
 * value per cell; NULL: none, the default): the init stage of
 * Vof::MakeIteration (src/solver/vof.ipp:504-514) first sets
 * u = u + dt * src * (1 - u) in every cell; the sweeps then start from that
 * field, cells that became interfacial through the source carrying the
 * plain flux v*u in the first sweep (they have no plane yet).  The
 * reference reads the source from its owner (Vof's fcs argument). */
int aphgpu_vof_set_source(aphgpu_ctx* ctx, const double* src);

/* Copies the VOF state to the host; any pointer may be NULL.
 * normals: AoS 3 per cell, NaN outside the interface; plane: plane
 * constant, NaN outside; mask: 1 in interfacial cells (0<alpha<1). */
int aphgpu_vof_get(aphgpu_ctx* ctx, double* alpha, double* normals,
                   double* plane, uint8_t* mask);

/* Height-function curvature of the current VOF state:
 * curvature::Heights::CalcCurvature (src/solver/curv.ipp:358-414), one
 * layer without colours.  kappa: NaN outside the interface; heights:
 * optional AoS 3 per cell (NaN where undefined).  Either may be NULL
 * (results stay resident for aphgpu_surface_tension). */
int aphgpu_curvature(aphgpu_ctx* ctx, double* kappa, double* heights);

/* Parameters of the particle-string curvature: PartStr::Par and
 * PartStrMeshM::Par (src/solver/partstr.h:38-45, partstrmeshm.h:26-36),
 * the part_* variables of the reference's configuration. */
typedef struct {
  int np;          /* particles per string, odd, 3..15 (part_np) */
  int ns;          /* strings (section planes) per cell (part_ns) */
  double leq;      /* string length in cells (part_h) */
  double relax;    /* relaxation factor (part_relax) */
  double tol;      /* tolerance on the correction (part_tol) */
  int itermax;     /* iterations at most (part_itermax) */
  double segcirc;  /* shift to a circular segment (part_segcirc) */
  int dn;          /* 1: normal displacement of the whole string (part_dn) */
} aphgpu_part_conf;

/* The defaults of deploy/scripts/sim_base.conf: np 7, ns 3, leq 4, relax
 * 0.5, tol 1e-5, itermax 20, segcirc 0, dn 0. */
void aphgpu_part_conf_default(aphgpu_part_conf* conf);

enum {
  APHGPU_CURV_HEIGHTS = 0,   /* curvature::Heights (aphgpu_curvature) */
  APHGPU_CURV_PARTICLES = 1, /* curvature::Particles */
  APHGPU_CURV_HYBRID = 2     /* curvature::Hybrid: heights, particles where
                                the heights give none */
};

/* Curvature of the current VOF state by the estimator that
 * curvature::MakeEstimator (src/solver/curv.ipp:604-622) selects by name:
 * Particles (curv.ipp:29-54 with partstrmeshm.ipp:266-395 and
 * partstr.h:57-646) seeds ns strings in every interfacial cell, one layer,
 * no colours (the single-field Vof gives the estimator none, vof.ipp:746-
 * 749), periodic, no contact angles.  conf: NULL for the defaults.  kappa:
 * host output (NaN where no estimate), or NULL to keep it resident (for
 * aphgpu_surface_tension).  Equal to the reference up to the last bits of
 * the device's cos and sin. */
int aphgpu_curvature_estimator(aphgpu_ctx* ctx, int estimator, const aphgpu_part_conf* conf,
                               double* kappa);

/* Surface-tension face force sigma*kappa*grad(alpha) of
 * AppendSurfaceTension (src/util/hydro.ipp:1289-1310) from the resident
 * volume fraction and curvature.  febp: 3 face blocks (host) or NULL to keep
 * it resident for the next aphgpu_assemble_projection(febp == NULL) call
 * with use_resident_force set by aphgpu_set_force_resident(). */
int aphgpu_surface_tension(aphgpu_ctx* ctx, double sigma, double* febp);

/* Makes the next assemble calls use the resident surface-tension force
 * (on != 0) when their febp argument is NULL. */
int aphgpu_set_force_resident(aphgpu_ctx* ctx, int on);

/* ---- projection fluid step ---- */

/* Sets up the projection fluid solver of aphros, Proj
 * (src/solver/proj.ipp) with the default ProjPar (BCG advection, implicit
 * diffusion, one iteration per step), periodic, without forces or
 * sources: density and dynamic viscosity are the mixtures rho1 (1 - a) +
 * rho2 a and mu1 (1 - a) + mu2 a of the gas volume fraction a (alpha, or
 * NULL for the resident VOF volume fraction, then re-read at every step);
 * vel: the cell velocity, 3 blocks of N (x, y, z components); the face
 * fluxes of the time layer are those of vel (Proj's constructor,
 * proj.ipp:96-101); pressures start at zero. */
int aphgpu_fluid_init(aphgpu_ctx* ctx, const double* alpha, double rho1, double rho2,
                      double mu1, double mu2, const double* vel);

/* One time step of Proj (StartStep, MakeIteration, FinishStep,
 * proj.ipp:309-322, 455-613): on the first step the initial pressure
 * (proj.ipp:111-127), then the acceleration of the pressure, the BCG
 * predicted face fluxes and their projection with dt/2 (proj.ipp:484-499),
 * the BCG advection of the velocity (proj.ipp:128-190), implicit
 * diffusion of each component (proj.ipp:241-307), the face fluxes of the
 * velocity projected with dt, and the new acceleration (proj.ipp:524-575).
 * Its five linear systems (four after the first step) are solved by
 * conf's solver (miniter 0, as Proj's solver is configured), each from
 * its guess (the pressure of the previous solve, the advected velocity).
 * The corrected fluxes become the resident advection fluxes of
 * aphgpu_vof_step(ctx, NULL, dt).  info->iter: total solver iterations;
 * info->converged: every solve converged. */
int aphgpu_fluid_step(aphgpu_ctx* ctx, double dt, const aphgpu_conf* conf, aphgpu_info* info);

/* Copies the fluid state to the host; any pointer may be NULL.  vel: 3
 * blocks of N; p: pressure; flux: the face fluxes, 3 face blocks. */
int aphgpu_fluid_get(aphgpu_ctx* ctx, double* vel, double* p, double* flux);

/* BCG face values of a cell field: UEmbed::InterpolateBcg
 * (src/solver/approx_eb.ipp:753-821) on the periodic mesh of the context,
 * the predictor of Proj; u: cell field, vflux: face volume fluxes (3 face
 * blocks), src: cell source, dt; out: 3 face blocks. */
int aphgpu_bcg_faces(aphgpu_ctx* ctx, const double* u, const double* vflux, const double* src,
                     double dt, double* out);

/* ---- timing of the last solve (CUDA events on the context stream) ---- */

/* Milliseconds of the last solve, VOF step or curvature
 * call measured on the device, and the number of kernels it launched. */
int aphgpu_last_timing(const aphgpu_ctx* ctx, double* ms, int64_t* launches);

/* Plain FP64 CG solve (the algorithm of aphgpu_solve with
 * APHGPU_SOLVER_CG) that allocates no memory at all.  This entry point has
 * no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc: a solver plug-in inside a host application that reserves the
 * GPU's memory for its own pool allocator, or a step loop with a fixed time
 * budget, where cudaMalloc/cudaFree would synchronize the device.  Such
 * callers already own their inputs and outputs; the solver's work vectors
 * live in one fixed device array inside the library (about 1.6 MB, held on
 * every GPU that loads the library until the process exits).
 *   d_expr8: device array, 8 doubles per cell (see aphgpu_set_system_expr);
 *   d_x0: device initial guess or NULL (zero), may equal d_x;
 *   d_x: device solution;  cellvol: h^3 of the residual norm;
 *   tol, miniter, maxiter, maxnorm: as in aphgpu_conf;  stream: the
 *   cudaStream_t to run on (NULL: the default stream).
 * Limits: at most 65536 cells (e.g. 64x32x32 or 40^3) and every dimension
 * >= 3; larger grids return APHGPU_ERR_ARG (no context, so no message).
 * The first call on a device looks up the array's device address while that
 * device is current: make it before any stream capture.  All calls share
 * the array: calls whose work overlaps on the GPU race and must be
 * serialized by the caller.  The call blocks: it synchronizes `stream`
 * every few iterations to read the convergence flag and returns after the
 * solve has finished. */
int aphgpu_cg_solve_noalloc(int nx, int ny, int nz, double cellvol,
                            const double* d_expr8, const double* d_x0,
                            double* d_x, double tol, int miniter, int maxiter,
                            int maxnorm, void* stream, aphgpu_info* info);

/* ---- serving loop ----
 *
 * Time-step requests for many simulations resident on one GPU, run with
 * continuous batching: `slots` worker threads start requests as they
 * arrive, requests of different simulations run concurrently on their own
 * streams (their kernels overlap on the device), steps of one simulation
 * run in submission order.  A request is one full step: projection
 * (assembly from the resident volume fraction, the request's predicted face
 * fluxes and the resident surface-tension force; solve warm-started from
 * the resident pressure; corrected fluxes), PLIC advection with the
 * corrected fluxes, height curvature, and the surface-tension force for the
 * next step.  Simulations are admitted while their device memory fits the
 * budget; to admit one, the least recently used idle simulations are
 * evicted to host memory and restored bit-exactly later.  There is no
 * counterpart in the reference (its time loop steps one simulation). */
typedef struct aphgpu_server aphgpu_server;

typedef struct {
  int64_t ticket;
  int sim;
  int status;          /* APHGPU_OK or the error of the step */
  int iters;           /* solver iterations (outer for the mixed solver) */
  int inner_iters;
  int converged;
  double residual;
  double queue_ms;     /* submission -> start */
  double latency_ms;   /* submission -> completion */
  double device_ms;    /* device time of solve + advection + curvature */
} aphgpu_step_result;

typedef struct {
  int sims;
  int resident;
  int64_t resident_bytes;
  int64_t budget_bytes;
  int64_t completed;
  int64_t queued;
  int64_t evictions;
  int64_t admissions;
} aphgpu_server_stats;

/* conf: solver of every step (NULL: mixed precision, rtol 1e-10). */
int aphgpu_server_create(aphgpu_server** server, int device, double budget_bytes,
                         int slots, const aphgpu_conf* conf);
void aphgpu_server_destroy(aphgpu_server* server);
/* Registers a simulation (periodic nx*ny*nz, cell h, gas volume fraction
 * alpha, densities, surface tension sigma); admitted at its first step. */
int aphgpu_server_add_sim(aphgpu_server* server, int nx, int ny, int nz, double h,
                          const double* alpha, double rho1, double rho2,
                          double sigma, int* sim);
/* Queues one step (vflux copied at submission: 3 face blocks). */
int aphgpu_server_submit(aphgpu_server* server, int sim, const double* vflux,
                         double dt, int64_t* ticket);
/* Waits for a step and returns its result (each ticket once). */
int aphgpu_server_wait(aphgpu_server* server, int64_t ticket,
                       aphgpu_step_result* result);
/* As aphgpu_server_wait, giving up after timeout_ms (< 0: no limit) with
 * APHGPU_ERR_TIMEOUT; the ticket then stays pending. */
int aphgpu_server_wait_timeout(aphgpu_server* server, int64_t ticket, double timeout_ms,
                               aphgpu_step_result* result);
/* Volume fraction and pressure of a simulation after its queued steps
 * that have started have finished (either pointer may be NULL). */
int aphgpu_server_get_state(aphgpu_server* server, int sim, double* alpha,
                            double* pressure);
int aphgpu_server_get_stats(aphgpu_server* server, aphgpu_server_stats* stats);

/* Batched solve of many independent periodic domains of uneven size, each
 * with its own context holding an assembled system (set_system_expr or
 * assemble_projection): the mixed-precision solver of every domain, with
 * every kernel launch covering all domains at one multigrid level through
 * per-level tile tables, per-domain reductions and stopping flags, and
 * batches of inner iterations replayed from a CUDA graph.  Domains converge
 * independently; each domain's result is what its own mixed solve computes
 * up to the order of floating-point sums.  The coarsest level of every
 * domain must be small enough for the dense direct solve (at most 1024
 * cells).  Every context must live on the same device; the batch runs on the
 * stream of the first context and waits for the others' pending work.  The
 * solution is left resident in each context (aphgpu_get_solution).  There
 * is no counterpart in the reference (it solves one domain per process). */
typedef struct aphgpu_batch aphgpu_batch;

int aphgpu_batch_create(aphgpu_batch** batch, int count, aphgpu_ctx* const* ctxs);
void aphgpu_batch_destroy(aphgpu_batch* batch);
const char* aphgpu_batch_last_error(const aphgpu_batch* batch);
/* Solves every domain from a zero initial guess with the mixed-precision
 * settings of conf (solver field ignored); infos (may be NULL) receives one
 * aphgpu_info per domain. */
int aphgpu_batch_solve(aphgpu_batch* batch, const aphgpu_conf* conf, aphgpu_info* infos);
/* Tiling of the batched launches: z planes per thread of a tile (1..64,
 * default 4) and the size in cells at or below which a domain's coarse
 * levels are cycled by one CTA per domain in a single launch (default
 * 4096; 0: only the coarsest level). */
int aphgpu_batch_set_tiles(aphgpu_batch* batch, int planes, int coarse_cells);
int aphgpu_batch_get_tiles(const aphgpu_batch* batch, int* planes, int* coarse_cells);
/* Cycle of the per-domain coarse levels: 1 (default) V, 2 W (each level
 * below the first per-domain level visited twice per visit of its parent). */
int aphgpu_batch_set_cycle(aphgpu_batch* batch, int cycle);
int aphgpu_batch_get_cycle(const aphgpu_batch* batch, int* cycle);
/* Autotuner: times solves over the tile planes, the coarse-level size and
 * the cycle, then over the smoothing sweeps; keeps the fastest tiling and
 * cycle in the batch and writes its sweeps into conf (mg_pre = mg_post);
 * best_ms may be NULL. */
int aphgpu_batch_tune(aphgpu_batch* batch, aphgpu_conf* conf, double* best_ms);
/* Device milliseconds of the last solve and kernels launched so far. */
int aphgpu_batch_last_ms(const aphgpu_batch* batch, double* ms, int64_t* launches);

/* Records event `slot` (0..7) on the context's stream; aphgpu_elapsed
 * returns the milliseconds between two recorded slots (waits for the
 * second). */
/* Execution options of a context (results do not depend on them; they
 * exist to measure and check the variants):
 *   APHGPU_OPT_GRAPHS        1 (default): replay batches of PCG iterations
 *                            from CUDA graphs; 0: launch every kernel
 *   APHGPU_OPT_FUSED_SWEEPS  fused out-of-place red-black sweeps (both
 *                            colours in one pass: half the DRAM traffic of
 *                            two half sweeps) on the FP32 levels: 1
 *                            the pipelined kernel, fed by asynchronous
 *                            copies into shared memory, on levels of at
 *                            least 2^21 cells with nx a multiple of 4,
 *                            nx >= 16, nz >= 8 and no stored diagonal; 2
 *                            the pipelined kernel on
 *                            every such level whatever its size; 3 the
 *                            synchronous fused kernel (latency-bound) on
 *                            every level with nx a multiple of 4, nx >= 8;
 *                            4 as 1 with bands of 6 rows (two CTAs per
 *                            SM instead of one); 5 the in-place wavefront
 *                            sweep (each CTA walks the planes of a tile
 *                            in chunks, the second colour one chunk
 *                            behind the first, waiting for its neighbour
 *                            tiles; cooperative launch) on
 *                            levels of at least 2^21 cells with nx a
 *                            multiple of 4 and nz >= 4; 6 the wavefront
 *                            sweep on every such level; 0 (default) two
 *                            in-place half sweeps everywhere.  Other
 *                            levels take the half sweeps
 *   APHGPU_OPT_HALF_COUPLINGS 1: the smoother and the restriction of the
 *                            finest FP32 level read an FP16 copy of the
 *                            couplings scaled by a power of two (the PCG
 *                            operator and the FP64 defect correction keep
 *                            FP32 / FP64: only the preconditioner changes,
 *                            and its rounding can cost inner iterations);
 *                            0 (default): FP32 couplings
 *   APHGPU_OPT_CYCLE         multigrid cycle below the finest level: 1
 *                            V-cycle, 2 W-cycle (each coarse level visited
 *                            twice per visit of the level above), 0
 *                            (default) W from 256^3 cells up, V below
 *   APHGPU_OPT_COARSE_SERIES weight in percent (0..100, default 60) of the
 *                            series combination of the fine couplings in
 *                            the coarse-level couplings; the rest is the
 *                            Galerkin coupling of constant prolongation
 *                            scaled by one half (0 = that operator alone).
 *                            Changes the preconditioner only; the coarse
 *                            operators are rebuilt at the next solve
 *   APHGPU_OPT_SWEEP_GROWTH  smoothing sweeps on level l below the finest
 *                            (mg_pre / mg_post on the finest): 1 the same
 *                            count, 2 count * (l + 1), 3 count * 2^l (at
 *                            most 16), 0 (default) 2 for V-cycles from
 *                            256^3 cells up and 1 otherwise
 *   APHGPU_OPT_CTA_COARSE    1 (default): the FP32 levels of at most 512
 *                            cells (8^3) below the finest are cycled by
 *                            one CTA per visit of their parent level,
 *                            staged in shared memory (the batch's
 *                            per-domain coarse cycle; a W-cycle at 512^3
 *                            launches 8 k kernels per solve instead of
 *                            16 k); 0: one launch per pass on every level
 *   APHGPU_OPT_WAVE_PLANES   planes per step of the wavefront sweep
 *                            (APHGPU_OPT_FUSED_SWEEPS 5 and 6); 0 (default):
 *                            as many as let three steps' worth of a level's
 *                            x, b and couplings fit in 60 MB of L2
 *   APHGPU_OPT_COLOR_SPLIT   1: the mixed solver keeps its finest
 *                            FP32 level (the right-hand side, the iterate
 *                            and the inner CG vectors) with each row's two
 *                            red-black colours in separate halves, so that
 *                            a half sweep reads and writes only the cells
 *                            it needs (18 instead of 24 bytes per cell);
 *                            taken when nx is a multiple of 8, ny and nz
 *                            are even, APHGPU_OPT_FUSED_SWEEPS is 0 and
 *                            APHGPU_OPT_HALF_COUPLINGS is off.  Same
 *                            smoothing, restriction and prolongation
 *                            values; the inner CG's FP32 dot products sum
 *                            in another order.  2 (default): so from
 *                            2^22 cells up (on smaller grids the split
 *                            kernels' 8 cells per thread leave too few
 *                            threads: the served 32^3-128^3 simulations
 *                            ran 10 % slower); 0: natural order
 *   APHGPU_OPT_DF_RESIDUAL   1: for flux-difference systems (every
 *                            diagonal minus the sum of its row's
 *                            couplings) the mixed solver updates its outer
 *                            residual after each inner solve as
 *                            r -= s A e in double-float arithmetic (pairs
 *                            of floats, 48 significant bits) on the FP32
 *                            pipe, with the correction x += s e in FP64;
 *                            the first residual is computed in FP64.  It
 *                            holds the couplings' FP32 low parts (12
 *                            bytes per cell, made again after each new
 *                            system).  2 (default): so from 2^22 cells up,
 *                            where the FP64 residual's time outweighs
 *                            that; 0: every outer residual b - A x in
 *                            FP64
 *   APHGPU_OPT_W_MIN_CELLS   with W-cycles: a level of at most this many
 *                            cells visits the level below it once (a V
 *                            below it); default 4096 (16^3: at 512^3 the
 *                            mixed solve takes 17 instead of 18 inner
 *                            iterations and 133 instead of 146 ms); 0: W
 *                            on every level */
enum {
  APHGPU_OPT_GRAPHS = 0,
  APHGPU_OPT_FUSED_SWEEPS = 1,
  APHGPU_OPT_HALF_COUPLINGS = 2,
  APHGPU_OPT_CYCLE = 3,
  APHGPU_OPT_COARSE_SERIES = 4,
  APHGPU_OPT_SWEEP_GROWTH = 5,
  APHGPU_OPT_CTA_COARSE = 6,
  APHGPU_OPT_WAVE_PLANES = 7,
  APHGPU_OPT_COLOR_SPLIT = 8,
  APHGPU_OPT_DF_RESIDUAL = 9,
  APHGPU_OPT_W_MIN_CELLS = 10
};
int aphgpu_set_option(aphgpu_ctx* ctx, int option, int value);

int aphgpu_mark(aphgpu_ctx* ctx, int slot);
int aphgpu_elapsed(aphgpu_ctx* ctx, int slot0, int slot1, double* ms);

/* Kernel identifiers for aphgpu_time_kernel. */
enum {
  APHGPU_K_SMOOTH32 = 0,   /* FP32 red-black half sweep, finest level */
  APHGPU_K_SMOOTH64 = 1,   /* FP64 red-black half sweep, finest level */
  APHGPU_K_APPLY64 = 2,    /* FP64 y = A p with the p.y reduction */
  APHGPU_K_APPLY32 = 3,    /* FP32 y = A p with the p.y reduction */
  APHGPU_K_RESTRICT32 = 4, /* FP32 residual + restriction, finest level */
  APHGPU_K_VOF_FLUX = 5,   /* VOF fluid fluxes of one direction through the
                              faces with an interfacial upwind cell */
  APHGPU_K_VOF_UPDATE = 6, /* VOF fluxes of the other faces and update of one
                              direction (one fused pass) */
  APHGPU_K_RECONSTRUCT = 7,/* interface normals and plane constants */
  APHGPU_K_HEIGHTS = 8,    /* height functions */
  APHGPU_K_CURVATURE = 9,  /* curvature from heights */
  APHGPU_K_SWEEP32 = 10    /* FP32 fused red-black sweep (both colours, out of
                              place), finest level */
};

/* Launches one kernel `reps` times on the context's stream on its resident
 * data (after a solve / VOF step has prepared it) and returns the mean
 * device milliseconds per launch, measured with CUDA events on that stream,
 * and the algorithmic bytes one launch moves (compulsory traffic: each
 * array element read or written once).  Kernels that update state in place
 * leave it modified. */
int aphgpu_time_kernel(aphgpu_ctx* ctx, int kernel, int reps, double* ms,
                       double* bytes);

/* Failure path of the wavefront sweep (APHGPU_OPT_FUSED_SWEEPS 5 and 6),
 * whose tiles wait on their neighbours' progress: runs its bounded wait
 * once (one warp) on a progress counter that nothing sets.  The wait gives
 * up after its bound (2^22 polls: one to a few seconds) and reports; the
 * call returns
 * APHGPU_ERR_TIMEOUT, as a solve does when a wait of its sweeps gave up,
 * and the context stays usable (the flag is cleared once reported). */
int aphgpu_wave_wait_check(aphgpu_ctx* ctx);

/* ---- connected-component colours of the volume fraction ---- */

/* Recolours the current volume fraction as Vof::MakeIteration does after
 * its sweeps (src/solver/vof.ipp:546-578, union-find recolouring of
 * src/util/vof.ipp:982-1150 with the stable colour map): gas cells (u >
 * 0.5) connected through faces, edges or corners, across the periodic
 * boundaries, share a colour; a bubble keeps its colour from the previous
 * call (or from aphgpu_vof_init: 0 where u > 0); cells with 0 < u <= 0.5
 * take the colour of a face neighbour with larger u.  Call after each
 * aphgpu_vof_step for the reference's colours.  Errors: APHGPU_ERR_STATE
 * before aphgpu_vof_init; APHGPU_ERR_UNSUPPORTED beyond 2^21 components;
 * APHGPU_ERR_TIMEOUT if the bounded union-find loop did not settle (the
 * colours are then left unchanged). */
int aphgpu_vof_recolor(aphgpu_ctx* ctx);
/* Colours of the cells (-1: none), N doubles (Vof::GetColor). */
int aphgpu_vof_colors(aphgpu_ctx* ctx, double* cl);

/* ---- field dumps (aphros raw + XMF format) ---- */

/* Fields of a context: pressure (the solution x), the right-hand side of
 * the system, the volume fraction and the curvature (after aphgpu_vof_init;
 * the curvature of the last aphgpu_curvature). */
enum {
  APHGPU_FIELD_PRESSURE = 0,
  APHGPU_FIELD_RHS = 1,
  APHGPU_FIELD_VF = 2,
  APHGPU_FIELD_CURVATURE = 3
};
/* Element types of a raw file, in the order of dump::Type (dump/xmf.h:13). */
enum { APHGPU_DUMP_UINT16 = 0, APHGPU_DUMP_FLOAT32 = 1, APHGPU_DUMP_FLOAT64 = 2 };

/* Writes `field` to `rawpath` (cells x-fastest, converted to `type` as C++
 * converts a double; UInt16 values outside [0, 65535] are clamped) and its
 * metadata, with dataset name `name` and binpath `rawpath`, to the path of
 * `rawpath` with the extension replaced by ".xmf".  Replaces
 * dump::Raw<M>::WriteWithXmf (src/dump/raw.ipp:204-226) on one block; the
 * files are those the reference writes. */
int aphgpu_dump_raw(aphgpu_ctx* ctx, int field, int type, const char* rawpath, const char* name);
/* Reads `field` from a raw file described by `xmfpath` (the binpath there,
 * or `rawpath` if not NULL): the whole array of the context's dimensions,
 * start 0 and stride 1, from byte `Seek`.  Replaces dump::Raw<M>::Read with
 * dump::Xmf::ReadXmf (src/dump/raw.ipp:257-363, src/dump/xmf.ipp:103-140)
 * for the sequential reader's case.  A volume fraction read back gets its
 * interface reconstructed (normals, plane constants) as at
 * aphgpu_vof_init; the context's step count (which orders the directional
 * sweeps, vof.ipp:428-435) is kept. */
int aphgpu_read_raw(aphgpu_ctx* ctx, int field, const char* xmfpath, const char* rawpath);
/* The XMF text aphgpu_dump_raw writes for an nx*ny*nz mesh of cell edge h
 * (host only; no GPU needed).  Copies at most cap-1 bytes and a NUL to out
 * (may be NULL) and the full length to *len (may be NULL). */
int aphgpu_xmf_text(int nx, int ny, int nz, double h, const char* name, const char* binpath,
                    int type, char* out, int cap, int* len);

#ifdef __cplusplus
}
#endif

#endif /* APHGPU_H_ */

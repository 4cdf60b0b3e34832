/*
 * CPU oracle: a plain-C restatement of aphros's projection-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by the parity tests, by `smoke()` as the
 * checker, and by the CPU-baseline legs of bench.py.
 *
 * Every function names the reference function (path:line inside the aphros
 * source tree) whose arithmetic it restates.  Floating-point expressions keep
 * the reference's association order so that, compiled without FMA
 * contraction (-ffp-contract=off), results agree with the reference bit for
 * bit wherever the reference itself is deterministic.
 *
 * Grid conventions (identical to the GPU library):
 *   - cells (i,j,k), 0<=i<nx etc., linear index i + nx*(j + ny*k) (x fastest,
 *     like geom/block.h:149-158 GIndex::GetIdx without halo cells);
 *   - periodic in all three directions (the configurations are periodic);
 *   - a face field for direction d stores, at the index of cell c, the value
 *     on the face between c-e_d and c (the "minus" face of c);
 *   - vector cell fields (normals, heights) are AoS, 3 doubles per cell,
 *     like FieldCell<Vect>.
 */
#ifndef APHROS_ORACLE_H_
#define APHROS_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- Poisson / projection ---------------- */

/* rho = rho1*(1-alpha) + rho2*alpha (kernel/hydro.ipp:1815-1822). */
void orc_mixture_density(
    int64_t ncells, const double* alpha, double rho1, double rho2, double* rho);

/* Harmonic face density (solver/approx_eb.h:351-363 InterpolateHarmonic via
 * solver/approx_eb.ipp:828-836 Interpolate). rho_f[d] has ncells entries. */
void orc_face_density(const int n[3], const double* rho, double* rho_f[3]);

/* Face force from surface tension (util/hydro.ipp:1289-1310
 * AppendSurfaceTension), added to ffst[d] (caller zeroes it). */
void orc_surface_tension(
    const int n[3], double h, const double* u, const double* kappa,
    double sigma, double* ffst[3]);

/* Face fluxes entering the projection, proj.ipp:556-562:
 *   v = vstar + febp/rho_f*dt*area   (febp may be NULL). */
void orc_face_flux_with_force(
    const int n[3], double h, double dt, double* const vstar[3],
    double* const febp[3], double* const rho_f[3], double* vout[3]);

/* Projection system assembly, proj.ipp:343-360 (GetFlux) and 367-383
 * (GetFluxSum), with GradientImplicit (approx_eb.ipp:1435-1468) and
 * AppendExpr (geom/mesh.h:575-579).
 *   expr8: 8 doubles per cell, e[0]*p[c] + sum_q e[1+q]*p[nb_q] + e[7] = 0,
 *          q = xm,xp,ym,yp,zm,zp.
 *   fk[d], fv[d]: face expression (k, -k, v) of proj.ipp:355-358, i.e.
 *          flux = k*p[cm] - k*p[cp] + v; may be NULL.
 *   src: volume source (NULL = 0). */
void orc_assemble_projection(
    const int n[3], double h, double dt, double* const rho_f[3],
    double* const vflux[3], const double* src, double* expr8, double* fk[3],
    double* fv[3]);

/* Removes the mean of e[7] over all cells (solver/pois.h:41-47). */
void orc_remove_rhs_mean(int64_t ncells, double* expr8);

typedef struct {
  double residual;
  int iter;
} orc_info;

/* Unpreconditioned CG, linear/linear.ipp:24-129 SolverConjugate::Imp::Solve.
 *   x0 may be NULL (zero guess) or equal to x.
 *   cellvol: m.GetCellSize().prod() used in the residual norm.
 *   maxnorm: 0 = L2 residual sqrt(sum r^2 / cellvol), 1 = max|r|/cellvol.
 *   res_hist: optional, receives the residual after every iteration
 *   (capacity maxiter+2).
 *   nthreads: OpenMP threads (<=0: library default). */
orc_info orc_cg_solve(
    const int n[3], double cellvol, const double* expr8, const double* x0,
    double* x, double tol, int miniter, int maxiter, int maxnorm,
    double* res_hist, int nthreads);

/* Runs exactly `iters` CG iterations (CPU baseline sampling), returns the
 * wall time in seconds. */
double orc_cg_time_iters(
    const int n[3], const double* expr8, double* x, int iters, int nthreads);

/* Residual r = -(A x + e7) (linear.ipp:42-58), returns sum r^2. */
double orc_residual(
    const int n[3], const double* expr8, const double* x, double* r);

/* Corrected face fluxes, proj.ipp:399-403 with UEmbed::Eval
 * (approx_eb.h:338-343): v = p[cm]*k + p[cp]*(-k) + v*. */
void orc_flux_correct(
    const int n[3], double* const fk[3], double* const fv[3], const double* p,
    double* vout[3]);

/* Cell acceleration, proj.ipp:408-433 GetAcceleration (no cell force, no
 * explicit viscosity): face (febp - grad p)/rho_f averaged to cells.
 * febp may be NULL. acc: AoS 3 per cell. */
void orc_acceleration(
    const int n[3], double h, const double* p, double* const rho_f[3],
    double* const febp[3], double* acc);

/* ---------------- PLIC geometry (solver/reconst.h) ---------------- */

double orc_solve_cubic(double a, double b, double c, double d, int k);
double orc_line_u(const double n[3], double a, const double h[3]);
double orc_line_a(const double n[3], double u, const double h[3]);
double orc_line_vol(
    const double n[3], double a, const double h[3], double dx, int d);
double orc_line_flux(
    const double n[3], double a, const double h[3], double q, double dt,
    int d);

/* ---------------- VOF ---------------- */

/* Interface normal of one cell (solver/normal.ipp:71-133 Youngs, then
 * 283-312 height update with force_overwrite=false), u3: 27 values of the
 * 3x3x3 neighbourhood, index (dx+1)+3*(dy+1)+9*(dz+1). */
void orc_normal_cell(const double u3[27], double nout[3]);

/* Vof::ReconstPlanes (solver/vof.ipp:70-90): mask = 0<u<1, normal
 * (UNormal::CalcNormal, normal.ipp:356-366) and plane constant
 * (Reconst::GetLineA) in interfacial cells, NaN elsewhere. */
void orc_vof_reconstruct(
    const int n[3], const double h[3], const double* u, uint8_t* mask,
    double* nrm, double* a);

/* One Weymouth sweep in direction d (solver/vof.ipp:212-327, type
 * weymouth, no embedded boundaries, no colour fields).
 *   ffv: mixture flux through the faces of direction d.
 *   u0: volume fraction at the start of the step (fcuu = u0<0.5?0:1). */
void orc_vof_sweep(
    const int n[3], const double h[3], double* u, const double* ffv, int d,
    const double* nrm, const double* a, const double* u0, double dt,
    double clipth);

/* Vof::MakeIteration (vof.ipp:498-583) for scheme weymouth and zero
 * source, preceded by the t=0 reconstruction of StartStep (vof.ipp:177-195)
 * when `reconstruct_first` is set.  u is updated in place; nrm, a, mask hold
 * the planes on entry (when reconstruct_first==0) and the planes of the
 * final field on exit (the state Vof keeps between steps).
 *   count: number of previous MakeIteration calls (selects split order). */
void orc_vof_step(
    const int n[3], const double h[3], double* u, double* const ffv[3],
    double dt, double clipth, int count, int reconstruct_first, uint8_t* mask,
    double* nrm, double* a);

/* orc_vof_step with a volume source src (per cell, NULL: none): the init
 * stage of Vof::MakeIteration (vof.ipp:504-514) first sets
 * u = u + dt * src * (1 - u) in every cell and takes fcuu from that field;
 * the first sweep then uses the planes reconstructed before the source
 * (cells that became interfacial through the source have none and carry
 * the plain flux v*u, as cells with an undefined normal do at
 * vof.ipp:233-255). */
void orc_vof_step_src(
    const int n[3], const double h[3], double* u, double* const ffv[3],
    const double* src, double dt, double clipth, int count,
    int reconstruct_first, uint8_t* mask, double* nrm, double* a);

/* ---------------- Curvature (height functions) ---------------- */

/* UHeight::Good(uu) (util/height.h:69-124) on a column of `si` values. */
double orc_height_good(const double* uu, int si);
/* UHeight::Good(uu, n) (util/height.h:19-62). */
double orc_height_good_n(const double* uu, int si, double nn);

/* Heights::CalcCurvature (solver/curv.ipp:358-414) for one layer without
 * colours: CalcDiff2/CalcDiff4/CalcHeight/CalcCurvHeight.
 *   nrm: normals of the PLIC state (AoS), kappa: output (NaN outside the
 *   interface), hgt: optional output heights (AoS, NaN where undefined). */
void orc_heights_curvature(
    const int n[3], const double h[3], const double* u, const double* nrm,
    double* kappa, double* hgt);

/* Parameters of the particle-string curvature (PartStr::Par and
 * PartStrMeshM::Par, src/solver/partstr.h:38-45, partstrmeshm.h:26-36):
 * particles per string (odd), strings per cell, string length in cells,
 * relaxation, tolerance, iterations at most, circular-segment factor,
 * normal displacement. */
typedef struct {
  int np, ns;
  double leq, relax, tol;
  int itermax;
  double segcirc;
  int dn;
} OrcPartPar;

/* The defaults of deploy/scripts/sim_base.conf (part_*). */
void orc_part_default(OrcPartPar* p);

/* curvature::Particles (src/solver/curv.ipp:29-54, partstrmeshm.ipp:266-395)
 * for one layer of a periodic domain of cubic cells h: strings seeded in the
 * interfacial cells (0 < u < 1) with a colour (cl NULL: no colours), lines
 * from the PLIC polygons (nrm AoS, pa) of the interfacial cells of the same
 * colour in the 5x5x5 stencil.  kappa: NaN where no string is seeded.
 * Returns 0, or -1 for parameters out of range. */
int orc_curv_particles(const int n[3], double h, const double* u, const double* nrm,
                       const double* pa, const double* cl, const OrcPartPar* p,
                       double* kappa, int nthreads);

/* Connected-component colours after a VOF step on one periodic block
 * (Vof::MakeIteration resetcolor + union-find recolor + propagate,
 * src/solver/vof.ipp:546-578): cl_prev the colours before, cl the result
 * (-1: no colour). */
void orc_recolor(const int n[3], const double* u, const double* cl_prev, double* cl);

/* BCG face predictor of a cell field, periodic, cubic cells of edge h
 * (UEmbed::InterpolateBcg, src/solver/approx_eb.ipp:753-821); face arrays
 * of direction d at the index of the plus cell. */
void orc_interpolate_bcg(const int n[3], double h, const double* u,
                         const double* const vflux[3], const double* src, double dt,
                         double* const out[3]);

/* One time step of the projection fluid solver Proj (src/solver/proj.ipp)
 * with the default ProjPar, periodic, no forces: state vel (3 blocks of N),
 * p, ppred and flux (3 face blocks) in/out; first at t = 0.  Returns the
 * total CG iterations.  orc_fluid_init: the initial fluxes of a velocity
 * (proj.ipp:62-67). */
void orc_fluid_init(const int n[3], double h, const double* vel, double* flux[3]);
int orc_fluid_step(const int n[3], double h, double dt, const double* rho, const double* mu,
                   double* vel, double* p, double* ppred, double* flux[3], int first,
                   double tol, int maxiter, int nthreads);

#ifdef __cplusplus
}
#endif

#endif

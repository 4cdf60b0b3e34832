// One time step of aphros's projection fluid solver on the device: Proj
// (src/solver/proj.ipp) with the default ProjPar -- BCG advection of the
// velocity, implicit diffusion, one iteration per step, periodic, no
// forces or sources -- with every field resident and the linear systems
// solved by the context's solvers.
//
//   StartStep (proj.ipp:309-322); on the first step CalcInitialPressure
//     (:111-127): face fluxes of the velocity, projected with dt.
//   MakeIteration (:455-603):
//     KAcceleration         cell acceleration of the pressure (:408-433)
//     KBcgFaces             BCG face predictor UEmbed::InterpolateBcg
//                           (approx_eb.ipp:753-821) of each velocity
//                           component with the time layer's fluxes; the
//                           predicted fluxes are its normal components
//     projection with dt/2  (:484-499, the predictor pressure)
//     KBcgFaces + KAdvect   BCG face values of each component with the
//                           predicted fluxes, flux sum, explicit update and
//                           acceleration (:128-190)
//     KDiffusionExpr        implicit-diffusion system of each component
//                           (:241-307, GradientImplicit with the correction
//                           term of approx_eb.ipp:1471-1480), solved from the
//                           advected velocity
//     KAddAcc, KFaceFlux    acceleration removed, face fluxes of the cell
//                           velocity (:524-560), projection with dt,
//                           acceleration added (:565-575)
//   FinishStep (:604-613): the iteration layer becomes the time layer.
//
// This translation unit is compiled without fused multiply-adds: every
// value outside the linear solves follows the reference's arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "stencil.cuh"

namespace aphgpu {
namespace {

__device__ __forceinline__ int64_t Nb(const Dims& d, int i, int j, int k, int dir, int s) {
  return dir == 0 ? d.idx(s < 0 ? wrapm(i - 1, d.nx) : wrapp(i + 1, d.nx), j, k)
       : dir == 1 ? d.idx(i, s < 0 ? wrapm(j - 1, d.ny) : wrapp(j + 1, d.ny), k)
                  : d.idx(i, j, s < 0 ? wrapm(k - 1, d.nz) : wrapp(k + 1, d.nz));
}

__device__ __forceinline__ void Ijk(const Dims& d, int64_t c, int& i, int& j, int& k) {
  i = (int)(c % d.nx);
  const int64_t r = c / d.nx;
  j = (int)(r % d.ny);
  k = (int)(r / d.ny);
}

// mixture rho1 (1 - a) + rho2 a (kernel/hydro.ipp:1815-1822)
__device__ __forceinline__ double Mix(double v1, double v2, double a) {
  return v1 * (1 - a) + v2 * a;
}

__global__ void KMixture(int64_t n, const double* __restrict__ a, double v1, double v2,
                         double* out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    out[c] = Mix(v1, v2, a[c]);
}

// Face fluxes of a cell velocity (3 blocks): face value (u[cp] + u[cm]) / 2
// (approx_eb.ipp:828-836) dotted with the face surface (proj.ipp:64-67),
// plus the balanced-force term 0 / rho_f * dt * area of proj.ipp:553-560.
__global__ void KFaceFlux(Dims d, double h, const double* __restrict__ vel,
                          const double* __restrict__ alpha, double rho1, double rho2,
                          double dt, int with_force, double* out) {
  const int64_t N = d.cells();
  const double area = h * h * h / h;  // the mesh's face area V / h
  TILE_LOOP_BEGIN(d)
  for (int dir = 0; dir < 3; ++dir) {
    const int64_t cm = Nb(d, i, j, k, dir, -1);
    // sum over the components: only the face-normal one has a nonzero
    // weight; 0 + x reproduces the sum with its zero terms
    const double v = (vel[dir * N + c] + vel[dir * N + cm]) * 0.5;
    double f = 0. + (v - 0.) * area;
    if (with_force) {
      const double rm = Mix(rho1, rho2, alpha[cm]), rp = Mix(rho1, rho2, alpha[c]);
      const double rf = 1 / ((1 / rp + 1 / rm) * 0.5);
      f += 0. / rf * dt * area;
    }
    out[dir * N + c] = f;
  }
  TILE_LOOP_END
}

// Gradient of u on the face of direction dir with index f (between f - e_dir
// and f): (u[f] - u[f - e_dir]) / h (UEmbed::Gradient, approx_eb.ipp:882-890)
__device__ __forceinline__ double FaceGrad(const Dims& d, const double* u, int64_t f, int dir,
                                           double h) {
  int i, j, k;
  Ijk(d, f, i, j, k);
  return (u[f] - u[Nb(d, i, j, k, dir, -1)]) / h;
}

// BCG face values of u (UEmbed::InterpolateBcg, approx_eb.ipp:753-821,
// periodic): faces of the directions in dirmask (bit d) of every cell (the
// face between c - e_d and c); src: cell source, stride `ss` (the
// acceleration component of an AoS field).
__global__ void KBcgFaces(Dims d, double h, double dt, const double* __restrict__ u,
                          const double* __restrict__ vflux, const double* __restrict__ src,
                          int ss, int dirmask, double* out, int64_t out_stride) {
  const int64_t N = d.cells();
  const double area = h * h;
  TILE_LOOP_BEGIN(d)
  const int64_t cp = c;
  for (int d0 = 0; d0 < 3; ++d0) {
    if (!((dirmask >> d0) & 1)) continue;
    const int64_t cm = Nb(d, i, j, k, d0, -1);
    const double v = vflux[d0 * N + cp];
    const double sgn = v > 0 ? 1 : -1;
    const int64_t cu = sgn > 0 ? cm : cp;  // upwind cell
    int iu, ju, ku;
    Ijk(d, cu, iu, ju, ku);
    double ut = (src[ss * cm] + src[ss * cp]) * 0.5;
    double ux = 0;
    int dd = d0;
    {
      const int64_t fm = cu, fp = Nb(d, iu, ju, ku, dd, 1);
      ux += (FaceGrad(d, u, fm, dd, h) + FaceGrad(d, u, fp, dd, h)) * 0.5;
      const double vel = v / area;
      ut -= ux * vel;
    }
    for (int t = 0; t < 2; ++t) {
      dd = (dd + 1) % 3;
      const int64_t fm = cu, fp = Nb(d, iu, ju, ku, dd, 1);
      const double vel = (vflux[dd * N + fm] + vflux[dd * N + fp]) / (area + area);
      ut -= FaceGrad(d, u, vel > 0 ? fm : fp, dd, h) * vel;
    }
    out[d0 * out_stride + cp] = u[cu] + ux * (sgn * 0.5 * h) + ut * (0.5 * dt);
  }
  TILE_LOOP_END
}

// Predicted fluxes from the BCG face values of component `dir` on the faces
// of direction `dir` (proj.ipp:490-495: the face velocity dotted with the
// surface, 0 + x as in KFaceFlux)
__global__ void KPredictedFlux(int64_t n, double area, const double* __restrict__ comp,
                               double* out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    out[c] = 0. + (comp[c] - 0.) * area;
}

// Advection of component `dir` (proj.ipp:128-190): flux sum of -ffu * ffv
// over the six faces, explicit update from the time layer, then the
// acceleration times dt (proj.ipp:517-522).
__global__ void KAdvect(Dims d, double dt, double vol, const double* __restrict__ u,
                        const double* __restrict__ ffu, const double* __restrict__ ffv,
                        const double* __restrict__ acc, int dir, double* vi) {
  const int64_t N = d.cells();
  TILE_LOOP_BEGIN(d)
  double sum = 0;
  for (int q = 0; q < 6; ++q) {
    const int dd = q / 2;
    const int64_t f = (q % 2 == 0) ? c : Nb(d, i, j, k, dd, 1);
    const double fl = -ffu[dd * N + f] * ffv[dd * N + f];
    sum += fl * (double)(-1 + (q % 2) * 2);
  }
  double v = u[c] + sum * dt / vol;
  v += acc[3 * c + dir] * dt;
  vi[c] = v;
  TILE_LOOP_END
}

// Implicit-diffusion system of one velocity component (proj.ipp:241-307):
// the flux of mu grad(u) on each face from GradientImplicit with the
// correction term at the guess g (approx_eb.ipp:1471-1480), summed with
// the outward factors (AppendExpr order), negated, plus the time term
// rho V (u - u_old) / dt; 8 coefficients per cell.
__global__ void KDiffusionExpr(Dims d, double h, double dt, const double* __restrict__ g,
                               const double* __restrict__ uold,
                               const double* __restrict__ mu,
                               const double* __restrict__ alpha, double rho1, double rho2,
                               double* e8) {
  const double vol = h * h * h;
  const double area = vol / h;  // the mesh's face area
  const double a = 1 / h;
  TILE_LOOP_BEGIN(d)
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int q = 0; q < 6; ++q) {
    const int dd = q / 2;
    const int64_t f = (q % 2 == 0) ? c : Nb(d, i, j, k, dd, 1);
    const int64_t fcm = (q % 2 == 0) ? Nb(d, i, j, k, dd, -1) : c;
    const int64_t fcp = f;
    int fi, fj, fk;
    Ijk(d, f, fi, fj, fk);
    const int64_t fm = Nb(d, fi, fj, fk, dd, -1);  // minus cell of face f
    const double muf = (mu[f] + mu[fm]) * 0.5;
    double fe[3] = {-a, a, 0};
    const double grad = (g[fcp] - g[fcm]) / h;
    const double ev = g[fcm] * fe[0] + g[fcp] * fe[1] + fe[2];
    fe[2] += grad - ev;
    const double o = (double)(-1 + (q % 2) * 2);
    double v[3];
    for (int t = 0; t < 3; ++t) v[t] = fe[t] * muf * area * o;
    s[0] += v[1 - q % 2];
    s[1 + q] += v[q % 2];
    s[7] += v[2];
  }
  double* ec = e8 + 8 * c;
  const double rho = Mix(rho1, rho2, alpha[c]);
  double td[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  td[0] = 1 / dt;
  td[7] = -uold[c] / dt;
  for (int t = 0; t < 8; ++t) ec[t] = -s[t] + td[t] * vol * rho;
  TILE_LOOP_END
}

// vi (3 blocks) += sign * acc (AoS) * dt
__global__ void KAddAcc(int64_t n, const double* __restrict__ acc, double dt, int sign,
                        double* vi) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    for (int e = 0; e < 3; ++e) {
      if (sign > 0)
        vi[e * n + c] += acc[3 * c + e] * dt;
      else
        vi[e * n + c] -= acc[3 * c + e] * dt;
    }
  }
}

int Copy(aphgpu_ctx* ctx, double* dst, const double* src, int64_t count) {
  APH_CUDA(ctx, cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToDevice,
                                ctx->stream));
  return APHGPU_OK;
}

// Proj::Project (proj.ipp:384-407): the projection system of the fluxes
// ffv with time step dt (no mean removal), solved from the guess in p, the
// corrected fluxes written back to ffv.
int Project(aphgpu_ctx* ctx, double* p, double* ffv, double dt, const aphgpu_conf* conf,
            int* iters) {
  auto& F = ctx->fluid;
  APH_TRY(AssembleProjectionDevice(ctx, ctx->alpha_proj, F.rho1, F.rho2, ffv, nullptr, dt, 0));
  APH_TRY(Copy(ctx, ctx->x, p, ctx->N));
  aphgpu_info info{};
  APH_TRY(aphgpu_solve_resident(ctx, conf, 0, &info));
  if (!info.converged) F.unconverged += 1;
  *iters += info.iter;
  APH_TRY(Copy(ctx, p, ctx->x, ctx->N));
  return FluxCorrect(ctx, ffv);
}

}  // namespace

int FluidStepDevice(aphgpu_ctx* ctx, double dt, const aphgpu_conf* conf_in, aphgpu_info* info,
                    double* d_res) {
  auto& F = ctx->fluid;
  const Dims d = ctx->d;
  const int64_t N = ctx->N;
  const double h = ctx->h;
  const double vol = h * h * h;
  const double area = vol / h;  // the mesh's face area
  cudaStream_t st = ctx->stream;
  const dim3 tg = TileGrid(d), tb = TileBlock();
  const int fb = FlatBlocks(N);
  aphgpu_conf conf = *conf_in;
  conf.miniter = 0;  // hypre_symm_miniter 0 of the fluid configuration
  conf.rtol = 0;
  int iters = 0;
  F.unconverged = 0;
  if (F.follow_vof) APH_TRY(Copy(ctx, ctx->alpha_proj, ctx->u, N));
  APH_TRY(Copy(ctx, F.vi, F.vel, 3 * N));
  APH_TRY(Copy(ctx, F.ffv, F.flux, 3 * N));
  if (F.steps == 0) {
    // CalcInitialPressure: fluxes of the cell velocity projected with dt
    KFaceFlux<<<tg, tb, 0, st>>>(d, h, F.vi, ctx->alpha_proj, F.rho1, F.rho2, dt, 1, F.ffv);
    APH_LAUNCHED(ctx);
    APH_TRY(Project(ctx, F.p, F.ffv, dt, &conf, &iters));
  }
  APH_TRY(Acceleration(ctx, F.acc, ctx->alpha_proj, F.rho1, F.rho2));
  // predicted fluxes: the BCG face value of component e on the faces of
  // direction e, with the time layer's fluxes
  for (int e = 0; e < 3; ++e) {
    KBcgFaces<<<tg, tb, 0, st>>>(d, h, dt, F.vel + e * N, F.flux, F.acc + e, 3, 1 << e,
                                 F.ffu, N);
    APH_LAUNCHED(ctx);
    KPredictedFlux<<<fb, kFlatThreads, 0, st>>>(N, area, F.ffu + e * N, F.ffv + e * N);
    APH_LAUNCHED(ctx);
  }
  APH_TRY(Project(ctx, F.ppred, F.ffv, dt * 0.5, &conf, &iters));
  // advection of each component with the predicted fluxes
  for (int e = 0; e < 3; ++e) {
    KBcgFaces<<<tg, tb, 0, st>>>(d, h, dt, F.vel + e * N, F.ffv, F.acc + e, 3, 7, F.ffu, N);
    APH_LAUNCHED(ctx);
    KAdvect<<<tg, tb, 0, st>>>(d, dt, vol, F.vel + e * N, F.ffu, F.ffv, F.acc, e,
                               F.vi + e * N);
    APH_LAUNCHED(ctx);
  }
  // implicit diffusion of each component from the advected velocity
  APH_TRY(Copy(ctx, F.guess, F.vi, 3 * N));
  for (int e = 0; e < 3; ++e) {
    KDiffusionExpr<<<tg, tb, 0, st>>>(d, h, dt, F.guess + e * N, F.vi + e * N, F.mu,
                                      ctx->alpha_proj, F.rho1, F.rho2, F.e8);
    APH_LAUNCHED(ctx);
    APH_TRY(SetSystemExprDevice(ctx, F.e8));
    APH_TRY(Copy(ctx, ctx->x, F.guess + e * N, N));
    aphgpu_info di{};
    APH_TRY(aphgpu_solve_resident(ctx, &conf, 0, &di));
    if (!di.converged) F.unconverged += 1;
    iters += di.iter;
    APH_TRY(Copy(ctx, F.vi + e * N, ctx->x, N));
  }
  // acceleration removed, face fluxes of the cell velocity, projection,
  // acceleration of the new pressure added
  KAddAcc<<<fb, kFlatThreads, 0, st>>>(N, F.acc, dt, -1, F.vi);
  APH_LAUNCHED(ctx);
  KFaceFlux<<<tg, tb, 0, st>>>(d, h, F.vi, ctx->alpha_proj, F.rho1, F.rho2, dt, 1, F.ffv);
  APH_LAUNCHED(ctx);
  APH_TRY(Project(ctx, F.p, F.ffv, dt, &conf, &iters));
  APH_TRY(Acceleration(ctx, F.acc, ctx->alpha_proj, F.rho1, F.rho2));
  KAddAcc<<<fb, kFlatThreads, 0, st>>>(N, F.acc, dt, 1, F.vi);
  APH_LAUNCHED(ctx);
  // FinishStep; the corrected fluxes are also the advection fluxes of the
  // next aphgpu_vof_step(ctx, NULL, dt)
  APH_TRY(Copy(ctx, F.vel, F.vi, 3 * N));
  APH_TRY(Copy(ctx, F.flux, F.ffv, 3 * N));
  APH_TRY(Copy(ctx, d_res, F.ffv, 3 * N));
  ctx->has_vflux_res = true;
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  F.steps += 1;
  info->iter = iters;
  info->inner_iter = 0;
  info->residual = 0;
  info->converged = F.unconverged == 0;
  return APHGPU_OK;
}

int FluidInitDevice(aphgpu_ctx* ctx, double rho1, double rho2, double mu1, double mu2) {
  auto& F = ctx->fluid;
  const int64_t N = ctx->N;
  F.rho1 = rho1;
  F.rho2 = rho2;
  KMixture<<<FlatBlocks(N), kFlatThreads, 0, ctx->stream>>>(N, ctx->alpha_proj, mu1, mu2,
                                                            F.mu);
  APH_LAUNCHED(ctx);
  // the time layer's fluxes: face fluxes of the initial velocity
  // (Proj's constructor, proj.ipp:96-101)
  KFaceFlux<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(
      ctx->d, ctx->h, F.vel, ctx->alpha_proj, rho1, rho2, 0., 0, F.flux);
  APH_LAUNCHED(ctx);
  APH_CUDA(ctx, cudaMemsetAsync(F.p, 0, sizeof(double) * N, ctx->stream));
  APH_CUDA(ctx, cudaMemsetAsync(F.ppred, 0, sizeof(double) * N, ctx->stream));
  F.steps = 0;
  return APHGPU_OK;
}

int BcgFacesDevice(aphgpu_ctx* ctx, const double* u, const double* vflux, const double* src,
                   double dt, double* out) {
  KBcgFaces<<<TileGrid(ctx->d), TileBlock(), 0, ctx->stream>>>(ctx->d, ctx->h, dt, u, vflux,
                                                               src, 1, 7, out, ctx->N);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

}  // namespace aphgpu

// Harness that runs aphros's OWN hot-path code (compiled from the reference
// sources by oracle/ref/Makefile) on inputs read from raw binary files, to
// pin the C oracle and to make golden fixtures.  Test infrastructure only.
//
// Modes (all arrays raw little-endian float64, cells x-fastest, periodic;
// face arrays hold, for each direction d, the value on the face between
// cell c-e_d and cell c at the index of c):
//
// n and bs are "N" or "NX,NY,NZ"; the domain extent (longest side) is 1.
//
//   proj  n bs h dt rho1 rho2 tol maxiter alpha.bin vflux.bin out
//     rho = CalcMixture formula (kernel/hydro.ipp:1818-1821),
//     rho_f = UEmbed::InterpolateHarmonic, system = Proj::GetFlux +
//     Proj::GetFluxSum (solver/proj.ipp:343-383) with the RHS mean removed,
//     solve with linear::SolverConjugate ("conjugate" module), fluxes by
//     UEmbed::Eval (proj.ipp:399-403).
//     Writes out.expr (8N), out.p (N), out.flux (3N), out.info (text).
//   cgtime n bs dt rho1 rho2 iters alpha.bin vflux.bin out
//     the system of `proj`, then linear::SolverConjugate for exactly
//     `iters` iterations (tolerance 0, miniter = maxiter = iters) on all
//     OpenMP threads; writes out.time (text: wall-clock seconds from the
//     end of the assembly to the end of the solve, and the iterations).
//     Nothing else is written (the timing mode of the CPU baseline).
//   vof   n bs h dt steps u.bin vflux.bin out
//     Vof (scheme weymouth) StartStep/MakeIteration/FinishStep/PostStep and
//     curvature::Heights::CalcCurvature per step, as in
//     test/advection/main.cpp:242-256.  Writes out.u, out.n (3N AoS),
//     out.a, out.k, out.cl (Vof::GetColor, the connected-component colours
//     of the default union-find recolouring; after the last step) and
//     out.sumu (text, per step).  With REF_VOF_SRC=path set, the volume
//     source field of the Vof (raw, N values) is read from that file.
//     REF_CURV=particles or hybrid replaces the estimator of out.k by
//     curvature::Particles or curvature::Hybrid (part_* defaults of
//     deploy/scripts/sim_base.conf).
//   overlap in out         rows (x y z hx hy hz cx cy cz r) -> GetSphereOverlap
//   reconst in out         rows (n0 n1 n2 u a h0 h1 h2 q dt d) ->
//                          GetLineA(n,u,h) GetLineU(n,a,h) GetLineFlux(...)
//   height  in out         rows (column, optional n=N) -> UHeight::Good
//   bcg   n bs dt u.bin vflux.bin src.bin out
//     UEmbed::InterpolateBcg (solver/approx_eb.ipp:753-821), periodic (no
//     boundary conditions): the cell field u advected to the faces by dt/2
//     with the face fluxes and the cell source src.  Writes out.ffu (3N).
//   fluid n bs dt steps rho1 rho2 mu1 mu2 tol maxiter alpha.bin vel.bin out
//     Proj (solver/proj.ipp, default ProjPar: BCG, implicit diffusion,
//     conjugate solver "symm") for `steps` time steps of one iteration each
//     (StartStep, MakeIteration, FinishStep) on a periodic mesh, density and
//     dynamic viscosity the mixtures rho1 (1 - alpha) + rho2 alpha and
//     mu1 (1 - alpha) + mu2 alpha, initial cell velocity vel (3 blocks of N),
//     no forces.  Writes out.vel (3 blocks), out.p, out.flux (3N).
//   xmf   n h name binpath type out.xmf
//     dump::Xmf::WriteXmf of the metadata that dump::Raw::WriteWithXmf
//     writes for a field of an n-cell mesh with cell size h (dump/raw.ipp:
//     204-226); type is Double, Float or UShort.
//   raw   n type in.f64 out.raw
//     dump::Raw::WriteBlocks of one block covering the mesh (the
//     sequential writer, dump/raw.ipp:73-158), values converted to type.
#include <omp.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "distr/distrbasic.h"
#include "dump/raw.h"
#include "dump/xmf.h"
#include "linear/linear.h"
#include "overlap/overlap.h"
#include "parse/vof.h"
#include "solver/approx_eb.h"
#include "solver/proj.h"
#include "solver/curv.h"
#include "solver/reconst.h"
#include "solver/vof.h"
#include "util/distr.h"
#include "util/height.h"

using M = MeshCartesian<double, 3>;
using Scal = typename M::Scal;
using Vect = typename M::Vect;
using MIdx = typename M::MIdx;
using Expr = typename M::Expr;
using ExprFace = typename M::ExprFace;
using UEB = UEmbed<M>;

namespace {

std::vector<double> ReadRaw(const std::string& path, size_t count) {
  std::vector<double> v(count);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::cerr << "cannot open " << path << std::endl;
    std::exit(2);
  }
  const size_t got = std::fread(v.data(), sizeof(double), count, f);
  std::fclose(f);
  if (got != count) {
    std::cerr << "short read " << path << std::endl;
    std::exit(2);
  }
  return v;
}

void WriteRaw(const std::string& path, const std::vector<double>& v) {
  FILE* f = std::fopen(path.c_str(), "wb");
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

struct Global {
  bool time_only = false;  // cgtime mode: no field outputs
  double t_solve0 = 0, t_solve1 = 0;
  int n = 0; // unused when nx,ny,nz set
  int nn[3] = {0, 0, 0};
  Scal dt = 0, rho1 = 1, rho2 = 1;
  int steps = 0;
  std::vector<double> alpha, vflux, u;
  std::vector<double> out_expr, out_p, out_flux, out_u, out_n, out_a, out_k, out_cl;
  std::vector<double> sumu;
  std::string out;
  Scal residual = 0;
  int iter = 0;
};
Global g;

size_t Wrap(int i, int n) {
  return size_t(((i % n) + n) % n);
}
size_t GIdx(const MIdx& w) {
  return Wrap(w[0], g.nn[0]) +
         size_t(g.nn[0]) *
             (Wrap(w[1], g.nn[1]) + size_t(g.nn[1]) * Wrap(w[2], g.nn[2]));
}
size_t NCells() {
  return size_t(g.nn[0]) * g.nn[1] * g.nn[2];
}
// parses "n" or "nx,ny,nz"
MIdx ParseSize(const char* s) {
  int a = 0, b = 0, c = 0;
  if (std::sscanf(s, "%d,%d,%d", &a, &b, &c) == 3) return MIdx(a, b, c);
  a = std::atoi(s);
  return MIdx(a, a, a);
}

// face value from the global face arrays: direction d, face of cell cp
template <class MM>
Scal FaceInput(const MM& m, IdxFace f, const std::vector<double>& arr) {
  const auto p = m.GetIndexFaces().GetMIdxDir(f);
  return arr[p.second.raw() * NCells() + GIdx(p.first)];
}

void RunProj(M& m, Vars& var) {
  auto sem = m.GetSem(__func__);
  struct {
    FieldCell<Scal> fcrho;
    FieldFace<Scal> ffdens;
    FieldFace<Scal> ffv;
    FieldFace<ExprFace> ffe;
    FieldCell<Expr> fcs;
    FieldCell<Scal> fcp;
    Scal sum7;
    Scal cnt;
    std::unique_ptr<linear::Solver<M>> solver;
    typename linear::Solver<M>::Info info;
  } * ctx(sem);
  auto& t = *ctx;
  if (sem("init")) {
    t.fcrho.Reinit(m);
    for (auto c : m.AllCells()) {
      const Scal a2 = g.alpha[GIdx(m.GetIndexCells().GetMIdx(c))];
      const Scal a1 = 1 - a2;
      t.fcrho[c] = g.rho1 * a1 + g.rho2 * a2;
    }
    t.ffdens = UEB::InterpolateHarmonic(t.fcrho, MapEmbed<BCond<Scal>>(), m);
    t.ffv.Reinit(m);
    for (auto f : m.AllFaces()) {
      t.ffv[f] = FaceInput(m, f, g.vflux);
    }
    // Proj::GetFlux (proj.ipp:343-360), periodic: no boundary conditions
    t.ffe = UEB::GradientImplicit(MapEmbed<BCond<Scal>>(), m);
    for (auto f : m.Faces()) {
      t.ffe[f] *= -m.GetArea(f) / t.ffdens[f] * g.dt;
      t.ffe[f][2] += t.ffv[f];
    }
    // Proj::GetFluxSum (proj.ipp:367-383), zero source
    t.fcs.Reinit(m, Expr::GetUnit(0));
    for (auto c : m.Cells()) {
      Expr sum(0);
      m.LoopNci(c, [&](auto q) {
        const auto cf = m.GetFace(c, q);
        const ExprFace v = t.ffe[cf] * m.GetOutwardFactor(c, q);
        m.AppendExpr(sum, v, q);
      });
      t.fcs[c] = sum;
    }
    t.sum7 = 0;
    t.cnt = 0;
    for (auto c : m.Cells()) {
      t.sum7 += t.fcs[c].back();
      t.cnt += 1;
    }
    m.Reduce(&t.sum7, Reduction::sum);
    m.Reduce(&t.cnt, Reduction::sum);
  }
  if (sem("mean")) {
    const Scal mean = t.sum7 / t.cnt;
    for (auto c : m.Cells()) {
      t.fcs[c].back() -= mean;
      if (g.time_only) continue;
      const size_t i = GIdx(m.GetIndexCells().GetMIdx(c));
      for (size_t q = 0; q < 8; ++q) {
        g.out_expr[8 * i + q] = t.fcs[c][q];
      }
    }
    t.fcp.Reinit(m, 0);
    auto factory = linear::ModuleLinear<M>::GetInstance("conjugate");
    fassert(factory, "conjugate solver not found");
    t.solver = factory->Make(var, "symm", m);
  }
  if (sem("clock0")) {
    if (m.IsRoot()) g.t_solve0 = omp_get_wtime();
  }
  if (sem.Nested("solve")) {
    t.info = t.solver->Solve(t.fcs, nullptr, t.fcp, m);
  }
  if (sem("clock1")) {
    if (m.IsRoot()) g.t_solve1 = omp_get_wtime();
  }
  if (g.time_only && sem("info")) {
    if (m.IsRoot()) {
      g.residual = t.info.residual;
      g.iter = t.info.iter;
    }
  }
  if (!g.time_only && sem("fluxes")) {
    for (auto c : m.Cells()) {
      g.out_p[GIdx(m.GetIndexCells().GetMIdx(c))] = t.fcp[c];
    }
    for (auto f : m.Faces()) {
      const auto p = m.GetIndexFaces().GetMIdxDir(f);
      const MIdx w = p.first;
      bool inner = true;
      for (int d = 0; d < 3; ++d) {
        if (w[d] < 0 || w[d] >= g.nn[d]) inner = false;
      }
      if (!inner) continue;
      g.out_flux[p.second.raw() * NCells() + GIdx(w)] =
          UEB::Eval(t.ffe[f], f, t.fcp, m);
    }
    if (m.IsRoot()) {
      g.residual = t.info.residual;
      g.iter = t.info.iter;
    }
  }
  if (sem()) {
  }
}

void RunBcg(M& m, Vars&) {
  auto sem = m.GetSem(__func__);
  if (sem("bcg")) {
    FieldCell<Scal> fcu(m), fcs(m);
    for (auto c : m.AllCells()) {
      const size_t i = GIdx(m.GetIndexCells().GetMIdx(c));
      fcu[c] = g.u[i];
      fcs[c] = g.alpha[i];
    }
    FieldFace<Scal> ffv(m, 0);
    for (auto f : m.AllFaces()) {
      ffv[f] = FaceInput(m, f, g.vflux);
    }
    const FieldFace<Scal> ffu =
        UEB::InterpolateBcg(fcu, MapEmbed<BCond<Scal>>(), ffv, fcs, g.dt, m);
    for (auto f : m.Faces()) {
      const auto p = m.GetIndexFaces().GetMIdxDir(f);
      const MIdx w = p.first;
      bool inner = true;
      for (int d = 0; d < 3; ++d) {
        if (w[d] < 0 || w[d] >= g.nn[d]) inner = false;
      }
      if (!inner) continue;
      g.out_flux[p.second.raw() * NCells() + GIdx(w)] = ffu[f];
    }
  }
  if (sem()) {
  }
}

struct FluidIn {
  Scal mu1 = 0, mu2 = 0;
  std::vector<double> vel;
} gf;

void RunFluid(M& m, Vars& var) {
  auto sem = m.GetSem(__func__);
  struct {
    FieldCell<Scal> fcr, fcd, fcsv, fcsm;
    FieldCell<Vect> fcf, fcvel;
    FieldEmbed<Scal> ffbp;
    MapEmbed<BCondFluid<Vect>> mebc;
    MapCell<std::shared_ptr<CondCellFluid>> mcc;
    std::unique_ptr<Proj<M>> fs;
    int step = 0;
  } * ctx(sem);
  auto& t = *ctx;
  if (sem("init")) {
    t.fcr.Reinit(m);
    t.fcd.Reinit(m);
    t.fcvel.Reinit(m);
    const size_t N = NCells();
    for (auto c : m.AllCells()) {
      const size_t i = GIdx(m.GetIndexCells().GetMIdx(c));
      const Scal a = g.alpha[i];
      t.fcr[c] = g.rho1 * (1 - a) + g.rho2 * a;
      t.fcd[c] = gf.mu1 * (1 - a) + gf.mu2 * a;
      t.fcvel[c] = Vect(gf.vel[i], gf.vel[N + i], gf.vel[2 * N + i]);
    }
    t.fcsv.Reinit(m, 0);
    t.fcsm.Reinit(m, 0);
    t.fcf.Reinit(m, Vect(0));
    t.ffbp = FieldEmbed<Scal>(m, 0);
    auto factory = linear::ModuleLinear<M>::GetInstance("conjugate");
    fassert(factory, "conjugate solver not found");
    std::shared_ptr<linear::Solver<M>> solver = factory->Make(var, "symm", m);
    ProjArgs<M> args{t.fcvel, t.mebc, t.mcc, &t.fcr, &t.fcd, &t.fcf, &t.ffbp,
                     &t.fcsv, &t.fcsm, 0., g.dt, solver, ProjPar<Vect>()};
    t.fs.reset(new Proj<M>(m, m, args));
  }
  sem.LoopBegin();
  if (sem("check")) {
    if (t.step >= g.steps) {
      sem.LoopBreak();
    }
  }
  if (sem.Nested("start")) {
    t.fs->StartStep();
  }
  if (sem.Nested("iter")) {
    t.fs->MakeIteration();
  }
  if (sem.Nested("finish")) {
    t.fs->FinishStep();
  }
  if (sem("inc")) {
    ++t.step;
  }
  sem.LoopEnd();
  if (sem("out")) {
    const size_t N = NCells();
    auto& vel = t.fs->GetVelocity();
    auto& p = t.fs->GetPressure();
    auto& ff = t.fs->GetVolumeFlux();
    for (auto c : m.Cells()) {
      const size_t i = GIdx(m.GetIndexCells().GetMIdx(c));
      for (int d = 0; d < 3; ++d) g.out_u[d * N + i] = vel[c][d];
      g.out_p[i] = p[c];
    }
    for (auto f : m.Faces()) {
      const auto q = m.GetIndexFaces().GetMIdxDir(f);
      const MIdx w = q.first;
      bool inner = true;
      for (int d = 0; d < 3; ++d) {
        if (w[d] < 0 || w[d] >= g.nn[d]) inner = false;
      }
      if (!inner) continue;
      g.out_flux[q.second.raw() * N + GIdx(w)] = ff[f];
    }
  }
  if (sem()) {
  }
}

void RunVof(M& m, Vars& var) {
  auto sem = m.GetSem(__func__);
  struct {
    FieldCell<Scal> fcu;
    FieldEmbed<Scal> ffv;
    FieldCell<Scal> fcsrc;
    MapEmbed<BCondAdvection<Scal>> bc; // empty: periodic (Vof keeps a reference)
    std::unique_ptr<Vof<M>> as;
    Multi<FieldCell<Scal>> fck;
    std::unique_ptr<curvature::Estimator<M>> curv;
    GRange<size_t> layers;
    int step = 0;
    Scal sumu;
  } * ctx(sem);
  auto& t = *ctx;
  if (sem("init")) {
    t.fcu.Reinit(m);
    for (auto c : m.AllCells()) {
      t.fcu[c] = g.u[GIdx(m.GetIndexCells().GetMIdx(c))];
    }
    t.ffv.Reinit(m, 0);
    for (auto f : m.AllFaces()) {
      t.ffv[f] = FaceInput(m, f, g.vflux);
    }
    t.fcsrc.Reinit(m, 0.);
    if (const char* srcpath = std::getenv("REF_VOF_SRC")) {
      // volume source of Vof::MakeIteration's init stage (vof.ipp:510-513)
      const std::vector<double> src = ReadRaw(srcpath, NCells());
      for (auto c : m.AllCells()) {
        t.fcsrc[c] = src[GIdx(m.GetIndexCells().GetMIdx(c))];
      }
    }
    VofPar<M> par; // defaults: weymouth, clipth 1e-10, dim 3 (solver/vof.h:13-53)
    (void)var;
    const FieldCell<Scal> fccl(m, 0);
    t.as.reset(new Vof<M>(
        m, m, t.fcu, fccl, t.bc, &t.ffv, &t.fcsrc,
        0., g.dt, par));
    t.layers = GRange<size_t>(1);
    t.fck.resize(t.layers);
    t.fck.InitAll(FieldCell<Scal>(m, GetNan<Scal>()));
    // REF_CURV=particles or hybrid selects the particle-string estimator
    // (curv.ipp:604-622) with the part_* defaults of sim_base.conf
    const char* est = std::getenv("REF_CURV");
    const std::string name = est ? est : "heights";
    if (name == "particles" || name == "hybrid") {
      typename PartStrMeshM<M>::Par pp;
      pp.ps.leq = 4;
      pp.ps.relax = 0.5;
      pp.ps.npmax = 7;
      pp.ps.segcirc = 0;
      pp.ps.dn = false;
      pp.ns = 3;
      pp.tol = 1e-5;
      pp.itermax = 20;
      pp.dim = 3;
      if (name == "particles") {
        t.curv = std::make_unique<curvature::Particles<M>>(m, pp, t.layers);
      } else {
        t.curv = std::make_unique<curvature::Hybrid<M>>(m, pp, t.layers);
      }
    } else {
      t.curv = std::make_unique<curvature::Heights<M>>();
    }
  }
  sem.LoopBegin();
  if (sem("empty")) {
    // an empty first stage in the loop, as test/advection/main.cpp:218-220
  }
  if (sem("check")) {
    if (t.step >= g.steps) {
      sem.LoopBreak();
    }
  }
  if (sem.Nested("start")) {
    t.as->StartStep();
  }
  if (sem.Nested("iter")) {
    t.as->MakeIteration();
  }
  if (sem.Nested("finish")) {
    t.as->FinishStep();
  }
  if (sem.Nested("post")) {
    t.as->PostStep();
  }
  if (sem.Nested("curv")) {
    t.curv->CalcCurvature(t.fck, t.as->GetPlic(), m, m);
  }
  if (sem("stat")) {
    t.sumu = 0;
    auto& u = t.as->GetField();
    for (auto c : m.Cells()) {
      t.sumu += u[c] * m.GetVolume(c);
    }
    m.Reduce(&t.sumu, Reduction::sum);
  }
  if (sem("stat2")) {
    if (m.IsRoot()) {
      g.sumu.push_back(t.sumu);
    }
    ++t.step;
  }
  sem.LoopEnd();
  if (sem("out")) {
    auto& u = t.as->GetField();
    auto& a = t.as->GetAlpha();
    auto& nn = t.as->GetNormal();
    auto& cl = t.as->GetColor();
    for (auto c : m.Cells()) {
      const size_t i = GIdx(m.GetIndexCells().GetMIdx(c));
      g.out_u[i] = u[c];
      g.out_cl[i] = cl[c];
      g.out_a[i] = a[c];
      g.out_k[i] = t.fck[0][c];
      for (int d = 0; d < 3; ++d) {
        g.out_n[3 * i + d] = nn[c][d];
      }
    }
  }
  if (sem()) {
  }
}

std::string MeshConf(MIdx n, MIdx bs) {
  Subdomains<MIdx> sub(n, bs, 1);
  std::string conf = sub.GetConfig();
  conf += "\nset string backend local";
  conf += "\nset double extent " + std::to_string(1.0);
  return conf;
}

int Main(int argc, const char** argv) {
  if (argc < 2) {
    std::cerr << "usage: ref_harness MODE ..." << std::endl;
    return 1;
  }
  const std::string mode = argv[1];
  if (mode == "proj") {
    if (argc != 13) return 1;
    const MIdx nsz = ParseSize(argv[2]);
    for (int d = 0; d < 3; ++d) g.nn[d] = nsz[d];
    const MIdx bs = ParseSize(argv[3]);
    const double h = std::atof(argv[4]);
    (void)h;
    g.dt = std::atof(argv[5]);
    g.rho1 = std::atof(argv[6]);
    g.rho2 = std::atof(argv[7]);
    const std::string tol = argv[8];
    const std::string maxiter = argv[9];
    g.alpha = ReadRaw(argv[10], NCells());
    g.vflux = ReadRaw(argv[11], 3 * NCells());
    g.out = argv[12];
    g.out_expr.assign(8 * NCells(), 0);
    g.out_p.assign(NCells(), 0);
    g.out_flux.assign(3 * NCells(), 0);
    std::string conf = MeshConf(nsz, bs);
    conf += "\nset double hypre_symm_tol " + tol;
    conf += "\nset int hypre_symm_maxiter " + maxiter;
    conf += "\nset int linsolver_symm_maxnorm 0";
    MpiWrapper mpi(&argc, &argv);
    int r = RunMpiBasicString<M>(mpi, RunProj, conf);
    return r;
  }
  if (mode == "cgtime") {
    if (argc != 11) return 1;
    const MIdx nsz = ParseSize(argv[2]);
    for (int d = 0; d < 3; ++d) g.nn[d] = nsz[d];
    const MIdx bs = ParseSize(argv[3]);
    g.dt = std::atof(argv[4]);
    g.rho1 = std::atof(argv[5]);
    g.rho2 = std::atof(argv[6]);
    const std::string iters = argv[7];
    g.alpha = ReadRaw(argv[8], NCells());
    g.vflux = ReadRaw(argv[9], 3 * NCells());
    g.out = argv[10];
    g.time_only = true;
    std::string conf = MeshConf(nsz, bs);
    conf += "\nset double hypre_symm_tol 0";
    conf += "\nset int hypre_symm_maxiter " + iters;
    conf += "\nset int hypre_symm_miniter " + iters;
    conf += "\nset int linsolver_symm_maxnorm 0";
    MpiWrapper mpi(&argc, &argv);
    return RunMpiBasicString<M>(mpi, RunProj, conf);
  }
  if (mode == "fluid") {
    if (argc != 15) return 1;
    const MIdx nsz = ParseSize(argv[2]);
    for (int d = 0; d < 3; ++d) g.nn[d] = nsz[d];
    const MIdx bs = ParseSize(argv[3]);
    g.dt = std::atof(argv[4]);
    g.steps = std::atoi(argv[5]);
    g.rho1 = std::atof(argv[6]);
    g.rho2 = std::atof(argv[7]);
    gf.mu1 = std::atof(argv[8]);
    gf.mu2 = std::atof(argv[9]);
    const std::string tol = argv[10];
    const std::string maxiter = argv[11];
    g.alpha = ReadRaw(argv[12], NCells());
    gf.vel = ReadRaw(argv[13], 3 * NCells());
    g.out = argv[14];
    g.out_u.assign(3 * NCells(), 0);
    g.out_p.assign(NCells(), 0);
    g.out_flux.assign(3 * NCells(), 0);
    std::string conf = MeshConf(nsz, bs);
    conf += "\nset double hypre_symm_tol " + tol;
    conf += "\nset int hypre_symm_maxiter " + maxiter;
    conf += "\nset int hypre_symm_miniter 0";
    conf += "\nset int linsolver_symm_maxnorm 0";
    MpiWrapper mpi(&argc, &argv);
    return RunMpiBasicString<M>(mpi, RunFluid, conf);
  }
  if (mode == "bcg") {
    if (argc != 9) return 1;
    const MIdx nsz = ParseSize(argv[2]);
    for (int d = 0; d < 3; ++d) g.nn[d] = nsz[d];
    const MIdx bs = ParseSize(argv[3]);
    g.dt = std::atof(argv[4]);
    g.u = ReadRaw(argv[5], NCells());
    g.vflux = ReadRaw(argv[6], 3 * NCells());
    g.alpha = ReadRaw(argv[7], NCells());  // the source
    g.out = argv[8];
    g.out_flux.assign(3 * NCells(), 0);
    MpiWrapper mpi(&argc, &argv);
    return RunMpiBasicString<M>(mpi, RunBcg, MeshConf(nsz, bs));
  }
  if (mode == "vof") {
    if (argc != 10) return 1;
    const MIdx nsz = ParseSize(argv[2]);
    for (int d = 0; d < 3; ++d) g.nn[d] = nsz[d];
    const MIdx bs = ParseSize(argv[3]);
    (void)std::atof(argv[4]);
    g.dt = std::atof(argv[5]);
    g.steps = std::atoi(argv[6]);
    g.u = ReadRaw(argv[7], NCells());
    g.vflux = ReadRaw(argv[8], 3 * NCells());
    g.out = argv[9];
    g.out_u.assign(NCells(), 0);
    g.out_a.assign(NCells(), 0);
    g.out_k.assign(NCells(), 0);
    g.out_cl.assign(NCells(), 0);
    g.out_n.assign(3 * NCells(), 0);
    std::string conf = MeshConf(nsz, bs);
    conf += "\nset string vof_scheme weymouth";
    conf += "\nset double vof_clipth 1e-10";
    if (std::getenv("REF_VERBOSE")) conf += "\nset int verbose_stages 1";
    MpiWrapper mpi(&argc, &argv);
    return RunMpiBasicString<M>(mpi, RunVof, conf);
  }
  return 1;
}

int Table(const std::string& mode, const char* in, const char* out) {
  std::ifstream fi(in);
  std::ofstream fo(out);
  fo.precision(17);
  std::string line;
  using R = Reconst<Scal>;
  while (std::getline(fi, line)) {
    std::istringstream s(line);
    if (mode == "overlap") {
      double v[10];
      for (auto& x : v) s >> x;
      fo << GetSphereOverlap(
                Vect(v[0], v[1], v[2]), Vect(v[3], v[4], v[5]),
                Vect(v[6], v[7], v[8]), v[9])
         << "\n";
    } else if (mode == "reconst") {
      double v[11];
      for (auto& x : v) s >> x;
      const Vect n(v[0], v[1], v[2]);
      const Vect h(v[5], v[6], v[7]);
      fo << R::GetLineA(n, v[3], h) << " " << R::GetLineU(n, v[4], h) << " "
         << R::GetLineFlux(n, v[4], h, v[8], v[9], size_t(v[10])) << "\n";
    } else if (mode == "height") {
      // a column of any length; with a leading "n=<value>" token the
      // two-argument Good(uu, n) is evaluated instead
      std::vector<double> uu;
      std::string tok;
      bool with_n = false;
      double nn = 0;
      while (s >> tok) {
        if (tok.rfind("n=", 0) == 0) {
          with_n = true;
          nn = std::atof(tok.c_str() + 2);
        } else {
          uu.push_back(std::atof(tok.c_str()));
        }
      }
      fo << (with_n ? UHeight<Scal>::Good(uu, nn) : UHeight<Scal>::Good(uu))
         << "\n";
    }
  }
  return 0;
}

} // namespace

int Dump(int argc, const char** argv) {
  const std::string mode = argv[1];
  const MIdx nsz = ParseSize(argv[2]);
  if (mode == "xmf") {
    if (argc != 8) return 1;
    using X = dump::Xmf<Vect>;
    X::Meta meta;
    meta.name = argv[4];
    meta.binpath = argv[5];
    meta.type = dump::StringToType(argv[6]);
    meta.dimensions = nsz;
    meta.count = nsz;
    meta.origin = Vect(0);
    meta.spacing = Vect(std::atof(argv[3]));
    X::WriteXmf(std::string(argv[7]), meta, false);
    return 0;
  }
  if (argc != 6) return 1;
  const size_t n = size_t(nsz.prod());
  const std::vector<double> v = ReadRaw(argv[4], n);
  MpiWrapper mpi;
  const std::vector<MIdx> starts{MIdx(0)}, sizes{nsz};
  const std::vector<std::vector<double>> data{v};
  dump::Raw<M>::WriteBlocks<double>(
      argv[5], starts, sizes, data, nsz, dump::StringToType(argv[3]), 0, mpi,
      true);
  return 0;
}

int main(int argc, const char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "";
  if (mode == "xmf" || mode == "raw") {
    if (argc < 3) return 1;
    return Dump(argc, argv);
  }
  if (mode == "overlap" || mode == "reconst" || mode == "height") {
    if (argc != 4) return 1;
    return Table(mode, argv[2], argv[3]);
  }
  const int r = Main(argc, argv);
  if (r != 0) return r;
  if (mode == "proj") {
    WriteRaw(g.out + ".expr", g.out_expr);
    WriteRaw(g.out + ".p", g.out_p);
    WriteRaw(g.out + ".flux", g.out_flux);
    std::ofstream fo(g.out + ".info");
    fo.precision(17);
    fo << g.residual << " " << g.iter << "\n";
  } else if (mode == "cgtime") {
    std::ofstream fo(g.out + ".time");
    fo.precision(17);
    fo << (g.t_solve1 - g.t_solve0) << " " << g.iter << " " << g.residual << "\n";
  } else if (mode == "bcg") {
    WriteRaw(g.out + ".ffu", g.out_flux);
  } else if (mode == "fluid") {
    WriteRaw(g.out + ".vel", g.out_u);
    WriteRaw(g.out + ".p", g.out_p);
    WriteRaw(g.out + ".flux", g.out_flux);
  } else if (mode == "vof") {
    WriteRaw(g.out + ".u", g.out_u);
    WriteRaw(g.out + ".n", g.out_n);
    WriteRaw(g.out + ".a", g.out_a);
    WriteRaw(g.out + ".k", g.out_k);
    WriteRaw(g.out + ".cl", g.out_cl);
    std::ofstream fo(g.out + ".sumu");
    fo.precision(17);
    for (auto s : g.sumu) fo << s << "\n";
  }
  return 0;
}

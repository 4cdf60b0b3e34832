// aphros's block framework stepping the reference-side VOF and curvature
// adapters (GpuVof, GpuCurvature) the way test/advection/main.cpp steps Vof
// and curvature::Heights (StartStep, MakeIteration, FinishStep, PostStep,
// CalcCurvature per step), on raw inputs; APHGPU_CURV=particles or hybrid
// selects the particle-string estimators.  Test infrastructure: its output
// is compared with oracle/_ref/ref_harness's `vof` mode (aphros's own Vof
// and Heights) on the same inputs and block layout.
//
//   vof_gpu n bs dt steps u.bin vflux.bin out   -> out.u, out.k (raw f64)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "distr/distrbasic.h"
#include "solver/curv.h"
#include "util/distr.h"

#include "curv_aphgpu.cpp"
#include "vof_aphgpu.cpp"

using M = MeshCartesian<double, 3>;
using Scal = typename M::Scal;
using MIdx = typename M::MIdx;

namespace {

struct Global {
  int n = 0;
  double dt = 0;
  int steps = 0;
  std::vector<double> u, vflux, out_u, out_k;
} g;

std::vector<double> ReadRaw(const std::string& path, size_t count) {
  std::vector<double> v(count);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(double), count, f) != count) {
    std::cerr << "cannot read " << path << std::endl;
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

void WriteRaw(const std::string& path, const std::vector<double>& v) {
  FILE* f = std::fopen(path.c_str(), "wb");
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

size_t Flat(const MIdx& w) {
  auto wrap = [](int i) { return size_t(((i % g.n) + g.n) % g.n); };
  return wrap(w[0]) + size_t(g.n) * (wrap(w[1]) + size_t(g.n) * wrap(w[2]));
}

void Run(M& m, Vars&) {
  auto sem = m.GetSem(__func__);
  struct {
    FieldCell<Scal> fcu;
    FieldEmbed<Scal> ffv;
    FieldCell<Scal> fcsrc;
    MapEmbed<BCondAdvection<Scal>> bc;  // empty: periodic
    std::unique_ptr<GpuVof<M>> as;
    Multi<FieldCell<Scal>> fck;
    std::unique_ptr<GpuCurvature<M>> curv;
    int step = 0;
  } * ctx(sem);
  auto& t = *ctx;
  const size_t N = size_t(g.n) * g.n * g.n;
  if (sem("init")) {
    t.fcu.Reinit(m);
    for (auto c : m.AllCells()) t.fcu[c] = g.u[Flat(m.GetIndexCells().GetMIdx(c))];
    t.ffv.Reinit(m, 0);
    const auto& indexf = m.GetIndexFaces();
    for (auto f : m.AllFaces()) {
      const auto p = indexf.GetMIdxDir(f);
      t.ffv[f] = g.vflux[p.second.raw() * N + Flat(p.first)];
    }
    t.fcsrc.Reinit(m, 0.);
    t.as.reset(new GpuVof<M>(m, t.fcu, t.bc, &t.ffv, &t.fcsrc, 0., g.dt, 1e-10));
    GpuVof<M>* as = t.as.get();
    // APHGPU_CURV=particles or hybrid selects the particle estimators (the
    // reference run takes REF_CURV with the same name)
    int est = APHGPU_CURV_HEIGHTS;
    if (const char* e = std::getenv("APHGPU_CURV")) {
      if (std::string(e) == "particles") est = APHGPU_CURV_PARTICLES;
      if (std::string(e) == "hybrid") est = APHGPU_CURV_HYBRID;
    }
    t.curv.reset(new GpuCurvature<M>([as]() { return as->GetContext(); }, est));
    t.fck.resize(GRange<size_t>(1));
    t.fck.InitAll(FieldCell<Scal>(m, GetNan<Scal>()));
  }
  sem.LoopBegin();
  if (sem("check")) {
    if (t.step >= g.steps) sem.LoopBreak();
  }
  if (sem.Nested("start")) t.as->StartStep();
  if (sem.Nested("iter")) t.as->MakeIteration();
  if (sem.Nested("finish")) t.as->FinishStep();
  if (sem.Nested("post")) t.as->PostStep();
  if (sem.Nested("curv")) t.curv->CalcCurvature(t.fck, t.as->GetPlic(), m, m);
  if (sem("next")) ++t.step;
  sem.LoopEnd();
  if (sem("out")) {
    const auto& u = t.as->GetField();
    for (auto c : m.Cells()) {
      const size_t i = Flat(m.GetIndexCells().GetMIdx(c));
      g.out_u[i] = u[c];
      g.out_k[i] = t.fck[0][c];
    }
  }
}

}  // namespace

int main(int argc, const char** argv) {
  if (argc != 8) {
    std::cerr << "usage: vof_gpu n bs dt steps u.bin vflux.bin out" << std::endl;
    return 1;
  }
  g.n = std::atoi(argv[1]);
  const int bs = std::atoi(argv[2]);
  g.dt = std::atof(argv[3]);
  g.steps = std::atoi(argv[4]);
  const size_t N = size_t(g.n) * g.n * g.n;
  g.u = ReadRaw(argv[5], N);
  g.vflux = ReadRaw(argv[6], 3 * N);
  g.out_u.assign(N, 0);
  g.out_k.assign(N, 0);
  MpiWrapper mpi(&argc, &argv);
  Subdomains<MIdx> sub(MIdx(g.n), MIdx(bs), 1);
  std::string conf = sub.GetConfig();
  conf += "\nset string backend local";
  conf += "\nset double extent 1";
  const int r = RunMpiBasicString<M>(mpi, Run, conf);
  if (r) return r;
  WriteRaw(std::string(argv[7]) + ".u", g.out_u);
  WriteRaw(std::string(argv[7]) + ".k", g.out_k);
  return 0;
}

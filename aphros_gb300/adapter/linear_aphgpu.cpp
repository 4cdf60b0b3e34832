// src/linear/linear_aphgpu.cpp (reference side)
#include <memory>
#include <vector>

#include "aphgpu.h"
#include "linear/linear.h"
#include "util/module.h"

namespace linear {

template <class M>
class SolverGpu : public Solver<M> {
 public:
  using Base = Solver<M>;
  using Scal = typename M::Scal;
  using Expr = typename M::Expr;
  using MIdx = typename M::MIdx;
  using Conf = typename Base::Conf;
  using Info = typename Base::Info;

  // Optional multigrid settings (gpu_<prefix>_* variables); negative or
  // zero values keep the library defaults.
  struct Tuning {
    int mg_pre = -1, mg_post = -1, inner_maxiter = -1;
    double inner_rtol = -1;
    int cycle = 0, sweep_growth = 0, coarse_series = -1;
  };

  SolverGpu(const Conf& conf, int kind, int maxnorm, const Tuning& tuning, const M& m)
      : Base(conf), kind_(kind), maxnorm_(maxnorm), tuning_(tuning) {
    if (m.IsLead()) {
      shared_obj_ = std::make_unique<Shared>();
      shared_ = shared_obj_.get();
    }
  }

  Info Solve(
      const FieldCell<Expr>& fc_system, const FieldCell<Scal>* fc_init,
      FieldCell<Scal>& fc_sol, M& m) override {
    auto sem = m.GetSem(__func__);
    auto& ms = m.GetShared();
    const MIdx gs = ms.GetGlobalSize();
    if (sem()) {
      // the lead sizes its buffers before any block writes into them (the
      // blocks of a rank run each stage concurrently)
      if (m.IsLead()) {
        const size_t n = size_t(gs.prod());
        shared_->expr.resize(8 * n);
        shared_->x0.resize(n);
        shared_->x.resize(n);
      }
      m.BcastFromLead(&shared_);  // every block sees the lead's buffers
    }
    // shared_ is valid on every block after the first stage (broadcast)
    auto flat = [&gs](MIdx w) {  // x fastest, as aphgpu expects
      return size_t(w[0]) + size_t(gs[0]) * (size_t(w[1]) + size_t(gs[1]) * w[2]);
    };
    if (sem("gather")) {
      Shared& s = *shared_;
      // blocks of one rank share memory: each writes its own cells
      for (auto c : m.CellsM()) {
        const size_t i = flat(MIdx(c));
        for (int q = 0; q < 8; ++q) s.expr[8 * i + q] = fc_system[c][q];
        s.x0[i] = fc_init ? (*fc_init)[c] : 0;
      }
    }
    if (sem("solve") && m.IsLead()) {
      Shared& s = *shared_;
      fassert(m.flags.is_periodic[0] && m.flags.is_periodic[1] &&
              m.flags.is_periodic[2], "gpu solver: periodic domains only");
      size_t ncells = 0;  // the rank must own the whole domain
      for (auto c : ms.CellsM()) {
        (void)c;
        ++ncells;
      }
      fassert_equal(ncells, size_t(gs.prod()));
      if (!s.ctx) {
        const auto h = ms.GetCellSize();
        fassert(h[0] == h[1] && h[1] == h[2], "gpu solver: cubic cells only");
        fassert_equal(aphgpu_create(&s.ctx, gs[0], gs[1], gs[2], h[0], 0), APHGPU_OK);
        fassert_equal(aphgpu_set_option(s.ctx, APHGPU_OPT_CYCLE, tuning_.cycle), APHGPU_OK);
        fassert_equal(
            aphgpu_set_option(s.ctx, APHGPU_OPT_SWEEP_GROWTH, tuning_.sweep_growth),
            APHGPU_OK);
        if (tuning_.coarse_series >= 0) {
          fassert_equal(
              aphgpu_set_option(s.ctx, APHGPU_OPT_COARSE_SERIES, tuning_.coarse_series),
              APHGPU_OK);
        }
      }
      int rc = aphgpu_set_system_expr(s.ctx, s.expr.data());
      aphgpu_conf c;
      aphgpu_conf_default(&c);
      c.solver = kind_;
      c.tol = this->conf.tol;
      c.miniter = this->conf.miniter;
      c.maxiter = this->conf.maxiter;
      c.maxnorm = maxnorm_;
      if (tuning_.mg_pre >= 0) c.mg_pre = tuning_.mg_pre;
      if (tuning_.mg_post >= 0) c.mg_post = tuning_.mg_post;
      if (tuning_.inner_maxiter > 0) c.inner_maxiter = tuning_.inner_maxiter;
      if (tuning_.inner_rtol > 0) c.inner_rtol = tuning_.inner_rtol;
      aphgpu_info info;
      if (rc == APHGPU_OK)
        rc = aphgpu_solve(s.ctx, &c, fc_init ? s.x0.data() : nullptr, s.x.data(), &info);
      fassert(rc == APHGPU_OK, std::string("aphgpu: ") + aphgpu_last_error(s.ctx));
      s.info.residual = info.residual;
      s.info.iter = info.iter;
    }
    if (sem("scatter")) {
      const Shared& s = *shared_;
      for (auto c : m.CellsM()) fc_sol[c] = s.x[flat(MIdx(c))];
      m.Comm(&fc_sol, M::CommStencil::direct_one);
    }
    // the result of the last stage (the value of earlier stages is unused)
    return shared_ ? shared_->info : Info{};
  }

 private:
  struct Shared {
    ~Shared() { aphgpu_destroy(ctx); }
    aphgpu_ctx* ctx = nullptr;
    std::vector<double> expr, x0, x;
    Info info{};
  };
  int kind_;
  int maxnorm_;
  Tuning tuning_;
  std::unique_ptr<Shared> shared_obj_;  // lead block only
  Shared* shared_ = nullptr;
};

template <class M, int Kind>
class ModuleLinearGpu : public ModuleLinear<M> {
 public:
  ModuleLinearGpu()
      : ModuleLinear<M>(Kind == APHGPU_SOLVER_CG      ? "gpu_cg"
                        : Kind == APHGPU_SOLVER_MGPCG ? "gpu"
                                                      : "gpu_mixed") {}
  std::unique_ptr<Solver<M>> Make(
      const Vars& var, std::string prefix, const M& m) override {
    const int maxnorm = var.Int["linsolver_" + prefix + "_maxnorm"];
    const std::string g = "gpu_" + prefix + "_";
    typename SolverGpu<M>::Tuning t;
    t.mg_pre = var.Int(g + "mg_pre", -1);
    t.mg_post = var.Int(g + "mg_post", -1);
    t.inner_maxiter = var.Int(g + "inner_maxiter", -1);
    t.inner_rtol = var.Double(g + "inner_rtol", -1.);
    t.cycle = var.Int(g + "cycle", 0);
    t.sweep_growth = var.Int(g + "sweep_growth", 0);
    t.coarse_series = var.Int(g + "coarse_series", -1);
    return std::make_unique<SolverGpu<M>>(
        this->GetConf(var, prefix), Kind, maxnorm, t, m);
  }
};

using M3 = MeshCartesian<double, 3>;
bool kReg_aphgpu[] = {
    RegisterModule<ModuleLinearGpu<M3, APHGPU_SOLVER_CG>>(),
    RegisterModule<ModuleLinearGpu<M3, APHGPU_SOLVER_MGPCG>>(),
    RegisterModule<ModuleLinearGpu<M3, APHGPU_SOLVER_MIXED>>(),
};

}  // namespace linear

// src/solver/curv_aphgpu.cpp (reference side): the curvature estimators of
// aphros behind their curvature::Estimator<M> interface (src/solver/curv.h:
// 16-37), computed by libaphgpu (aphgpu_curvature_estimator).
//
// MakeEstimator (src/solver/curv.ipp:604-622) selects the estimator with an
// if/else on the `curvature` variable; the branches for this class read
//   if (name == "gpu_heights")
//     return std::make_unique<GpuCurvature<M>>(ctx, APHGPU_CURV_HEIGHTS);
//   if (name == "gpu_particles" || name == "gpu_hybrid") {
//     aphgpu_part_conf pc;  // the part_* variables, as ParsePar reads them
//     aphgpu_part_conf_default(&pc);
//     pc.np = var.Int("part_np", pc.np);
//     pc.ns = var.Int("part_ns", pc.ns);
//     pc.leq = var.Double("part_h", pc.leq);
//     pc.relax = var.Double("part_relax", pc.relax);
//     pc.tol = var.Double("part_tol", pc.tol);
//     pc.itermax = var.Int("part_itermax", pc.itermax);
//     pc.segcirc = var.Double("part_segcirc", pc.segcirc);
//     pc.dn = var.Int("part_dn", pc.dn);
//     return std::make_unique<GpuCurvature<M>>(
//         ctx, name == "gpu_particles" ? APHGPU_CURV_PARTICLES : APHGPU_CURV_HYBRID, pc);
//   }
// where ctx is the GpuVof's GetContext() (the curvature is then computed on
// the volume fraction already resident on the device) or nullptr (the
// volume fraction of the Plic is copied to a context of this estimator).
// It replaces curvature::Heights (curv.ipp:358-414), curvature::Particles
// (curv.ipp:29-54) and curvature::Hybrid (curv.ipp:525-560) with one layer
// and no colours (the single-field Vof gives none), on periodic domains
// owned by one rank.
#include <functional>
#include <memory>
#include <vector>

#include "aphgpu.h"
#include "geom/mesh.h"
#include "solver/curv.h"

template <class M_>
class GpuCurvature final : public curvature::Estimator<M_> {
 public:
  using M = M_;
  using Scal = typename M::Scal;
  using Vect = typename M::Vect;
  using MIdx = typename M::MIdx;
  using Plic = generic::Plic<Vect>;

  // resident: returns the context holding the volume fraction (GpuVof's
  // GetContext), or is empty to copy the Plic's volume fraction;
  // estimator: APHGPU_CURV_HEIGHTS, _PARTICLES or _HYBRID; conf: the
  // particle parameters
  explicit GpuCurvature(std::function<aphgpu_ctx*()> resident = {},
                        int estimator = APHGPU_CURV_HEIGHTS,
                        const aphgpu_part_conf* conf = nullptr)
      : resident_(resident), estimator_(estimator) {
    aphgpu_part_conf_default(&conf_);
    if (conf) conf_ = *conf;
  }

  void CalcCurvature(
      const Multi<FieldCell<Scal>*>& fck, const Plic& plic, M& m,
      const M&) override {
    auto sem = m.GetSem("gpu-curvature");
    const MIdx gs = m.GetGlobalSize();
    const size_t n = size_t(gs.prod());
    if (sem()) {
      // the lead prepares its buffers before any block writes into them (the
      // blocks of a rank run each stage concurrently)
      if (m.IsLead()) {
        if (!shared_obj_) shared_obj_ = std::make_unique<Shared>();
        shared_ = shared_obj_.get();
        shared_->ctx = resident_ ? resident_() : nullptr;
        shared_->kappa.resize(n);
        if (!shared_->ctx) shared_->u.resize(n);
      }
      m.BcastFromLead(&shared_);
    }
    auto flat = [&gs](MIdx w) {  // x fastest, as aphgpu expects
      return size_t(w[0]) + size_t(gs[0]) * (size_t(w[1]) + size_t(gs[1]) * w[2]);
    };
    if (sem("gather")) {
      Shared& s = *shared_;
      if (!s.ctx) {
        const FieldCell<Scal>& fcu = *plic.vfcu[0];
        for (auto c : m.Cells()) s.u[flat(MIdx(m.GetIndexCells().GetMIdx(c)))] = fcu[c];
      }
    }
    if (sem("curvature") && m.IsLead()) {
      Shared& s = *shared_;
      aphgpu_ctx* ctx = s.ctx;
      if (!ctx) {
        fassert(m.flags.is_periodic[0] && m.flags.is_periodic[1] &&
                m.flags.is_periodic[2], "gpu curvature: periodic domains only");
        const auto h = m.GetCellSize();
        fassert(h[0] == h[1] && h[1] == h[2], "gpu curvature: cubic cells only");
        if (!own_.ctx) {
          fassert_equal(aphgpu_create(&own_.ctx, gs[0], gs[1], gs[2], h[0], 0), APHGPU_OK);
        }
        ctx = own_.ctx;
        const int rc = aphgpu_vof_init(ctx, s.u.data(), 1e-10);
        fassert(rc == APHGPU_OK, std::string("aphgpu: ") + aphgpu_last_error(ctx));
      }
      const int rc = aphgpu_curvature_estimator(ctx, estimator_, &conf_, s.kappa.data());
      fassert(rc == APHGPU_OK, std::string("aphgpu: ") + aphgpu_last_error(ctx));
    }
    if (sem("scatter")) {
      const Shared& s = *shared_;
      FieldCell<Scal>& fc = *fck[0];
      for (auto c : m.Cells()) fc[c] = s.kappa[flat(MIdx(m.GetIndexCells().GetMIdx(c)))];
      m.Comm(&fc);
    }
  }

  void CalcCurvature(
      const Multi<FieldCell<Scal>*>&, const Plic&, M&, const Embed<M>&) override {
    fassert(false, "gpu curvature: embedded boundaries are not supported");
  }

 private:
  struct Shared {
    aphgpu_ctx* ctx = nullptr;  // the context used by this call
    std::vector<double> u, kappa;
  };
  struct Own {
    ~Own() {
      aphgpu_destroy(ctx);
    }
    aphgpu_ctx* ctx = nullptr;  // this estimator's own context (lead block)
  };
  std::function<aphgpu_ctx*()> resident_;
  int estimator_;
  aphgpu_part_conf conf_;
  std::unique_ptr<Shared> shared_obj_;  // lead block only
  Shared* shared_ = nullptr;
  Own own_;
};

template class GpuCurvature<MeshCartesian<double, 3>>;

// the height-function estimator under its earlier name
template <class M>
using GpuHeights = GpuCurvature<M>;

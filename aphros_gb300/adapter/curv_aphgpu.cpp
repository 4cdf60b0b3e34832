// src/solver/curv_aphgpu.cpp (reference side): the height-function
// curvature of aphros behind its curvature::Estimator<M> interface
// (src/solver/curv.h:16-37), computed by libaphgpu (aphgpu_curvature).
//
// MakeEstimator (src/solver/curv.ipp:604-622) selects the estimator with an
// if/else on the `curvature` variable; the branch for this class reads
//   if (name == "gpu_heights") return std::make_unique<GpuHeights<M>>(ctx);
// where ctx is the GpuVof's GetContext() (the curvature is then computed on
// the volume fraction already resident on the device) or nullptr (the
// volume fraction of the Plic is copied to a context of this estimator).
// It replaces curvature::Heights (curv.ipp:358-414) with one layer and no
// colours, on periodic domains owned by one rank.
#include <functional>
#include <memory>
#include <vector>

#include "aphgpu.h"
#include "geom/mesh.h"
#include "solver/curv.h"

template <class M_>
class GpuHeights final : public curvature::Estimator<M_> {
 public:
  using M = M_;
  using Scal = typename M::Scal;
  using Vect = typename M::Vect;
  using MIdx = typename M::MIdx;
  using Plic = generic::Plic<Vect>;

  // resident: returns the context holding the volume fraction (GpuVof's
  // GetContext), or is empty to copy the Plic's volume fraction
  explicit GpuHeights(std::function<aphgpu_ctx*()> resident = {})
      : resident_(resident) {}

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
                m.flags.is_periodic[2], "gpu heights: periodic domains only");
        const auto h = m.GetCellSize();
        fassert(h[0] == h[1] && h[1] == h[2], "gpu heights: cubic cells only");
        if (!own_.ctx) {
          fassert_equal(aphgpu_create(&own_.ctx, gs[0], gs[1], gs[2], h[0], 0), APHGPU_OK);
        }
        ctx = own_.ctx;
        const int rc = aphgpu_vof_init(ctx, s.u.data(), 1e-10);
        fassert(rc == APHGPU_OK, std::string("aphgpu: ") + aphgpu_last_error(ctx));
      }
      const int rc = aphgpu_curvature(ctx, s.kappa.data(), nullptr);
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
    fassert(false, "gpu heights: embedded boundaries are not supported");
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
  std::unique_ptr<Shared> shared_obj_;  // lead block only
  Shared* shared_ = nullptr;
  Own own_;
};

template class GpuHeights<MeshCartesian<double, 3>>;

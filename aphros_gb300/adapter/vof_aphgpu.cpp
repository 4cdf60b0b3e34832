// src/solver/vof_aphgpu.cpp (reference side): the PLIC volume-of-fluid
// advection of aphros behind its AdvectionSolver<M> interface
// (src/solver/advection.h:58-100), computed by libaphgpu (aphgpu_vof_*).
//
// Hydro creates its advection solver with an if/else on `advection_solver`
// (src/kernel/hydro.ipp:742-800); the branch for this class reads
//   as_.reset(new GpuVof<M>(m, fcvf, bc_vf, &fev_, &fc_src_, t, dt, clipth));
// It replaces Vof<M> with scheme weymouth (the default of VofPar,
// src/solver/vof.h:13-53) on periodic domains owned by one rank.
//
// Staging follows the pattern of the reference's OpenCL solver
// (src/linear/conjugate_cl.ipp): every block of the rank writes its cells
// into buffers owned by the lead block, the lead block alone calls the C
// ABI, and every block reads its cells back.
#include <memory>
#include <vector>

#include "aphgpu.h"
#include "geom/mesh.h"
#include "solver/advection.h"

template <class M_>
class GpuVof final : public AdvectionSolver<M_> {
 public:
  using M = M_;
  using P = AdvectionSolver<M>;
  using Scal = typename M::Scal;
  using Vect = typename M::Vect;
  using MIdx = typename M::MIdx;
  using Plic = generic::Plic<Vect>;

  // fcu: initial volume fraction; fev: volume fluxes; fcs: volume source
  // (may be null); clipth: clipping threshold (VofPar::clipth)
  GpuVof(M& m, const FieldCell<Scal>& fcu, const MapEmbed<BCondAdvection<Scal>>& mebc,
         const FieldEmbed<Scal>* fev, const FieldCell<Scal>* fcs, double t, double dt,
         Scal clipth)
      : P(t, dt, m, fev, fcs, mebc), clipth_(clipth), layers_(1) {
    fcu_.time_curr = fcu;
    fcu_.time_prev = fcu;
    fcu_.iter_curr = fcu;
    fca_.Reinit(m, GetNan<Scal>());
    fcn_.Reinit(m, Vect(GetNan<Scal>()));
    fci_.Reinit(m, false);
    fccl_.Reinit(m, -1);
    fcim_.Reinit(m, MIdx(0));
    if (m.IsLead()) {
      shared_obj_ = std::make_unique<Shared>();
      shared_ = shared_obj_.get();
    }
  }

  void StartStep() override {
    auto sem = this->m.GetSem("start");
    if (sem("start")) {
      this->ClearIter();
      fcu_.time_prev = fcu_.time_curr;
      fcu_.iter_curr = fcu_.time_prev;
    }
    if (!started_ && sem.Nested("init")) {
      Upload(fcu_.time_curr, true);
    }
    if (sem("started")) {
      started_ = true;
    }
  }

  void MakeIteration() override {
    auto sem = this->m.GetSem("iter");
    auto& m = this->m;
    if (sem()) {
      // the lead sizes its buffers before any block writes into them (the
      // blocks of a rank run each stage concurrently)
      if (m.IsLead()) {
        const size_t n = size_t(m.GetGlobalSize().prod());
        shared_->flux.resize(3 * n);
        shared_->src.resize(n);
        shared_->has_src = this->fcs_ != nullptr;
      }
      m.BcastFromLead(&shared_);
    }
    if (sem("gather")) {
      Shared& s = *shared_;
      const MIdx gs = m.GetGlobalSize();
      const size_t n = size_t(gs.prod());
      const auto& ff = this->fev_->GetFieldFace();
      const auto& indexf = m.GetIndexFaces();
      for (auto f : m.Faces()) {
        const auto p = indexf.GetMIdxDir(f);
        const MIdx w = p.first;
        const size_t d = p.second.raw();
        if (w[d] == gs[d]) continue;  // the periodic image of face w[d] = 0
        s.flux[d * n + Flat(gs, w)] = ff[f];
      }
      if (this->fcs_) {
        for (auto c : m.Cells()) s.src[Flat(gs, MIdx(m.GetIndexCells().GetMIdx(c)))] =
            (*this->fcs_)[c];
      }
    }
    if (sem("advect") && m.IsLead()) {
      Shared& s = *shared_;
      Check(aphgpu_vof_set_source(s.ctx, s.has_src ? s.src.data() : nullptr));
      Check(aphgpu_vof_step(s.ctx, s.flux.data(), this->GetTimeStep()));
      Check(aphgpu_vof_get(s.ctx, s.u.data(), s.n.data(), s.a.data(), s.mask.data()));
    }
    if (sem("scatter")) {
      Scatter(fcu_.iter_curr);
      m.Comm(&fcu_.iter_curr);
      m.Comm(&fca_);
      m.Comm(&fcn_);
    }
    if (sem("inc")) {
      this->IncIter();
    }
  }

  void FinishStep() override {
    fcu_.time_curr = fcu_.iter_curr;
    this->IncTime();
  }

  const FieldCell<Scal>& GetField(Step l) const override {
    return fcu_.Get(l);
  }
  using P::GetField;

  Plic GetPlic() const override {
    return {layers_, &GetField(), &fca_, &fcn_, &fci_, nullptr, &fccl_, &fcim_,
            this->mebc_};
  }

  // The library context of this solver (valid on every block after the
  // first MakeIteration or StartStep); GpuHeights computes the curvature
  // on it without copying the volume fraction again.
  aphgpu_ctx* GetContext() const {
    return shared_ ? shared_->ctx : nullptr;
  }

 private:
  struct Shared {
    ~Shared() {
      aphgpu_destroy(ctx);
    }
    aphgpu_ctx* ctx = nullptr;
    std::vector<double> u, n, a, flux, src;
    std::vector<uint8_t> mask;
    bool has_src = false;
  };

  static size_t Flat(const MIdx& gs, const MIdx& w) {  // x fastest
    return size_t(w[0]) + size_t(gs[0]) * (size_t(w[1]) + size_t(gs[1]) * w[2]);
  }

  void Check(int rc) const {
    fassert(rc == APHGPU_OK,
            std::string("aphgpu: ") + aphgpu_last_error(shared_ ? shared_->ctx : nullptr));
  }

  // Volume fraction to the lead's context: aphgpu_vof_init reconstructs the
  // interface, the state of Vof after StartStep at t=0 (vof.ipp:177-195).
  void Upload(const FieldCell<Scal>& fcu, bool create) {
    auto sem = this->m.GetSem("upload");
    auto& m = this->m;
    if (sem()) {
      if (m.IsLead()) {
        const size_t n = size_t(m.GetGlobalSize().prod());
        shared_->u.resize(n);
        shared_->n.resize(3 * n);
        shared_->a.resize(n);
        shared_->mask.resize(n);
      }
      m.BcastFromLead(&shared_);
    }
    if (sem("gather")) {
      Shared& s = *shared_;
      const MIdx gs = m.GetGlobalSize();
      for (auto c : m.Cells()) s.u[Flat(gs, MIdx(m.GetIndexCells().GetMIdx(c)))] = fcu[c];
    }
    if (sem("init") && m.IsLead()) {
      Shared& s = *shared_;
      const MIdx gs = m.GetGlobalSize();
      fassert(m.flags.is_periodic[0] && m.flags.is_periodic[1] && m.flags.is_periodic[2],
              "gpu vof: periodic domains only");
      const auto h = m.GetCellSize();
      fassert(h[0] == h[1] && h[1] == h[2], "gpu vof: cubic cells only");
      if (create && !s.ctx) {
        fassert_equal(aphgpu_create(&s.ctx, gs[0], gs[1], gs[2], h[0], 0), APHGPU_OK);
      }
      Check(aphgpu_vof_init(s.ctx, s.u.data(), clipth_));
      Check(aphgpu_vof_get(s.ctx, nullptr, s.n.data(), s.a.data(), s.mask.data()));
    }
    if (sem("scatter")) {
      Scatter(fcu_.time_curr);
      m.Comm(&fca_);
      m.Comm(&fcn_);
    }
  }

  // Cells of this block from the lead's buffers (u, planes, mask).
  void Scatter(FieldCell<Scal>& fcu) {
    auto& m = this->m;
    const Shared& s = *shared_;
    const MIdx gs = m.GetGlobalSize();
    for (auto c : m.Cells()) {
      const size_t i = Flat(gs, MIdx(m.GetIndexCells().GetMIdx(c)));
      fcu[c] = s.u[i];
      fca_[c] = s.a[i];
      fcn_[c] = Vect(s.n[3 * i], s.n[3 * i + 1], s.n[3 * i + 2]);
      fci_[c] = s.mask[i] != 0;
    }
  }

  Scal clipth_;
  GRange<size_t> layers_;
  StepData<FieldCell<Scal>> fcu_;
  FieldCell<Scal> fca_;
  FieldCell<Vect> fcn_;
  FieldCell<bool> fci_;
  FieldCell<Scal> fccl_;
  FieldCell<MIdx> fcim_;
  bool started_ = false;
  std::unique_ptr<Shared> shared_obj_;  // lead block only
  Shared* shared_ = nullptr;
};

template class GpuVof<MeshCartesian<double, 3>>;

// glia/shim.hpp — header-only C++ layer with the reference's class and method names over the
// C-ABI of glia_rd.h, for code written against GLIA's PdeOperatorsRD / DerivativeOperatorsRD /
// DiffusionSolver API. PETSc is not needed: `Vec` is a host double vector (the C-ABI's default
// pointer mode) and PetscErrorCode is the C-ABI status (0 = success).
//
// Replaced interfaces (paths relative to the GLIA source tree):
//   Parameters / TumorParameters / OptimizerSettings  include/Parameters.h:17-109, 155-367
//   initializeGrid                                    src/grad/SpectralOperators.cpp:424-446
//   DiffCoef::setValues / setValuesSinusoidal         src/mat/DiffCoef.cpp:77-187
//   DiffusionSolver::precFactor / solve               src/pde/DiffusionSolver.cpp:119-250
//   Tumor (c_0_, c_t_, p_0_, p_t_), setSinusoidalCoefficients
//                                                     src/mat/Tumor.cpp:3-57, 102-112
//   DerivativeOperators::updateReactionAndDiffusion   src/grad/DerivativeOperators.cpp:323-367
//   PdeOperatorsRD::solveState / solveAdjoint         src/pde/PdeOperators.cpp:235-420
//   DerivativeOperatorsRD::evaluateObjective / evaluateGradient /
//                          evaluateObjectiveAndGradient src/grad/DerivativeOperatorsRD.cpp:7-226
#pragma once

#include <array>
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../glia_rd.h"

namespace glia_shim {

using PetscErrorCode = int;
using ScalarType = double;
using Vec = std::vector<double>;

struct TumorParameters {
  int np_ = 1, nk_ = 1, nr_ = 1, nt_ = 1, order_ = 2;
  ScalarType dt_ = 0.5, k_ = 0.0, rho_ = 10;
  ScalarType k_gm_wm_ratio_ = 0, k_glm_wm_ratio_ = 0, r_gm_wm_ratio_ = 0, r_glm_wm_ratio_ = 0;
  ScalarType phi_sigma_ = 2 * M_PI / 64, phi_spacing_factor_ = 1.5, smoothing_factor_ = 1;
  ScalarType obs_threshold_1_ = 0;
  std::array<ScalarType, 3> user_cm_{{M_PI, M_PI, M_PI}};
  bool adjoint_store_ = false, phi_store_ = false;
  bool two_time_points_ = false;  // objective with data at t = 0 as well (Data::dt0)
  bool time_history_off_ = false; // forward-only runs: no states kept
};

struct OptimizerSettings {
  ScalarType beta_ = 1e-4;
  int regularization_norm_ = 0;  // L2 = 0, L2b = 1
  bool diffusivity_inversion_ = true, flag_reaction_inv_ = false;
  ScalarType k_scale_ = 1, rho_scale_ = 1;
};

struct Grid {
  int n_[3] = {0, 0, 0};
  int64_t ng_ = 0;
  ScalarType h_[3] = {0, 0, 0}, lebesgue_measure_ = 0;
};

// Engine selection is not part of the reference API; it defaults to the fused mixed path.
struct EngineSettings {
  int precision = GLIA_MIXED;
  int engine = GLIA_ENGINE_FUSED;
  int history = GLIA_HISTORY_CHECKPOINT;
  int checkpoint_every = 10;
};

class Parameters {
 public:
  std::shared_ptr<TumorParameters> tu_ = std::make_shared<TumorParameters>();
  std::shared_ptr<OptimizerSettings> opt_ = std::make_shared<OptimizerSettings>();
  std::shared_ptr<Grid> grid_ = std::make_shared<Grid>();
  EngineSettings engine_;
};

// One context per grid: it stands for the reference's SpectralOperators + the PETSc objects.
class SpectralOperators {
 public:
  glia_ctx* ctx_ = nullptr;
  ~SpectralOperators() {
    if (ctx_) glia_destroy(ctx_);
  }
  void check(int rc, const char* where) const {
    if (rc != GLIA_OK)
      throw std::runtime_error(std::string(where) + ": " +
                               (ctx_ ? glia_last_error(ctx_) : "no context"));
  }
};

// initializeGrid(n, params, spec_ops)
inline PetscErrorCode initializeGrid(int n, std::shared_ptr<Parameters> params,
                                     std::shared_ptr<SpectralOperators> spec_ops) {
  int rc = glia_create(n, params->engine_.precision, params->engine_.engine, &spec_ops->ctx_);
  if (rc != GLIA_OK) return rc;
  auto& g = *params->grid_;
  g.n_[0] = g.n_[1] = g.n_[2] = n;
  g.ng_ = (int64_t)n * n * n;
  for (auto& h : g.h_) h = 2 * M_PI / n;
  g.lebesgue_measure_ = g.h_[0] * g.h_[1] * g.h_[2];
  // a freshly built DiffusionSolver reads TumorParameters::dt_
  return glia_set_time(spec_ops->ctx_, params->tu_->dt_, params->tu_->nt_, params->tu_->order_);
}

// MatProp: tissue probability maps (src/mat/MatProp.cpp)
class MatProp {
 public:
  MatProp(std::shared_ptr<Parameters> p, std::shared_ptr<SpectralOperators> s)
      : params_(p), spec_ops_(s) {}
  PetscErrorCode setValuesCustom(const Vec* gm, const Vec* wm, const Vec* csf, const Vec* vt,
                                 const Vec* /*bg*/, std::shared_ptr<Parameters>) {
    return glia_set_tissue(spec_ops_->ctx_, wm ? wm->data() : nullptr, gm ? gm->data() : nullptr,
                           csf ? csf->data() : nullptr, vt ? vt->data() : nullptr);
  }
  PetscErrorCode setValuesSinusoidal(std::shared_ptr<Parameters>) {
    return glia_set_tissue_sinusoidal(spec_ops_->ctx_);
  }
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<SpectralOperators> spec_ops_;
};

// DiffCoef (src/mat/DiffCoef.cpp)
class DiffCoef {
 public:
  DiffCoef(std::shared_ptr<Parameters> p, std::shared_ptr<SpectralOperators> s)
      : params_(p), spec_ops_(s) {}
  PetscErrorCode setValuesSinusoidal(std::shared_ptr<Parameters>, ScalarType scale) {
    return glia_set_diffusivity_sinusoidal(spec_ops_->ctx_, scale);
  }
  // DiffCoef::setSecondaryCoefficients (src/mat/DiffCoef.cpp:44-58), read by solveState(2)
  PetscErrorCode setSecondaryCoefficients(ScalarType k1, ScalarType k2, ScalarType k3,
                                          std::shared_ptr<MatProp>, std::shared_ptr<Parameters>) {
    return glia_set_secondary_coefficients(spec_ops_->ctx_, k1, k2, k3);
  }
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<SpectralOperators> spec_ops_;
};

// DiffusionSolver (src/pde/DiffusionSolver.cpp)
class DiffusionSolver {
 public:
  DiffusionSolver(std::shared_ptr<Parameters> p, std::shared_ptr<SpectralOperators> s,
                  std::shared_ptr<DiffCoef> k)
      : params_(p), spec_ops_(s), k_(k) {
    glia_prec_factor(spec_ops_->ctx_);
  }
  PetscErrorCode precFactor() { return glia_prec_factor(spec_ops_->ctx_); }
  PetscErrorCode solve(Vec& c, ScalarType dt) {
    return glia_diffusion_solve(spec_ops_->ctx_, c.data(), dt, &ksp_itr_);
  }
  int ksp_itr_ = 0;
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<SpectralOperators> spec_ops_;
  std::shared_ptr<DiffCoef> k_;
};

// Tumor: state vectors and the coefficient set-up it owns (src/mat/Tumor.cpp)
class Tumor {
 public:
  Tumor(std::shared_ptr<Parameters> p, std::shared_ptr<SpectralOperators> s)
      : params_(p), spec_ops_(s) {
    const size_t N = (size_t)p->grid_->ng_;
    c_0_.assign(N, 0.0);
    c_t_.assign(N, 0.0);
    p_0_.assign(N, 0.0);
    p_t_.assign(N, 0.0);
  }
  // k_->setValues + rho_->setValues + Phi set-up from the parameters (Tumor::initialize)
  PetscErrorCode initialize(const std::vector<double>* centers = nullptr) {
    auto& tu = *params_->tu_;
    int rc = glia_set_coefficients(spec_ops_->ctx_, tu.k_, tu.k_gm_wm_ratio_, tu.k_glm_wm_ratio_,
                                   tu.rho_, tu.r_gm_wm_ratio_, tu.r_glm_wm_ratio_);
    if (rc) return rc;
    std::vector<double> cm(3 * (size_t)tu.np_);
    if (centers) {
      cm = *centers;
    } else {
      rc = glia_phi_mesh(tu.np_, tu.user_cm_.data(), tu.phi_sigma_, tu.phi_spacing_factor_,
                         cm.data());
      if (rc) return rc;
    }
    return glia_set_phi(spec_ops_->ctx_, cm.data(), (int)(cm.size() / 3), tu.phi_sigma_,
                        tu.smoothing_factor_);
  }
  // Tumor::setSinusoidalCoefficients (src/mat/Tumor.cpp:102-112): sinusoidal tissue, then
  // k_->setValues and rho_->setValues from the parameters
  PetscErrorCode setSinusoidalCoefficients(std::shared_ptr<Parameters> params) {
    int rc = glia_set_tissue_sinusoidal(spec_ops_->ctx_);
    if (rc) return rc;
    auto& tu = *params->tu_;
    return glia_set_coefficients(spec_ops_->ctx_, tu.k_, tu.k_gm_wm_ratio_, tu.k_glm_wm_ratio_,
                                 tu.rho_, tu.r_gm_wm_ratio_, tu.r_glm_wm_ratio_);
  }
  Vec c_0_, c_t_, p_0_, p_t_;
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<SpectralOperators> spec_ops_;
};

inline glia_opt_settings to_opt(const Parameters& p, bool all_gradients = false) {
  glia_opt_settings s{};
  s.np = p.tu_->np_;
  s.nk = p.tu_->nk_;
  s.nr = p.tu_->nr_;
  s.flag_reaction_inv = p.opt_->flag_reaction_inv_;
  s.diffusivity_inversion = p.opt_->diffusivity_inversion_;
  s.regularization_norm = p.opt_->regularization_norm_;
  s.beta = p.opt_->beta_;
  s.k_scale = p.opt_->k_scale_;
  s.rho_scale = p.opt_->rho_scale_;
  s.phi_store = p.tu_->phi_store_;
  s.all_gradients = all_gradients;
  return s;
}

// PdeOperatorsRD (src/pde/PdeOperators.cpp)
class PdeOperatorsRD {
 public:
  PdeOperatorsRD(std::shared_ptr<Tumor> t, std::shared_ptr<Parameters> p,
                 std::shared_ptr<SpectralOperators> s)
      : tumor_(t), params_(p), spec_ops_(s) {
    auto& tu = *p->tu_;
    glia_set_time(s->ctx_, tu.dt_, tu.nt_, tu.order_);
    glia_set_history(s->ctx_, tu.time_history_off_ ? GLIA_HISTORY_OFF : p->engine_.history,
                     p->engine_.checkpoint_every, tu.adjoint_store_);
  }
  PetscErrorCode solveState(int linearized) {
    int rc = glia_solve_state(spec_ops_->ctx_, linearized, tumor_->c_0_.data(),
                              tumor_->c_t_.data());
    if (rc == GLIA_OK) diff_ksp_itr_state_ = (int)stats().diff_ksp_itr_state;
    return rc;
  }
  PetscErrorCode solveAdjoint(int linearized) {
    int rc = glia_solve_adjoint(spec_ops_->ctx_, linearized, tumor_->p_t_.data(),
                                tumor_->p_0_.data());
    if (rc == GLIA_OK) diff_ksp_itr_adj_ = (int)stats().diff_ksp_itr_adj;
    return rc;
  }
  glia_stats stats() const {
    glia_stats st{};
    glia_get_stats(spec_ops_->ctx_, &st);
    return st;
  }
  int diff_ksp_itr_state_ = 0, diff_ksp_itr_adj_ = 0;
  std::shared_ptr<Tumor> tumor_;
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<SpectralOperators> spec_ops_;
};

// Data (include/utils/Utils.h:99-124): the observations at t = 1 and (two snapshots) t = 0
struct Data {
  Vec t1, t0;
  const Vec& dt1() const { return t1; }
  const Vec& dt0() const { return t0; }
};

// DerivativeOperatorsRD (src/grad/DerivativeOperatorsRD.cpp)
class DerivativeOperatorsRD {
 public:
  DerivativeOperatorsRD(std::shared_ptr<PdeOperatorsRD> pde, std::shared_ptr<Parameters> p,
                        std::shared_ptr<Tumor> t)
      : pde_operators_(pde), params_(p), tumor_(t) {}
  // the optimizer settings and, when the parameters hold no p (flag_reaction_inv_: the
  // objective starts from Tumor::c_0_ instead of Phi p), the initial condition
  PetscErrorCode sync_settings() {
    glia_opt_settings s = to_opt(*params_, all_gradients_);
    int rc = glia_set_opt(ctx(), &s);
    if (!rc && params_->opt_->flag_reaction_inv_) rc = glia_set_c0(ctx(), tumor_->c_0_.data());
    return rc;
  }
  // DerivativeOperators::updateReactionAndDiffusion (src/grad/DerivativeOperators.cpp:323-367)
  // with DiffCoef / ReacCoef::updateIsotropicCoefficients (src/mat/DiffCoef.cpp:60-75,
  // src/mat/ReacCoef.cpp:40-50): k1 = x[np] k_scale, k2, k3 from x[np + 1], x[np + 2] when
  // nk > 1 (ratios k2 / k1, k3 / k1), else the parameters' ratios; rho likewise from x[np + nk]
  // under flag_reaction_inv_. Coefficients that are not inverted come from the parameters.
  PetscErrorCode updateReactionAndDiffusion(const Vec& x) {
    auto& tu = *params_->tu_;
    auto& op = *params_->opt_;
    const int np = tu.np_, nk = tu.nk_, nr = tu.nr_;
    if ((int)x.size() < np + nk + (op.flag_reaction_inv_ ? nr : 0)) return GLIA_ERR_INVALID;
    double k = tu.k_, kg = tu.k_gm_wm_ratio_, kc = tu.k_glm_wm_ratio_;
    if (op.diffusivity_inversion_ || op.flag_reaction_inv_) {
      k = x[np] * op.k_scale_;
      if (nk > 1) kg = x[np + 1] * op.k_scale_ / k;
      if (nk > 2) kc = x[np + 2] * op.k_scale_ / k;
    }
    double r = tu.rho_, rg = tu.r_gm_wm_ratio_, rc = tu.r_glm_wm_ratio_;
    if (op.flag_reaction_inv_) {
      r = x[np + nk] * op.rho_scale_;
      if (nr > 1) rg = x[np + nk + 1] * op.rho_scale_ / r;
      if (nr > 2) rc = x[np + nk + 2] * op.rho_scale_ / r;
    }
    return glia_set_coefficients(ctx(), k, kg, kc, r, rg, rc);
  }
  // the t = 0 data of the two-snapshot objective, or back to one snapshot
  PetscErrorCode sync_data(const Data& data) {
    const bool two = params_->tu_->two_time_points_ && !data.dt0().empty();
    return glia_set_data0(ctx(), two ? data.dt0().data() : nullptr);
  }
  PetscErrorCode evaluateObjective(ScalarType* J, const Vec& x, std::shared_ptr<Data> data) {
    int rc = sync_settings();
    if (!rc) rc = sync_data(*data);
    return rc ? rc : glia_eval_objective(ctx(), x.data(), (int)x.size(), data->dt1().data(), J);
  }
  PetscErrorCode evaluateGradient(Vec& dJ, const Vec& x, std::shared_ptr<Data> data) {
    int rc = sync_settings();
    if (!rc) rc = sync_data(*data);
    dJ.assign(x.size(), 0.0);
    return rc ? rc
              : glia_eval_gradient(ctx(), x.data(), (int)x.size(), data->dt1().data(), dJ.data());
  }
  PetscErrorCode evaluateObjectiveAndGradient(ScalarType* J, Vec& dJ, const Vec& x,
                                              std::shared_ptr<Data> data) {
    int rc = sync_settings();
    if (!rc) rc = sync_data(*data);
    dJ.assign(x.size(), 0.0);
    return rc ? rc
              : glia_eval_objective_and_gradient(ctx(), x.data(), (int)x.size(),
                                                 data->dt1().data(), J, dJ.data());
  }
  // DerivativeOperatorsRD::evaluateHessian(Vec y, Vec x) (src/grad/DerivativeOperatorsRD.cpp:
  // 229-438): the p block, or the p and kappa blocks with diffusivity inversion, linearised at
  // the last evaluation
  PetscErrorCode evaluateHessian(Vec& y, const Vec& x) {
    int rc = sync_settings();
    y.assign(x.size(), 0.0);
    return rc ? rc : glia_hessian_matvec(ctx(), x.data(), (int)x.size(), y.data());
  }
  glia_ctx* ctx() const { return pde_operators_->spec_ops_->ctx_; }
  bool all_gradients_ = false;  // extension: p, kappa and rho gradients in one sweep
  std::shared_ptr<PdeOperatorsRD> pde_operators_;
  std::shared_ptr<Parameters> params_;
  std::shared_ptr<Tumor> tumor_;
};

}  // namespace glia_shim

// engine.hpp — type-erased interface between the C-ABI (capi.cu) and the templated engines.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/glia_rd.h"

namespace glia {

class EngineBase {
 public:
  virtual ~EngineBase() = default;
  virtual void set_pointer_mode(int mode) = 0;
  virtual void set_stream(void* s) = 0;
  virtual void synchronize() = 0;
  virtual void set_launch_geometry(int pw_per_sm, int red_per_sm) = 0;
  virtual int64_t device_bytes() const = 0;
  virtual void set_time(double dt, int nt, int order) = 0;
  virtual void set_pcg(double rtol, int maxit, int pc_dt_mode, double pc_dt) = 0;
  virtual void set_history(int mode, int every, int adjoint_store) = 0;
  virtual void set_opt(const glia_opt_settings& s) = 0;
  virtual void set_tissue(const void* wm, const void* gm, const void* csf, const void* vt) = 0;
  virtual void set_tissue_sinusoidal() = 0;
  virtual void set_coefficients(double k, double kgm, double kglm, double rho, double rgm,
                                double rglm) = 0;
  virtual void set_diffusivity_sinusoidal(double scale) = 0;
  virtual void prec_factor() = 0;
  virtual int diffusion_solve(void* c, double dt) = 0;  // returns ksp iterations
  virtual void apply_d(const void* c, void* dc) = 0;
  virtual void smooth(void* out, const void* in, double sigma) = 0;
  virtual void set_phi(const double* centers, int np, double sigma, double smoothing_factor) = 0;
  virtual void phi_apply(const double* p, void* c0) = 0;
  virtual void phi_apply_transpose(const void* v, double* pout) = 0;
  virtual void phi_data_centers(const void* data, double sigma, double thr, double gvf,
                                double spacing_factor, int max_centers, double* centers,
                                int* np_out, void* frac) = 0;
  virtual void set_obs_threshold(const void* data, double thr) = 0;
  virtual void set_obs_filter(const void* f) = 0;
  virtual void set_obs_threshold0(const void* data, double thr) = 0;
  virtual void set_obs_filter0(const void* f) = 0;
  virtual void set_data0(const void* d0) = 0;
  virtual void set_c0(const void* c0) = 0;
  virtual void set_secondary_coefficients(double k1, double k2, double k3) = 0;
  virtual void solve_state(int linearized, const void* c0, void* c1) = 0;
  virtual void solve_adjoint(int linearized, const void* pt, void* a0) = 0;
  virtual void hessian_matvec(const double* x, int nx, double* y) = 0;
  virtual void get_state(int i, void* out) = 0;
  virtual void get_adjoint(int i, void* out) = 0;
  virtual void evaluate(const double* x, int nx, const void* d1, double* J, double* dJ) = 0;
  // An evaluation split for CUDA-graph capture (batches): eval_prepare does the host-dependent
  // part for x and d1 (coefficients, Phi p, data upload); eval_capture enqueues the forward,
  // residual, adjoint and gradient sweeps on the context's stream while that stream is being
  // captured, with no host synchronisation; eval_finish reads the results after the captured
  // graph has run.
  virtual void eval_prepare(const double* x, int nx, const void* d1) = 0;
  virtual void eval_capture() = 0;
  virtual void eval_finish(double* J, double* dJ) = 0;
  virtual void* stream() const = 0;
  virtual glia_stats stats() const = 0;
  virtual void selftest_bounded_wait() = 0;
  virtual void reset_stats() = 0;
  virtual void set_timing(bool on) = 0;
  virtual int timing(int slot, const char** name, int64_t* launches, double* ms,
                     double* bytes) = 0;
};

EngineBase* make_engine_f32(int n, bool reference_structured);
EngineBase* make_engine_f64(int n, bool reference_structured);

}  // namespace glia

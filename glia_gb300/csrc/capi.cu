// capi.cu — the extern "C" boundary declared in include/glia_rd.h. Every entry point catches
// all exceptions, stores the message on the context and returns a status code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.hpp"

struct glia_ctx {
  std::unique_ptr<glia::EngineBase> eng;
  std::string err;
  int precision = GLIA_FP64;
  int engine = GLIA_ENGINE_FUSED;
};

namespace {

template <class F>
int guarded(glia_ctx* ctx, F&& f) {
  if (!ctx || !ctx->eng) return GLIA_ERR_INVALID;
  try {
    f(*ctx->eng);
    return GLIA_OK;
  } catch (const glia::Error& e) {
    ctx->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    ctx->err = "host allocation failed";
    return GLIA_ERR_OOM;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return GLIA_ERR_INVALID;
  }
}

}  // namespace

extern "C" {

const char* glia_version(void) { return "glia-gb300 0.1 (sm_103a; cuFFT transforms)"; }

int glia_create(int n, int precision, int engine, glia_ctx** out) {
  if (!out) return GLIA_ERR_INVALID;
  *out = nullptr;
  if (n < 8 || n > 1024 || (n % 8) != 0) return GLIA_ERR_INVALID;
  if (precision != GLIA_FP64 && precision != GLIA_MIXED) return GLIA_ERR_INVALID;
  if (engine != GLIA_ENGINE_FUSED && engine != GLIA_ENGINE_REFERENCE) return GLIA_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return GLIA_ERR_NO_DEVICE;
  }
  glia_ctx* ctx = new (std::nothrow) glia_ctx();
  if (!ctx) return GLIA_ERR_OOM;
  ctx->precision = precision;
  ctx->engine = engine;
  try {
    const bool ref = engine == GLIA_ENGINE_REFERENCE;
    ctx->eng.reset(precision == GLIA_MIXED ? glia::make_engine_f32(n, ref)
                                           : glia::make_engine_f64(n, ref));
  } catch (const glia::Error& e) {
    delete ctx;
    return e.code;
  } catch (...) {
    delete ctx;
    return GLIA_ERR_OOM;
  }
  *out = ctx;
  return GLIA_OK;
}

int glia_destroy(glia_ctx* ctx) {
  if (!ctx) return GLIA_ERR_INVALID;
  try {
    ctx->eng.reset();
  } catch (...) {
  }
  delete ctx;
  return GLIA_OK;
}

const char* glia_last_error(const glia_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int glia_set_pointer_mode(glia_ctx* ctx, int mode) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_pointer_mode(mode); });
}
int glia_set_stream(glia_ctx* ctx, void* s) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_stream(s); });
}
int glia_set_launch_geometry(glia_ctx* ctx, int pointwise_blocks_per_sm,
                             int reduce_blocks_per_sm) {
  return guarded(ctx, [&](glia::EngineBase& e) {
    e.set_launch_geometry(pointwise_blocks_per_sm, reduce_blocks_per_sm);
  });
}
int glia_synchronize(glia_ctx* ctx) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.synchronize(); });
}
int glia_device_bytes(const glia_ctx* ctx, int64_t* bytes) {
  if (!ctx || !ctx->eng || !bytes) return GLIA_ERR_INVALID;
  *bytes = ctx->eng->device_bytes();
  return GLIA_OK;
}
int glia_set_time(glia_ctx* ctx, double dt, int nt, int order) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_time(dt, nt, order); });
}
int glia_set_pcg(glia_ctx* ctx, double rtol, int maxit, int pc_dt_mode, double pc_dt) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_pcg(rtol, maxit, pc_dt_mode, pc_dt); });
}
int glia_set_history(glia_ctx* ctx, int mode, int every, int adjoint_store) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_history(mode, every, adjoint_store); });
}
int glia_set_opt(glia_ctx* ctx, const glia_opt_settings* s) {
  if (!s) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_opt(*s); });
}
int glia_set_tissue(glia_ctx* ctx, const void* wm, const void* gm, const void* csf,
                    const void* vt) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_tissue(wm, gm, csf, vt); });
}
int glia_set_tissue_sinusoidal(glia_ctx* ctx) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_tissue_sinusoidal(); });
}
int glia_set_coefficients(glia_ctx* ctx, double k, double k_gm_wm, double k_glm_wm, double rho,
                          double r_gm_wm, double r_glm_wm) {
  return guarded(ctx, [&](glia::EngineBase& e) {
    e.set_coefficients(k, k_gm_wm, k_glm_wm, rho, r_gm_wm, r_glm_wm);
  });
}
int glia_set_diffusivity_sinusoidal(glia_ctx* ctx, double scale) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_diffusivity_sinusoidal(scale); });
}
int glia_prec_factor(glia_ctx* ctx) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.prec_factor(); });
}
int glia_diffusion_solve(glia_ctx* ctx, void* c, double dt, int* ksp_itr) {
  if (!c) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) {
    int its = e.diffusion_solve(c, dt);
    if (ksp_itr) *ksp_itr = its;
  });
}
int glia_apply_d(glia_ctx* ctx, const void* c, void* dc) {
  if (!c || !dc) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.apply_d(c, dc); });
}
int glia_smooth(glia_ctx* ctx, void* out, const void* in, double sigma) {
  if (!out || !in) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.smooth(out, in, sigma); });
}

// Phi::phiMesh (src/mat/Phi.cpp:148-234): cubic lattice of np = h^3 centres around cm; odd h is
// centred on cm, even h is offset by half a spacing.
int glia_phi_mesh(int np, const double cm[3], double sigma, double spacing_factor,
                  double* center) {
  if (np < 1 || !cm || !center) return GLIA_ERR_INVALID;
  const int h = (int)std::lround(std::pow((double)np, 1.0 / 3.0));
  const double space = spacing_factor * sigma;
  if (np == 1) {
    center[0] = cm[0];
    center[1] = cm[1];
    center[2] = cm[2];
    return GLIA_OK;
  }
  if (h * h * h != np) return GLIA_ERR_INVALID;
  int ptr = 0;
  if (np % 2 == 1) {
    for (int k = -(h - 1) / 2; k <= (h - 1) / 2; k++)
      for (int j = -(h - 1) / 2; j <= (h - 1) / 2; j++)
        for (int i = -(h - 1) / 2; i <= (h - 1) / 2; i++) {
          center[ptr + 0] = i * space + cm[0];
          center[ptr + 1] = j * space + cm[1];
          center[ptr + 2] = k * space + cm[2];
          ptr += 3;
        }
  } else {
    for (int k = -h / 2; k <= h / 2; k++)
      for (int j = -h / 2; j <= h / 2; j++)
        for (int i = -h / 2; i <= h / 2; i++) {
          if (i == 0 || j == 0 || k == 0) continue;
          const double m0 = (i < 0 ? -0.5 : 0.5), m1 = (j < 0 ? -0.5 : 0.5),
                       m2 = (k < 0 ? -0.5 : 0.5);
          center[ptr + 0] = (i - m0) * space + cm[0];
          center[ptr + 1] = (j - m1) * space + cm[1];
          center[ptr + 2] = (k - m2) * space + cm[2];
          ptr += 3;
        }
  }
  return GLIA_OK;
}
int glia_set_phi(glia_ctx* ctx, const double* centers, int np, double sigma,
                 double smoothing_factor) {
  if (!centers) return GLIA_ERR_INVALID;
  return guarded(ctx,
                 [&](glia::EngineBase& e) { e.set_phi(centers, np, sigma, smoothing_factor); });
}
int glia_phi_apply(glia_ctx* ctx, const double* p, void* c0) {
  if (!p || !c0) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.phi_apply(p, c0); });
}
int glia_phi_data_centers(glia_ctx* ctx, const void* data, double sigma, double data_threshold,
                          double gaussian_vol_frac, double spacing_factor, int max_centers,
                          double* centers, int* np_out, void* frac) {
  if (!data || !np_out || (max_centers > 0 && !centers) || max_centers < 0)
    return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) {
    e.phi_data_centers(data, sigma, data_threshold, gaussian_vol_frac, spacing_factor,
                       max_centers, centers, np_out, frac);
  });
}
int glia_phi_apply_transpose(glia_ctx* ctx, const void* v, double* pout) {
  if (!v || !pout) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.phi_apply_transpose(v, pout); });
}
int glia_set_obs_threshold(glia_ctx* ctx, const void* data, double thr) {
  if (!data) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_obs_threshold(data, thr); });
}
int glia_set_obs_filter(glia_ctx* ctx, const void* f) {
  if (!f) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_obs_filter(f); });
}
int glia_set_obs_threshold0(glia_ctx* ctx, const void* data, double thr) {
  if (!data) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_obs_threshold0(data, thr); });
}
int glia_set_obs_filter0(glia_ctx* ctx, const void* f) {
  if (!f) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_obs_filter0(f); });
}
int glia_set_data0(glia_ctx* ctx, const void* d0) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_data0(d0); });
}
int glia_set_c0(glia_ctx* ctx, const void* c0) {
  if (!c0) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_c0(c0); });
}
int glia_set_secondary_coefficients(glia_ctx* ctx, double k1, double k2, double k3) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_secondary_coefficients(k1, k2, k3); });
}
int glia_solve_state(glia_ctx* ctx, int linearized, const void* c0, void* c1) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.solve_state(linearized, c0, c1); });
}
int glia_solve_adjoint(glia_ctx* ctx, int linearized, const void* pt, void* a0) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.solve_adjoint(linearized, pt, a0); });
}
int glia_selftest_bounded_wait(glia_ctx* ctx) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.selftest_bounded_wait(); });
}
int glia_hessian_matvec(glia_ctx* ctx, const double* x, int nx, double* y) {
  if (!x || !y) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.hessian_matvec(x, nx, y); });
}
int glia_get_state(glia_ctx* ctx, int i, void* out) {
  if (!out) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.get_state(i, out); });
}
int glia_get_adjoint(glia_ctx* ctx, int i, void* out) {
  if (!out) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.get_adjoint(i, out); });
}
int glia_eval_objective(glia_ctx* ctx, const double* x, int nx, const void* d1, double* J) {
  if (!x || !d1 || !J) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.evaluate(x, nx, d1, J, nullptr); });
}
int glia_eval_gradient(glia_ctx* ctx, const double* x, int nx, const void* d1, double* dJ) {
  if (!x || !d1 || !dJ) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.evaluate(x, nx, d1, nullptr, dJ); });
}
int glia_eval_objective_and_gradient(glia_ctx* ctx, const double* x, int nx, const void* d1,
                                     double* J, double* dJ) {
  if (!x || !d1 || !J || !dJ) return GLIA_ERR_INVALID;
  return guarded(ctx, [&](glia::EngineBase& e) { e.evaluate(x, nx, d1, J, dJ); });
}
int glia_get_stats(const glia_ctx* ctx, glia_stats* st) {
  if (!ctx || !ctx->eng || !st) return GLIA_ERR_INVALID;
  *st = ctx->eng->stats();
  return GLIA_OK;
}
int glia_reset_stats(glia_ctx* ctx) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.reset_stats(); });
}
int glia_set_timing(glia_ctx* ctx, int enable) {
  return guarded(ctx, [&](glia::EngineBase& e) { e.set_timing(enable != 0); });
}
int glia_get_timing(glia_ctx* ctx, int slot, const char** name, int64_t* launches, double* ms,
                    double* algorithmic_bytes) {
  int count = 0;
  int rc = guarded(ctx, [&](glia::EngineBase& e) {
    count = e.timing(slot, name, launches, ms, algorithmic_bytes);
  });
  return rc == GLIA_OK ? count : rc;
}

}  // extern "C"

// ---- batches of evaluations in one CUDA graph ------------------------------------------------
struct glia_batch {
  std::vector<glia_ctx*> ctxs;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t root = nullptr;
  std::vector<cudaEvent_t> events;
  std::string err;
  ~glia_batch() { release(); }
  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    events.clear();
  }
  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      throw glia::Error(GLIA_ERR_CUDA, "cudaEventCreateWithFlags failed");
    events.push_back(e);
    return e;
  }
};

namespace {

#define BATCH_CUDA(call)                                                                  \
  do {                                                                                    \
    const cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) throw glia::Error(GLIA_ERR_CUDA, std::string(#call) + ": " +     \
                                                                cudaGetErrorString(e_));  \
  } while (0)

template <class F>
int batch_guarded(glia_batch* b, F&& f) {
  if (!b) return GLIA_ERR_INVALID;
  try {
    f();
    return GLIA_OK;
  } catch (const glia::Error& e) {
    b->err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    b->err = "host allocation failed";
    return GLIA_ERR_OOM;
  } catch (const std::exception& e) {
    b->err = e.what();
    return GLIA_ERR_INVALID;
  }
}

}  // namespace

extern "C" {

int glia_batch_create(glia_ctx* const* ctxs, int n, glia_batch** out) {
  if (!out) return GLIA_ERR_INVALID;
  *out = nullptr;
  if (!ctxs || n < 1) return GLIA_ERR_INVALID;
  for (int i = 0; i < n; i++)
    if (!ctxs[i] || !ctxs[i]->eng) return GLIA_ERR_INVALID;
  glia_batch* b = new (std::nothrow) glia_batch();
  if (!b) return GLIA_ERR_OOM;
  b->ctxs.assign(ctxs, ctxs + n);
  if (cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return GLIA_ERR_CUDA;
  }
  *out = b;
  return GLIA_OK;
}

int glia_batch_capture(glia_batch* b, const double* const* x, const int* nx,
                       const void* const* d1, const int* group) {
  if (!b || !x || !nx || !d1) return GLIA_ERR_INVALID;
  return batch_guarded(b, [&] {
    const int n = (int)b->ctxs.size();
    b->release();
    // host part of every evaluation (coefficients, Phi p, data), outside the capture
    for (int i = 0; i < n; i++) {
      glia_ctx* c = b->ctxs[i];
      if (!x[i] || !d1[i]) throw glia::Error(GLIA_ERR_INVALID, "null x or d1");
      if (!c->eng->stream())
        throw glia::Error(GLIA_ERR_INVALID, "contexts of a batch need a non-default stream");
      try {
        c->eng->eval_prepare(x[i], nx[i], d1[i]);
      } catch (const glia::Error& e) {
        c->err = e.what();
        throw glia::Error(e.code, "context " + std::to_string(i) + ": " + e.what());
      }
    }
    std::map<int, std::vector<int>> groups;
    for (int i = 0; i < n; i++) groups[group ? group[i] : 0].push_back(i);
    BATCH_CUDA(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeRelaxed));
    cudaGraph_t graph = nullptr;
    try {
      cudaEvent_t start = b->event();
      BATCH_CUDA(cudaEventRecord(start, b->root));
      for (auto& kv : groups) {
        for (int i : kv.second) {
          glia_ctx* c = b->ctxs[i];
          cudaStream_t s = static_cast<cudaStream_t>(c->eng->stream());
          BATCH_CUDA(cudaStreamWaitEvent(s, start, 0));  // fork: the branch joins the capture
          try {
            c->eng->eval_capture();
          } catch (const glia::Error& e) {
            c->err = e.what();
            throw glia::Error(e.code, "context " + std::to_string(i) + ": " + e.what());
          }
          cudaEvent_t done = b->event();
          BATCH_CUDA(cudaEventRecord(done, s));
          BATCH_CUDA(cudaStreamWaitEvent(b->root, done, 0));  // join
        }
        start = b->event();  // the next group starts when this one is done
        BATCH_CUDA(cudaEventRecord(start, b->root));
      }
      BATCH_CUDA(cudaStreamEndCapture(b->root, &graph));
    } catch (...) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(b->root, &junk);
      if (junk) cudaGraphDestroy(junk);
      cudaGetLastError();
      throw;
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      b->exec = nullptr;
      throw glia::Error(GLIA_ERR_CUDA, std::string("cudaGraphInstantiate: ") +
                                           cudaGetErrorString(ie));
    }
  });
}

int glia_batch_launch(glia_batch* b, void* stream) {
  if (!b) return GLIA_ERR_INVALID;
  return batch_guarded(b, [&] {
    if (!b->exec) throw glia::Error(GLIA_ERR_STATE, "no captured batch graph");
    BATCH_CUDA(cudaGraphLaunch(b->exec, stream ? static_cast<cudaStream_t>(stream) : b->root));
  });
}

int glia_batch_results(glia_batch* b, void* stream, double* J, double* const* dJ) {
  if (!b || !J) return GLIA_ERR_INVALID;
  return batch_guarded(b, [&] {
    BATCH_CUDA(cudaStreamSynchronize(stream ? static_cast<cudaStream_t>(stream) : b->root));
    for (size_t i = 0; i < b->ctxs.size(); i++) {
      glia_ctx* c = b->ctxs[i];
      try {
        c->eng->eval_finish(&J[i], dJ ? dJ[i] : nullptr);
      } catch (const glia::Error& e) {
        c->err = e.what();
        throw glia::Error(e.code, "context " + std::to_string(i) + ": " + e.what());
      }
    }
  });
}

const char* glia_batch_last_error(const glia_batch* b) { return b ? b->err.c_str() : "null batch"; }

int glia_batch_destroy(glia_batch* b) {
  if (!b) return GLIA_ERR_INVALID;
  if (b->root) cudaStreamSynchronize(b->root);
  b->release();
  if (b->root) cudaStreamDestroy(b->root);
  delete b;
  cudaGetLastError();
  return GLIA_OK;
}

}  // extern "C"

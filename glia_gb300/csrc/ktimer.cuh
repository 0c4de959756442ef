// ktimer.cuh — opt-in per-kernel device time with CUDA events on the launching stream.
//
// When enabled, each instrumented launch is bracketed by two events; the elapsed times are
// harvested after the stream has been synchronised (the engine synchronises once per PCG
// iteration anyway), so the timer adds no synchronisation of its own. Each slot also accumulates
// the algorithmic bytes its launches move (reads + writes of the arrays they must touch).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace glia {

enum KSlot {
  KS_SPEC_GRAD3_CG = 0,  // k_spec_grad3<CGDIR>: new PCG direction + gradient spectra
  KS_SPEC_GRAD3,         // k_spec_grad3: gradient spectra (solve set-up, D apply)
  KS_MUL_K3,             // k_mul_k3: k * grad
  KS_DIV_SETUP,          // k_spec_div<EPI_SETUP>
  KS_DIV_CGW,            // k_spec_div<EPI_CGW>
  KS_DIV_APPLYD,         // k_spec_div<EPI_APPLYD>
  KS_CG_UPDATE,          // k_cg_update
  KS_REACTION,           // k_reaction_fwd
  KS_REACTION_LIN,       // k_reaction_lin
  KS_GRAD_ACC,           // k_grad_rho_acc / k_grad_kappa_acc
  KS_OBS,                // k_obs_residual
  KS_PHI,                // k_phi_apply / k_phi_applyT
  KS_COPY,               // device-to-device copies (history, checkpoints)
  KS_FFT_R2C,            // cuFFT R2C/D2Z, single transform
  KS_FFT_C2R,            // cuFFT C2R/Z2D, single transform
  KS_FFT_R2C3,           // cuFFT R2C/D2Z, batch of 3
  KS_FFT_C2R3,           // cuFFT C2R/Z2D, batch of 3
  KS_REF_VEC,            // reference-structured vector kernels (axpy, pointwise, wave number)
  KS_REF_DOT,            // reference-structured inner products
  KS_ZPASS,              // k_zpass_mulk: fused z C2R, k multiply, z R2C
  KS_FFT_2D,             // cuFFT 2-D C2C over (x, y) for every kz
  KS_XINV,               // k_xinv: PCG direction, gradient spectra, inverse x transforms
  KS_XFWD_SETUP,         // k_xfwd<EPI_SETUP>: forward x transforms, divergence, solve set-up
  KS_XFWD_CGW,           // k_xfwd<EPI_CGW>: forward x transforms, divergence, w = A p
  KS_XFWD_APPLYD,        // k_xfwd<EPI_APPLYD>: forward x transforms, divergence, D u
  KS_YINV,               // k_yinv_bulk (or k_yinv): inverse y transforms, packed kz = 0 / n/2
  KS_ZFUSED,             // k_zpass2 (or k_zpass): z C2R, k multiply, z R2C per line
  KS_YFWD,               // k_yfwd: forward y transforms, unpacking
  KS_COUNT
};

static const char* const kSlotNames[KS_COUNT] = {
    "k_spec_grad3_cgdir", "k_spec_grad3",   "k_mul_k3",        "k_spec_div_setup",
    "k_spec_div_cgw",     "k_spec_div_applyd", "k_cg_update",   "k_reaction_fwd",
    "k_reaction_lin",     "k_grad_acc",     "k_obs_residual",  "k_phi",
    "copy_d2d",           "cufft_r2c",      "cufft_c2r",       "cufft_r2c_x3",
    "cufft_c2r_x3",       "ref_vector_ops", "ref_dot",         "k_zpass_mulk",
    "cufft_c2c_2d",       "k_xinv",         "k_xfwd_setup",    "k_xfwd_cgw",
    "k_xfwd_applyd",      "k_yinv_bulk",    "k_zpass2",         "k_yfwd"};

struct KTimer {
  bool on = false;
  struct Slot {
    int64_t launches = 0;
    double ms = 0, bytes = 0;
  };
  Slot slots[KS_COUNT];
  struct Pending {
    int slot;
    cudaEvent_t a, b;
    double bytes;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;

  ~KTimer() {
    for (auto& p : pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
  }
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t begin(cudaStream_t s) {
    if (!on) return nullptr;
    cudaEvent_t a = take();
    cudaEventRecord(a, s);
    return a;
  }
  void end(int slot, cudaEvent_t a, double bytes, cudaStream_t s) {
    if (!on || !a) return;
    cudaEvent_t b = take();
    cudaEventRecord(b, s);
    pending.push_back({slot, a, b, bytes});
  }
  // call only after the stream has been synchronised
  void harvest() {
    for (auto& p : pending) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
        slots[p.slot].launches++;
        slots[p.slot].ms += ms;
        slots[p.slot].bytes += p.bytes;
      }
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
  }
  void reset() {
    for (auto& p : pending) {
      pool.push_back(p.a);
      pool.push_back(p.b);
    }
    pending.clear();
    for (auto& s : slots) s = Slot{};
  }
};

}  // namespace glia

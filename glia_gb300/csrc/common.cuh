// common.cuh — shared types, error handling and index helpers of the GLIA RD CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/glia_rd.h"

namespace glia {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define GLIA_CUDA(call)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      int code_ = (e_ == cudaErrorMemoryAllocation) ? GLIA_ERR_OOM : GLIA_ERR_CUDA;        \
      throw ::glia::Error(code_, std::string(#call) + " failed: " + cudaGetErrorString(e_)); \
    }                                                                                      \
  } while (0)

#define GLIA_CUFFT(call)                                                             \
  do {                                                                               \
    cufftResult r_ = (call);                                                         \
    if (r_ != CUFFT_SUCCESS)                                                         \
      throw ::glia::Error(r_ == CUFFT_ALLOC_FAILED ? GLIA_ERR_OOM : GLIA_ERR_CUFFT,  \
                          std::string(#call) + " failed: cufftResult " +             \
                              std::to_string((int)r_));                              \
  } while (0)

#define GLIA_LAUNCH_CHECK() GLIA_CUDA(cudaPeekAtLastError())

template <typename R>
struct CT;
template <>
struct CT<float> {
  using C = float2;
  static constexpr cufftType kR2C = CUFFT_R2C;
  static constexpr cufftType kC2R = CUFFT_C2R;
};
template <>
struct CT<double> {
  using C = double2;
  static constexpr cufftType kR2C = CUFFT_D2Z;
  static constexpr cufftType kC2R = CUFFT_Z2D;
};

// Unsigned 32-bit division by a run-time constant through a multiply-high and a shift
// (round-up reciprocal method of Granlund & Montgomery, 1994). Exact for dividends < 2^31.
struct FastDiv {
  uint32_t d = 1, mul = 0, shr = 0;
  FastDiv() = default;
  explicit FastDiv(uint32_t div) : d(div) {
    uint32_t l = 0;
    while ((1ull << l) < div) l++;
    if (div == 1) {
      mul = 0;
      shr = 0;
    } else {
      uint64_t p = 31 + l;
      mul = (uint32_t)(((1ull << p) + div - 1) / div);
      shr = (uint32_t)(p - 32);
    }
  }
  __host__ __device__ __forceinline__ uint32_t div(uint32_t x) const {
#ifdef __CUDA_ARCH__
    return d == 1 ? x : (__umulhi(x, mul) >> shr);
#else
    return d == 1 ? x : (uint32_t)(((uint64_t)x * mul) >> 32) >> shr;
#endif
  }
};

// Geometry of the n^3 grid and its half spectrum (n, n, n/2+1), row-major, z fastest.
struct Geo {
  int n = 0, nh = 0;
  int64_t N = 0, Ns = 0;
  FastDiv fd_nh, fd_n;
  double invN = 0;
  Geo() = default;
  explicit Geo(int n_) : n(n_), nh(n_ / 2 + 1) {
    N = (int64_t)n * n * n;
    Ns = (int64_t)n * n * nh;
    fd_nh = FastDiv((uint32_t)nh);
    fd_n = FastDiv((uint32_t)n);
    invN = 1.0 / (double)N;
  }
};

// wave number of index K along a dimension of size n, Nyquist set to zero
// (src/cuda/SpectralOperators.cu:74-81).
__device__ __forceinline__ int wavenum(int K, int n) {
  const int h = n >> 1;
  return K < h ? K : (K == h ? 0 : K - n);
}

// Decomposes a half-spectrum element index e into (wx, wy, wz) and its Parseval multiplicity
// (1 on the kz = 0 and kz = n/2 planes, 2 elsewhere).
struct SpecIdx {
  int wx, wy, wz;
  double mult;
};
__device__ __forceinline__ SpecIdx spec_index(uint32_t e, const Geo& g) {
  uint32_t xy = g.fd_nh.div(e);
  uint32_t z = e - xy * (uint32_t)g.nh;
  uint32_t x = g.fd_n.div(xy);
  uint32_t y = xy - x * (uint32_t)g.n;
  SpecIdx s;
  s.wx = wavenum((int)x, g.n);
  s.wy = wavenum((int)y, g.n);
  s.wz = wavenum((int)z, g.n);
  s.mult = (z == 0 || (int)z == g.n / 2) ? 1.0 : 2.0;
  return s;
}

}  // namespace glia

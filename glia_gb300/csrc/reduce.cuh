// reduce.cuh — deterministic FP64 reductions for bandwidth-bound passes.
//
// Every reducing kernel runs a fixed number of blocks (grid-stride loops), folds its values with
// warp shuffles into one partial per block, and the last block to finish (atomic ticket) sums the
// partials in a fixed order and runs the kernel's scalar epilogue. The result does not depend on
// block scheduling, and no block ever waits on another.
#pragma once

#include "common.cuh"

namespace glia {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

// Sum of Q doubles over the block; the result is valid in thread 0. Uses shared memory `sh`.
template <int Q>
__device__ __forceinline__ void block_sum(double (&v)[Q], double (*sh)[kWarps]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    v[q] = x;
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < Q; q++) sh[q][warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < Q; q++) {
      double x = lane < kWarps ? sh[q][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[q] = x;
    }
  }
}

// Per-launch reduction workspace: partials[gridDim.x * Q] and one ticket counter (zero at rest).
struct RedWs {
  double* partials;
  unsigned int* counter;
};

// Returns true in the last block, where thread 0 holds the grid-wide sums in v.
template <int Q>
__device__ __forceinline__ bool grid_sum_last(double (&v)[Q], RedWs ws) {
  __shared__ double sh[Q][kWarps];
  __shared__ bool am_last;
  block_sum<Q>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < Q; q++) ws.partials[blockIdx.x * Q + q] = v[q];
    __threadfence();
    unsigned int t = atomicAdd(ws.counter, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double s[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) s[q] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
    for (int q = 0; q < Q; q++) s[q] += __ldcg(&ws.partials[b * Q + q]);
  }
  block_sum<Q>(s, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < Q; q++) v[q] = s[q];
    *ws.counter = 0u;
  }
  return true;
}

// Per-thread accumulator. For float data the terms are summed in FP32 with Kahan compensation
// (four FP32 operations per term, accurate to O(eps_32^2) of the summed magnitude), then widened
// to FP64 for the warp / block / grid combine. This keeps the FP64 units, which are scarce on
// GB300, out of the per-element path while the reduction stays at double-length accuracy.
template <typename R>
struct Acc;
template <>
struct Acc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};

// 16-byte vector access to real arrays.
template <typename R>
struct V16;
template <>
struct V16<float> {
  static constexpr int K = 4;
  __device__ __forceinline__ static void ld(const float* p, float (&v)[4]) {
    float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
  }
  __device__ __forceinline__ static void st(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct V16<double> {
  static constexpr int K = 2;
  __device__ __forceinline__ static void ld(const double* p, double (&v)[2]) {
    double2 t = *reinterpret_cast<const double2*>(p);
    v[0] = t.x;
    v[1] = t.y;
  }
  __device__ __forceinline__ static void st(double* p, const double (&v)[2]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
};

}  // namespace glia

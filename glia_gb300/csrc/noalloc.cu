// noalloc.cu — a data-mismatch reduction that allocates nothing.
//
// Some callers cannot let a library call cudaMalloc: code that records its loss evaluation into
// a CUDA graph (allocation is not allowed while a stream is being captured), processes that run
// under a fixed device-memory budget owned by their own allocator, and callers that have no glia
// context at all. glia_mismatch_f32_noalloc serves them: it computes the data term of
// DerivativeOperatorsRD (sum of (O c - d)^2 and, optionally, the adjoint final condition
// pt = -O^T (O c - d)) with the reduction scratch held in one file-scope __device__ array.
//
// The scratch is one FP64 partial per tile of kTile voxels plus a ticket counter, so a call
// handles at most kMaxTiles * kTile voxels (2^29); larger inputs are rejected. Every call on a
// device shares the same array and leaves its last contents behind; the counter is cleared at
// the start of every call. Calls that overlap on the GPU (different streams running at the same
// time) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/glia_rd.h"
#include "reduce.cuh"

namespace {

constexpr int kTile = 65536;       // voxels per block (and per FP64 partial)
constexpr int kMaxTiles = 8192;    // partials held by the scratch array
constexpr int kMaxDevices = 64;

struct NoallocScratch {
  double partials[kMaxTiles];
  unsigned int counter;
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device, resolved once per device (with that device
// current) by cudaGetSymbolAddress; host code never hands the symbol itself to a kernel.
NoallocScratch* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

__global__ void __launch_bounds__(glia::kThreads)
    k_mismatch_noalloc(const float* __restrict__ c, const float* __restrict__ O,
                       const float* __restrict__ d, float* __restrict__ pt, int64_t n,
                       NoallocScratch* __restrict__ scratch, double* __restrict__ sumsq) {
  const int64_t lo = (int64_t)blockIdx.x * kTile;
  const int64_t hi = lo + kTile < n ? lo + kTile : n;
  glia::Acc<float> acc;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const float r = c[i] * O[i] - d[i];
    acc.add(r * r);
    if (pt) pt[i] = -(r * O[i]);
  }
  double v[1] = {acc.value()};
  glia::RedWs ws{scratch->partials, &scratch->counter};
  if (!glia::grid_sum_last<1>(v, ws)) return;
  if (threadIdx.x == 0) *sumsq = v[0];
}

}  // namespace

extern "C" int glia_mismatch_f32_noalloc(const float* c, const float* obs, const float* d,
                                         float* pt, int64_t n, double* sumsq, void* stream) {
  if (!c || !obs || !d || !sumsq || n < 1) return GLIA_ERR_INVALID;
  if (n > (int64_t)kMaxTiles * kTile) return GLIA_ERR_INVALID;  // beyond the scratch capacity
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return GLIA_ERR_NO_DEVICE;
  }
  NoallocScratch* scratch;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return GLIA_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<NoallocScratch*>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(&scratch->counter, 0, sizeof(unsigned int), s) != cudaSuccess) {
    cudaGetLastError();
    return GLIA_ERR_CUDA;
  }
  const unsigned int blocks = (unsigned int)((n + kTile - 1) / kTile);
  k_mismatch_noalloc<<<blocks, glia::kThreads, 0, s>>>(c, obs, d, pt, n, scratch, sumsq);
  if (cudaPeekAtLastError() != cudaSuccess) {
    cudaGetLastError();
    return GLIA_ERR_CUDA;
  }
  return GLIA_OK;
}

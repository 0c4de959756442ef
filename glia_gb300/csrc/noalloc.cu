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
// time) race on the array and must be serialised by the caller. The array's address is looked
// up once per CUDA context, on the first call made with that context current; that first call
// must come before any stream capture.
#include <cuda.h>
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

// Device address of g_noalloc_scratch, resolved by cudaGetSymbolAddress once per CUDA context
// (with that context current) and cached under the context's process-unique ID, so that a
// non-primary context on the same device, or a primary context re-created after
// cudaDeviceReset, resolves its own module instance instead of reusing a stale address.
constexpr int kMaxContexts = 4 * kMaxDevices;
struct ScratchEntry {
  unsigned long long ctx_id;
  NoallocScratch* addr;
};
ScratchEntry g_scratch_cache[kMaxContexts];
int g_scratch_count = 0;
std::mutex g_scratch_mu;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// ID of the current CUDA context (0 when none is current or the driver lacks the query)
unsigned long long current_context_id() {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PfnCtxGetCurrent>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PfnCtxGetId>(fn);
    cudaGetLastError();
  }
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// The scratch address for the current context; nullptr on a CUDA error.
NoallocScratch* scratch_address() {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = current_context_id();
  if (id)
    for (int i = 0; i < g_scratch_count; i++)
      if (g_scratch_cache[i].ctx_id == id) return g_scratch_cache[i].addr;
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return nullptr;
  }
  if (!id) id = current_context_id();  // the runtime may have just made the primary current
  if (id && g_scratch_count < kMaxContexts) g_scratch_cache[g_scratch_count++] = {id, (NoallocScratch*)p};
  return static_cast<NoallocScratch*>(p);
}

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
  NoallocScratch* scratch = scratch_address();
  if (!scratch) return GLIA_ERR_CUDA;
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

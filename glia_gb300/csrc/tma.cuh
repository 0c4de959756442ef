// tma.cuh — tensor-memory-accelerator staging: 2-D tensor maps over the packed line arrays,
// mbarrier completion, bounded waits.
//
// A tile (NN rows x T complex) is one cp.async.bulk.tensor.2d issued by one thread; the copy
// engine signals the slot's mbarrier with the byte count. Every wait on an mbarrier is bounded
// by the SM clock (about one second at 2 GHz): a CTA whose copy does not arrive records
// DevScalars::dev_fault, waits (bounded again) for its other copies and returns, so the context
// stays usable and the host reports the fault.
#pragma once

#include <cuda.h>  // CUtensorMap and its enums (header only; the encoder comes from the runtime)
#include <cudaTypedefs.h>

#include "common.cuh"

namespace glia {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// true once phase `parity` of `bar` has completed; false after about 2^31 SM cycles
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (clock64() - t0 < (1LL << 31))
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// one 2-D tile of `map` at (x elements, y rows) into shared memory (128-byte aligned)
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// bytes (a multiple of 16) from global src to shared dst, both 16-byte aligned, completing on bar
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// One CTA waits on an mbarrier that nothing signals: the bounded wait must give up and record
// the fault (glia_selftest_bounded_wait).
static __global__ void k_selftest_wait(int* fault) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool ok = threadIdx.x != 0 || mbar_wait(&bar, 0);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(fault, 1);
}

// Host: FP32 2-D tensor map over `rows` rows of `inner` floats (row pitch = inner floats), box
// box_inner x box_rows, no swizzle, 256-byte L2 promotion, no out-of-range fill.
inline CUtensorMap make_tmap_f32_2d(const void* base, uint64_t inner, uint64_t rows,
                                    uint32_t box_inner, uint32_t box_rows) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    GLIA_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                               cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn)
      throw Error(GLIA_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  CUtensorMap map;
  const cuuint64_t dims[2] = {inner, rows};
  const cuuint64_t strides[1] = {inner * sizeof(float)};
  const cuuint32_t box[2] = {box_inner, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base),
                            dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(GLIA_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return map;
}

}  // namespace glia

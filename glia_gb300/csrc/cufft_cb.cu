// cufft_cb.cu — device callback linked into cuFFT plans at plan creation (LTO, JIT-linked by
// cuFFT). Built separately as an LTO-IR fatbin (glia_gb300/_build/cufft_cb.fatbin), never linked
// into libglia_rd.so.
//
// glia_store_times_k: store callback of the batched (x3) C2R of the gradient spectra; each real
// output value is multiplied by the diffusivity k at its voxel before it is written, which makes
// the separate k * grad pass unnecessary.
#include <cufftXt.h>

struct GliaCbInfo {
  const float* k;
  unsigned long long n3;  // voxels per transform
};

extern "C" __device__ void glia_store_times_k(void* dataOut, unsigned long long offset,
                                              cufftReal element, void* callerInfo,
                                              void* sharedPointer) {
  (void)sharedPointer;
  const GliaCbInfo* info = static_cast<const GliaCbInfo*>(callerInfo);
  static_cast<cufftReal*>(dataOut)[offset] = element * info->k[offset % info->n3];
}

// zpass.cuh — the z pass of the diffusion operator, fused: for every (x, y) line and each of the
// three gradient components, the half spectrum along z is transformed to the real line (C2R),
// multiplied by the diffusivity k, and transformed back (R2C), in place, in the registers of one
// warp. With cuFFT doing only the (x, y) passes (2-D C2C for each kz), the real-space gradient
// never touches HBM and the separate k-multiply pass disappears.
//
// Line length n = 2M, M = 32 * RR (RR = 1, 2, 4, 8 for n = 64 ... 512). Real transforms use the
// half-length packing identities (z[m] = a[2m] + i a[2m+1]); the M-point complex FFT is split as
// M = RR x 32: an RR-point DFT in registers, a twiddle, and a 32-point radix-2 FFT across the
// lanes with shuffles (decimation in frequency for the inverse, leaving lane L with index
// bitrev5(L); decimation in time for the forward, consuming that order). The C2R output pairs
// (2m, 2m+1) and the R2C input pairs coincide, so the k multiply needs no data exchange.
// Twiddles W_n^j = exp(-2 pi i j / n) come from a table computed on the host in double precision.
#pragma once

#include "reduce.cuh"

namespace glia {

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 shfl2(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ float2 shfl2_xor(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

template <int RR>
__global__ void __launch_bounds__(kThreads)
    k_zpass_mulk(int n, int lines, float* __restrict__ spec3, int64_t Ns,
                 const float* __restrict__ kfield, const float2* __restrict__ tw_g) {
  __shared__ float2 tw[32 * RR * 2];  // W_n^j, j < n
  constexpr int M = 32 * RR;
  constexpr int NN = 2 * M;
  for (int i = threadIdx.x; i < NN; i += blockDim.x) tw[i] = tw_g[i];
  __syncthreads();
  (void)n;
  const int nh = M + 1;
  const int lane = threadIdx.x & 31;
  const int br = (int)(__brev((unsigned)lane) >> 27);
  const int partner_lane = (32 - lane) & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int line = warp; line < lines; line += nwarps) {
    // k at the real positions 2m, 2m+1 with m = k1 + RR * bitrev5(lane): 2RR contiguous floats
    float kv[2 * RR];
    const float* kl = kfield + (int64_t)line * NN + 2 * RR * br;
    if constexpr (RR == 1) {
      const float2 t = *reinterpret_cast<const float2*>(kl);
      kv[0] = t.x;
      kv[1] = t.y;
    } else {
#pragma unroll
      for (int q = 0; q < RR / 2; q++) {
        const float4 t = *reinterpret_cast<const float4*>(kl + 4 * q);
        kv[4 * q] = t.x;
        kv[4 * q + 1] = t.y;
        kv[4 * q + 2] = t.z;
        kv[4 * q + 3] = t.w;
      }
    }
#pragma unroll 1
    for (int j = 0; j < 3; j++) {
      float2* Y = reinterpret_cast<float2*>(spec3) + j * Ns + (int64_t)line * nh;
      float2 y[RR], z[RR];
#pragma unroll
      for (int r = 0; r < RR; r++) y[r] = Y[lane + 32 * r];
      const float2 yM = lane == 0 ? Y[M] : make_float2(0.f, 0.f);
      // C2R packing: Z'[k] = (Y[k] + conj(Y[M-k])) + i (Y[k] - conj(Y[M-k])) W_n^{-k}
#pragma unroll
      for (int r = 0; r < RR; r++) {
        const float2 s1 = shfl2(y[RR - 1 - r], partner_lane);
        const float2 s2 = shfl2(y[(RR - r) % RR], partner_lane);
        const float2 p = lane == 0 ? (r == 0 ? yM : s2) : s1;
        const float2 a = y[r], b = cconj(p);
        const float2 dw = cmulf(make_float2(a.x - b.x, a.y - b.y), cconj(tw[lane + 32 * r]));
        z[r] = make_float2(a.x + b.x - dw.y, a.y + b.y + dw.x);
      }
      // inverse RR-point DFT over the registers
      float2 t[RR];
#pragma unroll
      for (int k1 = 0; k1 < RR; k1++) {
        float2 s = z[0];
#pragma unroll
        for (int r = 1; r < RR; r++) {
          const float2 w = cconj(tw[((NN / RR) * ((r * k1) % RR)) % NN]);
          const float2 v = cmulf(z[r], w);
          s.x += v.x;
          s.y += v.y;
        }
        // twiddle exp(+2 pi i lane k1 / M) = conj(W_n^{2 lane k1})
        t[k1] = k1 ? cmulf(s, cconj(tw[(2 * lane * k1) % NN])) : s;
      }
      // 32-point inverse DFT across the lanes, decimation in frequency
#pragma unroll
      for (int h = 16; h >= 1; h >>= 1) {
        const bool top = (lane & h) == 0;
        const float2 w = cconj(tw[(lane & (h - 1)) * (NN / (2 * h))]);
#pragma unroll
        for (int k1 = 0; k1 < RR; k1++) {
          const float2 o = shfl2_xor(t[k1], h);
          t[k1] = top ? make_float2(t[k1].x + o.x, t[k1].y + o.y)
                      : cmulf(make_float2(o.x - t[k1].x, o.y - t[k1].y), w);
        }
      }
      // t[k1] = z[k1 + RR * bitrev5(lane)]: real line values 2m, 2m+1 -> times k -> repacked
#pragma unroll
      for (int k1 = 0; k1 < RR; k1++) t[k1] = make_float2(t[k1].x * kv[2 * k1], t[k1].y * kv[2 * k1 + 1]);
      // 32-point forward DFT across the lanes, decimation in time (bit-reversed in, natural out)
#pragma unroll
      for (int h = 1; h <= 16; h <<= 1) {
        const bool top = (lane & h) == 0;
        const float2 w = tw[(lane & (h - 1)) * (NN / (2 * h))];
#pragma unroll
        for (int k1 = 0; k1 < RR; k1++) {
          const float2 o = shfl2_xor(t[k1], h);
          if (top) {
            const float2 v = cmulf(w, o);
            t[k1] = make_float2(t[k1].x + v.x, t[k1].y + v.y);
          } else {
            const float2 v = cmulf(w, t[k1]);
            t[k1] = make_float2(o.x - v.x, o.y - v.y);
          }
        }
      }
      // twiddle W_M^{lane k1} = W_n^{2 lane k1}, then the forward RR-point DFT over registers
#pragma unroll
      for (int k1 = 1; k1 < RR; k1++) t[k1] = cmulf(t[k1], tw[(2 * lane * k1) % NN]);
#pragma unroll
      for (int r = 0; r < RR; r++) {
        float2 s = t[0];
#pragma unroll
        for (int k1 = 1; k1 < RR; k1++) {
          const float2 v = cmulf(t[k1], tw[((NN / RR) * ((k1 * r) % RR)) % NN]);
          s.x += v.x;
          s.y += v.y;
        }
        z[r] = s;  // Z[lane + 32 r]
      }
      // R2C unpacking: X[k] = E + W_n^k O, E = (Z[k] + conj(Z[M-k])) / 2,
      // O = -i (Z[k] - conj(Z[M-k])) / 2, Z[M] = Z[0]
#pragma unroll
      for (int r = 0; r < RR; r++) {
        const float2 s1 = shfl2(z[RR - 1 - r], partner_lane);
        const float2 s2 = shfl2(z[(RR - r) % RR], partner_lane);
        const float2 zc = cconj(lane == 0 ? s2 : s1);
        const float2 E = make_float2(0.5f * (z[r].x + zc.x), 0.5f * (z[r].y + zc.y));
        const float2 O = make_float2(0.5f * (z[r].y - zc.y), -0.5f * (z[r].x - zc.x));
        const float2 v = cmulf(tw[lane + 32 * r], O);
        Y[lane + 32 * r] = make_float2(E.x + v.x, E.y + v.y);
        if (r == 0 && lane == 0) Y[M] = make_float2(E.x - O.x, E.y - O.y);
      }
    }
  }
}

}  // namespace glia

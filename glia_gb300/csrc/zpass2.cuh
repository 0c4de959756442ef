// zpass2.cuh — the z pass of the own-transform D apply with two real lines per complex transform.
//
// Per (x, y) line the z pass takes the packed half spectra H_x, H_y, H_0 (kz < n/2, slot 0
// holding the kz = 0 and kz = n/2 values as re / im), transforms them to real lines, multiplies
// by the diffusivity k and transforms back (H_0 with i w_z on both sides), in place. Two real
// lines a, b travel as one complex line z = a + i b through an n-point complex transform:
//   Z[k] = A[k] + i B[k] (A, B the Hermitian spectra of a, b), z = F^-1 Z = a + i b,
//   z' = k_a a + i k_b b, Z' = F z', A'[k] = (Z'[k] + conj Z'[n-k]) / 2,
//   B'[k] = (Z'[k] - conj Z'[n-k]) / 2i.
// H_x and H_y of one line form a pair (the same k on both parts); H_0 of two neighbouring lines
// form a pair (each part its own line's k). Unlike the even/odd split of a real transform through
// an n/2-point one there is no pre- or post-multiplication by twiddles, and the inverse
// transform's output order is the forward transform's input order, so no exchange between them.
//
// Work split: a group of R2 threads (one quarter or half warp) owns two lines of the block; each
// thread holds n / R2 complex values. The n-point transform is R1 x R2: an R1-point DFT over
// a (index R2 a + t) per thread, twiddles w^(t k1), an exchange through shared memory, R2-point
// DFTs over t for the thread's rows k1 = t + R2 ii. Exchanges use the group's two line regions of
// the staging slot whose inputs are already in registers; a group needs warp barriers only.
#pragma once

#include "ownfft.cuh"

namespace glia {

template <int NN>
struct Z2Decomp;
template <>
struct Z2Decomp<256> {
  static constexpr int R1 = 16, R2 = 16;
};
template <>
struct Z2Decomp<128> {
  static constexpr int R1 = 16, R2 = 8;
};
template <>
struct Z2Decomp<64> {
  static constexpr int R1 = 8, R2 = 8;
};

template <int NN>
struct Z2Geom {
  static constexpr int R1 = Z2Decomp<NN>::R1, R2 = Z2Decomp<NN>::R2;
  static constexpr int KPT = R1 / R2;          // stage-2 rows per thread
  static constexpr int NQ = NN / 2;
  static constexpr int NGRP = 256 / R2;        // thread groups per CTA
  static constexpr int LB = 2 * NGRP;          // lines per block (two per group)
  static constexpr int LS = NQ + 8;            // line stride (complex): lines 64 bytes apart mod 128
  static constexpr int SLOT = LB * LS;         // complex per staging slot
  static constexpr int NBLK = NN * NN / LB;
  static constexpr int PS = R1 + 2;            // twiddle row stride (complex)
  // groups of odd index shift their exchange area by 8 complex (64 bytes), so that groups of one
  // warp that write rows of R2 < 16 complex do not meet in the same banks
  static constexpr int SHIFT = R2 < 16 ? 8 : 0;
  static_assert(NQ + SHIFT <= LS, "exchange area must fit the line region");
  static_assert(R1 % R2 == 0 && R1 % 2 == 0, "decomposition");
};

template <int NN>
constexpr int zpass2_smem_bytes() {
  using Z = Z2Geom<NN>;
  return (3 * Z::SLOT + Z::R2 * Z::PS) * (int)sizeof(float2);
}

// Stages LB contiguous lines of NQ complex (or of n floats) into a slot of line stride LS.
template <int NN>
__device__ __forceinline__ void stage_lines2(float2* slot, const char* src) {
  using Z = Z2Geom<NN>;
  constexpr int CPL = Z::NQ / 2, NCH = Z::LB * CPL;
  static_assert(NCH % 256 == 0, "block must divide over 256 threads");
#pragma unroll
  for (int j = 0; j < NCH / 256; j++) {
    const int e = (int)threadIdx.x + 256 * j;
    const int line = e / CPL, ch = e - line * CPL;
    cp_async16(slot + line * Z::LS + 2 * ch, src + (size_t)e * 16);
  }
}

// One complex pair line through F^-1, the k multiply and F. u holds Z[R2 a + t] on entry; mulk
// (ii, k2, z) returns z times k at position t + R2 ii + R1 k2; out(ii, k2, A', B') receives the
// split result at q = t + R2 ii + R1 k2 for q < n/2. E0 / E1: the group's exchange halves.
template <int NN, class MulK, class Out>
__device__ __forceinline__ void pair_line(float2* E0, float2* E1, const float4* twr, int t,
                                          float2 (&u)[Z2Geom<NN>::R1], MulK&& mulk, Out&& out) {
  using Z = Z2Geom<NN>;
  constexpr int R1 = Z::R1, R2 = Z::R2, KPT = Z::KPT, H = NN / 2;
  auto row = [&](int k1) { return k1 < R1 / 2 ? E0 + k1 * R2 : E1 + (k1 - R1 / 2) * R2; };
  float2 v[KPT][R2];
  // inverse: R1-point DFTs over a, twiddles w^(+t k1), exchange, R2-point DFTs over t
  __syncwarp();  // the inputs of the exchange area are in registers
  reg_dft<R1, +1>(u);
#pragma unroll
  for (int k1 = 0; k1 < R1; k1 += 2) {
    const float4 w = twr[k1 / 2];
    if (k1) u[k1] = cmul2(u[k1], make_float2(w.x, w.y));
    u[k1 + 1] = cmul2(u[k1 + 1], make_float2(w.z, w.w));
    row(k1)[t ^ (k1 & (R2 - 1))] = u[k1];
    row(k1 + 1)[t ^ ((k1 + 1) & (R2 - 1))] = u[k1 + 1];
  }
  __syncwarp();
#pragma unroll
  for (int ii = 0; ii < KPT; ii++) {
    const int k1 = t + R2 * ii;
    const float2* r = row(k1);
#pragma unroll
    for (int tp = 0; tp < R2; tp++) v[ii][tp] = r[tp ^ (k1 & (R2 - 1))];
    reg_dft<R2, +1>(v[ii]);  // v[ii][k2] = z[k1 + R1 k2]
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) v[ii][k2] = mulk(ii, k2, v[ii][k2]);
  }
  __syncwarp();
  // forward: the thread holds z'[R2 a + t] at a = ii + KPT k2
#pragma unroll
  for (int ii = 0; ii < KPT; ii++)
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) u[ii + KPT * k2] = v[ii][k2];
  reg_dft<R1, -1>(u);
#pragma unroll
  for (int k1 = 0; k1 < R1; k1 += 2) {
    const float4 w = twr[k1 / 2];
    if (k1) u[k1] = cmul2(u[k1], make_float2(w.x, -w.y));
    u[k1 + 1] = cmul2(u[k1 + 1], make_float2(w.z, -w.w));
    row(k1)[t ^ (k1 & (R2 - 1))] = u[k1];
    row(k1 + 1)[t ^ ((k1 + 1) & (R2 - 1))] = u[k1 + 1];
  }
  __syncwarp();
#pragma unroll
  for (int ii = 0; ii < KPT; ii++) {
    const int k1 = t + R2 * ii;
    const float2* r = row(k1);
#pragma unroll
    for (int tp = 0; tp < R2; tp++) v[ii][tp] = r[tp ^ (k1 & (R2 - 1))];
    reg_dft<R2, -1>(v[ii]);  // v[ii][k2] = Z'[k1 + R1 k2]
  }
  __syncwarp();
  // natural order for the split: Z'[q] at e2(q)
  auto e2 = [&](int q) { return q < H ? E0 + q : E1 + (q - H); };
#pragma unroll
  for (int ii = 0; ii < KPT; ii++)
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) *e2(t + R2 * ii + R1 * k2) = v[ii][k2];
  __syncwarp();
#pragma unroll
  for (int ii = 0; ii < KPT; ii++)
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) {
      if (R2 * ii + R1 * k2 >= H) continue;  // q < n/2 only
      const int q = t + R2 * ii + R1 * k2;
      const float2 z = v[ii][k2], zq = *e2((NN - q) & (NN - 1));
      const float2 A = make_float2(0.5f * (z.x + zq.x), 0.5f * (z.y - zq.y));
      const float2 B = make_float2(0.5f * (z.y + zq.y), -0.5f * (z.x - zq.x));
      out(ii, k2, A, B);
    }
}

// In place on H = [H_x, H_y, H_0] -> [K_x, K_y, L_z]; k is the real diffusivity field. Items per
// block of LB lines: k, H_x, H_y, H_0, through a ring of three shared-memory slots (item i in
// slot i % 3). k goes to registers first and its slot takes H_0; the H_x / H_y pairs need both
// slots; then the next block's k and H_x are staged and H_0 is done; then the next H_y is staged.
// rev: blocks in descending order. The y-inverse pass writes the lines in ascending order and
// the y-forward pass reads them in ascending order, so in descending order the z pass starts on
// the lines still in L2 and ends on the ones the y-forward pass reads first.
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_zpass2(float* __restrict__ Hio, const float* __restrict__ kf,
             const float2* __restrict__ tw_g, bool rev) {
  using Z = Z2Geom<NN>;
  constexpr int R1 = Z::R1, R2 = Z::R2, KPT = Z::KPT, NQ = Z::NQ, LB = Z::LB, LS = Z::LS;
  constexpr int NP = NN * NN * NQ, PS = Z::PS;
  extern __shared__ float4 zpass2_dyn[];
  float2* slots = reinterpret_cast<float2*>(zpass2_dyn);
  float2* twt = slots + 3 * Z::SLOT;  // twt[t PS + k1] = exp(+2 pi i t k1 / n)
  for (int i = threadIdx.x; i < R2 * R1; i += blockDim.x) {
    const int tt = i / R1, k1 = i - tt * R1;
    twt[tt * PS + k1] = tw_n<NN, +1>(tw_g, tt * k1);
  }
  const int g = threadIdx.x / R2, t = threadIdx.x % R2;
  const int l0 = 2 * g, l1 = 2 * g + 1;
  const int sh = (g & 1) * Z::SHIFT;
  const float4* twr = reinterpret_cast<const float4*>(twt + t * PS);
  float2* Hc = reinterpret_cast<float2*>(Hio);
  const int nblk = (int)blockIdx.x < Z::NBLK
                       ? (Z::NBLK - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                       : 0;
  const int nitems = 4 * nblk;
  auto slot = [&](int i) { return slots + (i % 3) * Z::SLOT; };
  auto issue = [&](int i) {
    if (i < nitems) {
      const int bi = (int)blockIdx.x + (i / 4) * (int)gridDim.x, kind = i % 4;
      const int blk = rev ? Z::NBLK - 1 - bi : bi;
      const char* src =
          kind == 0 ? reinterpret_cast<const char*>(kf + (size_t)blk * LB * NN)
                    : reinterpret_cast<const char*>(Hc + (size_t)(kind - 1) * NP +
                                                    (size_t)blk * LB * NQ);
      stage_lines2<NN>(slot(i), src);
    }
    cp_async_commit();
  };
  issue(0);
  issue(1);
  issue(2);
  float kv[2][KPT][R2];  // k of lines l0, l1 at t + R2 ii + R1 k2
  for (int b = 0; b < nblk; b++) {
    const int i0 = 4 * b, bi = (int)blockIdx.x + b * (int)gridDim.x;
    const int blk = rev ? Z::NBLK - 1 - bi : bi;
    // k -> registers; its slot takes this block's H_0
    cp_async_wait<2>();
    __syncthreads();
    {
      const float* K0 = reinterpret_cast<const float*>(slot(i0) + l0 * LS);
      const float* K1 = reinterpret_cast<const float*>(slot(i0) + l1 * LS);
#pragma unroll
      for (int ii = 0; ii < KPT; ii++)
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) {
          kv[0][ii][k2] = K0[t + R2 * ii + R1 * k2];
          kv[1][ii][k2] = K1[t + R2 * ii + R1 * k2];
        }
    }
    __syncthreads();
    issue(i0 + 3);
    // H_x / H_y pairs of lines l0 and l1
    cp_async_wait<1>();
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int l = j ? l1 : l0;
      float2* X = slot(i0 + 1) + l * LS;
      float2* Y = slot(i0 + 2) + l * LS;
      float2 u[R1];
#pragma unroll
      for (int a = 0; a < R1; a++) {
        const int k = R2 * a + t;
        if (R2 * a < NQ) {  // 0 <= k < n/2
          const float2 hx = X[k], hy = Y[k];
          u[a] = make_float2(hx.x - hy.y, hx.y + hy.x);
          if (a == 0 && t == 0) u[a] = make_float2(hx.x, hy.x);  // kz = 0 of the packed slot
        } else {  // n/2 <= k < n: conjugates of kz = n - k
          const int m = (R2 * a == NQ && t == 0) ? 0 : NN - k;
          const float2 hx = X[m], hy = Y[m];
          u[a] = make_float2(hx.x + hy.y, hy.x - hx.y);
          if (R2 * a == NQ && t == 0) u[a] = make_float2(hx.y, hy.y);  // kz = n/2
        }
      }
      float2* OX = Hc + (size_t)(blk * LB + l) * NQ;
      float2* OY = OX + NP;
      pair_line<NN>(
          X + sh, Y + sh, twr, t, u,
          [&](int ii, int k2, float2 z) {
            const float kk = kv[j][ii][k2];
            return make_float2(z.x * kk, z.y * kk);
          },
          [&](int ii, int k2, float2 A, float2 B) {
            const int q = t + R2 * ii + R1 * k2;
            if (ii == 0 && k2 == 0 && t == 0) {
              // packed slot 0: (A'[0], A'[n/2]), (B'[0], B'[n/2]), all real; Z'[n/2] sits at
              // the start of the second exchange half
              const float2 zn = Y[sh];
              A.y = zn.x;
              B.y = zn.y;
            }
            OX[q] = A;
            OY[q] = B;
          });
    }
    __syncthreads();
    issue(i0 + 4);
    issue(i0 + 5);
    // H_0 of lines l0 and l1 as one pair: i w on the way in and out
    cp_async_wait<2>();
    __syncthreads();
    {
      float2* P0 = slot(i0 + 3) + l0 * LS;
      float2* P1 = slot(i0 + 3) + l1 * LS;
      float2 u[R1];
#pragma unroll
      for (int a = 0; a < R1; a++) {
        const int k = R2 * a + t;
        if (R2 * a < NQ) {
          const float w = (float)k;  // i w H, w = k (0 at k = 0: the packed slot drops out)
          const float2 h0 = P0[k], h1 = P1[k];
          // A = i w h0, B = i w h1, Z = A + i B
          u[a] = make_float2(-w * h0.y - w * h1.x, w * h0.x - w * h1.y);
        } else {
          const int m = (R2 * a == NQ && t == 0) ? 0 : NN - k;
          const float w = (float)m;  // conj(i w H) at kz = n - k
          const float2 h0 = P0[m], h1 = P1[m];
          // A = conj(i w h0) = (-w h0.y, -w h0.x), B = conj(i w h1)
          u[a] = make_float2(-w * h0.y + w * h1.x, -w * h0.x - w * h1.y);
          if (R2 * a == NQ && t == 0) u[a] = make_float2(0.f, 0.f);  // Nyquist: w = 0
        }
      }
      float2* O0 = Hc + (size_t)2 * NP + (size_t)(blk * LB + l0) * NQ;
      float2* O1 = O0 + NQ;
      pair_line<NN>(
          P0 + sh, P1 + sh, twr, t, u,
          [&](int ii, int k2, float2 z) {
            return make_float2(z.x * kv[0][ii][k2], z.y * kv[1][ii][k2]);
          },
          [&](int ii, int k2, float2 A, float2 B) {
            const int q = t + R2 * ii + R1 * k2;
            const float w = (float)q;  // L_z = i w A' (0 at q = 0)
            O0[q] = make_float2(-w * A.y, w * A.x);
            O1[q] = make_float2(-w * B.y, w * B.x);
          });
    }
    __syncthreads();
    issue(i0 + 6);
  }
  cp_async_wait<0>();
}

}  // namespace glia

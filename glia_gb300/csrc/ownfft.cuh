// ownfft.cuh — the y and z directions of the spectral D apply as own kernels (FP32, n = 64, 128,
// 256), between the x-pass kernels: with them the whole D apply runs without cuFFT.
//
//   k_xinv<OUT2>  p (or P r + b p) -> G_x = F_x^-1(i w_x p) / N, G_0 = F_x^-1(p) / N
//                 layout (x, ky, kz) with kz < n/2 + 1, the cuFFT half-spectrum order
//   k_yinv_bulk / k_yinv
//                 G -> H_x = F_y^-1 G_x, H_y = F_y^-1(i w_y G_0), H_0 = F_y^-1 G_0
//                 layout (x, y, kz'), kz' < n/2: the kz = 0 and kz = n/2 columns travel packed
//                 as one complex column G(kz = 0) + i G(kz = n/2); input rows staged by bulk
//                 copies (k_yinv_bulk, default) or cp.async (k_yinv)
//   k_zpass2 / k_zpass
//                 per (x, y) line: packed half spectrum -> real line, times k, back, packed;
//                 H_0 gets i w_z on both sides -> K_x, K_y, L_z = i w_z F_z(k d_z p), in place.
//                 k_zpass2 (default, zpass2.cuh): two real lines per complex transform;
//                 k_zpass (here): C2R / R2C through an n/2-point complex transform
//   k_yfwd        K -> M_x = F_y K_x, M_r = i w_y F_y K_y + F_y L_z, unpacked into the kz = 0
//                 and kz = n/2 columns, layout (x, ky, kz) with kz < n/2 + 1
//   k_xfwd<IN2>   divergence i w_x F_x M_x + F_x M_r and the PCG epilogue.
//
// Packing. After the x transform of a real field the kz = 0 and kz = n/2 planes are Hermitian in
// ky for every x, so the y transform of A + i B (A, B those planes) returns a + i b with a, b the
// real z = 0-frequency and Nyquist lines: exactly the two real values a packed n-point real
// transform keeps in its first complex slot. Diagonal multipliers act on A and B alike (w_z = 0
// on both planes, the Nyquist wave numbers being zero). On the way back the y-transformed packed
// column Z(ky) splits into the two planes by A = (Z(ky) + conj Z(-ky)) / 2,
// B = (Z(ky) - conj Z(-ky)) / 2i.
//
// Real transforms of length n through complex transforms of length n/2 (the classic even/odd
// split): C2R forms Z[k] = E[k] + i O[k] with E = X[k] + conj X[n/2 - k],
// O = (X[k] - conj X[n/2 - k]) exp(+2 pi i k / n), and its n/2-point inverse gives
// x[2m] + i x[2m + 1]; R2C transforms y[2m] + i y[2m + 1] and recombines
// Y[k] = Fe[k] + exp(-2 pi i k / n) Fo[k], Fe = (Z[k] + conj Z[n/2 - k]) / 2,
// Fo = (Z[k] - conj Z[n/2 - k]) / 2i.
#pragma once

#include "tma.cuh"
#include "xpass.cuh"

namespace glia {

// y transforms: N = R1 R2 rows (ky or y), T columns (kz') of one x plane per tile.
template <int NN>
struct YDecomp;
template <>
struct YDecomp<256> {
  static constexpr int N = 256, R1 = 16, R2 = 16, T = 16;
};
template <>
struct YDecomp<128> {
  static constexpr int N = 128, R1 = 16, R2 = 8, T = 32;
};
template <>
struct YDecomp<64> {
  static constexpr int N = 64, R1 = 8, R2 = 8, T = 32;
};

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}

// Stages the T-column block at column kz0 of NN half-spectrum rows (row r at src + r * nh,
// 8-byte aligned only: rows start 16-byte aligned when r is even) with 16-byte copies: row r is
// copied from column kz0 - (r & 1) as (T + 2) complex, so slot[r * (T + 2) + (r & 1) + col]
// holds column kz0 + col. The copied window stays inside the array or the memory right after it.
template <int NN, int T>
__device__ __forceinline__ void stage_rows_hs(float2* slot, const float2* src, int nh, int kz0) {
  constexpr int CR = T / 2 + 1, NCH = NN * CR;  // 16-byte chunks per row, per tile
#pragma unroll
  for (int j = 0; j < (NCH + 255) / 256; j++) {
    const int e = (int)threadIdx.x + 256 * j;
    if (NCH % 256 == 0 || e < NCH) {
      const int r = e / CR, ch = e - r * CR;
      cp_async16(slot + r * (T + 2) + 2 * ch, src + r * nh + kz0 - (r & 1) + 2 * ch);
    }
  }
}

template <int NN>
constexpr int yinv_smem_bytes() {
  return (2 * NN * (YDecomp<NN>::T + 2) + NN * YDecomp<NN>::T + 2 * NN + 256) *
         (int)sizeof(float2);
}

// G = [G_x, G_0] (half-spectrum layout per x plane) -> H = [H_x, H_y, H_0] (packed lines).
// Tiles (x, column block of T kz'); G_x and G_0 of the CTA's next tile are staged (cp.async,
// 16-byte chunks) behind the current tile's transforms.
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_yinv(const float* __restrict__ Gin, float* __restrict__ Hout,
           const float2* __restrict__ tw_g) {
  using D = YDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T, NB1 = R2 / GR;
  constexpr int NQ = NN / 2, NH = NN / 2 + 1, CB = NQ / T;
  constexpr int PS = NN * NH, NS = NN * PS, NP = NN * NN * NQ;
  constexpr int ntiles = NN * CB, TS = T + 2;
  extern __shared__ float4 yinv_dyn[];
  float2* slGx = reinterpret_cast<float2*>(yinv_dyn);
  float2* slG0 = slGx + NN * TS;
  float2* nyq = slG0 + NN * TS;  // kz = n/2 columns: [0, NN) of G_x, [NN, 2 NN) of G_0
  float2* sm = nyq + 2 * NN;
  float2* tw = sm + NN * T;
  fill_twb<D, +1>(tw, tw_g);
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const float2* Gx = reinterpret_cast<const float2*>(Gin);
  const float2* G0 = Gx + NS;
  float2* H = reinterpret_cast<float2*>(Hout);
  auto stage = [&](float2* slot, float2* ny, const float2* G, int t) {
    if (t < ntiles) {
      const int x = t / CB, cb = t - x * CB;
      stage_rows_hs<NN, T>(slot, G + x * PS, NH, cb * T);
      if (cb == 0 && (int)threadIdx.x < NN)
        cp_async8(ny + threadIdx.x, G + x * PS + (int)threadIdx.x * NH + NQ);
    }
    cp_async_commit();
  };
  stage(slGx, nyq, Gx, blockIdx.x);
  stage(slG0, nyq + NN, G0, blockIdx.x);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int x = tile / CB, kz = (tile - x * CB) * T + c;
    const bool pk = kz == 0;
    cp_async_wait<1>();  // G_x of this tile
    __syncthreads();
    xdft<D, +1>(
        sm, tw, c, gi,
        [&](int, int b, int a) {
          const int ky = R2 * a + b;
          float2 v = slGx[ky * TS + (ky & 1) + c];
          if (pk) {
            const float2 w = nyq[ky];
            v = make_float2(v.x - w.y, v.y + w.x);
          }
          return v;
        },
        [&] { stage(slGx, nyq, Gx, tile + gridDim.x); },
        [&](int, int k1, int k2, float2 y) { H[(x * NN + k1 + R1 * k2) * NQ + kz] = y; });
    cp_async_wait<1>();  // G_0 of this tile
    __syncthreads();
    float2 v[NB1][R1];
#pragma unroll
    for (int m = 0; m < NB1; m++) {
      const int b = gi + GR * m;
#pragma unroll
      for (int a = 0; a < R1; a++) {
        const int ky = R2 * a + b;
        float2 val = slG0[ky * TS + (ky & 1) + c];
        if (pk) {
          const float2 w = nyq[NN + ky];
          val = make_float2(val.x - w.y, val.y + w.x);
        }
        v[m][a] = val;
      }
    }
    __syncthreads();
    stage(slG0, nyq + NN, G0, tile + gridDim.x);
    xdft<D, +1>(
        sm, tw, c, gi, [&](int m, int, int a) { return v[m][a]; }, [] {},
        [&](int, int k1, int k2, float2 y) { H[2 * NP + (x * NN + k1 + R1 * k2) * NQ + kz] = y; });
    xdft<D, +1>(
        sm, tw, c, gi,
        [&](int m, int b, int a) {
          const float w = (float)wavenum(R2 * a + b, NN);
          return make_float2(-w * v[m][a].y, w * v[m][a].x);
        },
        [] {}, [&](int, int k1, int k2, float2 y) { H[NP + (x * NN + k1 + R1 * k2) * NQ + kz] = y; });
  }
  cp_async_wait<0>();
}

template <int NN>
constexpr int yinv_bulk_smem_bytes() {
  return yinv_smem_bytes<NN>() + 2 * (int)sizeof(uint64_t);
}

// k_yinv with the input rows staged by bulk copies (the copy engine, one 16-byte aligned window of
// T + 2 complex per row and thread, completing on one mbarrier per slot) instead of per-thread
// 16-byte cp.async chunks; the kz = n/2 column still by cp.async. The windows cross 128-byte
// lines (rows are n/2 + 1 complex long), which costs the load/store unit extra wavefronts per
// cp.async chunk. Waits are bounded; a timeout records DevScalars::dev_fault.
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_yinv_bulk(const float* __restrict__ Gin, float* __restrict__ Hout,
                const float2* __restrict__ tw_g, DevScalars* __restrict__ sc) {
  using D = YDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T, NB1 = R2 / GR;
  constexpr int NQ = NN / 2, NH = NN / 2 + 1, CB = NQ / T;
  constexpr int PS = NN * NH, NS = NN * PS, NP = NN * NN * NQ;
  constexpr int ntiles = NN * CB, TS = T + 2;
  constexpr unsigned SLOT_BYTES = NN * TS * sizeof(float2);
  extern __shared__ float4 yinv_dyn[];
  float2* slGx = reinterpret_cast<float2*>(yinv_dyn);
  float2* slG0 = slGx + NN * TS;
  float2* nyq = slG0 + NN * TS;
  float2* sm = nyq + 2 * NN;
  float2* tw = sm + NN * T;
  uint64_t* bars = reinterpret_cast<uint64_t*>(tw + 256);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  fill_twb<D, +1>(tw, tw_g);
  __syncthreads();
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const float2* Gx = reinterpret_cast<const float2*>(Gin);
  const float2* G0 = Gx + NS;
  float2* H = reinterpret_cast<float2*>(Hout);
  // after a CTA barrier that ends every read of the slot: rows by bulk copies, nyq by cp.async
  auto stage = [&](float2* slot, float2* ny, const float2* G, int t, uint64_t* bar) {
    if (t < ntiles) {
      const int x = t / CB, cb = t - x * CB;
      if (threadIdx.x == 0) mbar_arrive_expect_tx(bar, SLOT_BYTES);
      if ((int)threadIdx.x < NN) {
        const int r = threadIdx.x;
        fence_proxy_async();
        bulk_load(slot + r * TS, G + x * PS + r * NH + cb * T - (r & 1),
                  TS * (unsigned)sizeof(float2), bar);
        if (cb == 0) cp_async8(ny + r, G + x * PS + r * NH + NQ);
      }
    }
    cp_async_commit();
  };
  // The slot's rows of tile `it` (phase `it` of its barrier) have landed (uniform result). On a
  // timeout: record the fault and wait, bounded, for every copy of this CTA still in flight — the
  // late phase itself and the other slot's outstanding phase. When slot 0 is late, slot 1 holds
  // phase `it` (staged one tile ahead). When slot 1 is late, slot 0 was already re-staged for the
  // next tile during this tile's G_x transform: phase it + 1, pending only if that tile exists.
  auto ready = [&](int which, int it, bool next) {
    const bool ok = threadIdx.x != 0 || mbar_wait(&bars[which], (unsigned)(it & 1));
    if (!__syncthreads_or(!ok)) return true;
    if (threadIdx.x == 0) {
      atomicExch(&sc->dev_fault, 1);
      mbar_wait(&bars[which], (unsigned)(it & 1));
      if (which == 0)
        mbar_wait(&bars[1], (unsigned)(it & 1));
      else if (next)
        mbar_wait(&bars[0], (unsigned)((it + 1) & 1));
    }
    cp_async_wait<0>();
    __syncthreads();
    return false;
  };
  stage(slGx, nyq, Gx, blockIdx.x, &bars[0]);
  stage(slG0, nyq + NN, G0, blockIdx.x, &bars[1]);
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
    const int x = tile / CB, kz = (tile - x * CB) * T + c;
    const bool pk = kz == 0;
    const bool next = tile + (int)gridDim.x < ntiles;
    cp_async_wait<1>();  // nyq of G_x
    if (!ready(0, it, next)) return;
    xdft<D, +1>(
        sm, tw, c, gi,
        [&](int, int b, int a) {
          const int ky = R2 * a + b;
          float2 v = slGx[ky * TS + (ky & 1) + c];
          if (pk) {
            const float2 w = nyq[ky];
            v = make_float2(v.x - w.y, v.y + w.x);
          }
          return v;
        },
        [&] { stage(slGx, nyq, Gx, tile + gridDim.x, &bars[0]); },
        [&](int, int k1, int k2, float2 y) { H[(x * NN + k1 + R1 * k2) * NQ + kz] = y; });
    cp_async_wait<1>();  // nyq of G_0
    if (!ready(1, it, next)) return;
    float2 v[NB1][R1];
#pragma unroll
    for (int m = 0; m < NB1; m++) {
      const int b = gi + GR * m;
#pragma unroll
      for (int a = 0; a < R1; a++) {
        const int ky = R2 * a + b;
        float2 val = slG0[ky * TS + (ky & 1) + c];
        if (pk) {
          const float2 w = nyq[NN + ky];
          val = make_float2(val.x - w.y, val.y + w.x);
        }
        v[m][a] = val;
      }
    }
    __syncthreads();
    stage(slG0, nyq + NN, G0, tile + gridDim.x, &bars[1]);
    xdft<D, +1>(
        sm, tw, c, gi, [&](int m, int, int a) { return v[m][a]; }, [] {},
        [&](int, int k1, int k2, float2 y) { H[2 * NP + (x * NN + k1 + R1 * k2) * NQ + kz] = y; });
    xdft<D, +1>(
        sm, tw, c, gi,
        [&](int m, int b, int a) {
          const float w = (float)wavenum(R2 * a + b, NN);
          return make_float2(-w * v[m][a].y, w * v[m][a].x);
        },
        [] {}, [&](int, int k1, int k2, float2 y) { H[NP + (x * NN + k1 + R1 * k2) * NQ + kz] = y; });
  }
  cp_async_wait<0>();
}

template <int NN>
constexpr int yfwd_smem_bytes() {
  return (3 * NN * YDecomp<NN>::T + 2 * NN + 256) * (int)sizeof(float2);
}

// K = [K_x, K_y, L_z] (packed lines) -> M = [M_x, M_r] (half-spectrum layout per x plane).
// The CTA's inputs form a stream of items (K_x, K_y, L_z of its first tile, then of the next,
// ...) through two shared-memory slots: item i sits in slot i % 2 and, once the transform that
// reads it has its inputs in registers, item i + 2 is staged there (cp.async).
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_yfwd(const float* __restrict__ Kin, float* __restrict__ Mout,
           const float2* __restrict__ tw_g) {
  using D = YDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T, NB2 = R1 / GR;
  constexpr int NQ = NN / 2, NH = NN / 2 + 1, CB = NQ / T;
  constexpr int PS = NN * NH, NS = NN * PS, NP = NN * NN * NQ;
  constexpr int ntiles = NN * CB;
  extern __shared__ float4 yfwd_dyn[];
  float2* slots = reinterpret_cast<float2*>(yfwd_dyn);  // 2 x NN * T
  float2* sm = slots + 2 * NN * T;
  float2* zA = sm + NN * T;
  float2* zB = zA + NN;
  float2* tw = zB + NN;
  fill_twb<D, -1>(tw, tw_g);
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const float2* K = reinterpret_cast<const float2*>(Kin);
  float2* Mx = reinterpret_cast<float2*>(Mout);
  float2* Mr = Mx + NS;
  const int mytiles =
      (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                               : 0;
  const int nitems = 3 * mytiles;
  auto issue = [&](int i) {
    if (i < nitems) {
      const int t = (int)blockIdx.x + (i / 3) * (int)gridDim.x, j = i % 3;
      const int x = t / CB, cb = t - x * CB;
      stage_tile<NN, T>(slots + (i & 1) * NN * T, K + (size_t)j * NP + (size_t)x * NN * NQ, NQ, cb);
    }
    cp_async_commit();
  };
  issue(0);
  issue(1);
  for (int it = 0; it < mytiles; it++) {
    const int tile = (int)blockIdx.x + it * (int)gridDim.x;
    const int x = tile / CB, cb = tile - x * CB, kz = cb * T + c;
    const bool pk = kz == 0;
    const int i0 = 3 * it;
    auto slot = [&](int i) { return slots + (i & 1) * NN * T; };
    cp_async_wait<1>();
    __syncthreads();
    {
      const float2* S = slot(i0);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 2); },
          [&](int, int k1, int k2, float2 y) {
            const int ky = k1 + R1 * k2;
            if (pk)
              zA[ky] = y;
            else
              Mx[x * PS + ky * NH + kz] = y;
          });
    }
    float2 dsum[NB2][R2];
    cp_async_wait<1>();
    __syncthreads();
    {
      const float2* S = slot(i0 + 1);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 3); },
          [&](int m2, int k1, int k2, float2 y) {
            const float w = (float)wavenum(k1 + R1 * k2, NN);
            dsum[m2][k2] = make_float2(-w * y.y, w * y.x);
          });
    }
    cp_async_wait<1>();
    __syncthreads();
    {
      const float2* S = slot(i0 + 2);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 4); },
          [&](int m2, int k1, int k2, float2 y) {
            const int ky = k1 + R1 * k2;
            const float2 d = make_float2(dsum[m2][k2].x + y.x, dsum[m2][k2].y + y.y);
            if (pk)
              zB[ky] = d;
            else
              Mr[x * PS + ky * NH + kz] = d;
          });
    }
    if (cb == 0) {  // unpack the kz' = 0 column into kz = 0 and kz = n/2
      if (c == 0) {
        for (int ky = gi; ky < NN; ky += GR) {
          const int km = (NN - ky) & (NN - 1);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const float2 z = h ? zB[ky] : zA[ky];
            const float2 zm = h ? zB[km] : zA[km];
            const float2 s2 = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
            const float2 d2 = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
            float2* M = h ? Mr : Mx;
            M[x * PS + ky * NH] = s2;
            M[x * PS + ky * NH + NQ] = d2;
          }
        }
      }
    }
  }
  cp_async_wait<0>();
}

template <int NN>
constexpr int yfwd_tma_smem_bytes() {  // 128 bytes of alignment slack, slots, exchange, tables, barriers
  return 128 + (3 * NN * YDecomp<NN>::T + 2 * NN + 256) * (int)sizeof(float2) + 16;
}

// k_yfwd with its items loaded by the tensor-memory accelerator (GLIA_TMA=1): one tensor copy
// per item from kmap (the three arrays as 3 n^2 rows of n floats, a tile = the box of 2T floats x
// n rows), issued by one thread and completing on the slot's mbarrier. Same results as k_yfwd;
// measured 4.57 TB/s against k_yfwd's 4.86 at 256^3, so k_yfwd (cp.async) is the default.
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_yfwd_tma(const __grid_constant__ CUtensorMap kmap, float* __restrict__ Mout,
               const float2* __restrict__ tw_g, DevScalars* __restrict__ sc) {
  using D = YDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T, NB2 = R1 / GR;
  constexpr int NQ = NN / 2, NH = NN / 2 + 1, CB = NQ / T;
  constexpr int PS = NN * NH, NS = NN * PS;
  constexpr int ntiles = NN * CB;
  constexpr unsigned TILE_BYTES = NN * T * sizeof(float2);
  extern __shared__ float4 yfwd_dyn[];
  float2* slots = reinterpret_cast<float2*>(
      (reinterpret_cast<uintptr_t>(yfwd_dyn) + 127) & ~static_cast<uintptr_t>(127));
  float2* sm = slots + 2 * NN * T;
  float2* zA = sm + NN * T;
  float2* zB = zA + NN;
  float2* tw = zB + NN;
  uint64_t* bars = reinterpret_cast<uint64_t*>(tw + 256);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  fill_twb<D, -1>(tw, tw_g);
  __syncthreads();
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  float2* Mx = reinterpret_cast<float2*>(Mout);
  float2* Mr = Mx + NS;
  const int mytiles =
      (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                               : 0;
  const int nitems = 3 * mytiles;
  auto slot = [&](int i) { return slots + (i & 1) * NN * T; };
  auto issue = [&](int i) {  // after a CTA barrier that ends every read of the slot
    if (threadIdx.x == 0 && i < nitems) {
      const int t = (int)blockIdx.x + (i / 3) * (int)gridDim.x, j = i % 3;
      const int x = t / CB, cb = t - x * CB;
      fence_proxy_async();
      mbar_arrive_expect_tx(&bars[i & 1], TILE_BYTES);
      tma_load_2d(slot(i), &kmap, cb * 2 * T, j * NN * NN + x * NN, &bars[i & 1]);
    }
  };
  // item i has landed (all threads; uniform result). On a timeout: record the fault, wait
  // (bounded) for this CTA's copies still in flight (items i, i + 1) and report false.
  // The thread that observed the completed phase orders the copy before the CTA barrier.
  auto ready = [&](int i) {  // one thread waits on the barrier, the CTA barrier publishes it
    const bool ok = threadIdx.x != 0 || mbar_wait(&bars[i & 1], (unsigned)((i >> 1) & 1));
    if (!__syncthreads_or(!ok)) return true;
    if (threadIdx.x == 0) {
      atomicExch(&sc->dev_fault, 1);
      for (int q = i; q < i + 2 && q < nitems; q++)
        mbar_wait(&bars[q & 1], (unsigned)((q >> 1) & 1));
    }
    __syncthreads();
    return false;
  };
  issue(0);
  issue(1);
  for (int it = 0; it < mytiles; it++) {
    const int tile = (int)blockIdx.x + it * (int)gridDim.x;
    const int x = tile / CB, cb = tile - x * CB, kz = cb * T + c;
    const bool pk = kz == 0;
    const int i0 = 3 * it;
    if (!ready(i0)) return;
    {
      const float2* S = slot(i0);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 2); },
          [&](int, int k1, int k2, float2 y) {
            const int ky = k1 + R1 * k2;
            if (pk)
              zA[ky] = y;
            else
              Mx[x * PS + ky * NH + kz] = y;
          });
    }
    float2 dsum[NB2][R2];
    if (!ready(i0 + 1)) return;
    {
      const float2* S = slot(i0 + 1);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 3); },
          [&](int m2, int k1, int k2, float2 y) {
            const float w = (float)wavenum(k1 + R1 * k2, NN);
            dsum[m2][k2] = make_float2(-w * y.y, w * y.x);
          });
    }
    if (!ready(i0 + 2)) return;
    {
      const float2* S = slot(i0 + 2);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a) { return S[(R2 * a + b) * T + c]; },
          [&] { issue(i0 + 4); },
          [&](int m2, int k1, int k2, float2 y) {
            const int ky = k1 + R1 * k2;
            const float2 d = make_float2(dsum[m2][k2].x + y.x, dsum[m2][k2].y + y.y);
            if (pk)
              zB[ky] = d;
            else
              Mr[x * PS + ky * NH + kz] = d;
          });
    }
    if (cb == 0) {  // unpack the kz' = 0 column into kz = 0 and kz = n/2
      if (c == 0) {
        for (int ky = gi; ky < NN; ky += GR) {
          const int km = (NN - ky) & (NN - 1);
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const float2 z = h ? zB[ky] : zA[ky];
            const float2 zm = h ? zB[km] : zA[km];
            const float2 s2 = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
            const float2 d2 = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
            float2* M = h ? Mr : Mx;
            M[x * PS + ky * NH] = s2;
            M[x * PS + ky * NH + NQ] = d2;
          }
        }
      }
    }
  }
}

// z transforms: n/2 = R1 R2 complex points per line, R2 threads per line, 256 / R2 lines per
// block of the CTA.
template <int NN>
struct ZDecomp;
template <>
struct ZDecomp<256> {
  static constexpr int R1 = 16, R2 = 8;
};
template <>
struct ZDecomp<128> {
  static constexpr int R1 = 8, R2 = 8;
};
template <>
struct ZDecomp<64> {
  static constexpr int R1 = 8, R2 = 4;
};

template <int NN>
struct ZGeom {
  static constexpr int NQ = NN / 2, R1 = ZDecomp<NN>::R1, R2 = ZDecomp<NN>::R2;
  static constexpr int LB = 256 / R2;   // lines per block
  static constexpr int LS = NQ + 8;     // shared line stride (complex): lines 64 bytes apart mod 128
  static constexpr int SLOT = LB * LS;  // complex per slot
  static constexpr int NBLK = NN * NN / LB;
};

template <int NN>
constexpr int zpass_smem_bytes() {
  return (3 * ZGeom<NN>::SLOT + 256 + NN) * (int)sizeof(float2);
}

// Stages LB contiguous lines of NQ complex (or of n floats) into a slot of line stride LS.
template <int NN>
__device__ __forceinline__ void stage_lines(float2* slot, const char* src) {
  using Z = ZGeom<NN>;
  constexpr int CPL = Z::NQ / 2, NCH = Z::LB * CPL;
  static_assert(NCH % 256 == 0, "block must divide over 256 threads");
#pragma unroll
  for (int j = 0; j < NCH / 256; j++) {
    const int e = (int)threadIdx.x + 256 * j;
    const int line = e / CPL, ch = e - line * CPL;
    cp_async16(slot + line * Z::LS + 2 * ch, src + (size_t)e * 16);
  }
}

// In place on H = [H_x, H_y, H_0] -> [K_x, K_y, L_z]; k is the real diffusivity field. The CTA
// walks its blocks of LB lines as a stream of items (k, H_x, H_y, H_0 of block 0, then of block
// 1, ...) through a ring of three shared-memory slots: item i is consumed from slot i % 3 and,
// once consumed, its slot receives item i + 3 (cp.async), so every load runs behind at least one
// component's transforms. The k line is kept in registers for the block's three components; each
// component's exchanges run in its own slot.
template <int NN>
__global__ void __launch_bounds__(256, 2)
    k_zpass(float* __restrict__ Hio, const float* __restrict__ kf,
            const float2* __restrict__ tw_g) {
  using Z = ZGeom<NN>;
  constexpr int R1 = Z::R1, R2 = Z::R2, NQ = Z::NQ, LB = Z::LB, LS = Z::LS, KPT = R1 / R2;
  constexpr int NP = NN * NN * NQ;
  static_assert(R1 % R2 == 0, "stage-2 split");
  extern __shared__ float4 zpass_dyn[];
  float2* slots = reinterpret_cast<float2*>(zpass_dyn);
  float2* tw = slots + 3 * Z::SLOT;
  // per-stage twiddles in the order the threads of a line read them (conflict-free):
  // twA[k1 R2 + t] = exp(+2 pi i t k1 / (n/2)), twB[k2 R1 + m1] = exp(-2 pi i m1 k2 / (n/2))
  float2* twA = tw + 256;
  float2* twB = twA + NQ;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tw[i] = tw_g[i];
  for (int i = threadIdx.x; i < NQ; i += blockDim.x) {
    const int k1 = i / R2, tt = i - k1 * R2;
    twA[i] = tw_n<NQ, +1>(tw_g, tt * k1);
    const int k2 = i / R1, m1 = i - k2 * R1;
    twB[i] = tw_n<NQ, -1>(tw_g, m1 * k2);
  }
  const int l = threadIdx.x / R2, t = threadIdx.x % R2;
  float2* Hc = reinterpret_cast<float2*>(Hio);
  const int nblk = (int)blockIdx.x < Z::NBLK
                       ? (Z::NBLK - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                       : 0;
  const int nitems = 4 * nblk;
  auto issue = [&](int i) {
    if (i < nitems) {
      const int blk = (int)blockIdx.x + (i / 4) * (int)gridDim.x, kind = i % 4;
      const char* src =
          kind == 0 ? reinterpret_cast<const char*>(kf + (size_t)blk * LB * NN)
                    : reinterpret_cast<const char*>(Hc + (size_t)(kind - 1) * NP +
                                                    (size_t)blk * LB * NQ);
      stage_lines<NN>(slots + (i % 3) * Z::SLOT, src);
    }
    cp_async_commit();
  };
  issue(0);
  issue(1);
  issue(2);
  float2 kv[KPT][R2];  // (k[2m], k[2m + 1]) for m = k1 + R1 k2, k1 = t + R2 ii
  for (int i = 0; i < nitems; i++) {
    const int blk = (int)blockIdx.x + (i / 4) * (int)gridDim.x, kind = i % 4;
    cp_async_wait<2>();
    __syncthreads();
    float2* S = slots + (i % 3) * Z::SLOT + l * LS;  // this line's region of the slot
    if (kind == 0) {
#pragma unroll
      for (int ii = 0; ii < KPT; ii++)
#pragma unroll
        for (int k2 = 0; k2 < R2; k2++) kv[ii][k2] = S[t + R2 * ii + R1 * k2];
      __syncthreads();
      issue(i + 3);
      continue;
    }
    const int j = kind - 1;  // 0: H_x, 1: H_y, 2: H_0 (z derivative on both sides)
    const bool dz = j == 2;
    // C2R pre-processing: Z[k] for k = R2 a + t
    float2 u[R1];
#pragma unroll
    for (int a = 0; a < R1; a++) {
      const int k = R2 * a + t;
      if (k == 0) {
        const float2 p = S[0];
        const float x0 = dz ? 0.f : p.x, xn = dz ? 0.f : p.y;
        u[a] = make_float2(x0 + xn, x0 - xn);
      } else {
        float2 X = S[k], Xm = S[NQ - k];
        if (dz) {
          X = make_float2(-(float)k * X.y, (float)k * X.x);
          Xm = make_float2(-(float)(NQ - k) * Xm.y, (float)(NQ - k) * Xm.x);
        }
        Xm.y = -Xm.y;
        const float2 E = cadd(X, Xm);
        const float2 O = cmul2(csub(X, Xm), tw_n<NN, +1>(tw, k));
        u[a] = make_float2(E.x - O.y, E.y + O.x);
      }
    }
    // a line's 8 threads are lanes of one warp and touch only that line's region of the slot:
    // the exchanges below need warp barriers only
    __syncwarp();  // the line's region is this component's exchange area from here
    reg_dft<R1, +1>(u);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
      if (k1) u[k1] = cmul2(u[k1], twA[k1 * R2 + t]);
      S[k1 * R2 + (t ^ (k1 & (R2 - 1)))] = u[k1];
    }
    __syncwarp();
    float2 z[KPT][R2];
#pragma unroll
    for (int ii = 0; ii < KPT; ii++) {
      const int k1 = t + R2 * ii;
#pragma unroll
      for (int b = 0; b < R2; b++) z[ii][b] = S[k1 * R2 + (b ^ (k1 & (R2 - 1)))];
      reg_dft<R2, +1>(z[ii]);  // z[ii][k2] = x[2m] + i x[2m + 1], m = k1 + R1 k2
#pragma unroll
      for (int k2 = 0; k2 < R2; k2++)
        z[ii][k2] = make_float2(z[ii][k2].x * kv[ii][k2].x, z[ii][k2].y * kv[ii][k2].y);
      reg_dft<R2, -1>(z[ii]);  // forward, first stage: over m2 for m1 = k1
#pragma unroll
      for (int k2 = 1; k2 < R2; k2++)
        if (k1) z[ii][k2] = cmul2(z[ii][k2], twB[k2 * R1 + k1]);
    }
    __syncwarp();
#pragma unroll
    for (int ii = 0; ii < KPT; ii++) {
      const int m1 = t + R2 * ii;
#pragma unroll
      for (int k2 = 0; k2 < R2; k2++) S[k2 * R1 + (m1 ^ (k2 & (R1 - 1)))] = z[ii][k2];
    }
    __syncwarp();
#pragma unroll
    for (int m1 = 0; m1 < R1; m1++) u[m1] = S[t * R1 + (m1 ^ (t & (R1 - 1)))];
    reg_dft<R1, -1>(u);  // Z'[t + R2 k1'] = u[k1']
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) S[t + R2 * k1] = u[k1];
    __syncwarp();
    // R2C post-processing, packed, straight to global (in place)
    float2* out = Hc + (size_t)j * NP + (size_t)(blk * LB + l) * NQ;
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) {
      const int k = t + R2 * k1;
      float2 Y;
      if (k == 0) {
        const float2 z0 = S[0];
        Y = dz ? make_float2(0.f, 0.f) : make_float2(z0.x + z0.y, z0.x - z0.y);
      } else {
        const float2 Zk = S[k], Zq = S[NQ - k];
        const float2 Zm = make_float2(Zq.x, -Zq.y);
        const float2 Fe = make_float2(0.5f * (Zk.x + Zm.x), 0.5f * (Zk.y + Zm.y));
        const float2 Fo = make_float2(0.5f * (Zk.y - Zm.y), -0.5f * (Zk.x - Zm.x));
        const float2 W = cmul2(Fo, tw_n<NN, -1>(tw, k));
        Y = cadd(Fe, W);
        if (dz) Y = make_float2(-(float)k * Y.y, (float)k * Y.x);
      }
      out[k] = Y;
    }
    __syncthreads();
    issue(i + 3);
  }
  cp_async_wait<0>();
}

}  // namespace glia

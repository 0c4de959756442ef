// xpass.cuh — the x direction of the spectral D apply, fused into the kernels that already stream
// the spectra (FP32, n = 64, 128, 256).
//
// A three-dimensional transform is a 2-D transform over (y, z) for every x plus a 1-D transform
// along x. cuFFT does the (y, z) part as a contiguous batched 2-D transform; these kernels do the
// x part inside the passes around it:
//  k_xinv: new PCG direction p = P r + b p (or a plain spectrum), the three gradient spectra
//          i w_j p / N and their inverse transforms along x -> G_j(x, ky, kz) (two transforms);
//  k_xfwd: forward transforms along x of the three spectra of k grad p, the divergence
//          sum_j i w_j F_j (two transforms), and the epilogue of k_spec_div (CG operator / solve
//          set-up / plain D).
// Each CTA owns a tile: all n rows along x times T consecutive (ky, kz) columns of the flattened
// (ky, kz) plane (T complex = 128 to 512 contiguous bytes per row). The n-point DFT along x is
// R1 x R2: an R1-point DFT in registers over x = R2 a + b, a twiddle exp(s 2 pi i b k1 / n), one
// exchange through shared memory, and an R2-point DFT in registers giving k = k1 + R1 k2.
// Indices are 32-bit: 3 n^2 (n/2 + 1) < 2^31 for n <= 256. The grid is persistent (the resident
// CTA count), so every CTA walks the same number of tiles to within one.
#pragma once

#include "kernels.cuh"

namespace glia {

template <int NN>
struct XDecomp;
template <>
struct XDecomp<256> {
  static constexpr int N = 256, R1 = 16, R2 = 16, T = 16;
};
template <>
struct XDecomp<128> {
  static constexpr int N = 128, R1 = 16, R2 = 8, T = 32;
};
template <>
struct XDecomp<64> {
  static constexpr int N = 64, R1 = 8, R2 = 8, T = 64;
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul2(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// In-register DFTs, natural order in and out: X[k] = sum_j v[j] exp(S 2 pi i j k / R) for
// R = 2, 4, 8, 16, built from radix-4 butterflies (the factors +-i and -1 are sign changes and
// swaps, never multiplications).
template <int S>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = csub(a1, a3);
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = make_float2(t1.x - S * t3.y, t1.y + S * t3.x);  // t1 + S i t3
  a3 = make_float2(t1.x + S * t3.y, t1.y - S * t3.x);  // t1 - S i t3
}

// exp(S 2 pi i e / 16) times z for a compile-time e; e = 4 is S i (a swap)
template <int S, int E>
__device__ __forceinline__ float2 tw16(float2 z) {
  constexpr int e = E & 15;
  if constexpr (e == 0) {
    return z;
  } else if constexpr (e == 4) {
    return make_float2(-S * z.y, S * z.x);
  } else if constexpr (e == 8) {
    return make_float2(-z.x, -z.y);
  } else if constexpr (e == 12) {
    return make_float2(S * z.y, -S * z.x);
  } else {
    constexpr float c[16] = {1.000000000f,  0.923879533f,  0.707106781f,  0.382683432f,
                             0.000000000f,  -0.382683432f, -0.707106781f, -0.923879533f,
                             -1.000000000f, -0.923879533f, -0.707106781f, -0.382683432f,
                             0.000000000f,  0.382683432f,  0.707106781f,  0.923879533f};
    const float wc = c[e], ws = S * c[(e + 12) & 15];  // sin(2 pi e / 16) = cos(2 pi (e - 4) / 16)
    return make_float2(z.x * wc - z.y * ws, z.x * ws + z.y * wc);
  }
}

template <int R, int S>
__device__ __forceinline__ void reg_dft(float2 (&v)[R]) {
  static_assert(R == 2 || R == 4 || R == 8 || R == 16, "register DFT sizes 2 ... 16");
  if constexpr (R == 2) {
    const float2 a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
  } else if constexpr (R == 4) {
    dft4<S>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    // decimation in time: X[k] = E[k] + W^k O[k], X[k + 4] = E[k] - W^k O[k], W = w_16^2
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<S>(e0, e1, e2, e3);
    dft4<S>(o0, o1, o2, o3);
    o1 = tw16<S, 2>(o1);
    o2 = tw16<S, 4>(o2);
    o3 = tw16<S, 6>(o3);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
  } else {
    // 4 x 4: j = 4 j1 + j2; DFT over j1, twiddle w_16^(j2 k1), DFT over j2; k = k1 + 4 k2
    dft4<S>(v[0], v[4], v[8], v[12]);
    dft4<S>(v[1], v[5], v[9], v[13]);
    dft4<S>(v[2], v[6], v[10], v[14]);
    dft4<S>(v[3], v[7], v[11], v[15]);
    v[5] = tw16<S, 1>(v[5]);
    v[6] = tw16<S, 2>(v[6]);
    v[7] = tw16<S, 3>(v[7]);
    v[9] = tw16<S, 2>(v[9]);
    v[10] = tw16<S, 4>(v[10]);
    v[11] = tw16<S, 6>(v[11]);
    v[13] = tw16<S, 3>(v[13]);
    v[14] = tw16<S, 6>(v[14]);
    v[15] = tw16<S, 9>(v[15]);
    dft4<S>(v[0], v[1], v[2], v[3]);
    dft4<S>(v[4], v[5], v[6], v[7]);
    dft4<S>(v[8], v[9], v[10], v[11]);
    dft4<S>(v[12], v[13], v[14], v[15]);
    // v[4 k1 + k2] holds X[k1 + 4 k2]: transpose to natural order
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = t[i];
  }
}

// twiddle exp(S 2 pi i e / n) from the shared table W_256^j = exp(-2 pi i j / 256)
template <int NN, int S>
__device__ __forceinline__ float2 tw_n(const float2* tw, int e) {
  float2 w = tw[(e * (256 / NN)) & 255];
  if (S > 0) w.y = -w.y;
  return w;
}

// Asynchronous 16-byte global -> shared copies (cp.async, completion by commit / wait groups).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Stages tile `tile` of src (NN rows of T complex, rows `plane` complex apart) into shared memory
// as slot[row * T + col]: 2048 16-byte chunks, eight per thread, consecutive threads on
// consecutive chunks of a row.
template <int NN, int T>
__device__ __forceinline__ void stage_tile(float2* slot, const float2* src, int plane, int tile) {
  constexpr int CR = T / 2, NCH = NN * CR;
  static_assert(NCH % 256 == 0, "tile chunks must divide over 256 threads");
#pragma unroll
  for (int j = 0; j < NCH / 256; j++) {
    const int e = (int)threadIdx.x + 256 * j;
    const int row = e / CR, ch = e - row * CR;
    cp_async16(slot + row * T + 2 * ch, src + row * plane + tile * T + 2 * ch);
  }
}

// Dynamic shared memory of k_xinv: input slots (1 or 2), the exchange buffer, the twiddles.
template <int NN, int MODE>
constexpr int xinv_smem_bytes() {
  return ((MODE == 1 ? 3 : 2) * NN * XDecomp<NN>::T + 256) * (int)sizeof(float2);
}

// Column geometry of a tile: flattened (ky, kz) index q, its wave numbers and multiplicity.
struct XCol {
  int q;
  int wy, wz;
  float mult;
};
__device__ __forceinline__ XCol xcol(const Geo& g, int q) {
  XCol c;
  c.q = q;
  const uint32_t ky = g.fd_nh.div((uint32_t)q);
  const uint32_t kz = (uint32_t)q - ky * (uint32_t)g.nh;
  c.wy = wavenum((int)ky, g.n);
  c.wz = wavenum((int)kz, g.n);
  c.mult = (kz == 0 || (int)kz == g.n / 2) ? 1.f : 2.f;
  return c;
}

// Twiddles of the two-stage DFT in the order a thread reads them: twb[b R1 + k1] =
// exp(S 2 pi i b k1 / N) for b < R2, k1 < R1 (16-byte aligned rows, read in pairs).
template <class D, int S>
__device__ __forceinline__ void fill_twb(float2* twb, const float2* tw256) {
  for (int i = threadIdx.x; i < D::R1 * D::R2; i += blockDim.x) {
    const int b = i / D::R1, k1 = i - b * D::R1;
    twb[i] = tw_n<D::N, S>(tw256, b * k1);
  }
}

// One n-point DFT along the tile's rows for this thread's column, sign S, decomposition D
// (N = R1 R2 rows, T columns, 256 threads): in(m, b, a) is the input at row R2 a + b,
// out(m2, k1, k2, y) receives X[k1 + R1 k2]; twb is the table of fill_twb<D, S>. All threads of
// the CTA take part (two barriers); mid() runs after the first, when every input has been read.
template <class D, int S, class In, class Mid, class Out>
__device__ __forceinline__ void xdft(float2* sm, const float2* twb, int c, int gi, In&& in,
                                     Mid&& mid, Out&& out) {
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T;
  constexpr int NB1 = R2 / GR, NB2 = R1 / GR;
#pragma unroll
  for (int m = 0; m < NB1; m++) {
    const int b = gi + GR * m;
    float2 u[R1];
#pragma unroll
    for (int a = 0; a < R1; a++) u[a] = in(m, b, a);
    reg_dft<R1, S>(u);
    const float4* w4 = reinterpret_cast<const float4*>(twb + b * R1);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1 += 2) {
      const float4 w = w4[k1 / 2];
      if (k1) u[k1] = cmul2(u[k1], make_float2(w.x, w.y));
      u[k1 + 1] = cmul2(u[k1 + 1], make_float2(w.z, w.w));
      sm[(k1 * R2 + b) * T + c] = u[k1];
      sm[((k1 + 1) * R2 + b) * T + c] = u[k1 + 1];
    }
  }
  __syncthreads();
  mid();
#pragma unroll
  for (int m2 = 0; m2 < NB2; m2++) {
    const int k1 = gi + GR * m2;
    float2 y[R2];
#pragma unroll
    for (int b = 0; b < R2; b++) y[b] = sm[(k1 * R2 + b) * T + c];
    reg_dft<R2, S>(y);
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) out(m2, k1, k2, y[k2]);
  }
  __syncthreads();
}

// MODE 0: spectrum src -> G; MODE 1: PCG direction p = P r + b p (r = src, p = pdir, p written).
// The y and z gradient spectra differ from the plain spectrum only by factors constant along x,
// so two x transforms give the three components: G_x = F^-1(i w_x u) / N and
// G_y, G_z = i w_y, i w_z F^-1(u) / N. The inputs of the CTA's next tile are staged into shared
// memory (cp.async) while the current tile is transformed.
// OUT2 (own y / z passes): two arrays out, [G_x, G_0] with G_0 = F^-1(u) / N; otherwise three,
// [G_x, G_y, G_z].
template <int NN, int MODE, bool OUT2>
__global__ void __launch_bounds__(256, 2)
    k_xinv(Geo g, const float* __restrict__ src, float* __restrict__ pdir, float* __restrict__ G3,
           const DevScalars* __restrict__ sc, const float2* __restrict__ tw_g) {
  using D = XDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T;
  constexpr int NB1 = R2 / GR;
  extern __shared__ float4 xinv_dyn[];
  float2* slotS = reinterpret_cast<float2*>(xinv_dyn);
  float2* slotP = slotS + NN * T;
  float2* sm = slotP + (MODE == 1 ? NN * T : 0);
  float2* tw = sm + NN * T;
  if (MODE == 1 && sc->status != 0) return;
  fill_twb<D, +1>(tw, tw_g);
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const int plane = NN * g.nh, Ns = plane * NN;
  const int ntiles = plane / T;
  const float invN = (float)g.invN;
  const bool first = MODE == 1 ? sc->iter == 0 : true;
  const float bc = MODE == 1 ? (float)sc->bcoef : 0.f;
  const float pcc = MODE == 1 ? (float)sc->pc_c : 0.f;
  const float2* S = reinterpret_cast<const float2*>(src);
  float2* P = reinterpret_cast<float2*>(pdir);
  float2* Gc = reinterpret_cast<float2*>(G3);
  auto stage = [&](int t) {
    if (t < ntiles) {
      stage_tile<NN, T>(slotS, S, plane, t);
      if (MODE == 1 && !first) stage_tile<NN, T>(slotP, P, plane, t);
    }
    cp_async_commit();
  };
  stage(blockIdx.x);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    cp_async_wait<0>();
    __syncthreads();
    const XCol col = xcol(g, tile * T + c);
    float2 v[NB1][R1];
#pragma unroll
    for (int m = 0; m < NB1; m++) {
      const int b = gi + GR * m;
#pragma unroll
      for (int a = 0; a < R1; a++) {
        const int kx = R2 * a + b;
        float2 val = slotS[kx * T + c];
        if (MODE == 1) {
          const float pm = pc_mult<float>(pcc, wavenum(kx, NN), col.wy, col.wz);
          val.x *= pm;
          val.y *= pm;
          if (!first) {
            const float2 po = slotP[kx * T + c];
            val.x += bc * po.x;
            val.y += bc * po.y;
          }
          P[kx * plane + col.q] = val;
        }
        v[m][a] = val;
      }
    }
    __syncthreads();  // slots read: stage the next tile behind the transforms
    stage(tile + gridDim.x);
    xdft<D, +1>(
        sm, tw, c, gi,
        [&](int m, int b, int a) {
          const float w = (float)wavenum(R2 * a + b, NN) * invN;
          return make_float2(-w * v[m][a].y, w * v[m][a].x);
        },
        [] {},
        [&](int, int k1, int k2, float2 y) { Gc[(k1 + R1 * k2) * plane + col.q] = y; });
    if constexpr (OUT2) {
      xdft<D, +1>(
          sm, tw, c, gi, [&](int m, int, int a) { return v[m][a]; }, [] {},
          [&](int, int k1, int k2, float2 y) {
            Gc[Ns + (k1 + R1 * k2) * plane + col.q] = make_float2(y.x * invN, y.y * invN);
          });
    } else {
      const float fy = (float)col.wy * invN, fz = (float)col.wz * invN;
      xdft<D, +1>(
          sm, tw, c, gi, [&](int m, int, int a) { return v[m][a]; }, [] {},
          [&](int, int k1, int k2, float2 y) {
            const int i = (k1 + R1 * k2) * plane + col.q;
            Gc[Ns + i] = make_float2(-fy * y.y, fy * y.x);
            Gc[2 * Ns + i] = make_float2(-fz * y.y, fz * y.x);
          });
    }
  }
  cp_async_wait<0>();
}

// Epilogue of the forward x pass for one output element (k_spec_div semantics): d = the
// divergence sum_j i w_j F_j at (kx, column), av = the CG direction (CGW) or the spectrum of c
// (SETUP), xv = the spectrum of the caller's x (SETUP with cx).
template <int NN, int EPI>
__device__ __forceinline__ void xfwd_epilogue(float2 d, int kx, int idx, const XCol& col, float a,
                                              float pcc, float invN, float scale, float2 av,
                                              float2 xv, bool has_cx, float2* O, float2* AO,
                                              Acc<float> (&acc)[4]) {
  if (EPI == EPI_APPLYD) {
    O[idx] = make_float2(d.x * scale, d.y * scale);
  } else if (EPI == EPI_SETUP) {
    const float br = av.x + a * d.x, bi = av.y + a * d.y;
    const float rr = 2.f * a * d.x, ri = 2.f * a * d.y;
    const float pm = pc_mult<float>(pcc, wavenum(kx, NN), col.wy, col.wz);
    const float r2 = rr * rr + ri * ri;
    acc[0].add(col.mult * pm * pm * (br * br + bi * bi));
    acc[1].add(col.mult * pm * pm * r2);
    acc[2].add(col.mult * pm * r2);
    if (has_cx) acc[3].add(col.mult * (xv.x * d.x + xv.y * d.y));
    O[idx] = make_float2(av.x * invN, av.y * invN);
    AO[idx] = make_float2(rr, ri);
  } else {  // EPI_CGW
    const float wr = av.x - a * d.x, wi = av.y - a * d.y;
    acc[0].add(col.mult * (av.x * wr + av.y * wi));
    O[idx] = make_float2(wr, wi);
  }
}

template <int EPI>
__device__ __forceinline__ void xfwd_finish(Acc<float> (&acc)[4], Geo g, DevScalars* sc, RedWs ws,
                                            bool has_cx) {
  if constexpr (EPI == EPI_SETUP) {
    double sums[4] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
    if (!grid_sum_last<4>(sums, ws)) return;
    if (threadIdx.x == 0) div_setup_finish(sums, sc, g.invN, has_cx);
  } else if constexpr (EPI == EPI_CGW) {
    double sums[1] = {acc[0].value()};
    if (!grid_sum_last<1>(sums, ws)) return;
    if (threadIdx.x == 0) div_cgw_finish(sums[0], sc, g.invN);
  }
}

// Forward transforms along x of the three spectra F_j of k grad u (the cuFFT 2-D path: layout
// (x, ky, kz) per component), the divergence sum_j i w_j F_j = i w_x F(K_x) +
// F(i w_y K_y + i w_z K_z) (two x transforms), and the epilogue of k_spec_div.
template <int NN, int EPI>
__global__ void __launch_bounds__(256, 2)
    k_xfwd(Geo g, const float* __restrict__ G3, const float* __restrict__ aux_in,
           const float* __restrict__ cx, float* __restrict__ out, float* __restrict__ aux_out,
           float scale, DevScalars* __restrict__ sc, RedWs ws, const float2* __restrict__ tw_g) {
  using D = XDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T;
  constexpr int NB2 = R1 / GR;
  __shared__ float2 sm[NN * T];
  __shared__ __align__(16) float2 tw[256];
  fill_twb<D, -1>(tw, tw_g);
  __syncthreads();
  if (EPI == EPI_CGW && sc->status != 0) return;
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const int plane = NN * g.nh, Ns = plane * NN;
  const int ntiles = plane / T;
  const float a = EPI == EPI_APPLYD ? 0.f : (float)sc->a_cn;
  const float pcc = (float)sc->pc_c;
  const float invN = (float)g.invN;
  const float2* Gc = reinterpret_cast<const float2*>(G3);
  const float2* AX = reinterpret_cast<const float2*>(aux_in);
  const float2* CX = reinterpret_cast<const float2*>(cx);
  float2* O = reinterpret_cast<float2*>(out);
  float2* AO = reinterpret_cast<float2*>(aux_out);
  Acc<float> acc[4];
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const XCol col = xcol(g, tile * T + c);
    float2 dsum[NB2][R2];
    xdft<D, -1>(
        sm, tw, c, gi, [&](int, int b, int a1) { return Gc[(R2 * a1 + b) * plane + col.q]; },
        [] {},
        [&](int m2, int k1, int k2, float2 y) {
          const float w = (float)wavenum(k1 + R1 * k2, NN);
          dsum[m2][k2] = make_float2(-w * y.y, w * y.x);
        });
    const float wy = (float)col.wy, wz = (float)col.wz;
    xdft<D, -1>(
        sm, tw, c, gi,
        [&](int, int b, int a1) {
          const int i = (R2 * a1 + b) * plane + col.q;
          const float2 gy = Gc[Ns + i], gz = Gc[2 * Ns + i];
          return make_float2(-(wy * gy.y + wz * gz.y), wy * gy.x + wz * gz.x);
        },
        [] {},
        [&](int m2, int, int k2, float2 y) {
          dsum[m2][k2].x += y.x;
          dsum[m2][k2].y += y.y;
        });
#pragma unroll
    for (int m2 = 0; m2 < NB2; m2++) {
      const int k1 = gi + GR * m2;
#pragma unroll
      for (int k2 = 0; k2 < R2; k2++) {
        const int kx = k1 + R1 * k2;
        const int idx = kx * plane + col.q;
        const float2 av = EPI == EPI_APPLYD ? make_float2(0.f, 0.f) : AX[idx];
        const float2 xv = (EPI == EPI_SETUP && CX) ? CX[idx] : make_float2(0.f, 0.f);
        xfwd_epilogue<NN, EPI>(dsum[m2][k2], kx, idx, col, a, pcc, invN, scale, av, xv,
                               CX != nullptr, O, AO, acc);
      }
    }
  }
  xfwd_finish<EPI>(acc, g, sc, ws, cx != nullptr);
}

template <int NN>
constexpr int xfwd_own_smem_bytes() {
  return (3 * NN * XDecomp<NN>::T + 256) * (int)sizeof(float2);
}

// Forward x pass of the own-transform path: M = [M_x, M_r] in the half-spectrum layout,
// divergence i w_x F_x M_x + F_x M_r, epilogue of k_spec_div. The CTA's inputs form a stream of
// items (M_x, M_r and the epilogue's spectra of its first tile, then of the next, ...) through
// two shared-memory slots: item i sits in slot i % 2 and, once consumed, its slot receives item
// i + 2 (cp.async).
template <int NN, int EPI>
__global__ void __launch_bounds__(256, 2)
    k_xfwd_own(Geo g, const float* __restrict__ M2, const float* __restrict__ aux_in,
               const float* __restrict__ cx, float* __restrict__ out, float* __restrict__ aux_out,
               float scale, DevScalars* __restrict__ sc, RedWs ws,
               const float2* __restrict__ tw_g) {
  using D = XDecomp<NN>;
  constexpr int R1 = D::R1, R2 = D::R2, T = D::T, GR = 256 / T;
  constexpr int NB2 = R1 / GR;
  extern __shared__ float4 xfwd_dyn[];
  float2* slots = reinterpret_cast<float2*>(xfwd_dyn);  // 2 x NN * T
  float2* sm = slots + 2 * NN * T;
  float2* tw = sm + NN * T;
  if (EPI == EPI_CGW && sc->status != 0) return;
  fill_twb<D, -1>(tw, tw_g);
  const int c = threadIdx.x % T, gi = threadIdx.x / T;
  const int plane = NN * g.nh, Ns = plane * NN;
  const int ntiles = plane / T;
  const float a = EPI == EPI_APPLYD ? 0.f : (float)sc->a_cn;
  const float pcc = (float)sc->pc_c;
  const float invN = (float)g.invN;
  const float2* Mx = reinterpret_cast<const float2*>(M2);
  const float2* Mr = Mx + Ns;
  const float2* AX = reinterpret_cast<const float2*>(aux_in);
  const float2* CX = reinterpret_cast<const float2*>(cx);
  float2* O = reinterpret_cast<float2*>(out);
  float2* AO = reinterpret_cast<float2*>(aux_out);
  const int naux = EPI == EPI_APPLYD ? 0 : (EPI == EPI_SETUP && CX ? 2 : 1);
  const int NI = 2 + naux;
  const int mytiles =
      (int)blockIdx.x < ntiles ? (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                               : 0;
  const int nitems = NI * mytiles;
  auto slot = [&](int i) { return slots + (i & 1) * NN * T; };
  auto issue = [&](int i) {
    if (i < nitems) {
      const int t = (int)blockIdx.x + (i / NI) * (int)gridDim.x, kind = i % NI;
      const float2* src = kind == 0 ? Mx : (kind == 1 ? Mr : (kind == 2 ? AX : CX));
      stage_tile<NN, T>(slot(i), src, plane, t);
    }
    cp_async_commit();
  };
  issue(0);
  issue(1);
  Acc<float> acc[4];
  for (int it = 0; it < mytiles; it++) {
    const int tile = (int)blockIdx.x + it * (int)gridDim.x;
    const int i0 = NI * it;
    const XCol col = xcol(g, tile * T + c);
    float2 dsum[NB2][R2];
    cp_async_wait<1>();
    __syncthreads();
    {
      const float2* S = slot(i0);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a1) { return S[(R2 * a1 + b) * T + c]; },
          [&] { issue(i0 + 2); },
          [&](int m2, int k1, int k2, float2 y) {
            const float w = (float)wavenum(k1 + R1 * k2, NN);
            dsum[m2][k2] = make_float2(-w * y.y, w * y.x);
          });
    }
    cp_async_wait<1>();
    __syncthreads();
    {
      const float2* S = slot(i0 + 1);
      xdft<D, -1>(
          sm, tw, c, gi, [&](int, int b, int a1) { return S[(R2 * a1 + b) * T + c]; },
          [&] { issue(i0 + 3); },
          [&](int m2, int, int k2, float2 y) {
            dsum[m2][k2].x += y.x;
            dsum[m2][k2].y += y.y;
          });
    }
    if (naux == 2)
      cp_async_wait<0>();
    else
      cp_async_wait<1>();
    __syncthreads();
    const float2* SA = slot(i0 + 2);
    const float2* SX = slot(i0 + 3);
#pragma unroll
    for (int m2 = 0; m2 < NB2; m2++) {
      const int k1 = gi + GR * m2;
#pragma unroll
      for (int k2 = 0; k2 < R2; k2++) {
        const int kx = k1 + R1 * k2;
        const float2 av = naux ? SA[kx * T + c] : make_float2(0.f, 0.f);
        const float2 xv = naux == 2 ? SX[kx * T + c] : make_float2(0.f, 0.f);
        xfwd_epilogue<NN, EPI>(dsum[m2][k2], kx, kx * plane + col.q, col, a, pcc, invN, scale, av,
                               xv, naux == 2, O, AO, acc);
      }
    }
    if (naux) {
      __syncthreads();  // the epilogue's slots are read: stage the next tile's M_x (and M_r)
      issue(i0 + 4);
      if (naux == 2) issue(i0 + 5);
    }
  }
  cp_async_wait<0>();
  xfwd_finish<EPI>(acc, g, sc, ws, naux == 2);
}

}  // namespace glia

// kernels.cuh — sm_103a kernels of the GLIA reaction–diffusion path.
//
// All kernels are bandwidth-bound: 16-byte vector loads/stores, grid-stride loops over a fixed
// grid, FP64 accumulation in every reduction (warp shuffles + deterministic last-block combine).
// R is the storage / transform type (float for the mixed path, double for FP64); spectra are
// interleaved complex R on the half grid (n, n, n/2+1).
#pragma once

#include "reduce.cuh"

namespace glia {

// ---------------------------------------------------------------------------------------------
// Device-resident PCG state. Mirrors PETSc KSPSolve_CG + KSPConvergedDefault (left PC,
// preconditioned norm, nonzero initial guess) as used by DiffusionSolver::solve
// (src/pde/DiffusionSolver.cpp:217-250). The host writes the configuration; kernels update the
// rest, so no scalar leaves the device inside a solve except `status`.
// ---------------------------------------------------------------------------------------------
struct DevScalars {
  double a_cn;    // dt_solve / 2 (operator A = I - a_cn * D)
  double pc_c;    // 0.25 * dt_pc * kbar: preconditioner 1 / (1 + pc_c |w|^2)
  double rtol, abstol, divtol;
  int maxit;
  int pad0;
  double beta, beta_old, dpi, dpi_old, alpha, bcoef, dp, rnorm0, ttol;
  int it;      // KSP iteration number (ksp->its)
  int iter;    // loop index of the next iteration
  int status;  // 0 running, 1 converged rtol, 2 converged (beta == 0), -3 maxit, -4 dtol,
               // -8 indefinite, -9 NaN/Inf
  int pad1;
  double kdot_weight;  // weight of the next <c, D alpha> contribution
  double acc[8];       // [0..2] kappa (wm, gm, csf) explicit, [3..5] rho, [6] kappa via <c, D a>
  double red[4];       // generic reduction results
  // per-sweep solve statistics, accumulated on the device (read once per sweep)
  long long sum_its[3];  // PCG iterations of state / adjoint / other solves
  long long nsolves;
  int max_its;
  int err_status;        // first failing solve's status (0 = none)
  int err_its;
  int guard;             // WHILE-loop body executions of the current solve
  double last_dp;
  int dev_fault;         // a bounded device wait ran out (1: TMA copy did not arrive)
  int pad2;
  double m1_keep;        // ||O c(1) - d||^2 of a graph-captured evaluation (read after it ran)
};

__device__ __forceinline__ int conv_test(double rn, const DevScalars* s) {
  if (isnan(rn) || isinf(rn)) return -9;
  if (rn <= s->ttol) return 1;
  if (rn >= s->divtol * s->rnorm0) return -4;
  return 0;
}

// spectral preconditioner multiplier 1 / (1 + pcc |w|^2) (precFactorDiffusion,
// src/cuda/DiffCoef.cu:11-64, without the 1/N^3 factor, which the spectral-space PCG absorbs)
template <typename R>
__device__ __forceinline__ R pc_mult(R pcc, int wx, int wy, int wz) {
  const R v = (R)1 + pcc * (R)(wx * wx + wy * wy + wz * wz);
  return v == (R)0 ? (R)1 : (R)1 / v;
}

#define GRID_STRIDE(t, total)                                                    \
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (total); \
       t += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------------------------
// Fused spectral-space kernels
// ---------------------------------------------------------------------------------------------

// Gradient spectra: out_j = i w_j v / N (j = x, y, z) in one pass over v, batched for one
// 3-way C2R. CGDIR: v is the new PCG direction p = P r + b p_old, computed here from r and the
// previous direction and written back to `pdir` (first iteration: p = P r).
template <typename R, bool CGDIR>
__global__ void __launch_bounds__(kThreads)
    k_spec_grad3(Geo g, const R* __restrict__ src, R* __restrict__ pdir, R* __restrict__ out3,
                 const DevScalars* __restrict__ sc) {
  using V = V16<R>;
  constexpr int K = V::K, CPV = K / 2;
  if (CGDIR && sc->status != 0) return;
  const int64_t nvec = g.Ns * 2 / K;
  const int64_t ss = g.Ns * 2;
  const R invN = (R)g.invN;
  const bool first = CGDIR ? (sc->iter == 0) : true;
  const R b = CGDIR ? (R)sc->bcoef : R(0);
  const R pcc = CGDIR ? (R)sc->pc_c : R(0);
  GRID_STRIDE(t, nvec) {
    R v[K], pv[K], o0[K], o1[K], o2[K];
    V::ld(src + t * K, v);
    if (CGDIR && !first) V::ld(pdir + t * K, pv);
#pragma unroll
    for (int j = 0; j < CPV; j++) {
      SpecIdx s = spec_index((uint32_t)(t * CPV + j), g);
      R re = v[2 * j], im = v[2 * j + 1];
      if (CGDIR) {
        const R P = pc_mult<R>(pcc, s.wx, s.wy, s.wz);
        re *= P;
        im *= P;
        if (!first) {
          re += b * pv[2 * j];
          im += b * pv[2 * j + 1];
        }
        v[2 * j] = re;
        v[2 * j + 1] = im;
      }
      const R rx = re * invN, ix = im * invN;
      o0[2 * j] = -(R)s.wx * ix;
      o0[2 * j + 1] = (R)s.wx * rx;
      o1[2 * j] = -(R)s.wy * ix;
      o1[2 * j + 1] = (R)s.wy * rx;
      o2[2 * j] = -(R)s.wz * ix;
      o2[2 * j + 1] = (R)s.wz * rx;
    }
    if (CGDIR) V::st(pdir + t * K, v);
    V::st(out3 + t * K, o0);
    V::st(out3 + ss + t * K, o1);
    V::st(out3 + 2 * ss + t * K, o2);
  }
}

// g_j *= k for the three gradient components (one pass, batched layout).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_mul_k3(int64_t N, R* __restrict__ g3, const R* __restrict__ k, const DevScalars* sc,
             int check_status) {
  using V = V16<R>;
  constexpr int K = V::K;
  if (check_status && sc->status != 0) return;
  const int64_t nvec = N / K;
  GRID_STRIDE(t, nvec) {
    R kv[K], a[K];
    V::ld(k + t * K, kv);
#pragma unroll
    for (int j = 0; j < 3; j++) {
      V::ld(g3 + j * N + t * K, a);
#pragma unroll
      for (int q = 0; q < K; q++) a[q] *= kv[q];
      V::st(g3 + j * N + t * K, a);
    }
  }
}

enum DivEpi { EPI_APPLYD = 0, EPI_SETUP = 1, EPI_CGW = 2 };

// Scalar epilogue of a solve set-up (last block, thread 0): PETSc's n = 0 convergence test from
// sums = [||B b||^2, ||z0||^2, <z0, r0>, <cx, D c>] (Parseval sums, times 1/N).
__device__ __forceinline__ void div_setup_finish(const double (&sums)[4], DevScalars* sc,
                                                 double invN, bool has_cx) {
  double dp = sqrt(sums[1] * invN), snorm = sqrt(sums[0] * invN);
  if (snorm == 0.0) snorm = dp;
  sc->rnorm0 = snorm;
  sc->ttol = fmax(sc->rtol * snorm, sc->abstol);
  sc->dp = dp;
  sc->it = 0;
  sc->iter = 0;
  sc->dpi = 0.0;
  sc->bcoef = 0.0;
  sc->beta = sums[2] * invN;
  int st = conv_test(dp, sc);
  if (st == 0 && sc->beta == 0.0) {
    st = 2;
    sc->it = 1;
  }
  sc->status = st;
  if (has_cx) sc->acc[6] += sc->kdot_weight * sums[3] * invN;
}

// Scalar epilogue of w = A p (last block, thread 0): PETSc's indefiniteness check, alpha.
__device__ __forceinline__ void div_cgw_finish(double pw_sum, DevScalars* sc, double invN) {
  const double dpi = pw_sum * invN;
  sc->dpi_old = sc->dpi;
  sc->dpi = dpi;
  sc->beta_old = sc->beta;
  sc->it = sc->iter + 1;
  if (dpi == 0.0 || (sc->iter > 0 && dpi * sc->dpi_old <= 0.0))
    sc->status = -8;
  else if (isnan(dpi) || isinf(dpi))
    sc->status = -9;
  else
    sc->alpha = sc->beta / dpi;
}

// Divergence in spectral space, D = sum_j i w_j G_j (the spectrum of div(k grad u)), fused with
// the epilogue of its caller:
//  EPI_APPLYD: out = scale * D.
//  EPI_SETUP : Crank–Nicolson set-up of one diffusion solve from c = F^-1 chat / N:
//              b = c + a D c, r0 = b - A c = 2 a D c, x0 = c; writes r (aux) and x' = chat / N
//              (out); reduces ||B b||^2, ||z0||^2, <z0, r0> and optionally <cx, D c> for the
//              kappa gradient; the last block runs PETSc's n = 0 convergence test.
//  EPI_CGW   : w = p - a D p (aux = p, out = w); reduces <p, w>; the last block does the
//              PETSc indefiniteness check and alpha = beta / <p, w>.
template <typename R, int EPI>
__global__ void __launch_bounds__(kThreads)
    k_spec_div(Geo g, const R* __restrict__ G3, const R* __restrict__ aux_in,
               const R* __restrict__ cx, R* __restrict__ out, R* __restrict__ aux_out, R scale,
               DevScalars* __restrict__ sc, RedWs ws) {
  using V = V16<R>;
  constexpr int K = V::K, CPV = K / 2;
  if (EPI == EPI_CGW && sc->status != 0) return;
  const int64_t nvec = g.Ns * 2 / K;
  const int64_t ss = g.Ns * 2;
  const R a = (R)(EPI == EPI_APPLYD ? 0.0 : sc->a_cn);
  const R pcc = (R)sc->pc_c;
  const R invN = (R)g.invN;
  Acc<R> acc[4];
  GRID_STRIDE(t, nvec) {
    R g0[K], g1[K], g2[K], o[K], ax[K], cv[K];
    V::ld(G3 + t * K, g0);
    V::ld(G3 + ss + t * K, g1);
    V::ld(G3 + 2 * ss + t * K, g2);
    if (EPI != EPI_APPLYD) V::ld(aux_in + t * K, ax);
    if (EPI == EPI_SETUP && cx) V::ld(cx + t * K, cv);
#pragma unroll
    for (int j = 0; j < CPV; j++) {
      SpecIdx s = spec_index((uint32_t)(t * CPV + j), g);
      // i * (wx G0 + wy G1 + wz G2)
      const R sr = (R)s.wx * g0[2 * j] + (R)s.wy * g1[2 * j] + (R)s.wz * g2[2 * j];
      const R si = (R)s.wx * g0[2 * j + 1] + (R)s.wy * g1[2 * j + 1] + (R)s.wz * g2[2 * j + 1];
      const R dr = -si, di = sr;
      if (EPI == EPI_APPLYD) {
        o[2 * j] = dr * scale;
        o[2 * j + 1] = di * scale;
      } else if (EPI == EPI_SETUP) {
        const R cr = ax[2 * j], ci = ax[2 * j + 1];
        const R br = cr + a * dr, bi = ci + a * di;
        const R rr = (R)2 * a * dr, ri = (R)2 * a * di;
        const R P = pc_mult<R>(pcc, s.wx, s.wy, s.wz), m = (R)s.mult;
        const R r2 = rr * rr + ri * ri;
        acc[0].add(m * P * P * (br * br + bi * bi));
        acc[1].add(m * P * P * r2);
        acc[2].add(m * P * r2);
        if (cx) acc[3].add(m * (cv[2 * j] * dr + cv[2 * j + 1] * di));
        o[2 * j] = cr * invN;
        o[2 * j + 1] = ci * invN;
        ax[2 * j] = rr;
        ax[2 * j + 1] = ri;
      } else {  // EPI_CGW
        const R pr = ax[2 * j], pi = ax[2 * j + 1];
        const R wr = pr - a * dr, wi = pi - a * di;
        acc[0].add((R)s.mult * (pr * wr + pi * wi));
        o[2 * j] = wr;
        o[2 * j + 1] = wi;
      }
    }
    V::st(out + t * K, o);
    if (EPI == EPI_SETUP) V::st(aux_out + t * K, ax);
  }
  if constexpr (EPI == EPI_APPLYD) {
    return;
  } else if constexpr (EPI == EPI_SETUP) {
    double sums[4] = {acc[0].value(), acc[1].value(), acc[2].value(), acc[3].value()};
    if (!grid_sum_last<4>(sums, ws)) return;
    if (threadIdx.x == 0) div_setup_finish(sums, sc, g.invN, cx != nullptr);
  } else {
    double a1[1] = {acc[0].value()};
    if (!grid_sum_last<1>(a1, ws)) return;
    if (threadIdx.x == 0) div_cgw_finish(a1[0], sc, g.invN);
  }
}

// PCG update in spectral space: x' += (alpha / N) p, r -= alpha w, z = P r; reduces ||z||^2 and
// <z, r>; the last block runs PETSc's convergence test and prepares the next direction.
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_cg_update(Geo g, R* __restrict__ x, const R* __restrict__ p, R* __restrict__ r,
                const R* __restrict__ w, DevScalars* __restrict__ sc, RedWs ws) {
  using V = V16<R>;
  constexpr int K = V::K, CPV = K / 2;
  if (sc->status != 0) return;
  const int64_t nvec = g.Ns * 2 / K;
  const R al = (R)sc->alpha;
  const R alN = (R)(sc->alpha * g.invN);
  const R pcc = (R)sc->pc_c;
  Acc<R> acc[2];
  GRID_STRIDE(t, nvec) {
    R xv[K], pv[K], rv[K], wv[K];
    V::ld(x + t * K, xv);
    V::ld(p + t * K, pv);
    V::ld(r + t * K, rv);
    V::ld(w + t * K, wv);
#pragma unroll
    for (int q = 0; q < K; q++) {
      xv[q] += alN * pv[q];
      rv[q] -= al * wv[q];
    }
#pragma unroll
    for (int j = 0; j < CPV; j++) {
      SpecIdx s = spec_index((uint32_t)(t * CPV + j), g);
      const R P = pc_mult<R>(pcc, s.wx, s.wy, s.wz);
      const R m2 = (R)s.mult * (rv[2 * j] * rv[2 * j] + rv[2 * j + 1] * rv[2 * j + 1]);
      acc[0].add(P * P * m2);
      acc[1].add(P * m2);
    }
    V::st(x + t * K, xv);
    V::st(r + t * K, rv);
  }
  double sums[2] = {acc[0].value(), acc[1].value()};
  if (!grid_sum_last<2>(sums, ws)) return;
  if (threadIdx.x == 0) {
    const double dp = sqrt(sums[0] * g.invN);
    sc->dp = dp;
    int st = conv_test(dp, sc);
    if (st == 0) {
      const double bnew = sums[1] * g.invN;
      sc->beta = bnew;
      sc->bcoef = bnew / sc->beta_old;
      sc->iter = sc->iter + 1;
      if (bnew == 0.0) {
        st = 2;
        sc->it = sc->iter + 1;
      } else if (sc->iter >= sc->maxit) {
        st = -3;
      }
    }
    sc->status = st;
  }
}

// ---------------------------------------------------------------------------------------------
// Reaction (PdeOperatorsRD::reaction / reactionAdjoint, src/pde/PdeOperators.cpp:140-190,
// 318-370; kernels src/cuda/PdeOperators.cu:4-25). The forward logistic step is written as
// c e / (c e + 1 - c), algebraically equal to the reference's alpha e / (alpha e + 1) with
// alpha = c / (1 - c) and its c = 1 guard, and free of the 1 / (1 - c) cancellation.
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_reaction_fwd(int64_t N, R* __restrict__ c, const R* __restrict__ rho, R dt,
                   R* __restrict__ chalf_out) {
  using V = V16<R>;
  constexpr int K = V::K;
  GRID_STRIDE(t, N / K) {
    R cv[K], rv[K];
    V::ld(c + t * K, cv);
    V::ld(rho + t * K, rv);
    if (chalf_out) V::st(chalf_out + t * K, cv);
#pragma unroll
    for (int q = 0; q < K; q++) {
      const R e = exp(rv[q] * dt);
      const R ce = cv[q] * e;
      cv[q] = ce / (ce + (R)1 - cv[q]);
    }
    V::st(c + t * K, cv);
  }
}

// a *= e / (c e + 1 - c)^2 with c the half-step state (linearised logistic step; the adjoint
// of the diagonal forward linearisation).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_reaction_lin(int64_t N, R* __restrict__ a, const R* __restrict__ rho,
                   const R* __restrict__ c, R dt) {
  using V = V16<R>;
  constexpr int K = V::K;
  GRID_STRIDE(t, N / K) {
    R av[K], rv[K], cv[K];
    V::ld(a + t * K, av);
    V::ld(rho + t * K, rv);
    V::ld(c + t * K, cv);
#pragma unroll
    for (int q = 0; q < K; q++) {
      const R e = exp(rv[q] * dt);
      const R al = cv[q] * e + (R)1 - cv[q];
      av[q] = av[q] * e / (al * al);
    }
    V::st(a + t * K, av);
  }
}

// ---------------------------------------------------------------------------------------------
// Gradient time accumulation (DerivativeOperators::gradDiffusion / gradReaction,
// src/grad/DerivativeOperators.cpp:189-321), reduced straight to FP64 scalars per tissue class.
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_grad_rho_acc(int64_t N, const R* __restrict__ c, const R* __restrict__ a,
                   const R* __restrict__ wm, const R* __restrict__ gm,
                   const R* __restrict__ csf, double weight, DevScalars* sc, RedWs ws) {
  using V = V16<R>;
  constexpr int K = V::K;
  Acc<R> acc[3];
  GRID_STRIDE(t, N / K) {
    R cv[K], av[K], w[K], gg[K], f[K];
    V::ld(c + t * K, cv);
    V::ld(a + t * K, av);
    V::ld(wm + t * K, w);
    V::ld(gm + t * K, gg);
    V::ld(csf + t * K, f);
#pragma unroll
    for (int q = 0; q < K; q++) {
      const R v = (cv[q] * cv[q] - cv[q]) * av[q];
      acc[0].add(w[q] * v);
      acc[1].add(gg[q] * v);
      acc[2].add(f[q] * v);
    }
  }
  double sums[3] = {acc[0].value(), acc[1].value(), acc[2].value()};
  if (!grid_sum_last<3>(sums, ws)) return;
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; q++) sc->acc[3 + q] += weight * sums[q];
}

template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_grad_kappa_acc(int64_t N, const R* __restrict__ gc3, const R* __restrict__ ga3,
                     const R* __restrict__ wm, const R* __restrict__ gm,
                     const R* __restrict__ csf, double weight, DevScalars* sc, RedWs ws) {
  using V = V16<R>;
  constexpr int K = V::K;
  Acc<R> acc[3];
  GRID_STRIDE(t, N / K) {
    R c0[K], c1[K], c2[K], a0[K], a1[K], a2[K], w[K], gg[K], f[K];
    V::ld(gc3 + t * K, c0);
    V::ld(gc3 + N + t * K, c1);
    V::ld(gc3 + 2 * N + t * K, c2);
    V::ld(ga3 + t * K, a0);
    V::ld(ga3 + N + t * K, a1);
    V::ld(ga3 + 2 * N + t * K, a2);
    V::ld(wm + t * K, w);
    V::ld(gm + t * K, gg);
    V::ld(csf + t * K, f);
#pragma unroll
    for (int q = 0; q < K; q++) {
      R v = c0[q] * a0[q];
      v += c1[q] * a1[q];
      v += c2[q] * a2[q];
      acc[0].add(w[q] * v);
      acc[1].add(gg[q] * v);
      acc[2].add(f[q] * v);
    }
  }
  double sums[3] = {acc[0].value(), acc[1].value(), acc[2].value()};
  if (!grid_sum_last<3>(sums, ws)) return;
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; q++) sc->acc[q] += weight * sums[q];
}

// ---------------------------------------------------------------------------------------------
// Observation residual (Obs::apply / applyT, src/mat/Obs.cpp:71-132, and the mismatch of
// DerivativeOperatorsRD, src/grad/DerivativeOperatorsRD.cpp:153-162): r = O c - d,
// m1 = ||r||^2 into sc->red[0], pt = -O^T r (pt may be null).
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_obs_residual(int64_t N, const R* __restrict__ c, const R* __restrict__ O,
                   const R* __restrict__ d, R* __restrict__ pt, DevScalars* sc, RedWs ws) {
  using V = V16<R>;
  constexpr int K = V::K;
  Acc<R> acc;
  GRID_STRIDE(t, N / K) {
    R cv[K], ov[K], dv[K], pv[K];
    V::ld(c + t * K, cv);
    V::ld(O + t * K, ov);
    V::ld(d + t * K, dv);
#pragma unroll
    for (int q = 0; q < K; q++) {
      const R r = cv[q] * ov[q] - dv[q];
      acc.add(r * r);
      pv[q] = -(r * ov[q]);
    }
    if (pt) V::st(pt + t * K, pv);
  }
  double sums[1] = {acc.value()};
  if (!grid_sum_last<1>(sums, ws)) return;
  if (threadIdx.x == 0) sc->red[0] = sums[0];
}

// ---------------------------------------------------------------------------------------------
// Generic reductions and vector kernels (also the building blocks of the reference-structured
// baseline path, which launches one kernel per PETSc vector operation).
// ---------------------------------------------------------------------------------------------
// slot: red[slot] = sum(x*y) (y null -> sum(x)); mode 1: max(x)
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_dot(int64_t N, const R* __restrict__ x, const R* __restrict__ y, DevScalars* sc, int slot,
          RedWs ws) {
  Acc<R> acc;
  GRID_STRIDE(i, N) { acc.add(y ? x[i] * y[i] : x[i]); }
  double sums[1] = {acc.value()};
  if (!grid_sum_last<1>(sums, ws)) return;
  if (threadIdx.x == 0) sc->red[slot] = sums[0];
}

template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_max(int64_t N, const R* __restrict__ x, double* __restrict__ partials, int slot,
          DevScalars* sc, unsigned int* counter) {
  __shared__ double sh[kWarps];
  __shared__ bool am_last;
  double m = -INFINITY;
  GRID_STRIDE(i, N) { m = fmax(m, (double)x[i]); }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = sh[0];
    for (int w = 1; w < kWarps; w++) b = fmax(b, sh[w]);
    partials[blockIdx.x] = b;
    __threadfence();
    am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!am_last || threadIdx.x != 0) return;
  __threadfence();
  double b = -INFINITY;
  for (int k = 0; k < (int)gridDim.x; k++) b = fmax(b, __ldcg(&partials[k]));
  sc->red[slot] = b;
  *counter = 0u;
}

template <typename R>
__global__ void k_axpy(int64_t N, R* __restrict__ y, double a, const R* __restrict__ x) {
  GRID_STRIDE(i, N) { y[i] += (R)a * x[i]; }
}
template <typename R>
__global__ void k_aypx(int64_t N, R* __restrict__ y, double b, const R* __restrict__ x) {
  GRID_STRIDE(i, N) { y[i] = x[i] + (R)b * y[i]; }
}
template <typename R>
__global__ void k_pointwise_mult(int64_t N, R* __restrict__ z, const R* __restrict__ x,
                                 const R* __restrict__ y) {
  GRID_STRIDE(i, N) { z[i] = x[i] * y[i]; }
}
template <typename R>
__global__ void k_scale(int64_t N, R* __restrict__ x, double a) {
  GRID_STRIDE(i, N) { x[i] *= (R)a; }
}
template <typename R>
__global__ void k_fill(int64_t N, R* __restrict__ x, double v) {
  GRID_STRIDE(i, N) { x[i] = (R)v; }
}
template <typename Rin, typename Rout>
__global__ void k_convert(int64_t N, const Rin* __restrict__ in, Rout* __restrict__ out) {
  GRID_STRIDE(i, N) { out[i] = (Rout)in[i]; }
}

// multiply{X,Y,Z}WaveNumber (src/cuda/SpectralOperators.cu:54-124): out = i w_dim f / N
template <typename R>
__global__ void k_mult_wavenumber(Geo g, int dim, const R* __restrict__ f, R* __restrict__ out) {
  const R invN = (R)g.invN;
  GRID_STRIDE(e, g.Ns) {
    SpecIdx s = spec_index((uint32_t)e, g);
    const R w = (R)(dim == 0 ? s.wx : (dim == 1 ? s.wy : s.wz));
    const R re = f[2 * e], im = f[2 * e + 1];
    out[2 * e] = -invN * w * im;
    out[2 * e + 1] = invN * w * re;
  }
}
// precFactorDiffusion (src/cuda/DiffCoef.cu:11-64), isotropic tensor, stored factor
template <typename R>
__global__ void k_precfactor(Geo g, R* __restrict__ P, double dt, double kbar) {
  const R factor = (R)g.invN;
  GRID_STRIDE(e, g.Ns) {
    SpecIdx s = spec_index((uint32_t)e, g);
    const R wx = (R)s.wx, wy = (R)s.wy, wz = (R)s.wz, kb = (R)kbar;
    R v = (R)1 + (R)0.25 * (R)dt * (kb * wx * wx + kb * wy * wy + kb * wz * wz);
    P[e] = (v == (R)0) ? factor : factor / v;
  }
}
// hadamardComplexProduct (complex x real, src/cuda/UtilsCuda.cu:14-19)
template <typename R>
__global__ void k_hadamard_real(int64_t Ns, R* __restrict__ f, const R* __restrict__ P) {
  GRID_STRIDE(e, Ns) {
    f[2 * e] *= P[e];
    f[2 * e + 1] *= P[e];
  }
}
// complex x complex with a real scale (smoother convolution)
template <typename R>
__global__ void k_spec_mul(int64_t Ns, int batch, R* __restrict__ f, const R* __restrict__ kern) {
  GRID_STRIDE(e, Ns * batch) {
    const int64_t k = e % Ns;
    const R ar = f[2 * e], ai = f[2 * e + 1], br = kern[2 * k], bi = kern[2 * k + 1];
    f[2 * e] = ar * br - ai * bi;
    f[2 * e + 1] = ar * bi + ai * br;
  }
}

// ---------------------------------------------------------------------------------------------
// Material properties and coefficient assembly
// ---------------------------------------------------------------------------------------------
// MatProp::setValuesCustom tail (src/mat/MatProp.cpp:171-189): clip >= 0, bg, filter; sum(filter)
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_matprop(int64_t N, R* wm, R* gm, R* csf, R* vt, R* bg, R* filter, DevScalars* sc, int slot,
              RedWs ws) {
  double acc[1] = {0.0};
  GRID_STRIDE(i, N) {
    R w = wm[i], g2 = gm[i], c = csf[i], v = vt[i];
    g2 = (g2 <= (R)0) ? (R)0 : g2;
    w = (w <= (R)0) ? (R)0 : w;
    v = (v <= (R)0) ? (R)0 : v;
    c = (c <= (R)0) ? (R)0 : c;
    wm[i] = w;
    gm[i] = g2;
    csf[i] = c;
    vt[i] = v;
    bg[i] = -(((g2 + w) + v + c) - (R)1);
    const R f = ((w > (R)0.1 || g2 > (R)0.1) && v < (R)0.8) ? (R)1 : (R)0;
    filter[i] = f;
    acc[0] += (double)f;
  }
  if (!grid_sum_last<1>(acc, ws)) return;
  if (threadIdx.x == 0) sc->red[slot] = acc[0];
}

// DiffCoef::setValues / ReacCoef::setValues: out = dgm gm + dwm wm + dglm csf; sum(out)
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_assemble(int64_t N, R* __restrict__ out, const R* __restrict__ wm, const R* __restrict__ gm,
               const R* __restrict__ csf, double dwm, double dgm, double dglm, DevScalars* sc,
               int slot, RedWs ws) {
  double acc[1] = {0.0};
  GRID_STRIDE(i, N) {
    R v = (R)0;
    v += (R)dgm * gm[i];
    v += (R)dwm * wm[i];
    v += (R)dglm * csf[i];
    out[i] = v;
    acc[0] += (double)v;
  }
  if (!grid_sum_last<1>(acc, ws)) return;
  if (threadIdx.x == 0) sc->red[slot] = acc[0];
}

// DiffCoef::setSecondaryCoefficients (src/mat/DiffCoef.cpp:44-58): k~ = k1 wm + k2 gm + k3 csf.
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_assemble_secondary(int64_t N, R* __restrict__ out, const R* __restrict__ wm,
                         const R* __restrict__ gm, const R* __restrict__ csf, double k1,
                         double k2, double k3) {
  GRID_STRIDE(i, N) {
    R v = wm[i] * (R)k1;
    v += (R)k2 * gm[i];
    v += (R)k3 * csf[i];
    out[i] = v;
  }
}

// solveIncremental's mixture (src/pde/PdeOperators.cpp:200-220): out = 0.5 (a + b) + e, e = a
// before the step (mode 1) or b after it (mode 2), in the reference's operation order.
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_incr_mix(int64_t N, R* __restrict__ out, const R* __restrict__ a, const R* __restrict__ b,
               int mode) {
  const R* e = mode == 1 ? a : b;
  GRID_STRIDE(i, N) {
    R v = a[i] + b[i];
    v *= (R)0.5;
    v += e[i];
    out[i] = v;
  }
}

// MatProp::setValuesSinusoidal (src/mat/MatProp.cpp:34-68) and
// DiffCoef::setValuesSinusoidal (src/mat/DiffCoef.cpp:134-187); sum of the k field.
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_sinusoid(Geo g, R* wm, R* gm, R* csf, R* vt, R* bg, R* filter, R* kxx, double kscale,
               DevScalars* sc, int slot, RedWs ws) {
  double acc[1] = {0.0};
  const double tp = 2.0 * 3.14159265358979323846 / g.n;
  GRID_STRIDE(i, g.N) {
    const int64_t n = g.n;
    const int x = (int)(i / (n * n)), y = (int)((i / n) % n), z = (int)(i % n);
    const double s = 0.5 + 0.5 * sin(4.0 * tp * x) * sin(4.0 * tp * y) * sin(4.0 * tp * z);
    if (kxx) {
      const double kv = kscale * s;
      kxx[i] = (R)kv;
      acc[0] += (double)(R)kv;
    } else {
      wm[i] = (R)s;
      gm[i] = (R)(1.0 - s);
      csf[i] = vt[i] = bg[i] = (R)0;
      filter[i] = (R)1;
    }
  }
  if (!grid_sum_last<1>(acc, ws)) return;
  if (threadIdx.x == 0) sc->red[slot] = acc[0];
}

// Obs::setDefaultFilter (src/mat/Obs.cpp:26-55)
template <typename R>
__global__ void k_threshold(int64_t N, const R* __restrict__ d, double thr, R* __restrict__ f) {
  GRID_STRIDE(i, N) { f[i] = ((double)d[i] > thr) ? (R)1 : (R)0; }
}

// computeWeierstrassFilter (src/cuda/SpectralOperators.cu:12-50): periodised Gaussian with its
// eight images, NaN guarded; sum into red[slot].
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_weierstrass(Geo g, R* __restrict__ f, double sigma, DevScalars* sc, int slot, RedWs ws) {
  double acc[1] = {0.0};
  const double twopi = 2.0 * 3.14159265358979323846, h = twopi / g.n;
  GRID_STRIDE(p, g.N) {
    const int64_t n = g.n;
    const double X = (double)(p / (n * n)) * h, Y = (double)((p / n) % n) * h,
                 Z = (double)(p % n) * h;
    const double Xp = X - twopi, Yp = Y - twopi, Zp = Z - twopi, s2 = sigma;
    double v = exp((-X * X - Y * Y - Z * Z) / s2 / s2 / 2.0) +
               exp((-Xp * Xp - Yp * Yp - Zp * Zp) / s2 / s2 / 2.0);
    v += exp((-Xp * Xp - Y * Y - Z * Z) / s2 / s2 / 2.0) +
         exp((-X * X - Yp * Yp - Z * Z) / s2 / s2 / 2.0);
    v += exp((-X * X - Y * Y - Zp * Zp) / s2 / s2 / 2.0) +
         exp((-Xp * Xp - Yp * Yp - Z * Z) / s2 / s2 / 2.0);
    v += exp((-Xp * Xp - Y * Y - Zp * Zp) / s2 / s2 / 2.0) +
         exp((-X * X - Yp * Yp - Zp * Zp) / s2 / s2 / 2.0);
    if (v != v) v = 0.0;
    f[p] = (R)v;
    acc[0] += (double)(R)v;
  }
  if (!grid_sum_last<1>(acc, ws)) return;
  if (threadIdx.x == 0) sc->red[slot] = acc[0];
}

// ---------------------------------------------------------------------------------------------
// Gaussian basis Phi (src/mat/Phi.cpp; kernels src/cuda/Phi.cu:11-83)
// ---------------------------------------------------------------------------------------------
// Phi::initialize times the brain filter for a batch of centres: out[b] = exp(-(r/R)^2) filter,
// R = sqrt(2) sigma, non-periodic distance.
template <typename R>
__global__ void k_phi_gauss(Geo g, int batch, const double* __restrict__ centers, double sigma,
                            const R* __restrict__ filter, R* __restrict__ out) {
  const double h = 2.0 * 3.14159265358979323846 / g.n, Rr = sqrt(2.0) * sigma;
  GRID_STRIDE(e, g.N * batch) {
    const int b = (int)(e / g.N);
    const int64_t p = e - (int64_t)b * g.N, n = g.n;
    const double dx = h * (double)(p / (n * n)) - centers[3 * b];
    const double dy = h * (double)((p / n) % n) - centers[3 * b + 1];
    const double dz = h * (double)(p % n) - centers[3 * b + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz), ratio = r / Rr;
    out[e] = (R)exp(-ratio * ratio) * filter[p];
  }
}

struct PhiBox {
  int lo[3], ext[3];
  int64_t off;  // offset of the box values in the box store
};

// Phi::truncate (r / sigma <= 5) and extraction of the compact box of each batched field;
// per-box maximum of the truncated values (zero outside the ball included) into boxmax[b].
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_phi_extract(Geo g, int batch, const R* __restrict__ full, const PhiBox* __restrict__ boxes,
                  const double* __restrict__ centers, double sigma, R* __restrict__ store,
                  double* __restrict__ boxmax) {
  __shared__ double sh[kWarps];
  const int b = blockIdx.y;
  if (b >= batch) return;
  const PhiBox B = boxes[b];
  const int64_t nb = (int64_t)B.ext[0] * B.ext[1] * B.ext[2];
  const double h = 2.0 * 3.14159265358979323846 / g.n;
  double m = 0.0;  // the grid always holds voxels outside the ball, where the value is zero
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nb;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int ez = B.ext[2], ey = B.ext[1];
    const int x = B.lo[0] + (int)(q / ((int64_t)ey * ez));
    const int y = B.lo[1] + (int)((q / ez) % ey);
    const int z = B.lo[2] + (int)(q % ez);
    const double dx = h * x - centers[3 * b], dy = h * y - centers[3 * b + 1],
                 dz = h * z - centers[3 * b + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    R v = full[(int64_t)b * g.N + ((int64_t)x * g.n + y) * g.n + z];
    v = (r / sigma <= 5.0) ? v : (R)0;
    store[B.off + q] = v;
    m = fmax(m, (double)v);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double bm = sh[0];
    for (int w = 1; w < kWarps; w++) bm = fmax(bm, sh[w]);
    // one slot per (box, x-block); combined on the host
    boxmax[(int64_t)b * gridDim.x + blockIdx.x] = bm;
  }
}

// Phi::setValues on the compact boxes only. The smoother's periodised Gaussian (eight images,
// unit sum) is the product of three 1-D kernels w(d) = exp(-(dh)^2 / 2s^2) + exp(-(dh - 2pi)^2 /
// 2s^2) (d = offset mod n) over their sum, so W * f is three 1-D convolutions; w is cut at
// |d| <= Rh voxels, where it is below 1e-20 of its peak. Four passes per batch of boxes (grid
// (blocks per box, batch), one scratch region per box at scr_off[b]):
//  0: f = exp(-(r / (sqrt 2 sigma))^2) filter on the box widened by Rh on each side (periodic
//     grid indices, non-periodic distances, as Phi::initialize on the full grid);
//  1, 2: convolution along z, then y, each narrowing that axis to the box;
//  3: convolution along x, Phi::truncate (r / sigma <= 5), the box values into store, and the
//     per-box maximum into boxmax[b * gridDim.x + blockIdx.x].
// taps[d] multiplies the input at local index (output index + d), d = 0 ... 2 Rh (w is even).
// Everything is FP64; store is R.
template <typename R, int PASS>
__global__ void __launch_bounds__(kThreads)
    k_phi_box(Geo g, int batch, const PhiBox* __restrict__ boxes,
              const double* __restrict__ centers, double sigma, int Rh,
              const double* __restrict__ taps, const R* __restrict__ filter,
              const int64_t* __restrict__ scr_off, const double* __restrict__ in,
              double* __restrict__ out, R* __restrict__ store, double* __restrict__ boxmax) {
  __shared__ double sh[kWarps];
  const int b = blockIdx.y;
  if (b >= batch) return;
  const PhiBox B = boxes[b];
  const int n = g.n, W = 2 * Rh + 1;
  // extents of this pass's output: axes already convolved are box-sized, the others widened
  const int ex = B.ext[0] + (PASS < 3 ? 2 * Rh : 0);
  const int ey = B.ext[1] + (PASS < 2 ? 2 * Rh : 0);
  const int ez = B.ext[2] + (PASS < 1 ? 2 * Rh : 0);
  const int64_t cnt = (int64_t)ex * ey * ez;
  const double h = 2.0 * 3.14159265358979323846 / n;
  const double cx = centers[3 * b], cy = centers[3 * b + 1], cz = centers[3 * b + 2];
  const double* src = PASS > 0 ? in + scr_off[b] : nullptr;
  double* dst = PASS < 3 ? out + scr_off[b] : nullptr;
  double m = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(q / ((int64_t)ey * ez)), iy = (int)((q / ez) % ey), iz = (int)(q % ez);
    if (PASS == 0) {
      const int x = ((B.lo[0] - Rh + ix) % n + n) % n, y = ((B.lo[1] - Rh + iy) % n + n) % n,
                z = ((B.lo[2] - Rh + iz) % n + n) % n;
      const double dx = h * x - cx, dy = h * y - cy, dz = h * z - cz;
      const double ratio = sqrt(dx * dx + dy * dy + dz * dz) / (sqrt(2.0) * sigma);
      dst[q] = exp(-ratio * ratio) * (double)filter[((int64_t)x * n + y) * n + z];
    } else if (PASS == 1) {  // input (ex, ey, ez + 2Rh)
      const double* s = src + ((int64_t)ix * ey + iy) * (ez + 2 * Rh) + iz;
      double v = 0.0;
      for (int d = 0; d < W; d++) v += taps[d] * s[d];
      dst[q] = v;
    } else if (PASS == 2) {  // input (ex, ey + 2Rh, ez)
      const double* s = src + ((int64_t)ix * (ey + 2 * Rh) + iy) * ez + iz;
      double v = 0.0;
      for (int d = 0; d < W; d++) v += taps[d] * s[(int64_t)d * ez];
      dst[q] = v;
    } else {  // input (ex + 2Rh, ey, ez); box output
      const double* s = src + ((int64_t)ix * ey + iy) * ez + iz;
      double v = 0.0;
      for (int d = 0; d < W; d++) v += taps[d] * s[(int64_t)d * ey * ez];
      const double dx = h * (B.lo[0] + ix) - cx, dy = h * (B.lo[1] + iy) - cy,
                   dz = h * (B.lo[2] + iz) - cz;
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const R rv = (r / sigma <= 5.0) ? (R)v : (R)0;
      store[B.off + q] = rv;
      m = fmax(m, (double)rv);
    }
  }
  if (PASS == 3) {
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double bm = sh[0];
      for (int w = 1; w < kWarps; w++) bm = fmax(bm, sh[w]);
      boxmax[(int64_t)b * gridDim.x + blockIdx.x] = bm;
    }
  }
}

// checkTumorExistence (src/mat/Phi.cpp:457-520) for every lattice point of Phi::setGaussians(Vec
// data): counts[t] = number of ball offsets o (|o| <= r, from offs) with the point + o inside the
// grid and data > thr there. Lattice point t = (a, b, c) in x-major order over axis[0 .. nax).
static __global__ void __launch_bounds__(kThreads)
    k_data_centers(const double* __restrict__ data, int n, const int* __restrict__ axis, int nax,
                   const int* __restrict__ offs, int noff, double thr, int* __restrict__ counts) {
  const int64_t L = (int64_t)nax * nax * nax;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int x = axis[t / ((int64_t)nax * nax)], y = axis[(t / nax) % nax], z = axis[t % nax];
    int c = 0;
    for (int o = 0; o < noff; o++) {
      const int i = x + offs[3 * o], j = y + offs[3 * o + 1], k = z + offs[3 * o + 2];
      if (i < 0 || j < 0 || k < 0 || i >= n || j >= n || k >= n) continue;
      if (data[((int64_t)i * n + j) * n + k] > thr) c++;
    }
    counts[t] = c;
  }
}

// num_tumor_output of Phi::setGaussians(Vec data): counts / interior at the lattice points
template <typename R>
__global__ void k_data_frac(const int* __restrict__ counts, int n, const int* __restrict__ axis,
                            int nax, double interior, R* __restrict__ out) {
  const int64_t L = (int64_t)nax * nax * nax;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int x = axis[t / ((int64_t)nax * nax)], y = axis[(t / nax) % nax], z = axis[t % nax];
    out[((int64_t)x * n + y) * n + z] = (R)((double)counts[t] / interior);
  }
}

// Phi::apply: out = scale * sum_i p_i phi_i, gathered per output cell (cells of 8^3 voxels, box
// lists in CSR order of increasing index), each output voxel written exactly once.
template <typename R>
__global__ void __launch_bounds__(512)
    k_phi_apply(Geo g, int cells_per_dim, const int* __restrict__ cell_ptr,
                const int* __restrict__ cell_list, const PhiBox* __restrict__ boxes,
                const R* __restrict__ store, const double* __restrict__ p, double scale,
                R* __restrict__ out) {
  const int cell = blockIdx.x;
  const int cz = cell % cells_per_dim, cy = (cell / cells_per_dim) % cells_per_dim,
            cx = cell / (cells_per_dim * cells_per_dim);
  const int x = cx * 8 + (threadIdx.x >> 6), y = cy * 8 + ((threadIdx.x >> 3) & 7),
            z = cz * 8 + (threadIdx.x & 7);
  if (x >= g.n || y >= g.n || z >= g.n) return;
  double acc = 0.0;
  for (int k = cell_ptr[cell]; k < cell_ptr[cell + 1]; k++) {
    const int i = cell_list[k];
    const PhiBox B = boxes[i];
    const int lx = x - B.lo[0], ly = y - B.lo[1], lz = z - B.lo[2];
    if (lx < 0 || ly < 0 || lz < 0 || lx >= B.ext[0] || ly >= B.ext[1] || lz >= B.ext[2])
      continue;
    acc += p[i] * (double)store[B.off + ((int64_t)lx * B.ext[1] + ly) * B.ext[2] + lz];
  }
  out[((int64_t)x * g.n + y) * g.n + z] = (R)(acc * scale);
}

// Phi::applyTranspose: pout_i = sum over box i of phi_i v (one block per box, FP64).
template <typename R>
__global__ void __launch_bounds__(kThreads)
    k_phi_applyT(Geo g, const PhiBox* __restrict__ boxes, const R* __restrict__ store,
                 const R* __restrict__ v, double* __restrict__ pout) {
  __shared__ double sh[1][kWarps];
  const PhiBox B = boxes[blockIdx.x];
  const int64_t nb = (int64_t)B.ext[0] * B.ext[1] * B.ext[2];
  double acc[1] = {0.0};
  for (int64_t q = threadIdx.x; q < nb; q += blockDim.x) {
    const int ez = B.ext[2], ey = B.ext[1];
    const int x = B.lo[0] + (int)(q / ((int64_t)ey * ez));
    const int y = B.lo[1] + (int)((q / ez) % ey);
    const int z = B.lo[2] + (int)(q % ez);
    acc[0] += (double)store[B.off + q] * (double)v[((int64_t)x * g.n + y) * g.n + z];
  }
  block_sum<1>(acc, sh);
  if (threadIdx.x == 0) pout[blockIdx.x] = acc[0];
}

}  // namespace glia

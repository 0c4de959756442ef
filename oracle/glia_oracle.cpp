// glia_oracle.cpp — TEST INFRASTRUCTURE ONLY: the FP64 CPU oracle of GLIA's reaction–diffusion
// forward / adjoint / gradient path.
//
// This file restates, in plain C++17 + OpenMP and double precision, the algorithm of the
// reference (ShashankSubramanian/GLIA): the state and adjoint solves (including the linearised
// ones of the Hessian), the objective (one or two snapshots), the gradient, both Hessian branches.
// It is what the CUDA library is tested against, and the timed CPU baseline; the product never
// links, loads or calls it. Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use it.
//
// Pins (see tests/test_oracle_pins.py):
//  - src/test/pdesolver.cpp:46-48 known answer: 64^3, sinusoidal k (scale 1e-2), Gaussian test
//    function, 10 Crank–Nicolson solves with dt = 0.02 -> ||c||_2 == Approx(2.0487) and 5 CG
//    iterations on the last solve.
//  - src/test/grad.cpp:74-77: J < 1e-7 at the generating parameters, J > 0 with zero data.
//  - the hand-written FFT against numpy.fft.
// What stays unpinned: PETSc's KSPCG / KSPConvergedDefault (third-party, PETSc 3.7-3.11, not in
// the reference tree) is restated from its published algorithm; the known answer above is the
// only in-tree check of it. accFFT's CPU gradient/divergence are not vendored; the spectral
// operators follow the reference's CUDA kernels (src/cuda/SpectralOperators.cu:54-124).
//
// Exported C functions are named oracle_glia_* and mirror include/glia_rd.h one to one (host
// double pointers only).

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../include/glia_rd.h"

namespace orc {

using cplx = std::complex<double>;
static const double kPi = 3.14159265358979323846;

// ------------------------------------------------------------------------------------------
// FFT: iterative radix-2 complex transform, unnormalised, sign -1 forward / +1 inverse.
// ------------------------------------------------------------------------------------------
struct FFT1 {
  int n = 0, logn = 0;
  std::vector<cplx> tw;  // tw[k] = exp(-2 pi i k / n), k < n/2
  std::vector<int> rev;
  void init(int n_) {
    n = n_;
    logn = 0;
    while ((1 << logn) < n) logn++;
    if ((1 << logn) != n) throw std::runtime_error("oracle FFT: n must be a power of two");
    tw.resize(std::max(1, n / 2));
    for (int k = 0; k < n / 2; k++) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / n;
      tw[k] = cplx((double)cosl(a), (double)sinl(a));
    }
    rev.resize(n);
    for (int i = 0; i < n; i++) {
      int r = 0;
      for (int b = 0; b < logn; b++)
        if (i & (1 << b)) r |= 1 << (logn - 1 - b);
      rev[i] = r;
    }
  }
  void exec(cplx* a, int sign) const {
    for (int i = 0; i < n; i++)
      if (i < rev[i]) std::swap(a[i], a[rev[i]]);
    for (int len = 2; len <= n; len <<= 1) {
      int half = len >> 1, step = n / len;
      for (int i = 0; i < n; i += len)
        for (int j = 0; j < half; j++) {
          cplx w = tw[j * step];
          if (sign > 0) w = std::conj(w);
          cplx u = a[i + j], v = a[i + j + half] * w;
          a[i + j] = u + v;
          a[i + j + half] = u - v;
        }
    }
  }
};

// 3-D real-to-complex / complex-to-real transforms on an n^3 grid with the half spectrum
// (n, n, n/2+1), row-major, unnormalised (the cuFFT R2C/C2R convention the reference uses).
struct FFT3 {
  int n = 0, nh = 0, M = 0;
  FFT1 fn, fm;
  std::vector<cplx> wz;  // exp(-2 pi i k / n), k <= n/2
  void init(int n_) {
    n = n_;
    nh = n / 2 + 1;
    M = n / 2;
    fn.init(n);
    fm.init(M);
    wz.resize(M + 1);
    for (int k = 0; k <= M; k++) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / n;
      wz[k] = cplx((double)cosl(a), (double)sinl(a));
    }
  }
  // transform along y and x for every kz (sign as FFT1)
  void xy_pass(cplx* s, int sign) const {
    const int64_t plane = (int64_t)n * nh;
#pragma omp parallel
    {
      std::vector<cplx> buf((size_t)n * nh);
#pragma omp for schedule(static)
      for (int x = 0; x < n; x++) {  // y lines of plane x
        cplx* p = s + x * plane;
        for (int y = 0; y < n; y++)
          for (int k = 0; k < nh; k++) buf[(size_t)k * n + y] = p[(int64_t)y * nh + k];
        for (int k = 0; k < nh; k++) fn.exec(&buf[(size_t)k * n], sign);
        for (int y = 0; y < n; y++)
          for (int k = 0; k < nh; k++) p[(int64_t)y * nh + k] = buf[(size_t)k * n + y];
      }
#pragma omp for schedule(static)
      for (int y = 0; y < n; y++) {  // x lines at fixed y
        for (int x = 0; x < n; x++)
          for (int k = 0; k < nh; k++) buf[(size_t)k * n + x] = s[x * plane + (int64_t)y * nh + k];
        for (int k = 0; k < nh; k++) fn.exec(&buf[(size_t)k * n], sign);
        for (int x = 0; x < n; x++)
          for (int k = 0; k < nh; k++) s[x * plane + (int64_t)y * nh + k] = buf[(size_t)k * n + x];
      }
    }
  }
  void r2c(const double* in, cplx* out) const {
    const int64_t lines = (int64_t)n * n;
#pragma omp parallel
    {
      std::vector<cplx> z(M);
#pragma omp for schedule(static)
      for (int64_t l = 0; l < lines; l++) {
        const double* a = in + l * n;
        for (int m = 0; m < M; m++) z[m] = cplx(a[2 * m], a[2 * m + 1]);
        fm.exec(z.data(), -1);
        cplx* X = out + l * nh;
        for (int k = 0; k <= M; k++) {
          cplx Zk = z[k % M], Zc = std::conj(z[(M - k) % M]);
          cplx E = 0.5 * (Zk + Zc);
          cplx O = cplx(0, -0.5) * (Zk - Zc);
          X[k] = E + wz[k] * O;
        }
      }
    }
    xy_pass(out, -1);
  }
  void c2r(const cplx* in, double* out) const {
    const int64_t total = (int64_t)n * n * nh;
    std::vector<cplx> s(in, in + total);
    xy_pass(s.data(), +1);
    const int64_t lines = (int64_t)n * n;
#pragma omp parallel
    {
      std::vector<cplx> z(M);
#pragma omp for schedule(static)
      for (int64_t l = 0; l < lines; l++) {
        const cplx* X = s.data() + l * nh;
        for (int k = 0; k < M; k++) {
          cplx a = X[k], b = std::conj(X[M - k]);
          z[k] = (a + b) + cplx(0, 1) * ((a - b) * std::conj(wz[k]));
        }
        fm.exec(z.data(), +1);
        double* o = out + l * n;
        for (int m = 0; m < M; m++) {
          o[2 * m] = z[m].real();
          o[2 * m + 1] = z[m].imag();
        }
      }
    }
  }
};

// ------------------------------------------------------------------------------------------
// Deterministic reductions (fixed chunking, independent of the thread count).
// ------------------------------------------------------------------------------------------
static const int kChunks = 1024;
template <class F>
static double chunked_sum(int64_t N, F f) {
  std::vector<double> part(kChunks, 0.0);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < kChunks; c++) {
    int64_t lo = N * c / kChunks, hi = N * (c + 1) / kChunks;
    double s = 0;
    for (int64_t i = lo; i < hi; i++) s += f(i);
    part[c] = s;
  }
  double s = 0;
  for (double v : part) s += v;
  return s;
}
static double vdot(const double* a, const double* b, int64_t N) {
  return chunked_sum(N, [&](int64_t i) { return a[i] * b[i]; });
}
static double vnorm(const double* a, int64_t N) { return std::sqrt(vdot(a, a, N)); }
static double vsum(const double* a, int64_t N) {
  return chunked_sum(N, [&](int64_t i) { return a[i]; });
}
static double vmax(const double* a, int64_t N) {
  double m = -INFINITY;
  for (int64_t i = 0; i < N; i++) m = std::max(m, a[i]);
  return m;
}
static void vaxpy(double* y, double a, const double* x, int64_t N) {  // y += a x
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; i++) y[i] += a * x[i];
}
static void vaypx(double* y, double b, const double* x, int64_t N) {  // y = x + b y
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < N; i++) y[i] = x[i] + b * y[i];
}
static void vcopy(double* y, const double* x, int64_t N) { std::memcpy(y, x, N * sizeof(double)); }

using Field = std::vector<double>;

// wave number of index K along a dimension of size n (Nyquist -> 0), as in
// src/cuda/SpectralOperators.cu:74-81 and src/pde/DiffusionSolver.cpp:149-157.
static inline double wavenum(int64_t K, int n) {
  int64_t w = K;
  if (K > n / 2.0) w -= n;
  if (K == n / 2.0) w = 0;
  return (double)w;
}

// ------------------------------------------------------------------------------------------
// Context: the reference's Tumor + MatProp + DiffCoef + ReacCoef + Phi + Obs + DiffusionSolver
// + PdeOperatorsRD + DerivativeOperatorsRD state for one grid.
// ------------------------------------------------------------------------------------------
struct Ctx {
  int n;
  int64_t N, Ns;
  double h, h3;
  FFT3 fft;
  std::string err;

  // TumorParameters
  double dt = 0.5;
  int nt = 1, order = 2;
  bool adjoint_store = false;
  double k_gm_wm = 0, k_glm_wm = 0, r_gm_wm = 0, r_glm_wm = 0;
  glia_opt_settings opt{};

  // MatProp
  Field wm, gm, csf, vt, bg, filter;
  bool tissue_set = false;
  // DiffCoef (isotropic: kxx = kyy = kzz; the off-diagonal fields stay zero)
  Field kxx;
  double k_scale = 1e-2, kxx_avg = 0, filter_avg = 0;
  // ReacCoef
  Field rho_vec;
  double rho_scale = 0;
  // DiffusionSolver
  double rtol = 1e-6, abstol = 1e-50, divtol = 1e4;
  int maxit = 5000;
  int pc_dt_mode = GLIA_PC_DT_REFERENCE;
  double pc_dt_fixed = 0;
  double ctx_dt = 0.5;  // DiffusionSolver::Ctx::dt_
  std::vector<double> precfactor;
  int ksp_itr = 0;
  double last_rnorm = 0;
  // Phi (stored un-normalised, per-function maxima kept for both normalisation modes)
  int np = 0;
  double phi_sigma = 0;
  std::vector<double> centers;
  std::vector<double> phi_max_each;
  // Obs
  Field obs_filter;
  // two snapshots (TumorParameters::two_time_points_): Obs::filter_0_ and Data::dt0
  Field obs_filter0, data0;
  bool two_tp = false;
  // Tumor state
  Field c0, ct, p0, pt;
  // PdeOperatorsRD history
  std::vector<Field> c_hist, p_hist, c_half;
  bool state_done = false;
  bool history_off = false;  // TumorParameters::time_history_off_: no states kept
  // DiffCoef::temp_[7]: sum_i m_i k~_i of the Hessian's diffusivity direction
  Field ksec;
  // scratch
  std::vector<cplx> xh, wh;
  Field d1;
  Field t[8];
  glia_stats st{};

  explicit Ctx(int n_) : n(n_) {
    N = (int64_t)n * n * n;
    Ns = (int64_t)n * n * (n / 2 + 1);
    h = 2.0 * kPi / n;
    h3 = h * h * h;
    fft.init(n);
    for (Field* f : {&wm, &gm, &csf, &vt, &bg, &filter, &kxx, &rho_vec, &obs_filter, &c0, &ct,
                     &p0, &pt, &d1})
      f->assign(N, 0.0);
    for (auto& f : t) f.assign(N, 0.0);
    std::fill(obs_filter.begin(), obs_filter.end(), 1.0);
    xh.resize(Ns);
    wh.resize(Ns);
    precfactor.assign(Ns, 0.0);
    opt.np = 1;
    opt.nk = 1;
    opt.nr = 1;
    opt.diffusivity_inversion = 1;
    opt.beta = 1e-4;
    opt.k_scale = 1;
    opt.rho_scale = 1;
    // MatProp::setValues defaults (src/mat/MatProp.cpp:20-33): wm = 1, filter = 1
    std::fill(wm.begin(), wm.end(), 1.0);
    std::fill(filter.begin(), filter.end(), 1.0);
  }

  // ---- spectral operators (src/grad/SpectralOperators.cpp:100-261, CUDA semantics) ----
  void mult_wavenumber(int dim, const cplx* f, cplx* w) const {
    const int nh = n / 2 + 1;
    const double factor = 1.0 / ((double)n * n * n);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < nh; z++) {
          int64_t i = ((int64_t)x * n + y) * nh + z;
          double wv = dim == 0 ? wavenum(x, n) : dim == 1 ? wavenum(y, n) : wavenum(z, n);
          w[i] = cplx(-factor * wv * f[i].imag(), factor * wv * f[i].real());
        }
  }
  void gradient(double* gx, double* gy, double* gz, const double* x) {
    fft.r2c(x, xh.data());
    st.total_fft_execs++;
    double* out[3] = {gx, gy, gz};
    for (int d = 0; d < 3; d++) {
      mult_wavenumber(d, xh.data(), wh.data());
      fft.c2r(wh.data(), out[d]);
      st.total_fft_execs++;
    }
  }
  void divergence(double* div, const double* vx, const double* vy, const double* vz, double* tmp) {
    // order x, z, y as in src/grad/SpectralOperators.cpp:202-238
    fft.r2c(vx, xh.data());
    mult_wavenumber(0, xh.data(), wh.data());
    fft.c2r(wh.data(), div);
    fft.r2c(vz, xh.data());
    mult_wavenumber(2, xh.data(), wh.data());
    fft.c2r(wh.data(), tmp);
    vaxpy(div, 1.0, tmp, N);
    fft.r2c(vy, xh.data());
    mult_wavenumber(1, xh.data(), wh.data());
    fft.c2r(wh.data(), tmp);
    vaxpy(div, 1.0, tmp, N);
    st.total_fft_execs += 6;
  }
  // DiffCoef::applyD (src/mat/DiffCoef.cpp:249-271): dc = div(K grad c). Uses t[1..6],t[7].
  void applyD(double* dc, const double* c) {
    gradient(t[4].data(), t[5].data(), t[6].data(), c);
    // applyK (src/mat/DiffCoef.cpp:206-247) with kxy = kxz = kyz = 0
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      t[1][i] = kxx[i] * t[4][i];
      t[2][i] = kxx[i] * t[5][i];
      t[3][i] = kxx[i] * t[6][i];
    }
    divergence(dc, t[1].data(), t[2].data(), t[3].data(), t[7].data());
  }
  // DiffCoef::setSecondaryCoefficients (src/mat/DiffCoef.cpp:44-58): k~ = k1 wm + k2 gm + k3 csf,
  // with k2, k3 from the current ratios when nk = 1
  void setSecondaryCoefficients(double k1, double k2, double k3) {
    if (opt.nk == 1) {
      k2 = k_gm_wm * k1;
      k3 = k_glm_wm * k1;
    }
    ksec.assign(N, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      double v = wm[i] * k1;
      v += k2 * gm[i];
      v += k3 * csf[i];
      ksec[i] = v;
    }
  }
  // DiffCoef::applyDWithSecondaryCoeffs (:273-300): dc = div(k~ grad c); dc may alias c
  void applyDsec(double* dc, const double* c) {
    gradient(t[4].data(), t[5].data(), t[6].data(), c);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      t[1][i] = ksec[i] * t[4][i];
      t[2][i] = ksec[i] * t[5][i];
      t[3][i] = ksec[i] * t[6][i];
    }
    divergence(dc, t[1].data(), t[2].data(), t[3].data(), t[7].data());
  }
  // SpectralOperators::weierstrassSmoother (src/grad/SpectralOperators.cpp:264-381)
  void smooth(double* out, const double* in, double sigma) {
    if (sigma == 0) {
      if (out != in) vcopy(out, in, N);
      return;
    }
    const double twopi = 2.0 * kPi, hx = twopi / n;
    Field f(N);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) {
          double X = i * hx, Xp = X - twopi, Y = j * hx, Yp = Y - twopi, Z = k * hx,
                 Zp = Z - twopi;
          int64_t p = ((int64_t)i * n + j) * n + k;
          double s2 = sigma;
          double v = std::exp((-X * X - Y * Y - Z * Z) / s2 / s2 / 2.0) +
                     std::exp((-Xp * Xp - Yp * Yp - Zp * Zp) / s2 / s2 / 2.0);
          v += std::exp((-Xp * Xp - Y * Y - Z * Z) / s2 / s2 / 2.0) +
               std::exp((-X * X - Yp * Yp - Z * Z) / s2 / s2 / 2.0);
          v += std::exp((-X * X - Y * Y - Zp * Zp) / s2 / s2 / 2.0) +
               std::exp((-Xp * Xp - Yp * Yp - Z * Z) / s2 / s2 / 2.0);
          v += std::exp((-Xp * Xp - Y * Y - Zp * Zp) / s2 / s2 / 2.0) +
               std::exp((-X * X - Yp * Yp - Zp * Zp) / s2 / s2 / 2.0);
          if (v != v) v = 0.;
          f[p] = v;
        }
    double sum_f = vsum(f.data(), N);
    double nf = 1. / (sum_f * hx * hx * hx);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) f[i] *= nf;
    std::vector<cplx> fh(Ns), ch(Ns);
    fft.r2c(f.data(), fh.data());
    fft.r2c(in, ch.data());
    const double alp = (1.0 / ((double)N)) * hx * hx * hx;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < Ns; i++) fh[i] *= (ch[i] * alp);
    fft.c2r(fh.data(), out);
    st.total_fft_execs += 3;
  }

  // ---- DiffusionSolver (src/pde/DiffusionSolver.cpp) ----
  double pc_dt_now() const {
    if (pc_dt_mode == GLIA_PC_DT_FIXED) return pc_dt_fixed;
    return ctx_dt;
  }
  // precFactor (:119-180) for the isotropic tensor, dt_pc given
  void precFactor_dt(double dtpc) {
    const int nh = n / 2 + 1;
    const double factor = 1.0 / ((double)n * n * n);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < nh; z++) {
          double wx = wavenum(x, n), wy = wavenum(y, n), wz = wavenum(z, n);
          double v = (1 + 0.25 * dtpc *
                              (kxx_avg * wx * wx + 2.0 * 0.0 * wx * wy + 2.0 * 0.0 * wx * wz +
                               2.0 * 0.0 * wy * wz + kxx_avg * wy * wy + kxx_avg * wz * wz));
          int64_t i = ((int64_t)x * n + y) * nh + z;
          precfactor[i] = (v == 0) ? factor : factor / v;
        }
  }
  void precFactor() { precFactor_dt(pc_dt_now()); }
  // applyPC (:182-215): y = F^-1 [P F x]
  void applyPC(double* y, const double* x) {
    fft.r2c(x, xh.data());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < Ns; i++) xh[i] *= precfactor[i];
    fft.c2r(xh.data(), y);
    st.total_fft_execs += 2;
  }
  // operatorA (:97-117): y = x - dt/2 * D x, dt = ctx dt
  void operatorA(double* y, const double* x, Field& tmp) {
    vcopy(y, x, N);
    applyD(tmp.data(), y);
    vaxpy(y, -0.5 * ctx_dt, tmp.data(), N);
  }
  // solve (:217-250): (I - dt/2 D) c+ = (I + dt/2 D) c by KSPCG with nonzero initial guess.
  // The CG mirrors PETSc's KSPSolve_CG with KSP_NORM_PRECONDITIONED and KSPConvergedDefault
  // (rtol on ||B b|| because the initial guess is nonzero).
  int solve(double* c, double dts) {
    ctx_dt = dts;
    if (pc_dt_mode == GLIA_PC_DT_MATCHED) precFactor_dt(2.0 * dts);
    st.total_diffusion_solves++;
    if (k_scale == 0) {
      ksp_itr = 0;
      return 0;
    }
    Field b(N), r(N), z(N), p(N), w(N), tmp(N);
    vcopy(b.data(), c, N);
    applyD(tmp.data(), b.data());
    vaxpy(b.data(), 0.5 * dts, tmp.data(), N);
    // r = b - A x
    operatorA(r.data(), c, tmp);
    vaypx(r.data(), -1.0, b.data(), N);
    applyPC(z.data(), r.data());
    double dp = vnorm(z.data(), N);
    // KSPConvergedDefault at n = 0 with a nonzero guess: rnorm0 = ||B b||
    applyPC(tmp.data(), b.data());
    double snorm = vnorm(tmp.data(), N);
    if (snorm == 0) snorm = dp;
    double rnorm0 = snorm, ttol = std::max(rtol * rnorm0, abstol);
    int reason = 0, its = 0;
    auto conv = [&](int k, double rn) {
      if (std::isnan(rn) || std::isinf(rn)) return -9;
      if (rn <= ttol) return 2;
      if (rn >= divtol * rnorm0) return -4;
      (void)k;
      return 0;
    };
    reason = conv(0, dp);
    last_rnorm = dp;
    if (reason == 0) {
      double beta = vdot(z.data(), r.data(), N), betaold = 0, dpi = 0, dpiold = 0;
      int i = 0;
      do {
        its = i + 1;
        if (beta == 0.0) {
          reason = 3;
          break;
        }
        if (i == 0)
          vcopy(p.data(), z.data(), N);
        else
          vaypx(p.data(), beta / betaold, z.data(), N);
        dpiold = dpi;
        operatorA(w.data(), p.data(), tmp);
        dpi = vdot(p.data(), w.data(), N);
        betaold = beta;
        if (dpi == 0.0 || (i > 0 && dpi * dpiold <= 0.0)) {
          reason = -8;
          break;
        }
        double a = beta / dpi;
        vaxpy(c, a, p.data(), N);
        vaxpy(r.data(), -a, w.data(), N);
        applyPC(z.data(), r.data());
        dp = vnorm(z.data(), N);
        last_rnorm = dp;
        reason = conv(i + 1, dp);
        if (reason) break;
        beta = vdot(z.data(), r.data(), N);
        i++;
      } while (i < maxit);
      if (i >= maxit && reason == 0) reason = -3;
    }
    ksp_itr = its;
    st.last_ksp_itr = its;
    st.max_ksp_itr = std::max(st.max_ksp_itr, its);
    st.total_pcg_iterations += its;
    st.last_rnorm = last_rnorm;
    if (reason < 0) {
      err = "oracle PCG did not converge (reason " + std::to_string(reason) + ")";
      return GLIA_ERR_NOT_CONVERGED;
    }
    return 0;
  }

  // ---- DiffCoef / ReacCoef / MatProp ----
  // DiffCoef::setValues (src/mat/DiffCoef.cpp:77-132)
  void diffcoef_setValues(double ks, double kgm, double kglm) {
    k_scale = ks;
    k_gm_wm = kgm;
    k_glm_wm = kglm;
    double dgm = ks * kgm, dwm = ks, dglm = ks * kglm;
    dgm = (dgm <= 0) ? 0.0 : dgm;
    dglm = (dglm <= 0) ? 0.0 : dglm;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) kxx[i] = 0.0 + dgm * gm[i] + dwm * wm[i] + dglm * csf[i];
    kxx_avg = vsum(kxx.data(), N);
    filter_avg = vsum(filter.data(), N);
    kxx_avg *= 1.0 / filter_avg;
  }
  // DiffCoef::setValuesSinusoidal (src/mat/DiffCoef.cpp:134-187)
  void diffcoef_setValuesSinusoidal(double scale) {
    k_scale = scale;
    const double freq = 4;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < n; z++) {
          int64_t i = ((int64_t)x * n + y) * n + z;
          kxx[i] = scale * (0.5 + 0.5 * std::sin(freq * 2.0 * kPi / n * x) *
                                      std::sin(freq * 2.0 * kPi / n * y) *
                                      std::sin(freq * 2.0 * kPi / n * z));
        }
    kxx_avg = vsum(kxx.data(), N) * (1.0 / (double)N);
  }
  // ReacCoef::setValues (src/mat/ReacCoef.cpp:13-38)
  void reaccoef_setValues(double rs, double rgm, double rglm) {
    rho_scale = rs;
    r_gm_wm = rgm;
    r_glm_wm = rglm;
    double dgm = rs * rgm, dwm = rs, dglm = rs * rglm;
    dgm = (dgm <= 0) ? 0.0 : dgm;
    dglm = (dglm <= 0) ? 0.0 : dglm;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) rho_vec[i] = 0.0 + dgm * gm[i] + dwm * wm[i] + dglm * csf[i];
  }
  // MatProp::setValuesCustom (src/mat/MatProp.cpp:134-203)
  void matprop_setValuesCustom(const double* w, const double* g, const double* cs,
                               const double* v) {
    for (int64_t i = 0; i < N; i++) {
      wm[i] = w ? w[i] : 0.0;
      gm[i] = g ? g[i] : 0.0;
      csf[i] = cs ? cs[i] : 0.0;
      vt[i] = v ? v[i] : 0.0;
      gm[i] = (gm[i] <= 0.) ? 0. : gm[i];
      wm[i] = (wm[i] <= 0.) ? 0. : wm[i];
      vt[i] = (vt[i] <= 0.) ? 0. : vt[i];
      csf[i] = (csf[i] <= 0.) ? 0. : csf[i];
      bg[i] = -((gm[i] + wm[i] + vt[i] + csf[i]) - 1.0);
      filter[i] = ((wm[i] > 0.1 || gm[i] > 0.1) && vt[i] < 0.8) ? 1.0 : 0.0;
    }
    tissue_set = true;
  }
  // MatProp::setValuesSinusoidal (src/mat/MatProp.cpp:34-68)
  void matprop_setValuesSinusoidal() {
    const double freq = 4;
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < n; z++) {
          int64_t i = ((int64_t)x * n + y) * n + z;
          wm[i] = 0.5 + 0.5 * std::sin(freq * 2.0 * kPi / n * x) *
                            std::sin(freq * 2.0 * kPi / n * y) *
                            std::sin(freq * 2.0 * kPi / n * z);
          gm[i] = 1 - wm[i];
          vt[i] = 0;
          csf[i] = 0;
          bg[i] = 0;
          filter[i] = 1;
        }
    tissue_set = true;
  }

  // ---- reaction (src/pde/PdeOperators.cpp:140-190, CPU branch) ----
  void reaction(double* c, const double* cl, int linearized) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      double factor = std::exp(rho_vec[i] * dt);
      if (linearized == 0) {
        double alph = c[i] / (1.0 - c[i]);
        if (std::isinf(alph))
          c[i] = 1.0;
        else
          c[i] = alph * factor / (alph * factor + 1.0);
      } else {
        double alph = (cl[i] * factor + 1.0 - cl[i]);
        c[i] = c[i] * factor / (alph * alph);
      }
    }
  }

  // ---- Phi (src/mat/Phi.cpp) ----
  // Each basis function is zero outside the ball r <= 5 sigma (Phi::truncate, :238-260), so it
  // is kept as the grid box [centre - 5 sigma, centre + 5 sigma] clipped to the domain (the
  // Gaussians use non-periodic distances, :294-301). Boxes are stored un-normalised with their
  // maxima, which serves both normalisation modes of Phi::apply / applyTranspose.
  struct Box {
    int lo[3], ext[3];
    Field v;
  };
  std::vector<Box> boxes;
  double phi_smooth_factor = 1.0;
  void box_bounds(const double* cc, int* lo, int* ext) const {
    for (int d = 0; d < 3; d++) {
      double a = (cc[d] - 5.0 * phi_sigma) / h, b = (cc[d] + 5.0 * phi_sigma) / h;
      int l = (int)std::ceil(a - 1e-9), u = (int)std::floor(b + 1e-9);
      l = std::max(l, 0);
      u = std::min(u, n - 1);
      lo[d] = l;
      ext[d] = std::max(0, u - l + 1);
    }
  }
  // Phi::initialize + filter + weierstrassSmoother + truncate for one centre (:96-115)
  void phi_build(Field& out, const double* cc) {
    const double R = std::sqrt(2.) * phi_sigma;
    const double xc = cc[0], yc = cc[1], zc = cc[2];
    out.assign(N, 0.0);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < n; z++) {
          int64_t i = ((int64_t)x * n + y) * n + z;
          double dx = h * x - xc, dy = h * y - yc, dz = h * z - zc;
          double r = std::sqrt(dx * dx + dy * dy + dz * dz);
          double ratio = r / R;
          out[i] = std::exp(-ratio * ratio) * filter[i];
        }
    double sigma_smooth = phi_smooth_factor * 2.0 * kPi / n;
    smooth(out.data(), out.data(), sigma_smooth);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < n; x++)
      for (int y = 0; y < n; y++)
        for (int z = 0; z < n; z++) {
          int64_t i = ((int64_t)x * n + y) * n + z;
          double dx = h * x - xc, dy = h * y - yc, dz = h * z - zc;
          double r = std::sqrt(dx * dx + dy * dy + dz * dz);
          out[i] = (r / phi_sigma <= 5) ? out[i] : 0.0;
        }
  }
  void phi_setValues() {
    boxes.assign(np, Box());
    phi_max_each.assign(np, 0.0);
    Field full;
    for (int i = 0; i < np; i++) {
      phi_build(full, &centers[3 * i]);
      phi_max_each[i] = vmax(full.data(), N);
      Box& b = boxes[i];
      box_bounds(&centers[3 * i], b.lo, b.ext);
      b.v.assign((size_t)b.ext[0] * b.ext[1] * b.ext[2], 0.0);
      for (int a = 0; a < b.ext[0]; a++)
        for (int c = 0; c < b.ext[1]; c++)
          for (int e = 0; e < b.ext[2]; e++)
            b.v[((size_t)a * b.ext[1] + c) * b.ext[2] + e] =
                full[((int64_t)(b.lo[0] + a) * n + (b.lo[1] + c)) * n + (b.lo[2] + e)];
    }
  }
  double phi_max_all() const {
    double m = 0;
    for (double v : phi_max_each) m = std::max(m, v);
    return m;
  }
  void box_axpy(double* out, double a, const Box& b) const {
#pragma omp parallel for schedule(static)
    for (int x = 0; x < b.ext[0]; x++)
      for (int y = 0; y < b.ext[1]; y++)
        for (int z = 0; z < b.ext[2]; z++)
          out[((int64_t)(b.lo[0] + x) * n + (b.lo[1] + y)) * n + (b.lo[2] + z)] +=
              a * b.v[((size_t)x * b.ext[1] + y) * b.ext[2] + z];
  }
  double box_dot(const Box& b, const double* in) const {
    double s = 0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int x = 0; x < b.ext[0]; x++) {
      double sx = 0;
      for (int y = 0; y < b.ext[1]; y++)
        for (int z = 0; z < b.ext[2]; z++)
          sx += b.v[((size_t)x * b.ext[1] + y) * b.ext[2] + z] *
                in[((int64_t)(b.lo[0] + x) * n + (b.lo[1] + y)) * n + (b.lo[2] + z)];
      s += sx;
    }
    return s;
  }
  // Phi::apply (:313-377). stored mode: global max; on-the-fly: max over active functions
  void phi_apply(double* out, const double* p) {
    std::fill(out, out + N, 0.0);
    double pm = 0;
    bool nnz = false;
    for (int i = 0; i < np; i++) {
      if (opt.phi_store) {
        box_axpy(out, p[i], boxes[i]);
      } else if (p[i] != 0) {
        nnz = true;
        pm = std::max(pm, phi_max_each[i]);
        box_axpy(out, p[i], boxes[i]);
      }
    }
    double scale;
    if (opt.phi_store)
      scale = 1.0 / phi_max_all();
    else
      scale = 1.0 / (nnz ? pm : 1.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) out[i] *= scale;
  }
  // Phi::applyTranspose (:379-439): both modes normalise by the max over all functions
  void phi_applyT(double* pout, const double* in) {
    double pm = phi_max_all();
    for (int i = 0; i < np; i++) pout[i] = box_dot(boxes[i], in) * (1.0 / pm);
  }

  // ---- PdeOperatorsRD (src/pde/PdeOperators.cpp) ----
  // solveIncremental (:192-233): c~ += dts / 2 * D~(0.5 (c_i + c_i+1) + c_i) before the step
  // (mode 1) or ... + c_i+1 after it (mode 2); dts is the half step the caller passes
  void solveIncremental(double* ctil, double dts, int iter, int mode) {
    Field temp(N);
    const double* a = c_hist[iter].data();
    const double* b = c_hist[iter + 1].data();
    const double* e = mode == 1 ? a : b;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      double v = a[i] + b[i];
      v *= 0.5;
      v += e[i];
      temp[i] = v;
    }
    applyDsec(temp.data(), temp.data());
    vaxpy(ctil, dts / 2, temp.data(), N);
  }
  // linearized = 0 fills the history; linearized = 1 is the incremental forward around it, the
  // reaction linearised at c_[i] (reaction(1, i) reads c_[iter], :153-156), history untouched;
  // linearized = 2 adds the diffusivity direction's source terms (solveIncremental) around each
  // step, before the first and after the second diffusion half step.
  int solveState(int linearized) {
    if (linearized != 0 && (!state_done || (int)c_hist.size() != nt + 1)) {
      err = "solveState(1) needs a preceding solveState(0)";
      return GLIA_ERR_STATE;
    }
    if (linearized == 2 && (int64_t)ksec.size() != N) {
      err = "solveState(2) needs the secondary diffusion coefficients";
      return GLIA_ERR_STATE;
    }
    st.nb_state_solves++;
    vcopy(ct.data(), c0.data(), N);
    if (linearized == 0 && history_off) {  // the state only (solveState(0), :252-254, 295-298)
      c_hist.clear();
      c_half.clear();
      state_done = false;
      st.diff_ksp_itr_state = 0;
      for (int i = 0; i < nt; i++) {
        int rc;
        if (order == 2) {
          if ((rc = solve(ct.data(), dt / 2.0))) return rc;
          st.diff_ksp_itr_state += ksp_itr;
          reaction(ct.data(), nullptr, 0);
          if ((rc = solve(ct.data(), dt / 2.0))) return rc;
          st.diff_ksp_itr_state += ksp_itr;
        } else {
          if ((rc = solve(ct.data(), dt))) return rc;
          st.diff_ksp_itr_state += ksp_itr;
          reaction(ct.data(), nullptr, 0);
        }
      }
      return 0;
    }
    if (linearized == 0) {
      c_hist.assign(nt + 1, Field());
      c_half.assign(adjoint_store ? nt : 0, Field());
      c_hist[0] = ct;
    }
    st.diff_ksp_itr_state = 0;
    for (int i = 0; i < nt; i++) {
      int rc;
      if (linearized == 2) solveIncremental(ct.data(), dt / 2, i, 1);
      if (order == 2) {
        if ((rc = solve(ct.data(), dt / 2.0))) return rc;
        st.diff_ksp_itr_state += ksp_itr;
        if (linearized == 0 && adjoint_store) c_half[i] = ct;
        reaction(ct.data(), c_hist[i].data(), linearized);
        if ((rc = solve(ct.data(), dt / 2.0))) return rc;
        st.diff_ksp_itr_state += ksp_itr;
        if (linearized == 2) solveIncremental(ct.data(), dt / 2, i, 2);
      } else {
        if ((rc = solve(ct.data(), dt))) return rc;
        st.diff_ksp_itr_state += ksp_itr;
        if (linearized == 0 && adjoint_store) c_half[i] = ct;
        reaction(ct.data(), c_hist[i].data(), linearized);
      }
      if (linearized == 0) c_hist[i + 1] = ct;
    }
    if (linearized == 0) state_done = true;
    return 0;
  }
  // reactionAdjoint (:318-370)
  int reactionAdjoint(int iter) {
    Field tmp;
    if (adjoint_store) {
      tmp = c_half[iter];
    } else {
      tmp = c_hist[iter];
      int rc = solve(tmp.data(), order == 2 ? dt / 2.0 : dt);
      st.diff_ksp_itr_adj += ksp_itr;
      if (rc) return rc;
    }
    reaction(p0.data(), tmp.data(), 1);
    return 0;
  }
  int solveAdjoint(int linearized) {
    if (history_off) {
      err = "solveAdjoint: no time history (GLIA_HISTORY_OFF)";
      return GLIA_ERR_STATE;
    }
    if (!state_done) {
      err = "solveAdjoint needs a preceding solveState";
      return GLIA_ERR_STATE;
    }
    st.nb_adjoint_solves++;
    vcopy(p0.data(), pt.data(), N);
    // the history vectors live as long as nt does (resizeTimeHistory, :49-103, VecSet to 0);
    // p_[nt] changes only in a linearized = 1 sweep
    if ((int)p_hist.size() != nt + 1) p_hist.assign(nt + 1, Field(N, 0.0));
    if (linearized == 1) p_hist[nt] = p0;
    st.diff_ksp_itr_adj = 0;
    for (int i = 0; i < nt; i++) {
      int rc;
      if (order == 2) {
        if ((rc = solve(p0.data(), dt / 2.0))) return rc;
        st.diff_ksp_itr_adj += ksp_itr;
        if ((rc = reactionAdjoint(nt - i - 1))) return rc;
        if ((rc = solve(p0.data(), dt / 2.0))) return rc;
        st.diff_ksp_itr_adj += ksp_itr;
      } else {
        if ((rc = solve(p0.data(), dt))) return rc;
        st.diff_ksp_itr_adj += ksp_itr;
        if ((rc = reactionAdjoint(nt - i - 1))) return rc;
      }
      p_hist[nt - i - 1] = p0;
    }
    return 0;
  }

  // evaluateHessian with diffusivity inversion (src/grad/DerivativeOperatorsRD.cpp:244-397):
  // [Hpp p~ + Hpk k~; Hkp p~ + Hkk k~], each block from its own incremental forward / adjoint
  // pair. The kappa rows are the time integral of grad c_i . grad a~_i over the stored histories,
  // where p_[nt] is the final condition of the last linearized = 1 adjoint (solveAdjoint(2) does
  // not write it). Rows past np + nk (rho) are 0: the reference leaves them as the caller's y.
  int hessianDiffusivity(const double* x, double* y) {
    const int np_ = opt.np, nk = opt.nk;
    std::fill(y, y + nx(), 0.0);
    auto incremental_pair = [&](int lin) -> int {
      int rc = solveState(lin);
      if (rc) return rc;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < N; i++) pt[i] = -(obs_filter[i] * (obs_filter[i] * ct[i]));
      return solveAdjoint(2);
    };
    auto kappa_rows = [&](bool add) {
      Field T(N, 0.0);
      kappaIntegral(T);
      const double v = vdot(wm.data(), T.data(), N) * h3;
      y[np_] = add ? y[np_] + v : v;
      if (nk == 1) y[np_] += vdot(gm.data(), T.data(), N) * h3 * k_gm_wm;
      if (nk > 1) y[np_ + 1] += vdot(gm.data(), T.data(), N) * h3;
      if (nk > 2) y[np_ + 2] += vdot(csf.data(), T.data(), N) * h3;
    };
    std::vector<double> pa(std::max(np_, 1));
    // Hpp p~ (:253-268): c~0 = Phi p~
    phi_apply(c0.data(), x);
    int rc = incremental_pair(1);
    if (rc) return rc;
    phi_applyT(pa.data(), p0.data());
    phi_applyT(y, c0.data());
    for (int i = 0; i < np_; i++) y[i] = (opt.beta * y[i] - pa[i]) * h3;
    // Hkp p~ (:270-316)
    kappa_rows(false);
    // Hpk k~ (:318-349): c~0 = 0, k~ from x's kappa entries, solveState(2)
    std::fill(c0.begin(), c0.end(), 0.0);
    setSecondaryCoefficients(x[np_], nk > 1 ? x[np_ + 1] : 0.0, nk > 2 ? x[np_ + 2] : 0.0);
    if ((rc = incremental_pair(2))) return rc;
    phi_applyT(pa.data(), p0.data());
    for (int i = 0; i < np_; i++) y[i] += -h3 * pa[i];
    // Hkk k~ (:351-397)
    kappa_rows(true);
    return 0;
  }
  // evaluateHessian (src/grad/DerivativeOperatorsRD.cpp:229-438); without diffusivity inversion
  // (:398-425) the Gauss-Newton matvec of the p block around the current history.
  int hessian(const double* x, double* y) {
    if (!state_done) {
      err = "evaluateHessian needs a preceding state solve or gradient";
      return GLIA_ERR_STATE;
    }
    if (two_tp) {  // :234
      err = "evaluateHessian is not implemented for two snapshots";
      return GLIA_ERR_INVALID;
    }
    if (opt.diffusivity_inversion) return hessianDiffusivity(x, y);
    const int np_ = opt.np;
    phi_apply(c0.data(), x);
    int rc = solveState(1);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) pt[i] = -(obs_filter[i] * (obs_filter[i] * ct[i]));
    if ((rc = solveAdjoint(2))) return rc;
    std::vector<double> pa(std::max(np_, 1));
    phi_applyT(pa.data(), p0.data());
    if (opt.regularization_norm != 0) {
      for (int i = 0; i < nx(); i++) y[i] = opt.beta * x[i] - (i < np_ ? h3 * pa[i] : 0.0);
    } else {
      phi_applyT(y, c0.data());
      for (int i = 0; i < np_; i++) y[i] = opt.beta * h3 * y[i] - h3 * pa[i];
      for (int i = np_; i < nx(); i++) y[i] = 0.0;
    }
    return 0;
  }

  // ---- DerivativeOperators (src/grad/DerivativeOperators.cpp, DerivativeOperatorsRD.cpp) ----
  bool update_kappa() const { return opt.diffusivity_inversion || opt.flag_reaction_inv || opt.all_gradients; }
  bool update_rho() const { return opt.flag_reaction_inv || opt.all_gradients; }
  bool apply_phi() const { return !opt.flag_reaction_inv || opt.all_gradients; }
  // updateReactionAndDiffusion (:323-367)
  void updateReactionAndDiffusion(const double* x) {
    const int np_ = opt.np, nk = opt.nk, nr = opt.nr;
    if (update_kappa()) {
      double k1 = x[np_] * opt.k_scale;
      double k2 = nk > 1 ? x[np_ + 1] * opt.k_scale : 0;
      double k3 = nk > 2 ? x[np_ + 2] * opt.k_scale : 0;
      // DiffCoef::updateIsotropicCoefficients (src/mat/DiffCoef.cpp:60-75)
      double rgm = nk == 1 ? k_gm_wm : k2 / k1;
      double rglm = nk == 1 ? k_glm_wm : k3 / k1;
      diffcoef_setValues(k1, rgm, rglm);
      precFactor();
    }
    if (update_rho()) {
      double r1 = x[np_ + nk] * opt.rho_scale;
      double r2 = nr > 1 ? x[np_ + nk + 1] * opt.rho_scale : 0;
      double r3 = nr > 2 ? x[np_ + nk + 2] * opt.rho_scale : 0;
      double rgm = nr == 1 ? r_gm_wm : r2 / r1;
      double rglm = nr == 1 ? r_glm_wm : r3 / r1;
      reaccoef_setValues(r1, rgm, rglm);
    }
  }
  // gradDiffusion (:189-256)
  void gradDiffusion(double* dJ) {
    if (!update_kappa()) return;
    const int np_ = opt.np, nk = opt.nk;
    Field T(N, 0.0);
    kappaIntegral(T);
    dJ[np_] = vdot(wm.data(), T.data(), N) * h3;
    if (nk == 1) dJ[np_] += vdot(gm.data(), T.data(), N) * h3 * k_gm_wm;
    if (nk > 1) dJ[np_ + 1] = vdot(gm.data(), T.data(), N) * h3;
    if (nk > 2) dJ[np_ + 2] = vdot(csf.data(), T.data(), N) * h3;
  }
  // T = sum_i w_i dt grad c_i . grad p_i over the histories (trapezoid, w = 1/2 at the ends)
  void kappaIntegral(Field& T) {
    Field g1(N), g2(N), g3(N), a1(N), a2(N), a3(N);
    for (int i = 0; i < nt + 1; i++) {
      double wgt = (i == 0 || i == nt) ? 0.5 : 1.0;
      gradient(g1.data(), g2.data(), g3.data(), c_hist[i].data());
      gradient(a1.data(), a2.data(), a3.data(), p_hist[i].data());
      const double s = dt * wgt;
#pragma omp parallel for schedule(static)
      for (int64_t j = 0; j < N; j++) {
        double v = g1[j] * a1[j];
        v += g2[j] * a2[j];
        v += g3[j] * a3[j];
        T[j] += s * v;
      }
    }
  }
  // gradReaction (:258-321)
  void gradReaction(double* dJ) {
    if (!update_rho()) return;
    const int np_ = opt.np, nk = opt.nk, nr = opt.nr;
    Field R(N, 0.0);
    for (int i = 0; i < nt + 1; i++) {
      double wgt = (i == 0 || i == nt) ? 0.5 : 1.0;
      const double* c = c_hist[i].data();
      const double* a = p_hist[i].data();
      const double s = dt * wgt;
#pragma omp parallel for schedule(static)
      for (int64_t j = 0; j < N; j++) R[j] += s * ((c[j] * c[j] - c[j]) * a[j]);
    }
    dJ[np_ + nk] = vdot(wm.data(), R.data(), N) * h3;
    if (nr == 1) dJ[np_ + nk] += vdot(gm.data(), R.data(), N) * h3 * r_gm_wm;
    if (nr > 1) dJ[np_ + nk + 1] = vdot(gm.data(), R.data(), N) * h3;
    if (nr > 2) dJ[np_ + nk + 2] = vdot(csf.data(), R.data(), N) * h3;
  }
  int nx() const { return opt.np + opt.nk + opt.nr; }
  // evaluateObjectiveAndGradient (src/grad/DerivativeOperatorsRD.cpp:130-226); want_grad
  // false gives evaluateObjective (:7-61).
  int evaluate(const double* x, const double* data1, double* J, double* dJ, bool want_grad) {
    st.nb_obj_evals += J ? 1 : 0;
    st.nb_grad_evals += want_grad ? 1 : 0;
    const int np_ = opt.np;
    if (want_grad) std::fill(dJ, dJ + nx(), 0.0);
    updateReactionAndDiffusion(x);
    if (apply_phi()) phi_apply(c0.data(), x);
    // ||O0 c(0) - d0||^2 (:148-152)
    double m0 = 0;
    Field r0;
    if (two_tp) {
      r0.assign(N, 0.0);
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < N; i++) r0[i] = c0[i] * obs_filter0[i] - data0[i];
      m0 = vdot(r0.data(), r0.data(), N);
    }
    int rc = solveState(0);
    if (rc) return rc;
    Field tmp(N);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) tmp[i] = ct[i] * obs_filter[i] - data1[i];
    double m1 = vdot(tmp.data(), tmp.data(), N);
    if (want_grad) {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < N; i++) pt[i] = -(tmp[i] * obs_filter[i]);
      if ((rc = solveAdjoint(1))) return rc;
      if (apply_phi()) {
        if (!opt.phi_store) {
          vaxpy(p0.data(), -opt.beta, c0.data(), N);
          phi_applyT(dJ, p0.data());
          for (int i = 0; i < np_; i++) dJ[i] *= -h3;
        } else {
          std::vector<double> pta(np_);
          phi_applyT(pta.data(), p0.data());
          for (int i = 0; i < np_; i++) pta[i] *= h3;
          if (opt.regularization_norm == 0) {
            phi_applyT(dJ, c0.data());
            for (int i = 0; i < np_; i++) dJ[i] = dJ[i] * opt.beta * h3 - pta[i];
          } else {
            for (int i = 0; i < nx(); i++) dJ[i] = x[i] * opt.beta - (i < np_ ? pta[i] : 0.0);
          }
        }
      }
      if (two_tp) {  // dJ += h^3 Phi^T O0^T (O0 c(0) - d0) (:189-196)
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; i++) r0[i] *= obs_filter0[i];
        std::vector<double> pr(std::max(np_, 1));
        phi_applyT(pr.data(), r0.data());
        for (int i = 0; i < np_; i++) dJ[i] += h3 * pr[i];
      }
    }
    double reg = 0;
    if (opt.regularization_norm == 0) {
      reg = vdot(c0.data(), c0.data(), N) * 0.5 * opt.beta * h3;
    } else {
      for (int i = 0; i < np_; i++) reg += x[i] * x[i];
      reg *= 0.5 * opt.beta;
    }
    if (J) *J = h3 * 0.5 * (m1 + m0) + reg;
    if (want_grad) {
      gradDiffusion(dJ);
      gradReaction(dJ);
    }
    return 0;
  }
};

}  // namespace orc

using orc::Ctx;

#define ORC_TRY(expr)                                  \
  try {                                                \
    expr;                                              \
  } catch (const std::exception& e) {                  \
    if (ctx) ctx->err = e.what();                      \
    return GLIA_ERR_INVALID;                           \
  }

struct glia_ctx : public orc::Ctx {
  using orc::Ctx::Ctx;
};

extern "C" {

int oracle_glia_create(int n, int precision, int engine, glia_ctx** out) {
  (void)precision;
  (void)engine;
  if (!out || n < 8 || n > 1024 || (n & (n - 1))) return GLIA_ERR_INVALID;
  try {
    *out = new glia_ctx(n);
  } catch (...) {
    return GLIA_ERR_OOM;
  }
  return GLIA_OK;
}
int oracle_glia_destroy(glia_ctx* ctx) {
  delete ctx;
  return GLIA_OK;
}
const char* oracle_glia_last_error(const glia_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }
int oracle_glia_set_num_threads(int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
}
int oracle_glia_set_time(glia_ctx* ctx, double dt, int nt, int order) {
  if (!ctx || dt <= 0 || nt < 1 || (order != 1 && order != 2)) return GLIA_ERR_INVALID;
  ctx->dt = dt;
  ctx->nt = nt;
  ctx->order = order;
  ctx->ctx_dt = dt;  // a freshly built DiffusionSolver starts from TumorParameters::dt_
  ctx->state_done = false;
  return GLIA_OK;
}
int oracle_glia_set_pcg(glia_ctx* ctx, double rtol, int maxit, int pc_dt_mode, double pc_dt) {
  if (!ctx || rtol <= 0 || maxit < 1) return GLIA_ERR_INVALID;
  ctx->rtol = rtol;
  ctx->maxit = maxit;
  ctx->pc_dt_mode = pc_dt_mode;
  ctx->pc_dt_fixed = pc_dt;
  return GLIA_OK;
}
int oracle_glia_set_history(glia_ctx* ctx, int mode, int every, int adjoint_store) {
  (void)every;  // the oracle keeps every state; checkpointing changes no result
  if (!ctx || mode < GLIA_HISTORY_FULL || mode > GLIA_HISTORY_OFF) return GLIA_ERR_INVALID;
  ctx->adjoint_store = adjoint_store != 0;
  ctx->history_off = mode == GLIA_HISTORY_OFF;
  ctx->state_done = false;
  return GLIA_OK;
}
int oracle_glia_set_opt(glia_ctx* ctx, const glia_opt_settings* s) {
  if (!ctx || !s || s->nk < 1 || s->nk > 3 || s->nr < 1 || s->nr > 3 || s->np < 0)
    return GLIA_ERR_INVALID;
  ctx->opt = *s;
  return GLIA_OK;
}
int oracle_glia_set_tissue(glia_ctx* ctx, const double* wm, const double* gm, const double* csf,
                           const double* vt) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->matprop_setValuesCustom(wm, gm, csf, vt);
  return GLIA_OK;
}
int oracle_glia_set_tissue_sinusoidal(glia_ctx* ctx) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->matprop_setValuesSinusoidal();
  return GLIA_OK;
}
int oracle_glia_set_coefficients(glia_ctx* ctx, double k, double k_gm_wm, double k_glm_wm,
                                 double rho, double r_gm_wm, double r_glm_wm) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->diffcoef_setValues(k, k_gm_wm, k_glm_wm);
  ctx->reaccoef_setValues(rho, r_gm_wm, r_glm_wm);
  ctx->precFactor();
  return GLIA_OK;
}
int oracle_glia_set_diffusivity_sinusoidal(glia_ctx* ctx, double scale) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->diffcoef_setValuesSinusoidal(scale);
  return GLIA_OK;
}
int oracle_glia_prec_factor(glia_ctx* ctx) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->precFactor();
  return GLIA_OK;
}
int oracle_glia_diffusion_solve(glia_ctx* ctx, double* c, double dt, int* its) {
  if (!ctx || !c || dt <= 0) return GLIA_ERR_INVALID;
  int rc = ctx->solve(c, dt);
  if (its) *its = ctx->ksp_itr;
  return rc;
}
int oracle_glia_apply_d(glia_ctx* ctx, const double* c, double* dc) {
  if (!ctx || !c || !dc) return GLIA_ERR_INVALID;
  ctx->applyD(dc, c);
  return GLIA_OK;
}
int oracle_glia_smooth(glia_ctx* ctx, double* out, const double* in, double sigma) {
  if (!ctx || !out || !in) return GLIA_ERR_INVALID;
  ctx->smooth(out, in, sigma);
  return GLIA_OK;
}
int oracle_glia_set_phi(glia_ctx* ctx, const double* centers, int np, double sigma,
                        double smoothing_factor) {
  if (!ctx || !centers || np < 1 || sigma <= 0) return GLIA_ERR_INVALID;
  ctx->np = np;
  ctx->phi_sigma = sigma;
  ctx->phi_smooth_factor = smoothing_factor;
  ctx->centers.assign(centers, centers + 3 * np);
  ORC_TRY(ctx->phi_setValues());
  return GLIA_OK;
}
int oracle_glia_phi_apply(glia_ctx* ctx, const double* p, double* c0) {
  if (!ctx || !p || !c0 || ctx->np < 1) return GLIA_ERR_INVALID;
  ctx->phi_apply(c0, p);
  return GLIA_OK;
}
int oracle_glia_phi_apply_transpose(glia_ctx* ctx, const double* v, double* pout) {
  if (!ctx || !v || !pout || ctx->np < 1) return GLIA_ERR_INVALID;
  ctx->phi_applyT(pout, v);
  return GLIA_OK;
}
int oracle_glia_set_obs_threshold(glia_ctx* ctx, const double* data, double thr) {
  if (!ctx || !data) return GLIA_ERR_INVALID;
  for (int64_t i = 0; i < ctx->N; i++) ctx->obs_filter[i] = double(data[i] > thr);
  return GLIA_OK;
}
int oracle_glia_set_obs_filter(glia_ctx* ctx, const double* f) {
  if (!ctx || !f) return GLIA_ERR_INVALID;
  std::copy(f, f + ctx->N, ctx->obs_filter.begin());
  return GLIA_OK;
}
int oracle_glia_set_obs_threshold0(glia_ctx* ctx, const double* data, double thr) {
  if (!ctx || !data) return GLIA_ERR_INVALID;
  ctx->obs_filter0.assign(ctx->N, 0.0);
  for (int64_t i = 0; i < ctx->N; i++) ctx->obs_filter0[i] = double(data[i] > thr);
  return GLIA_OK;
}
int oracle_glia_set_obs_filter0(glia_ctx* ctx, const double* f) {
  if (!ctx || !f) return GLIA_ERR_INVALID;
  ctx->obs_filter0.assign(f, f + ctx->N);
  return GLIA_OK;
}
int oracle_glia_set_data0(glia_ctx* ctx, const double* d0) {
  if (!ctx) return GLIA_ERR_INVALID;
  if (!d0) {
    ctx->two_tp = false;
    return GLIA_OK;
  }
  ctx->data0.assign(d0, d0 + ctx->N);
  if ((int64_t)ctx->obs_filter0.size() != ctx->N) ctx->obs_filter0.assign(ctx->N, 1.0);
  ctx->two_tp = true;
  return GLIA_OK;
}
int oracle_glia_set_c0(glia_ctx* ctx, const double* c0) {
  if (!ctx || !c0) return GLIA_ERR_INVALID;
  std::copy(c0, c0 + ctx->N, ctx->c0.begin());
  return GLIA_OK;
}
int oracle_glia_set_secondary_coefficients(glia_ctx* ctx, double k1, double k2, double k3) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->setSecondaryCoefficients(k1, k2, k3);
  return GLIA_OK;
}
int oracle_glia_solve_state(glia_ctx* ctx, int linearized, const double* c0, double* c1) {
  if (!ctx || linearized < 0 || linearized > 2) return GLIA_ERR_INVALID;
  if (c0) std::copy(c0, c0 + ctx->N, ctx->c0.begin());
  int rc = ctx->solveState(linearized);
  if (rc) return rc;
  if (c1) std::copy(ctx->ct.begin(), ctx->ct.end(), c1);
  return GLIA_OK;
}
int oracle_glia_solve_adjoint(glia_ctx* ctx, int linearized, const double* pt, double* a0) {
  if (!ctx || (linearized != 1 && linearized != 2)) return GLIA_ERR_INVALID;
  if (pt) std::copy(pt, pt + ctx->N, ctx->pt.begin());
  int rc = ctx->solveAdjoint(linearized);
  if (rc) return rc;
  if (a0) std::copy(ctx->p0.begin(), ctx->p0.end(), a0);
  return GLIA_OK;
}
int oracle_glia_hessian_matvec(glia_ctx* ctx, const double* x, int nx, double* y) {
  if (!ctx || !x || !y || nx != ctx->nx()) return GLIA_ERR_INVALID;
  if (!ctx->state_done) {
    ctx->err = "evaluateHessian needs a preceding state solve or gradient";
    return GLIA_ERR_STATE;
  }
  return ctx->hessian(x, y);
}
int oracle_glia_get_state(glia_ctx* ctx, int i, double* out) {
  if (!ctx || !out || i < 0 || i >= (int)ctx->c_hist.size()) return GLIA_ERR_INVALID;
  std::copy(ctx->c_hist[i].begin(), ctx->c_hist[i].end(), out);
  return GLIA_OK;
}
int oracle_glia_get_adjoint(glia_ctx* ctx, int i, double* out) {
  if (!ctx || !out || i < 0 || i >= (int)ctx->p_hist.size() || ctx->p_hist[i].empty())
    return GLIA_ERR_INVALID;
  std::copy(ctx->p_hist[i].begin(), ctx->p_hist[i].end(), out);
  return GLIA_OK;
}
int oracle_glia_eval_objective(glia_ctx* ctx, const double* x, int nx, const double* d1,
                               double* J) {
  if (!ctx || !x || !d1 || !J || nx != ctx->nx()) return GLIA_ERR_INVALID;
  return ctx->evaluate(x, d1, J, nullptr, false);
}
int oracle_glia_eval_gradient(glia_ctx* ctx, const double* x, int nx, const double* d1,
                              double* dJ) {
  if (!ctx || !x || !d1 || !dJ || nx != ctx->nx()) return GLIA_ERR_INVALID;
  return ctx->evaluate(x, d1, nullptr, dJ, true);
}
int oracle_glia_eval_objective_and_gradient(glia_ctx* ctx, const double* x, int nx,
                                            const double* d1, double* J, double* dJ) {
  if (!ctx || !x || !d1 || !J || !dJ || nx != ctx->nx()) return GLIA_ERR_INVALID;
  return ctx->evaluate(x, d1, J, dJ, true);
}
int oracle_glia_get_stats(const glia_ctx* ctx, glia_stats* st) {
  if (!ctx || !st) return GLIA_ERR_INVALID;
  *st = ctx->st;
  return GLIA_OK;
}
int oracle_glia_reset_stats(glia_ctx* ctx) {
  if (!ctx) return GLIA_ERR_INVALID;
  ctx->st = glia_stats{};
  return GLIA_OK;
}
const char* oracle_glia_version(void) { return "glia-oracle 1 (fp64 cpu)"; }
int oracle_glia_set_pointer_mode(glia_ctx* ctx, int mode) {
  return (ctx && mode == GLIA_PTR_HOST_F64) ? GLIA_OK : GLIA_ERR_INVALID;
}
int oracle_glia_set_stream(glia_ctx* ctx, void* s) {
  (void)s;
  return ctx ? GLIA_OK : GLIA_ERR_INVALID;
}
int oracle_glia_synchronize(glia_ctx* ctx) { return ctx ? GLIA_OK : GLIA_ERR_INVALID; }
int oracle_glia_device_bytes(const glia_ctx* ctx, int64_t* b) {
  if (!ctx || !b) return GLIA_ERR_INVALID;
  *b = 0;
  return GLIA_OK;
}
// Phi::phiMesh (src/mat/Phi.cpp:148-234)
int oracle_glia_phi_mesh(int np, const double cm[3], double sigma, double spacing_factor,
                         double* center) {
  if (np < 1 || !cm || !center) return GLIA_ERR_INVALID;
  int h = (int)std::lround(std::pow((double)np, 1.0 / 3.0));
  double space = spacing_factor * sigma;
  if (np == 1) {
    center[0] = cm[0];
    center[1] = cm[1];
    center[2] = cm[2];
    return GLIA_OK;
  }
  if (h * h * h != np) return GLIA_ERR_INVALID;
  int ptr = 0;
  if (np % 2 == 1) {
    for (int k = -(h - 1) / 2; k <= (h - 1) / 2; k++)
      for (int j = -(h - 1) / 2; j <= (h - 1) / 2; j++)
        for (int i = -(h - 1) / 2; i <= (h - 1) / 2; i++) {
          center[ptr + 0] = i * space + cm[0];
          center[ptr + 1] = j * space + cm[1];
          center[ptr + 2] = k * space + cm[2];
          ptr += 3;
        }
  } else {
    for (int k = -h / 2; k <= h / 2; k++)
      for (int j = -h / 2; j <= h / 2; j++)
        for (int i = -h / 2; i <= h / 2; i++) {
          double mu0 = ((i < 0) ? -1 : ((i > 0) ? 1 : 0)) * 0.5;
          double mu1 = ((j < 0) ? -1 : ((j > 0) ? 1 : 0)) * 0.5;
          double mu2 = ((k < 0) ? -1 : ((k > 0) ? 1 : 0)) * 0.5;
          if (i != 0 && j != 0 && k != 0) {
            center[ptr + 0] = (i - mu0) * space + cm[0];
            center[ptr + 1] = (j - mu1) * space + cm[1];
            center[ptr + 2] = (k - mu2) * space + cm[2];
            ptr += 3;
          }
        }
  }
  return GLIA_OK;
}
// Phi::setGaussians(Vec data) (src/mat/Phi.cpp:615-1004) on one process, where every lattice point
// is local and the neighbour exchange sends nothing: gaussian_interior from the offset loops
// (:646-653), the first and last lattice index (:679-712), the lattice loops with x += space on
// an int (:717-719), checkTumorExistenceOutOfProc's clipped ball count (:486-520; with one
// process every point is in range exactly when it lies on the grid), the selection
// marker > gvf * interior in index order with X * h coordinates (:870-891) and
// num_tumor_output = marker / interior (:871).
int oracle_glia_phi_data_centers(glia_ctx* ctx, const double* data, double sigma, double thr,
                                 double gvf, double spacing_factor, int max_centers,
                                 double* centers, int* np_out, double* frac) {
  if (!ctx || !data || !np_out || max_centers < 0 || (max_centers > 0 && !centers))
    return GLIA_ERR_INVALID;
  const int n = ctx->n;
  const double hx = 2.0 * M_PI / n;
  const double space = spacing_factor * sigma / hx;
  if (!(sigma > 0) || !(space >= 1.0) || !(gvf >= 0)) return GLIA_ERR_INVALID;
  int gaussian_interior = 0;
  for (int i = -sigma / hx; i <= sigma / hx; i++)
    for (int j = -sigma / hx; j <= sigma / hx; j++)
      for (int k = -sigma / hx; k <= sigma / hx; k++)
        if (std::sqrt((double)(i * i + j * j + k * k)) <= sigma / hx) gaussian_interior++;
  std::vector<int> marker((size_t)ctx->N, 0);
  int start = -1, end = -1;
  for (int x = 0; x < n && start < 0; x++)
    if (std::fmod((double)x, space) == 0) start = x;
  for (int x = n - 1; x >= 0 && end < 0; x--)
    if (std::fmod((double)x, space) == 0) end = x;
  const double radius = sigma / hx;
  for (int x = start; start >= 0 && x <= end; x += space)
    for (int y = start; y <= end; y += space)
      for (int z = start; z <= end; z += space) {
        int num_tumor = 0;
        for (int i = x - radius; i <= x + radius; i++)
          for (int j = y - radius; j <= y + radius; j++)
            for (int k = z - radius; k <= z + radius; k++) {
              if (i < 0 || j < 0 || k < 0 || i >= n || j >= n || k >= n) continue;
              const double distance =
                  std::sqrt((double)((i - x) * (i - x) + (j - y) * (j - y) + (k - z) * (k - z)));
              if (distance <= radius && data[((int64_t)i * n + j) * n + k] > thr) num_tumor++;
            }
        marker[((size_t)x * n + y) * n + z] = num_tumor;
      }
  int count = 0;
  for (int64_t i = 0; i < ctx->N; i++) {
    if (frac) frac[i] = (double)marker[(size_t)i] / gaussian_interior;
    if (marker[(size_t)i] > gvf * gaussian_interior) {
      const int64_t X = i / ((int64_t)n * n), Y = (i / n) % n, Z = i % n;
      if (count < max_centers) {
        centers[3 * count] = X * hx;
        centers[3 * count + 1] = Y * hx;
        centers[3 * count + 2] = Z * hx;
      }
      count++;
    }
  }
  *np_out = count;
  return count > max_centers ? GLIA_ERR_INVALID : GLIA_OK;
}
// Raw FFT access for the numpy cross-check.
int oracle_fft_r2c(int n, const double* in, double* out_interleaved) {
  orc::FFT3 f;
  f.init(n);
  f.r2c(in, reinterpret_cast<orc::cplx*>(out_interleaved));
  return GLIA_OK;
}
int oracle_fft_c2r(int n, const double* in_interleaved, double* out) {
  orc::FFT3 f;
  f.init(n);
  f.c2r(reinterpret_cast<const orc::cplx*>(in_interleaved), out);
  return GLIA_OK;
}
}  // extern "C"

/*
 * glia_rd.h — C-ABI of the GB300-native reaction–diffusion forward / adjoint path.
 *
 * Model: dc/dt = div(k(x) grad c) + rho(x) c (1 - c) on the periodic grid [0, 2*pi)^3 with n^3
 * voxels (row-major, z fastest: idx = x*n*n + y*n + z). Strang splitting (order 2) or Lie
 * splitting (order 1); each diffusion sub-step is Crank–Nicolson solved by PCG with the spectral
 * mean-diffusivity preconditioner; the logistic reaction sub-step is analytic.
 *
 * Every entry point replaces one method of the reference's C++/PETSc classes; the replaced
 * interface is cited next to each declaration (paths are relative to the GLIA source tree).
 *
 * Conventions
 *  - Every function returns an int status: GLIA_OK (0) or a negative GLIA_ERR_* code.
 *    glia_last_error(ctx) returns the message of the last failure on that context.
 *    No C++ exception crosses this boundary.
 *  - A context owns its device work buffers, cuFFT plans, time history and checkpoints.
 *    The caller owns every buffer it passes. A context is not thread-safe: use one per host
 *    thread (and per CUDA stream).
 *  - Grid fields (n^3 values) are passed as `const void*` / `void*`; their location and element
 *    type follow the context's pointer mode (glia_set_pointer_mode): host double (default),
 *    device double or device float. Parameter vectors (p, x, dJ, centers) are always host double.
 *  - Floating-point state is FP64 (GLIA_FP64) or FP32 bulk with FP64 reductions and FP64
 *    scalars (GLIA_MIXED). GLIA_ENGINE_REFERENCE restates the reference's GPU structure
 *    (real-space PCG, one kernel per vector operation, 10 transforms per diffusion apply) and
 *    exists as the plain baseline; GLIA_ENGINE_FUSED is the fused spectral-space path.
 */
#ifndef GLIA_RD_H_
#define GLIA_RD_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------ */
#define GLIA_OK 0
#define GLIA_ERR_INVALID (-1)       /* bad argument or unsupported size                        */
#define GLIA_ERR_CUDA (-2)          /* CUDA runtime error (message has the CUDA error string)  */
#define GLIA_ERR_CUFFT (-3)         /* cuFFT plan or execution error                           */
#define GLIA_ERR_NOT_CONVERGED (-4) /* PCG reached maxit, diverged or hit a NaN                */
#define GLIA_ERR_STATE (-5)         /* call order: e.g. adjoint before a state solve           */
#define GLIA_ERR_OOM (-6)           /* device allocation failed                                */
#define GLIA_ERR_NONFINITE (-7)     /* a non-finite value reached a reduction                  */
#define GLIA_ERR_NO_DEVICE (-8)     /* no CUDA device is visible                               */

/* ---- context configuration --------------------------------------------------------------- */
#define GLIA_FP64 0  /* all fields, transforms and reductions in double                        */
#define GLIA_MIXED 1 /* fields and transforms in float; reductions, PCG scalars, gradients FP64 */

#define GLIA_ENGINE_FUSED 0     /* fused spectral-space PCG (the product path)                  */
#define GLIA_ENGINE_REFERENCE 1 /* reference-structured plain path (baseline, FP64 or float)    */

#define GLIA_PTR_HOST_F64 0   /* grid fields are host double arrays                            */
#define GLIA_PTR_DEVICE_F64 1 /* grid fields are device double arrays                          */
#define GLIA_PTR_DEVICE_F32 2 /* grid fields are device float arrays                           */

/* Time history kept for the adjoint (PdeOperatorsRD ctor, src/pde/PdeOperators.cpp:17-55). */
#define GLIA_HISTORY_FULL 0       /* every state c_[0..nt] (and c_half_ when adjoint_store) */
#define GLIA_HISTORY_CHECKPOINT 1 /* every k-th state; segments recomputed in the adjoint    */
#define GLIA_HISTORY_OFF 2        /* time_history_off_: no states kept (forward-only runs);  */
                                  /* adjoint, gradient and Hessian return GLIA_ERR_STATE     */

/* Which dt the spectral preconditioner is built with (DiffusionSolver::precFactor,
 * src/pde/DiffusionSolver.cpp:119-180, reads ctx_->dt_, which solve() overwrites at :226). */
#define GLIA_PC_DT_REFERENCE 0 /* reference rule: dt of the last solve, full dt before any   */
#define GLIA_PC_DT_FIXED 1     /* the value given to glia_set_pcg                            */
#define GLIA_PC_DT_MATCHED 2   /* twice the dt of each solve (exact for constant k)          */

typedef struct glia_ctx glia_ctx;

/* Optimizer-side settings read by the derivative operators (include/Parameters.h:17-109). */
typedef struct glia_opt_settings {
  int np;                    /* number of Gaussian coefficients p                               */
  int nk;                    /* number of diffusivity parameters (1..3)                         */
  int nr;                    /* number of reaction parameters (1..3)                            */
  int flag_reaction_inv;     /* OptimizerSettings::flag_reaction_inv_: no Phi apply, rho grad   */
  int diffusivity_inversion; /* OptimizerSettings::diffusivity_inversion_: kappa from x, grad   */
  int regularization_norm;   /* 0 = L2 (on Phi p), 1 = L2b (on p)                              */
  double beta;               /* OptimizerSettings::beta_                                        */
  double k_scale;            /* OptimizerSettings::k_scale_ (x entries are multiplied by it)    */
  double rho_scale;          /* OptimizerSettings::rho_scale_                                   */
  int phi_store;             /* TumorParameters::phi_store_: stored-Phi gradient formula        */
  int all_gradients;         /* extension: p, kappa and rho gradients from one sweep            */
} glia_opt_settings;

/* Counters (TumorStatistics, include/utils/Utils.h:43-96, and PdeOperators::diff_ksp_itr_*). */
typedef struct glia_stats {
  int64_t nb_state_solves;
  int64_t nb_adjoint_solves;
  int64_t nb_obj_evals;
  int64_t nb_grad_evals;
  int64_t diff_ksp_itr_state; /* PCG iterations accumulated over the last solveState          */
  int64_t diff_ksp_itr_adj;   /* PCG iterations accumulated over the last solveAdjoint        */
  int64_t total_diffusion_solves;
  int64_t total_pcg_iterations;
  int64_t total_fft_execs; /* 3-D transforms executed (a batch of b counts b)               */
  int last_ksp_itr;        /* DiffusionSolver::ksp_itr_ of the last solve                   */
  int max_ksp_itr;
  double last_rnorm; /* final preconditioned residual norm of the last solve              */
} glia_stats;

/* ---- lifecycle ----------------------------------------------------------------------------- */
/* initializeGrid(n, params, spec_ops) + SpectralOperators::setup
 * (src/grad/SpectralOperators.cpp:19-66, 424-446). n must be even, 8 <= n <= 1024. */
int glia_create(int n, int precision, int engine, glia_ctx** out);
int glia_destroy(glia_ctx* ctx);
const char* glia_last_error(const glia_ctx* ctx);
const char* glia_version(void);
int glia_set_pointer_mode(glia_ctx* ctx, int mode);
int glia_set_stream(glia_ctx* ctx, void* cuda_stream); /* NULL = the context's own stream */
int glia_synchronize(glia_ctx* ctx);
/* Launch shape (extension; no counterpart in the reference): CTAs per SM of the bandwidth
 * kernels (1..16, default 8) and of the reducing kernels (1..8, default 4). Smaller grids let
 * several contexts on different streams share the GPU (batches of small problems). */
int glia_set_launch_geometry(glia_ctx* ctx, int pointwise_blocks_per_sm,
                             int reduce_blocks_per_sm);
/* Device bytes currently held by the context (fields, spectra, history, plans). */
int glia_device_bytes(const glia_ctx* ctx, int64_t* bytes);

/* ---- parameters ---------------------------------------------------------------------------- */
/* TumorParameters::dt_, nt_, order_ (include/Parameters.h:164-166, 226). Resizes the history
 * like PdeOperatorsRD::resizeTimeHistory (src/pde/PdeOperators.cpp:57-103). */
int glia_set_time(glia_ctx* ctx, double dt, int nt, int order);
/* KSPSetTolerances(ksp_, 1e-6, default, default, 5000) (src/pde/DiffusionSolver.cpp:27). */
int glia_set_pcg(glia_ctx* ctx, double rtol, int maxit, int pc_dt_mode, double pc_dt);
/* TumorParameters::adjoint_store_ / time_history_off_ plus the checkpoint extension. */
int glia_set_history(glia_ctx* ctx, int mode, int checkpoint_every, int adjoint_store);
int glia_set_opt(glia_ctx* ctx, const glia_opt_settings* s);

/* ---- material properties and coefficients -------------------------------------------------- */
/* MatProp::setValuesCustom (src/mat/MatProp.cpp:134-203): NULL maps are zero; clip >= 0,
 * bg = 1 - sum, filter = [(wm > 0.1 or gm > 0.1) and vt < 0.8]. */
int glia_set_tissue(glia_ctx* ctx, const void* wm, const void* gm, const void* csf, const void* vt);
/* MatProp::setValuesSinusoidal (src/mat/MatProp.cpp:34-68). */
int glia_set_tissue_sinusoidal(glia_ctx* ctx);
/* DiffCoef::setValues (src/mat/DiffCoef.cpp:77-132) + ReacCoef::setValues
 * (src/mat/ReacCoef.cpp:13-38) + DiffusionSolver::precFactor. */
int glia_set_coefficients(glia_ctx* ctx, double k, double k_gm_wm, double k_glm_wm, double rho,
                          double r_gm_wm, double r_glm_wm);
/* DiffCoef::setValuesSinusoidal (src/mat/DiffCoef.cpp:134-187); does not refactor the PC. */
int glia_set_diffusivity_sinusoidal(glia_ctx* ctx, double scale);
/* DiffusionSolver::precFactor() (src/pde/DiffusionSolver.cpp:119-180). */
int glia_prec_factor(glia_ctx* ctx);
/* DiffusionSolver::solve(Vec c, dt) (src/pde/DiffusionSolver.cpp:217-250); c in/out. */
int glia_diffusion_solve(glia_ctx* ctx, void* c, double dt, int* ksp_itr);
/* DiffCoef::applyD(dc, c) (src/mat/DiffCoef.cpp:249-271). */
int glia_apply_d(glia_ctx* ctx, const void* c, void* dc);
/* SpectralOperators::weierstrassSmoother (src/grad/SpectralOperators.cpp:264-381). */
int glia_smooth(glia_ctx* ctx, void* out, const void* in, double sigma);

/* ---- Gaussian basis (Phi) ------------------------------------------------------------------ */
/* Phi::phiMesh (src/mat/Phi.cpp:148-234): np lattice centres around cm, spacing = factor*sigma.
 * Host-only helper; centers_out holds 3*np doubles. */
int glia_phi_mesh(int np, const double cm[3], double sigma, double spacing_factor,
                  double* centers_out);
/* Phi::setGaussians (explicit centres) + Phi::setValues (src/mat/Phi.cpp:33-144): each basis
 * function is trunc_5sigma(W_smooth * (filter * gaussian)); normalised by the global max.
 * Requires tissue. smoothing_factor: sigma_smooth = factor * 2*pi/n. */
int glia_set_phi(glia_ctx* ctx, const double* centers, int np, double sigma,
                 double smoothing_factor);
/* Phi::apply (src/mat/Phi.cpp:313-377): c0 = Phi p. */
int glia_phi_apply(glia_ctx* ctx, const double* p, void* c0);
/* Phi::applyTranspose (src/mat/Phi.cpp:379-439): pout = Phi^T v. */
int glia_phi_apply_transpose(glia_ctx* ctx, const void* v, double* pout);
/* Phi::setGaussians(Vec data) (src/mat/Phi.cpp:615-1004, checkTumorExistence :457-520) for one
 * process: Gaussian centres placed where the data has tumour. Lattice points X (each axis from
 * the first to the last index with fmod(X, space) == 0, advancing by X += space on an integer;
 * space = spacing_factor * sigma / h voxels) keep a centre when more than
 * gaussian_vol_frac * (grid points of the ball of radius sigma / h) points of the ball around
 * them, clipped to the grid, hold data > data_threshold (compared in FP64). data is in the
 * context's pointer mode. centers receives up to max_centers (x, y, z) triples in [0, 2 pi),
 * in the reference's x-major order; *np_out the number found (GLIA_ERR_INVALID, with *np_out
 * set, when it exceeds max_centers). frac (may be NULL; pointer mode) receives the
 * reference's num_tumor_output: count / ball size at the lattice points, 0 elsewhere.
 * sigma > 0, gaussian_vol_frac >= 0 and a spacing of at least one voxel are required. */
int glia_phi_data_centers(glia_ctx* ctx, const void* data, double sigma, double data_threshold,
                          double gaussian_vol_frac, double spacing_factor, int max_centers,
                          double* centers, int* np_out, void* frac);

/* ---- observation operator ------------------------------------------------------------------ */
/* Obs::setDefaultFilter (src/mat/Obs.cpp:26-55): filter = [data > thr]. */
int glia_set_obs_threshold(glia_ctx* ctx, const void* data, double thr);
/* Obs::setCustomFilter (src/mat/Obs.cpp:57-69). */
int glia_set_obs_filter(glia_ctx* ctx, const void* filter);
/* The same two for the observation operator at t = 0 of the two-snapshot objective
 * (Obs::setDefaultFilter / setCustomFilter with time_point 0, filter_0_; 1 until set). */
int glia_set_obs_threshold0(glia_ctx* ctx, const void* data, double thr);
int glia_set_obs_filter0(glia_ctx* ctx, const void* filter);
/* Data::dt0 with TumorParameters::two_time_points_ (include/utils/Utils.h:99-124): the data at
 * t = 0. With it the objective gains h^3/2 ||O0 c(0) - d0||^2 and the p gradient
 * h^3 Phi^T O0^T (O0 c(0) - d0) (src/grad/DerivativeOperatorsRD.cpp:29-33, 114-120, 148-152,
 * 189-196); the Hessian returns GLIA_ERR_INVALID as the reference's (:234). d0 = NULL goes back to
 * one snapshot. */
int glia_set_data0(glia_ctx* ctx, const void* d0);

/* ---- PDE operators --------------------------------------------------------------------------- */
/* Tumor::c_0_ (used by the derivative operators when flag_reaction_inv is set). */
int glia_set_c0(glia_ctx* ctx, const void* c0);
/* DiffCoef::setSecondaryCoefficients (src/mat/DiffCoef.cpp:44-58): the diffusivity direction
 * k~ = k1 wm + k2 gm + k3 csf of the incremental forward with linearized = 2 (k2, k3 from the
 * current gm / glm ratios when nk = 1). */
int glia_set_secondary_coefficients(glia_ctx* ctx, double k1, double k2, double k3);
/* PdeOperatorsRD::solveState(int linearized) (src/pde/PdeOperators.cpp:235-316).
 * c0 may be NULL (use Tumor::c_0_); c1 may be NULL. linearized = 0: the state equation (fills
 * the history); 1: the incremental forward around the history of the last linearized = 0 solve,
 * the logistic step linearised at the state at each step's start (reaction(1, i), :140-190);
 * 2: as 1 plus the sources of the diffusivity direction (solveIncremental, :192-233) around each
 * step, dt/4 div(k~ grad(0.5 (c_i + c_i+1) + c_i)) before the first diffusion half step and
 * ... + c_i+1 after the second (needs glia_set_secondary_coefficients). */
int glia_solve_state(glia_ctx* ctx, int linearized, const void* c0, void* c1);
/* PdeOperatorsRD::solveAdjoint(int linearized) (src/pde/PdeOperators.cpp:372-420).
 * Needs a preceding glia_solve_state. a0 may be NULL. linearized = 1: adjoint; 2: incremental
 * adjoint of the Hessian matvec (same sweep, p_[nt] of the history left as it was). */
int glia_solve_adjoint(glia_ctx* ctx, int linearized, const void* pt, void* a0);
/* PdeOperatorsRD::c_[i] (FULL history only) / p_[i] (after an adjoint, FULL history only). */
int glia_get_state(glia_ctx* ctx, int i, void* out);
int glia_get_adjoint(glia_ctx* ctx, int i, void* out);

/* ---- derivative operators -------------------------------------------------------------------- */
/* DerivativeOperatorsRD::evaluateObjective (src/grad/DerivativeOperatorsRD.cpp:7-61).
 * x = [p (np), kappa (nk), rho (nr)], d1 = data at t = 1 (grid field). */
int glia_eval_objective(glia_ctx* ctx, const double* x, int nx, const void* d1, double* J);
/* DerivativeOperatorsRD::evaluateGradient (src/grad/DerivativeOperatorsRD.cpp:63-127). */
int glia_eval_gradient(glia_ctx* ctx, const double* x, int nx, const void* d1, double* dJ);
/* DerivativeOperatorsRD::evaluateObjectiveAndGradient
 * (src/grad/DerivativeOperatorsRD.cpp:130-226). */
int glia_eval_objective_and_gradient(glia_ctx* ctx, const double* x, int nx, const void* d1,
                                     double* J, double* dJ);
/* DerivativeOperatorsRD::evaluateHessian (src/grad/DerivativeOperatorsRD.cpp:229-438): the
 * Gauss-Newton matvec y = H x, linearised at the state history of the last gradient evaluation
 * or state solve (so call it after glia_eval_* at the current iterate). x and y have
 * nx = np + nk + nr entries (host doubles).
 * Without diffusivity inversion (:398-425), the p block: c~0 = Phi x, incremental forward
 * (glia_solve_state 1), p~_t = -O^T O c~(1), incremental adjoint (glia_solve_adjoint 2),
 * y = h^3 (beta Phi^T c~0 - Phi^T a~0), or beta x - h^3 Phi^T a~0 with the L2b regulariser;
 * entries past np are beta x (L2b) or 0.
 * With diffusivity inversion (:244-397), the p and kappa blocks [Hpp p~ + Hpk k~;
 * Hkp p~ + Hkk k~]: a second incremental pair from c~0 = 0 with k~ = x's kappa entries
 * (glia_set_secondary_coefficients, glia_solve_state 2); the kappa rows integrate
 * grad c . grad a~ in time like the gradient, where the t = 1 term reads p_[nt] as the reference
 * leaves it: the final condition of the last linearized = 1 adjoint (0 before the first). The
 * p rows use the L2 form. Rows past np + nk (rho) are 0. */
int glia_hessian_matvec(glia_ctx* ctx, const double* x, int nx, double* y);

int glia_get_stats(const glia_ctx* ctx, glia_stats* st);
int glia_reset_stats(glia_ctx* ctx);

/* ---- kernel timing (extension; no counterpart in the reference) ----------------------------
 * While enabled, every launch of this library (kernels, cuFFT executions, copies) is bracketed
 * by CUDA events on the context's stream and accumulated per kernel slot together with the
 * algorithmic bytes the launch must move. Enabling clears the counters. glia_get_timing returns
 * the number of slots (>= 1) or a negative status; slot names are static strings. */
int glia_set_timing(glia_ctx* ctx, int enable);
int glia_get_timing(glia_ctx* ctx, int slot, const char** name, int64_t* launches, double* ms,
                    double* algorithmic_bytes);

/* ---- batches of gradient evaluations in one CUDA graph ---------------------------------------
 * The batched form of DerivativeOperatorsRD::evaluateObjectiveAndGradient
 * (src/grad/DerivativeOperatorsRD.cpp:130-226) over independent problems, one context each (the
 * reference has no batch interface: it evaluates one problem per process). glia_batch_capture
 * runs the host part of every evaluation at its x and d1 (coefficient update, Phi p, data in the
 * contexts' pointer modes), then captures all evaluations into one graph: a fork from the
 * batch's stream into every context's stream, each context's forward, adjoint and gradient
 * sweeps with its PCG loops as conditional WHILE nodes, a join. group[i] (NULL: all 0) orders
 * the branches: contexts of one group run as parallel branches, groups one after another in
 * increasing order. glia_batch_launch launches the graph once (stream NULL = the batch's own
 * stream); every launch recomputes the evaluations captured at those x and d1 from the
 * coefficients, Phi p and data that the capture left in each context: a call on a context
 * between capture and launch that changes them (coefficients, Phi, data, an ordinary
 * evaluation at another x) changes what the next launch computes, so capture again after such
 * calls; a new x needs a new capture. Until glia_batch_results has read a launch, the contexts
 * report no state history (get_state / solve_adjoint refuse). glia_batch_results waits for
 * the launch and writes J[i] and dJ[i] (np + nk + nr entries each; dJ NULL: objectives only).
 * Requirements: the fused engine, one snapshot, phi_store = 0, a history mode other than OFF,
 * timing disabled, every context on its own non-default stream, and one ordinary evaluation of
 * each context beforehand (its first call sets up the plans and graphs a capture cannot
 * create). Errors name the failing context; its own message is in glia_last_error. */
typedef struct glia_batch glia_batch;
int glia_batch_create(glia_ctx* const* ctxs, int n, glia_batch** out);
int glia_batch_capture(glia_batch* b, const double* const* x, const int* nx,
                       const void* const* d1, const int* group);
int glia_batch_launch(glia_batch* b, void* stream);
int glia_batch_results(glia_batch* b, void* stream, double* J, double* const* dJ);
const char* glia_batch_last_error(const glia_batch* b);
int glia_batch_destroy(glia_batch* b);

/* ---- data mismatch without allocation (extension; no counterpart in the reference) ---------
 * For callers that cannot let a library allocate device memory: code that captures its loss
 * evaluation into a CUDA graph (cudaMalloc is not allowed during stream capture), processes
 * that run under a fixed device-memory budget held by their own allocator, and callers with no
 * glia context. Computes *sumsq = sum_i (obs_i c_i - d_i)^2 (the ||O c(1) - d||^2 term of
 * DerivativeOperatorsRD::evaluateObjective, before the h^3/2 factor) and, when pt is not NULL,
 * pt_i = -obs_i (obs_i c_i - d_i) (the adjoint final condition). All pointers are device
 * pointers (float fields, one double result); work is ordered on `stream` (NULL = the legacy
 * default stream). It needs no context and calls no allocator: its reduction scratch is a
 * static 64 KiB device array shared by every call, which limits n to 2^29 voxels (larger n
 * returns GLIA_ERR_INVALID). The first call in each CUDA context (the device's primary context,
 * or any other context current at the call) resolves that array's address with
 * cudaGetSymbolAddress and must come before any stream capture. Calls that overlap on the GPU
 * race on the shared scratch; serialise them. */
int glia_mismatch_f32_noalloc(const float* c, const float* obs, const float* d, float* pt,
                              int64_t n, double* sumsq, void* stream);

/* Diagnostic (extension; no counterpart in the reference): checks the bounded device waits the
 * TMA staging relies on. One CTA waits on an mbarrier that no copy signals; the wait gives up
 * after about 2^31 SM cycles (one second at 2 GHz) and records the fault in the context's device
 * scalars, which this call reads and clears. Returns GLIA_OK when the fault was recorded and the
 * context still runs kernels afterwards, GLIA_ERR_CUDA otherwise. FP32 contexts only. */
int glia_selftest_bounded_wait(glia_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* GLIA_RD_H_ */

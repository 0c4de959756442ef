// The reference's "Running diffusion solver" test (src/test/pdesolver.cpp:7-56), written
// against the C++ shim over the C-ABI: the same calls in the same order and the same two
// assertions. Exit status 0 = pass. argv[1]: 0 = FP64 (default), 1 = mixed precision.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "glia/shim.hpp"

using namespace glia_shim;

// createTestFunction (src/test/helper.cpp:17-45)
static void createTestFunction(Vec& x, const Parameters& params) {
  const int n = params.grid_->n_[0];
  const ScalarType R = std::sqrt(2.) * (2 * M_PI) / 64;
  for (int X = 0; X < n; X++)
    for (int Y = 0; Y < n; Y++)
      for (int Z = 0; Z < n; Z++) {
        const ScalarType dx = params.grid_->h_[0] * X - M_PI, dy = params.grid_->h_[1] * Y - M_PI,
                         dz = params.grid_->h_[2] * Z - M_PI;
        const ScalarType ratio = std::sqrt(dx * dx + dy * dy + dz * dz) / R;
        x[((size_t)X * n + Y) * n + Z] = std::exp(-ratio * ratio);
      }
}

int main(int argc, char** argv) {
  auto params = std::make_shared<Parameters>();
  params->engine_.precision = argc > 1 ? std::atoi(argv[1]) : GLIA_FP64;
  auto spec_ops = std::make_shared<SpectralOperators>();
  if (initializeGrid(64, params, spec_ops) != 0) {
    std::printf("initializeGrid failed\n");
    return 2;
  }
  auto k = std::make_shared<DiffCoef>(params, spec_ops);
  k->setValuesSinusoidal(params, 1E-2);
  auto diff_solver = std::make_shared<DiffusionSolver>(params, spec_ops, k);
  Vec c(params->grid_->ng_, 0.0);
  createTestFunction(c, *params);
  diff_solver->precFactor();
  for (int i = 0; i < 10; i++) spec_ops->check(diff_solver->solve(c, 0.02), "solve");
  double s = 0;
  for (double v : c) s += v * v;
  const double nrm = std::sqrt(s);
  // Catch2 Approx default epsilon (100 * float epsilon) for FP64; 1e-4 relative when mixed
  const double eps = params->engine_.precision == GLIA_FP64 ? 100 * FLT_EPSILON : 1e-4;
  const bool ok_norm = std::fabs(nrm - 2.0487) <= eps * 2.0487;
  const bool ok_its = diff_solver->ksp_itr_ == 5;
  std::printf("||c||_2 = %.7f (expect 2.0487), ksp_itr_ = %d (expect 5)\n", nrm,
              diff_solver->ksp_itr_);
  return (ok_norm && ok_its) ? 0 : 1;
}

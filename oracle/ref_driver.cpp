/*
 * ref_driver.cpp - runs the reference's own multicore engine
 * (MulticoreEngineExecutor with the loss plugins of lossFunction 0-3,
 * compiled from the reference sources with the GSL shim) on arrays passed in,
 * so tests can pin the oracle against the reference itself.
 *
 * TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by `make -C oracle ref`
 * when the reference sources are present; nothing on the product path or on
 * the GPU machine needs it.
 *
 * The engine is driven as cpp/src/solver/Solver.h:43-65 drives it: repeated
 * executeBulkOfIterations() calls with getObjectiveValue() after each bulk.
 * The settings are set directly (the pattern of
 * cpp/src/experiments/minibatch_sdca_experiment.cpp:20-51).
 */
#include "solver/MulticoreEngineExecutor.h"
#include "solver/Solver.h"

#include <cstdint>

namespace {
void reset_sampler(uint64_t seed) {
  // gsl_rng_r is the reference's per-thread generator
  // (cpp/src/utils/randomNumbersUtil.h:11-13); restart every thread's stream.
#pragma omp parallel
  { gsl_rng_set(gsl_rng_r, (unsigned long)seed); }
}
}  // namespace

extern "C" int ref_lasso_run(int m, int n, const int* col_ptr, const int* row_idx,
                             const double* vals, const double* b, double lambda, int threads,
                             uint64_t seed, int bulks, unsigned long inner, double* x_out,
                             double* r_out, double* obj_out) {
  OptimizationSettings settings;
  settings.lossFunction = 0;
  settings.totalThreads = threads;
  settings.innerIterations = inner;
  settings.verbose = false;
  ProblemData<int, double> inst;
  const int nnz = col_ptr[n];
  inst.A_csc_col_ptr.assign(col_ptr, col_ptr + n + 1);
  inst.A_csc_row_idx.assign(row_idx, row_idx + nnz);
  inst.A_csc_values.assign(vals, vals + nnz);
  inst.b.assign(b, b + m);
  inst.m = m;
  inst.n = n;
  inst.lambda = lambda;
  inst.sigma = 1;
  MulticoreEngineExecutor<int, double> executor(inst, &settings);
  reset_sampler(seed);
  obj_out[0] = executor.getObjectiveValue();
  for (int k = 0; k < bulks; ++k) {
    executor.executeBulkOfIterations();
    obj_out[k + 1] = executor.getObjectiveValue();
  }
  for (int i = 0; i < n; ++i) x_out[i] = inst.x[i];
  for (int i = 0; i < m; ++i) r_out[i] = executor.residuals[i];
  return 0;
}

/* eval_out holds 4 doubles per evaluation (bulks+1 of them): gap, primal,
 * dual, 0-1 accuracy, as in SVMDualLoss::getResultLogRow
 * (cpp/src/solver/lossFunctions/SVMDualLoss/SVMDualLoss.h:31-42). */
extern "C" int ref_svm_run(int d, int n, const int* row_ptr, const int* col_idx,
                           const double* vals, const double* y, double lambda, double sigma,
                           int threads, uint64_t seed, int bulks, unsigned long inner,
                           double* alpha_out, double* w_out, double* eval_out) {
  OptimizationSettings settings;
  settings.lossFunction = 2;
  settings.totalThreads = threads;
  settings.innerIterations = inner;
  settings.verbose = false;
  ProblemData<int, double> inst;
  const int nnz = row_ptr[n];
  inst.A_csr_row_ptr.assign(row_ptr, row_ptr + n + 1);
  inst.A_csr_col_idx.assign(col_idx, col_idx + nnz);
  inst.A_csr_values.assign(vals, vals + nnz);
  inst.b.assign(y, y + n);
  inst.m = d;
  inst.n = n;
  inst.lambda = lambda;
  inst.sigma = sigma;
  MulticoreEngineExecutor<int, double> executor(inst, &settings);
  // The SVM loss keeps its own copy of the instance and of w
  // (MulticoreSVMDualLoss.h:19-29); read alpha and w from it.
  auto* loss = dynamic_cast<Loss::MulticoreSVMDualLoss<int, double>*>(executor.loss);
  if (!loss) return -1;
  reset_sampler(seed);
  for (int k = 0; k <= bulks; ++k) {
    if (k > 0) executor.executeBulkOfIterations();
    executor.getObjectiveValue();
    eval_out[4 * k + 0] = loss->lastComputedObjectiveValue;
    eval_out[4 * k + 1] = loss->lastPrimalObjectiveValue;
    eval_out[4 * k + 2] = loss->lastDualObjectiveValue;
    eval_out[4 * k + 3] = loss->lastZeroOneAccuracy;
  }
  for (int i = 0; i < n; ++i) alpha_out[i] = loss->instance.x[i];
  for (int i = 0; i < d; ++i) w_out[i] = loss->residuals[i];
  return 0;
}

/* Losses 1 (MulticoreL2SquareRegSquareLoss) and 3 (MulticoreL2SquareRegLogisticLoss)
 * through the same engine (MulticoreEngineExecutor.h:32-58).  A is CSC over the
 * coordinates (for loss 3 the features, rows = samples, b = labels); sigma is
 * instance.sigma, which loss 3's Lipschitz constants use.  The logistic
 * objective walks A_test_csr_row_ptr.size() - 1 test rows, so that vector gets
 * one entry (no test set). */
extern "C" int ref_smooth_run(int loss, int m, int n, const int* col_ptr, const int* row_idx,
                              const double* vals, const double* b, double lambda, double sigma,
                              int threads, uint64_t seed, int bulks, unsigned long inner,
                              double* x_out, double* r_out, double* obj_out) {
  if (loss != 1 && loss != 3) return -1;
  OptimizationSettings settings;
  settings.lossFunction = loss;
  settings.totalThreads = threads;
  settings.innerIterations = inner;
  settings.verbose = false;
  ProblemData<int, double> inst;
  const int nnz = col_ptr[n];
  inst.A_csc_col_ptr.assign(col_ptr, col_ptr + n + 1);
  inst.A_csc_row_idx.assign(row_idx, row_idx + nnz);
  inst.A_csc_values.assign(vals, vals + nnz);
  inst.b.assign(b, b + m);
  inst.A_test_csr_row_ptr.assign(1, 0);
  inst.m = m;
  inst.n = n;
  inst.lambda = lambda;
  inst.sigma = sigma;
  MulticoreEngineExecutor<int, double> executor(inst, &settings);
  reset_sampler(seed);
  obj_out[0] = executor.getObjectiveValue();
  for (int k = 0; k < bulks; ++k) {
    executor.executeBulkOfIterations();
    obj_out[k + 1] = executor.getObjectiveValue();
  }
  for (int i = 0; i < n; ++i) x_out[i] = inst.x[i];
  for (int i = 0; i < m; ++i) r_out[i] = executor.residuals[i];
  return 0;
}

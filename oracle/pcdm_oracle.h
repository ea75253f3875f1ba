/*
 * pcdm_oracle.h - CPU restatement of optml/ac-dc's PCDM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GPU library:
 * only the tests, the smoke check and the CPU-baseline leg of the benchmark
 * use it.  The product path never calls it.
 *
 * Parity is pinned by compiling the reference's own multicore engine from its
 * sources (oracle/Makefile, target ref) and checking bit-for-bit equality of
 * this oracle's serial trajectory against it on seeded inputs
 * (tests/golden/make_golden.py writes the fixtures).
 *
 * Index types: int64 offsets, int32 indices, FP64 values (ProblemData<int,double>
 * widened).  Evaluation results are written to double out[ORC_EVAL_LEN]:
 *   [0] primal  [1] dual  [2] gap  [3] rel_gap  [4] zero_one_accuracy
 *   [5] reg_norm (||x||_1 or sum alpha)  [6] sq_norm (||r||^2 or ||w||^2)
 *   [7] max_abs_grad (||A^T r||_inf, Lasso)  [8] support (nonzeros of x)
 */
#ifndef PCDM_ORACLE_H_
#define PCDM_ORACLE_H_

#include <stdint.h>

#define ORC_EVAL_LEN 9

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 (Salmon et al., SC'11) and the coordinate sampler:
 * update k draws floor(philox64(seed, k) * n / 2^64). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t orc_sample(uint64_t seed, uint64_t k, uint64_t n);

/* ---- Lasso (loss 0) ---- */
void orc_lasso_lipschitz(int64_t n, const int64_t* col_ptr, const double* vals, double beta,
                         double* Li);
void orc_lasso_residuals(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, const double* b, const double* x, double* r);
void orc_lasso_updates(int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                       const double* vals, double lambda, const double* Li, double* x, double* r,
                       uint64_t seed, uint64_t k0, uint64_t count);
void orc_lasso_eval(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                    const double* vals, const double* b, double lambda, const double* x,
                    const double* r, int threads, double* out);
/* Serial solve: epochs of n updates, refresh + evaluation after every
 * check_every epochs, until the (relative if rel) gap <= target or max_epochs.
 * x must hold the start point; r is written.  Returns epochs run. */
int64_t orc_lasso_solve(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                        const double* vals, const double* b, double lambda, double beta,
                        uint64_t seed, double target, int rel, int64_t max_epochs,
                        int64_t check_every, double* x, double* r, double* out);

/* q-shrinking (the build's definition; the reference has only the settings
 * fields use_shrinking / shrinking_probability / shrinking_starting_iter,
 * cpp/src/solver/settingsAndStatistics.h:60-62): after start_epoch epochs,
 * update k draws from the active list with probability q (Philox word 2 below
 * q * 2^32; index umulhi(word 3, |A|)), else uniformly (words 0-1).  The list
 * {j : x_j != 0 or |a_j^T r| > (1 - eps) lambda} is rebuilt in column order at
 * every check.  Serial, FP64; the step uses Li * step_scale while drawing from
 * the list.  Parity of this rule is unpinned: the reference has no shrinking. */
int64_t orc_lasso_solve_shrink(int64_t m, int64_t n, const int64_t* col_ptr,
                               const int32_t* row_idx, const double* vals, const double* b,
                               double lambda, double beta, uint64_t seed, double target, int rel,
                               int64_t max_epochs, int64_t check_every, double q, double eps,
                               int64_t start_epoch, double step_scale, double* x, double* r,
                               double* out, double* gap_trace);

/* Working-set solve for fixtures of large instances (the optimum, not a
 * sampler trajectory): cyclic sweeps of the reference's exact-step update over
 * W = {j : x_j != 0 or |a_j^T r| > (1 - eps) lambda}, `sweeps` of them between
 * checks; every check refreshes r exactly, evaluates the gap over all columns
 * (OpenMP, threads) and rebuilds W; anderson = K > 1 adds an Anderson
 * extrapolation after every K + 1 sweeps.  Returns the sweeps made. */
int64_t orc_lasso_solve_ws(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                           const double* vals, const double* b, double lambda, double target,
                           int rel, int64_t max_checks, int64_t sweeps, double eps, int threads,
                           int anderson, double* x, double* r, double* out, int64_t* checks_out);

/* ---- losses 1 (L2-regularised square) and 3 (L2-regularised logistic); the
 *      matrix is CSC over coordinates, m = residual entries (samples for 3) ---- */
#define ORC_LOSS_RIDGE 1
#define ORC_LOSS_LOGISTIC 3
void orc_smooth_lipschitz(int loss, int64_t n, const int64_t* col_ptr, const double* vals,
                          double lambda, double beta, double sigma, double* Li);
void orc_smooth_residuals(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                          const int32_t* row_idx, const double* vals, const double* b,
                          const double* x, double* r);
void orc_smooth_updates(int loss, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                        const double* vals, const double* b, double lambda, const double* Li,
                        double* x, double* r, uint64_t seed, uint64_t k0, uint64_t count);
void orc_smooth_eval(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, const double* b, double lambda,
                     const double* x, const double* r, double* out);
int64_t orc_smooth_solve(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                         const int32_t* row_idx, const double* vals, const double* b,
                         double lambda, double beta, double sigma, uint64_t seed, double target,
                         int rel, int64_t max_epochs, double* x, double* r, double* out);

/* ---- SVM dual (loss 2); the matrix is CSR by sample, m = features ---- */
void orc_svm_lipschitz(int64_t n, const int64_t* row_ptr, const double* vals, double sigma,
                       double* Li);
void orc_svm_residuals(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, double* alpha,
                       double* w);
void orc_svm_updates(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                     const double* vals, const double* y, double lambda, const double* Li,
                     double* alpha, double* w, uint64_t seed, uint64_t k0, uint64_t count);
void orc_svm_eval(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                  const double* vals, const double* y, double lambda, const double* alpha,
                  const double* w, int threads, double* out);
int64_t orc_svm_solve(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                      const double* vals, const double* y, double lambda, double sigma,
                      uint64_t seed, double target, int64_t max_epochs, int64_t check_every,
                      double* alpha, double* w, double* out);

/* Synchronous mini-batch SDCA (hinge dual): tau-nice draws as the reference's
 * mini-batch loop makes them (first tau distinct values of the uniform stream,
 * counter *k), every delta of a step from the same w, then all applied in the
 * order drawn.  orc_tau_nice writes one step's draws. */
void orc_tau_nice(uint64_t seed, uint64_t* k, int64_t n, int64_t tau, int32_t* S);
void orc_svm_minibatch(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, const double* Li,
                       double* alpha, double* w, uint64_t seed, uint64_t* k, int64_t tau,
                       int64_t steps);
int64_t orc_svm_minibatch_solve(int64_t m, int64_t n, const int64_t* row_ptr,
                                const int32_t* col_idx, const double* vals, const double* y,
                                double lambda, double sigma, uint64_t seed, int64_t tau,
                                double target, int64_t max_epochs, int64_t check_every,
                                double* alpha, double* w, double* out);

/* ---- OpenMP asynchronous form (the reference's multicore engine:
 * omp parallel for over updates, CAS-loop atomic adds).  Returns seconds. */
double orc_lasso_hogwild(int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, double lambda, const double* Li, double* x,
                         double* r, uint64_t seed, uint64_t k0, uint64_t count, int threads);
double orc_svm_hogwild(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, const double* Li,
                       double* alpha, double* w, uint64_t seed, uint64_t k0, uint64_t count,
                       int threads);

/* omega: max number of entries in one residual row (MultiCoreSolver.cpp:32-38). */
int64_t orc_omega(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx);
/* ESO parameter 1 + (omega-1)(tau-1)/(n-1) (MultiCoreSolver.cpp:108-110). */
double orc_eso_beta(double omega, double tau, double n);

#ifdef __cplusplus
}
#endif
#endif

/*
 * acdc_gpu.h - C-ABI of the GB300 (sm_103a) PCDM library, libacdc_gpu.so.
 *
 * The library replaces the hot path of optml/ac-dc's multicore engine:
 * randomized parallel coordinate descent (PCDM) for
 *   loss 0: L1-regularised least squares  min_x 0.5||Ax-b||^2 + lambda||x||_1
 *   loss 1: L2-regularised least squares  min_x 0.5||Ax-b||^2 + (lambda/2)||x||^2
 *   loss 2: hinge-loss SVM dual (SDCA)    max_a (1/n)sum a_i - (lambda/2)||w(a)||^2,
 *                                          w(a) = (1/(lambda n)) sum_i a_i y_i x_i
 *   loss 3: L2-regularised logistic       min_x sum_i log(1 + exp(-b_i A_i. x))
 *                                                + (lambda/2)||x||^2
 * behind plain pointers and sizes.  A C++ engine (CudaEngineExecutor.h) plugs
 * these calls into the reference's AbstractEngineExecutor / Solver structure.
 *
 * Conventions
 *  - Every function returns 0 (ACDC_OK) or a negative ACDC_E* status; no C++
 *    exception crosses this boundary.  acdc_last_error() gives the message.
 *  - Matrices arrive as compressed columns of the coordinate operand:
 *      losses 0, 1: CSC of A (m rows x n columns), vector b of length m;
 *      loss 2: CSR of X by sample == CSC of X^T (m = features, n = samples),
 *              labels y of length n;
 *      loss 3: CSC of A with samples as rows and features as columns, labels
 *              b (+-1) of length m (MultiCoreSolver.cpp:80-105 arranges LIBSVM
 *              data this way for this loss).
 *    This matches ProblemData<L,D> (cpp/src/solver/structures.h:31-97): the
 *    multicore Lasso reads A_csc_*, the SVM dual reads A_csr_*, and in both
 *    instance.m is the residual length and instance.n the coordinate count.
 *  - Host arrays are only read during the call that takes them; the library
 *    owns every device buffer until the matching *_destroy.
 *  - One context per host thread; calls on one context are serialised.
 */
#ifndef ACDC_GPU_H_
#define ACDC_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define ACDC_OK 0
#define ACDC_EINVAL (-1)      /* invalid argument (sizes, pointers, indices)        */
#define ACDC_ENOMEM (-2)      /* device or host allocation failed                   */
#define ACDC_EUNSUPPORTED (-3)/* loss 1 or 3 in a batched path or the server        */
#define ACDC_ECUDA (-4)       /* CUDA runtime error                                 */
#define ACDC_ETIMEOUT (-5)    /* a bounded device wait ran out                      */
#define ACDC_EDEVICE (-6)     /* a kernel reported a bad index or state             */
#define ACDC_EBUSY (-7)       /* server admission refused (budget or slots)         */
#define ACDC_ENOTFOUND (-8)   /* unknown ticket                                     */
#define ACDC_ENODEV (-9)      /* no CUDA device                                     */
#define ACDC_ECANCELED (-10)  /* a served request cancelled before it finished      */

/* ---- loss codes (OptimizationSettings::lossFunction,
 *      cpp/src/solver/MulticoreEngineExecutor.h:32-58) ------------------- */
#define ACDC_LOSS_L1_SQUARE 0 /* MulticoreL1RegSquareLoss                          */
#define ACDC_LOSS_L2_SQUARE 1 /* MulticoreL2SquareRegSquareLoss                    */
#define ACDC_LOSS_SVM_DUAL 2  /* MulticoreSVMDualLoss                              */
#define ACDC_LOSS_LOGISTIC 3  /* MulticoreL2SquareRegLogisticLoss                  */
/* q-shrinking, screened evaluations, batched paths and the server cover losses
 * 0 and 2; losses 1 and 3 solve one problem at a time (batched calls with them
 * return ACDC_EUNSUPPORTED). */

typedef struct acdc_ctx acdc_ctx;
typedef struct acdc_problem acdc_problem;
typedef struct acdc_server acdc_server;

/* Solver settings: the OptimizationSettings fields this path reads
 * (cpp/src/solver/settingsAndStatistics.h:11-93) plus the device knobs. */
typedef struct acdc_settings {
  int32_t loss;                   /* lossFunction: 0, 1, 2 or 3                    */
  int32_t tau;                    /* updates in flight (= totalThreads); >= 1      */
  int32_t warps_per_block;        /* CTA size in warps for the update kernel       */
  int32_t refresh_every;          /* epochs between FP64 refresh + gap in solve    */
  uint64_t seed;                  /* sampler key                                   */
  double sigma;                   /* ESO beta; <= 0: 1+(omega-1)(tau-1)/(n-1)      */
  double gap_target;              /* solve stops when the gap reaches this         */
  int32_t gap_relative;           /* 1: compare (P-D)/max(1,|P|); 0: P-D           */
  int32_t max_epochs;             /* solve gives up after this many epochs         */
  int32_t use_shrinking;          /* q-shrinking (use_shrinking)                   */
  int32_t shrinking_starting_iter;/* epochs before shrinking starts                */
  double shrinking_probability;   /* q: probability of drawing from the active set */
  double shrink_eps;              /* Lasso active test |a_j^T r| > (1-eps) lambda   */
  int32_t precision;              /* ACDC_PREC_*: arithmetic of x and the residual  */
  int32_t tau_active;             /* updates in flight while shrinking (0 = tau)   */
  double polish_rel_gap;          /* AUTO: switch to FP64 below this relative gap  */
  int32_t active_passes;          /* > 0: while shrinking, each bulk is this many
                                     passes over the active set (|A|/q updates each)
                                     instead of refresh_every epochs               */
  int32_t screened_eval;          /* Lasso with shrinking, 1 (default): between
                                     full passes, solve evaluates only the active
                                     columns and bounds the others by
                                     |a_j^T r| <= |a_j^T r0| + ||a_j|| ||r - r0||
                                     (r0 = residual of the last full pass); a full
                                     pass (and active-set rebuild) runs whenever
                                     that bound reaches (1 - eps/2) lambda.  The
                                     certificate stays a valid duality gap.       */
  int32_t polish_stall_epochs;     /* AUTO: also switch to FP64 once the relative
                                     gap (below 1e-2) has not halved over this
                                     many epochs; 0 = 10                          */
  int32_t hot_polish_sweeps;      /* with the hot set and x in FP32: at each
                                     evaluation whose relative gap is below
                                     polish_rel_gap, x is copied to FP64, one
                                     warp makes hot_polish_sweeps * |H| updates
                                     drawn from the hot list with the exact step
                                     1/||a_j||^2 in FP64 (nothing else in
                                     flight) and the gap is evaluated again: kept
                                     if it meets the target (the solution is then
                                     the FP64 x), else x is rounded back to FP32
                                     and the bulks go on.  0 = off, default 16    */
  double hot_threshold;           /* Lasso with shrinking and screened_eval: after
                                     each evaluation the active columns whose KKT
                                     violation exceeds hot_threshold times the
                                     largest one, plus the active columns sharing
                                     a row with them, form a hot set that gets
                                     about one draw each per tau_active updates
                                     (at most half of the active-set draws,
                                     ESO-scaled for the hot set); 0 = off,
                                     default 0.1                                  */
  int32_t polish_active_passes;   /* with hot_polish_sweeps: before the hot sweep,
                                     this many passes (|A|/q updates each) of the
                                     q-shrinking draws in FP64, tau_active in
                                     flight; 0 = none, default 2                  */
  int32_t lanes_per_update;       /* update kernel, one warp per update unless
                                     8/16/32: -1 = the ring kernel (records and
                                     entries staged through shared-memory copy
                                     rings) for every launch; 1 = the lean kernel
                                     (the records of a chunk of draws staged at
                                     once, an entry ring, columns of at most 4
                                     entries summed in one lane) for every
                                     launch; 0 (default) = the lean kernel for
                                     the q-shrinking launches, the ring kernel
                                     for the others; 8, 16 or 32 = the grouped
                                     kernel, in which that many lanes perform one
                                     update (32/lanes updates per warp) with
                                     records and entries prefetched into
                                     registers.  The iterates do not depend on
                                     the kernel at one update in flight; tau
                                     counts the updates in flight in every case. */
  int32_t minibatch;              /* SVM dual (loss 2) only, 1: synchronous
                                     mini-batch SDCA as the reference's mini-batch
                                     loop runs it (cpp/src/experiments/mSDCA.cpp:
                                     60-105): each step draws tau distinct samples
                                     (the first tau distinct values of the sampler
                                     stream), computes every delta from the same w,
                                     then applies them all; beta is the ESO value
                                     for tau and an epoch is ceil(n / tau) steps.
                                     q-shrinking is off in this mode.  0 (default):
                                     asynchronous, tau updates in flight.         */
  int32_t reserved3;
} acdc_settings;

/* precision: FP32 x and residual with FP64 refresh and gap (FP32), the same
 * with the updates switched to FP64 x and residual once the relative gap falls
 * below polish_rel_gap (AUTO, the default), or FP64 throughout (FP64).  The
 * matrix values are stored in FP32 in every mode. */
#define ACDC_PREC_AUTO 0
#define ACDC_PREC_FP32 1
#define ACDC_PREC_FP64 2

/* FP64 evaluation of the current iterate (after an FP64 refresh).  The duality
 * gaps of losses 0, 1 and 3 are this library's (the reference reports a gap
 * for the SVM dual only):
 *   loss 0: dual point s r, s = min(1, lambda/||A^T r||_inf);
 *   loss 1: P - D = sum_j (a_j^T r + lambda x_j)^2 / (2 lambda), dual point r;
 *   loss 3: D(a) = -sum_i [a_i log a_i + (1-a_i) log(1-a_i)]
 *                  - ||sum_i a_i b_i A_i.||^2 / (2 lambda) at a_i = sigmoid(r_i),
 *           with r_i = -b_i A_i. x. */
typedef struct acdc_eval {
  double primal;            /* P                                                  */
  double dual;              /* D                                                  */
  double gap;               /* P - D                                              */
  double rel_gap;           /* (P - D) / max(1, |P|)                              */
  double zero_one_accuracy; /* SVM: fraction of y_i x_i^T w > 0; logistic: fraction
                               of correctly signed samples; 0 otherwise           */
  double reg_norm;          /* loss 0: ||x||_1; 1, 3: ||x||^2; SVM: sum alpha_i    */
  double sq_norm;           /* loss 0, 1: ||Ax-b||^2; SVM: ||w||^2; logistic:
                               sum log(1 + exp(r_i))                              */
  double max_abs_grad;      /* Lasso ||A^T r||_inf (an upper bound of it after a
                               screened evaluation); SVM 0                        */
  int64_t support;          /* nonzeros of x (alpha)                              */
  int64_t active;           /* size of the q-shrinking active set                 */
} acdc_eval;

/* Work counters of the update kernel since the last reset. */
typedef struct acdc_stats {
  uint64_t updates;         /* coordinate updates                                 */
  uint64_t nonzero_updates; /* updates whose step was nonzero                     */
  uint64_t nnz_read;        /* matrix entries gathered                            */
  uint64_t nnz_scattered;   /* matrix entries scattered into the residual         */
  double update_ms;         /* device time of update kernels (CUDA events)        */
  double eval_ms;           /* device time of refresh + gap kernels               */
  int64_t update_launches;
  int64_t eval_launches;
  int64_t screened_evals;   /* evaluations that read only the active columns      */
} acdc_stats;

typedef struct acdc_solve_result {
  acdc_eval eval;
  int32_t converged;
  int32_t epochs;
  double seconds;           /* host wall time of the call                         */
  acdc_stats stats;
  double device_ms;         /* CUDA-event time on the context stream, first launch
                               to the last gap read-back (includes host decisions) */
  int32_t fp64_epochs;      /* epochs run in the FP64 polish stage                */
  int32_t reserved;
} acdc_solve_result;

typedef struct acdc_problem_info {
  int64_t m, n, nnz, nnz_padded;
  int64_t omega;            /* max entries per residual row                       */
  double sigma;             /* ESO beta in use                                    */
  double lambda;
  int64_t device_bytes;
  int32_t loss;
  int32_t tau;
  int64_t omega_active;     /* omega over the last active set                     */
  double active_step_scale; /* step scale while drawing from the active set       */
  int64_t long_columns;     /* columns with more than 32 entries                  */
} acdc_problem_info;

/* ---- context ---------------------------------------------------------- */
void acdc_settings_default(acdc_settings* s);
/* ACDC_OK when every field of s lies in its range, else ACDC_EINVAL: the check
 * acdc_problem_set_settings makes (which also names the field in
 * acdc_last_error).  Needs no device, so a caller can refuse bad settings
 * before uploading a matrix. */
int acdc_settings_check(const acdc_settings* s);
int acdc_ctx_create(int device, acdc_ctx** out);
int acdc_ctx_destroy(acdc_ctx* ctx);
/* Device memory of the context's pool (every problem, staging buffer and
 * table of the context comes from it): bytes the pool holds from the driver,
 * and bytes handed out now.  No reference counterpart: the reference engine
 * has no device memory. */
int acdc_ctx_memory(acdc_ctx* ctx, int64_t* reserved, int64_t* used);
const char* acdc_last_error(const acdc_ctx* ctx);
const char* acdc_status_string(int status);

/* ---- problem upload (replaces InputOuputHelper::loadCSCData /
 *      loadDistributedSparseSVMRowData feeding MulticoreEngineExecutor's
 *      constructor, cpp/src/solver/MulticoreEngineExecutor.h:25-66) ------- */
/* col_ptr: n+1 offsets; row_idx/vals: col_ptr[n] entries; rhs: b (losses 0,
 * 1: m entries), y (loss 2: n entries, +-1) or the labels (loss 3: m entries,
 * +-1).  Values are stored on the device as FP32 in 16-byte aligned column
 * segments (loss 3: b_i A_ij); x starts at 0. */
int acdc_problem_create(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n, const int64_t* col_ptr,
                        const int32_t* row_idx, const double* vals, const double* rhs,
                        double lambda, acdc_problem** out);
/* The same with the reference's ProblemData<int,double> index type. */
int acdc_problem_create_i32(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n,
                            const int32_t* col_ptr, const int32_t* row_idx, const double* vals,
                            const double* rhs, double lambda, acdc_problem** out);
/* The same matrix A (m x n) given by rows: row_ptr[0..m] (row i's entries at
 * row_ptr[i]..row_ptr[i+1]-1), their column indices col_idx (0-based, < n)
 * and values.  The device turns the rows into its column layout, keeping each
 * column's entries in row order: the transposition the reference makes on the
 * host for the logistic loss (getCSR_from_CSC, helpers/matrix_conversions.h:65-104,
 * at frontends/solvers/MultiCoreSolver.cpp:89-93), so LIBSVM rows (samples x
 * features, labels as rhs) go in as read.  A column index outside [0, n)
 * returns ACDC_EDEVICE. */
int acdc_problem_create_rows(acdc_ctx* ctx, int32_t loss, int64_t m, int64_t n,
                             const int64_t* row_ptr, const int32_t* col_idx, const double* vals,
                             const double* rhs, double lambda, acdc_problem** out);
int acdc_problem_destroy(acdc_problem* p);
int acdc_problem_info_get(acdc_problem* p, acdc_problem_info* info);

/* Settings: computes beta and the reciprocal Lipschitz constants
 * Li = 1/(beta ||a_j||^2) (MulticoreSquareLoss.h:27-40 without, and
 * MulticoreSVMDualLoss.h:48-61 with, the sigma factor). */
int acdc_problem_set_settings(acdc_problem* p, const acdc_settings* s);
int acdc_problem_set_lambda(acdc_problem* p, double lambda);

/* ---- the engine (AbstractEngineExecutor, cpp/src/solver/AbstractEngineExecutor.h:14-37) */
/* executeBulkOfIterations: n_updates sampled coordinate updates
 * (MulticoreEngineExecutor.h:83-89 with the loss updates of
 * MulticoreL1RegSquareLoss.h:41-63 / MulticoreSVMDualLoss.h:119-141).
 * Asynchronous on the context's stream. */
int acdc_run_updates(acdc_problem* p, uint64_t n_updates);
/* recomputeResiduals in FP64 (MulticoreSquareLoss.h:42-53, MulticoreSVMDualLoss.h:31-46);
 * the FP32 working residual is replaced by the rounded FP64 one. */
int acdc_recompute_residuals(acdc_problem* p);
/* FP64 refresh + objective and duality gap (MulticoreL1RegSquareLoss.h:30-39,
 * MulticoreSVMDualLoss.h:63-117; the Lasso dual point is theta = -s r,
 * s = min(1, lambda/||A^T r||_inf)).  Synchronises. */
int acdc_evaluate(acdc_problem* p, acdc_eval* out);
/* Bulks of refresh_every epochs, each followed by refresh + gap, until the gap
 * target or max_epochs. */
int acdc_solve(acdc_problem* p, acdc_solve_result* out);

/* One row per evaluation of a solve: the reference's Solver prints one log row
 * per bulk of updates (Solver.h:23-77, getResultLogRow); row 0 is the
 * evaluation before the first bulk. */
typedef struct acdc_trace_row {
  uint64_t updates;         /* updates of this solve call before the evaluation   */
  double primal;            /* P at the evaluation                                */
  double gap;               /* P - D                                              */
  double rel_gap;           /* (P - D) / max(1, |P|)                              */
  int64_t active;           /* active-set size (q-shrinking), else 0              */
  int64_t hot;              /* hot-set size, else 0                               */
  int64_t omega_active;     /* max active columns in one row                      */
  int64_t omega_hot;        /* max hot columns in one row                         */
  float update_ms;          /* device time of the bulk before the evaluation      */
  float eval_ms;            /* device time of the evaluation                      */
  int32_t shrink;           /* 1: the bulk drew from the active (and hot) set     */
  int32_t fp64;             /* 1: the bulk ran with FP64 x and residual           */
  int32_t screened;         /* 1: the evaluation was a screened one               */
  int32_t reserved;
} acdc_trace_row;

/* acdc_solve that also records its evaluations: rows receives the first cap of
 * them and *n_rows (if not null) their number, which may exceed cap. */
int acdc_solve_traced(acdc_problem* p, acdc_solve_result* out, acdc_trace_row* rows,
                      int64_t cap, int64_t* n_rows);

/* Restarts the solve on the resident data: x = 0, residual refreshed, sampler
 * counter 0, FP32 stage, active set cleared (the state the engine constructor
 * leaves, MulticoreEngineExecutor.h:25-66). */
int acdc_problem_reset(acdc_problem* p);

int acdc_get_x(acdc_problem* p, double* x);        /* n entries (alpha for loss 2) */
int acdc_set_x(acdc_problem* p, const double* x);  /* warm start; refreshes r      */

/* Checkpoint and resume of a problem's solver state: x (FP64), the sampler's
 * update counter (and the mini-batch draw counter), the updates and epochs
 * done, lambda and the precision stage
 * (FP32 or FP64 x).  acdc_checkpoint_size gives the bytes (0 for a null
 * problem); acdc_checkpoint_save writes them to host memory; acdc_checkpoint_load
 * restores them into a problem of the same loss and sizes, recomputing the
 * residuals from x (the active and hot sets are rebuilt at its next
 * evaluation), so that the updates continue from the same draw.  A buffer
 * of another size, loss or shape returns ACDC_EINVAL.  The reference only dumps
 * x per lambda (experiments/lasso_console_solver.cpp:164-171) and has no resume. */
int64_t acdc_checkpoint_size(const acdc_problem* p);
int acdc_checkpoint_save(acdc_problem* p, void* buf, int64_t size);
int acdc_checkpoint_load(acdc_problem* p, const void* buf, int64_t size);
int acdc_get_residuals(acdc_problem* p, double* r);/* m entries: Ax-b or w, FP32 working copy */
int acdc_get_stats(acdc_problem* p, acdc_stats* s);
/* 0-1 accuracy of the current model on n_test held-out samples given as CSR
 * (row_ptr[n_test + 1], 0-based feature indices, labels +-1): the fraction with
 * label * (sample . weights) > 0.  Weights: the SVM dual's w, refreshed from the
 * current alpha in FP64 (the test loop of MulticoreSVMDualLoss.h:95-112), or the
 * logistic loss's x (MulticoreL2SquareRegLogisticLoss.h:65-81).  Features beyond
 * the weights' length count as zero.  Losses 0 and 1: ACDC_EUNSUPPORTED. */
int acdc_test_accuracy(acdc_problem* p, int64_t n_test, const int64_t* row_ptr,
                       const int32_t* col_idx, const double* vals, const double* labels,
                       double* accuracy);
int acdc_reset_stats(acdc_problem* p);
int acdc_synchronize(acdc_problem* p);

/* Diagnostic: the coordinates the device sampler draws for updates
 * k0 .. k0+count-1 of a solve keyed by seed over n coordinates (shrinking
 * off); out receives count entries.  Lets a caller check the device stream
 * against acdc_sample_coordinate (acdc_host.h). */
int acdc_debug_sample(acdc_ctx* ctx, uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                      int64_t* out);

/* The tau-nice draws of the synchronous mini-batch (settings.minibatch):
 * `steps` steps of tau distinct coordinates in [0, n), each the first tau
 * distinct values of the sampler stream from counter k0 on, into out
 * (steps x tau, in the order drawn); *k_out gets the counter after the last
 * step.  Replaces the draw loop of cpp/src/experiments/mSDCA.cpp:60-74
 * (gsl_rng_uniform_int drawn again while it repeats a value of the step). */
int acdc_debug_tau_nice(acdc_ctx* ctx, uint64_t seed, uint64_t k0, int64_t n, int32_t tau,
                        int32_t steps, int32_t* out, uint64_t* k_out);

/* acdc_debug_sample without any allocation (no counterpart in the reference,
 * whose sampler is a host GSL call), for callers that must not allocate device
 * memory while they run: one whose memory is already committed to resident
 * problems (an allocation may fail, or grow the context's pool past the
 * budget), or one checking the sampler beside running solves that wants no
 * allocation call on their stream.  The draws go to a fixed device array of
 * ACDC_NOALLOC_MAX_SAMPLES entries (512 KiB) instead of a per-call allocation;
 * count beyond that returns ACDC_EINVAL.  The first call on a device looks up
 * the array's address (cudaGetSymbolAddress, may load the module): make it
 * before any stream capture.  One array per device: calls that overlap on a
 * device race and must be serialised by the caller. */
#define ACDC_NOALLOC_MAX_SAMPLES 65536
int acdc_debug_sample_noalloc(acdc_ctx* ctx, uint64_t seed, uint64_t k0, uint64_t count,
                              int64_t n, int64_t* out);

/* ---- batched lambda paths (many instances, one launch sequence) --------- */
typedef struct acdc_batch_options {
  int32_t path_len;         /* lambdas per instance                               */
  int32_t max_epochs;       /* per lambda                                         */
  double gap_target;        /* per lambda, relative gap                           */
  int32_t refresh_every;    /* epochs between gap checks                          */
  int32_t autotune;         /* 1: tau per instance by timed probe launches of
                               each candidate (powers of two with ESO beta <= 4):
                               the smallest beta / measured updates per second,
                               cached per size class on the context; 2: the
                               closed-form rule (largest tau with beta <= 1.3)   */
  int32_t tau_override;     /* > 0: fixed tau for every instance                  */
  int32_t plain;            /* 1: solve one instance per launch sequence (baseline) */
  int32_t use_shrinking;    /* 1: q-shrinking (q = 0.9) for Lasso instances, from
                               the second round of each lambda                    */
  int32_t active_passes;    /* while shrinking, passes over the active set per
                               round (default 20 when 0)                          */
  int32_t reserved[6];
} acdc_batch_options;

typedef struct acdc_batch_result {
  acdc_eval eval;           /* at the end of this lambda                          */
  double lambda;
  int32_t converged;
  int32_t epochs;
  int32_t tau;
  int32_t reserved;
} acdc_batch_result;

/* Solves problems[i] along lambdas[i*path_len + k] (k = 0..path_len-1), each
 * lambda warm-started from the previous solution (the pattern of
 * cpp/src/experiments/lasso_console_solver.cpp:149-172).  results has
 * count*path_len entries; x_out (optional) receives each problem's final x
 * at x_out[i] (n_i entries each). */
int acdc_batch_solve_path(acdc_ctx* ctx, int32_t count, acdc_problem* const* problems,
                          const double* lambdas, const acdc_batch_options* opt,
                          acdc_batch_result* results, double* const* x_out);

/* ---- serving: continuous batching of solve requests -------------------- */
typedef struct acdc_server_options {
  int64_t memory_budget_bytes;  /* device bytes admitted at once                  */
  int32_t max_slots;            /* requests on the device at once                 */
  int32_t quantum_epochs;       /* rounds per acdc_server_step (a round is one
                                   epoch, or with shrinking at most one)          */
  int32_t max_epochs;           /* per request                                    */
  int32_t use_shrinking;        /* 1: q-shrinking for Lasso requests              */
  int32_t reserved[6];
} acdc_server_options;

typedef struct acdc_request {
  int32_t loss;
  int32_t reserved0;
  int64_t m, n;
  const int64_t* col_ptr;
  const int32_t* row_idx;
  const double* vals;
  const double* rhs;
  double lambda;
  double gap_target;
  uint64_t seed;
} acdc_request;

typedef struct acdc_request_result {
  int32_t state;            /* 0 queued, 1 running, 2 done, 3 failed              */
  int32_t converged;
  int32_t epochs;
  int32_t status;           /* ACDC_* code for failed requests                    */
  acdc_eval eval;
  double submit_time, start_time, finish_time; /* seconds, host monotonic clock   */
} acdc_request_result;

int acdc_server_create(acdc_ctx* ctx, const acdc_server_options* opt, acdc_server** out);
/* Returns a ticket; the request's arrays are read only during the call.  When
 * no request waits ahead of it and a slot and the memory budget are free, the
 * request is admitted at once (its device copy made from the caller's arrays,
 * state 1); otherwise its arrays are copied and it waits in arrival order
 * (state 0).  ACDC_EBUSY if the request can never fit the memory budget. */
int acdc_server_submit(acdc_server* s, const acdc_request* req, int64_t* ticket);
/* Runs one scheduling round: admits queued requests that fit, advances every
 * resident request by quantum_epochs, retires converged ones.  Returns the
 * number of requests still queued or running in *pending. */
int acdc_server_step(acdc_server* s, int32_t* pending);
/* Result of a ticket; x (optional, n entries) once done.  A done ticket is
 * released by acdc_server_release. */
int acdc_server_poll(acdc_server* s, int64_t ticket, acdc_request_result* res, double* x);
int acdc_server_release(acdc_server* s, int64_t ticket);
/* Cancels a queued or running request: it leaves the queue or the device (its
 * memory is released and the slot tables are rebuilt at the next step) and
 * ends in state 3 with status ACDC_ECANCELED.  A finished request is left as
 * it is.  Call between steps, like every server call. */
int acdc_server_cancel(acdc_server* s, int64_t ticket);
int acdc_server_destroy(acdc_server* s);

/* Where the server's host time went since its creation (seconds on the host
 * monotonic clock; each phase includes the device work it waits for).  No
 * counterpart in the reference, which has no server. */
typedef struct acdc_server_stats {
  int64_t steps;            /* acdc_server_step calls                             */
  int64_t builds;           /* slot-table rebuilds (the resident set changed)     */
  int64_t rounds;           /* rounds run                                         */
  int64_t admitted;         /* requests made resident                             */
  int64_t retired;          /* requests finished and released from the device    */
  double admit_s;           /* device copies and layouts of admitted requests    */
  double build_s;           /* slot-table rebuilds                                */
  double rounds_s;          /* rounds                                             */
  double retire_s;          /* result collection, x read-back, device release     */
} acdc_server_stats;
int acdc_server_get_stats(acdc_server* s, acdc_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* ACDC_GPU_H_ */

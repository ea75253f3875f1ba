// CudaEngineExecutor<L,D>: the GB300 engine behind the reference's engine
// interface (AbstractEngineExecutor, cpp/src/solver/AbstractEngineExecutor.h:14-37),
// a drop-in for MulticoreEngineExecutor (cpp/src/solver/MulticoreEngineExecutor.h:17-138)
// so that Solver<L,D>::runSolver (cpp/src/solver/Solver.h:23-77) drives it unchanged.
//
// It reads only members that the reference's ProblemData and
// OptimizationSettings declare, so it compiles against the reference's own
// headers as well as against the mirrors in this directory.  Device knobs that
// the reference's settings lack come through CudaEngineOptions.
//
// Behaviour per reference member:
//  * constructor: loss switch on settings->lossFunction (0: L1-regularised
//    square loss on A_csc_*; 1: L2-regularised square loss on A_csc_*; 2: SVM
//    dual on A_csr_* with labels in b; 3: L2-regularised logistic loss on
//    A_csc_* after the samples were made rows; any other code throws
//    std::runtime_error), x = 0, residual refreshed, reciprocal
//    Lipschitz constants Li = 1/(sigma ||a_j||^2) with sigma = forcedSigma when
//    positive, instance.sigma for the SVM, else the ESO value for
//    tau = totalThreads;
//  * executeBulkOfIterations: innerIterations sampled updates on the device;
//  * recomputeResiduals: FP64 recomputation of the residual;
//  * getObjectiveValue: FP64 objective (Lasso) or duality gap (SVM), and x
//    (alpha) copied back into instance.x;
//  * getResultLogHeaders / getResultLogRow: the row formats of
//    cpp/src/solver/lossFunctions/squareLoss/SquareLoss.h:28-38 and
//    cpp/src/solver/lossFunctions/SVMDualLoss/SVMDualLoss.h:31-42.
// One deliberate difference: for the SVM the reference keeps alpha inside its
// loss object (MulticoreSVMDualLoss.h:19-29) and leaves instance.x at zero;
// this engine writes alpha to instance.x.
#ifndef ACDC_CUDA_ENGINE_EXECUTOR_H_
#define ACDC_CUDA_ENGINE_EXECUTOR_H_

#include <cstdint>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "acdc_gpu.h"

struct CudaEngineOptions {
  int device = 0;
  int warps_per_block = 8;
  unsigned long long seed = 0;
  int refresh_every = 5;         // solve(): epochs between FP64 gap checks
  double gap_target = 1e-6;      // solve(): relative gap (Lasso), absolute (SVM)
  int max_epochs = 1000;         // solve()
  int precision = ACDC_PREC_AUTO;
  int tau_active = 0;
  int active_passes = 0;
};

template <typename L, typename D>
class CudaEngineExecutor : public AbstractEngineExecutor<L, D> {
 public:
  ProblemData<L, D>& instance;

  CudaEngineExecutor(ProblemData<L, D>& inst, OptimizationSettings* s,
                     const CudaEngineOptions& opt = CudaEngineOptions())
      : instance(inst), opt_(opt) {
    this->settings = s;
    loss_ = s->lossFunction;
    if (loss_ < ACDC_LOSS_L1_SQUARE || loss_ > ACDC_LOSS_LOGISTIC)
      throw std::runtime_error("unknown lossFunction " + std::to_string(loss_));
    // Settings first: a bad value is refused before any device work.
    acdc_settings st;
    acdc_settings_default(&st);
    st.loss = loss_;
    st.tau = s->totalThreads > 0 ? s->totalThreads : 1;
    st.warps_per_block = opt.warps_per_block;
    st.seed = opt.seed;
    // The SVM dual and the logistic loss take the engine's sigma into their
    // Lipschitz constants (MulticoreSVMDualLoss.h:48-61,
    // MulticoreL2SquareRegLogisticLoss.h:30-44); losses 0 and 1 let the library
    // choose the ESO beta for tau.
    const bool uses_sigma = loss_ == ACDC_LOSS_SVM_DUAL || loss_ == ACDC_LOSS_LOGISTIC;
    st.sigma = s->forcedSigma > 0 ? s->forcedSigma : (uses_sigma ? (double)inst.sigma : 0.0);
    st.gap_target = opt.gap_target;
    st.gap_relative = loss_ == ACDC_LOSS_SVM_DUAL ? 0 : 1;
    st.max_epochs = opt.max_epochs;
    st.refresh_every = opt.refresh_every;
    st.use_shrinking = s->use_shrinking ? 1 : 0;
    st.shrinking_probability = s->shrinking_probability;
    st.shrinking_starting_iter = s->shrinking_starting_iter;
    st.precision = opt.precision;
    st.tau_active = opt.tau_active;
    st.active_passes = opt.active_passes;
    if (acdc_settings_check(&st) != ACDC_OK)
      throw std::runtime_error("OptimizationSettings out of range for the GPU engine");
    check(acdc_ctx_create(opt.device, &ctx_), "acdc_ctx_create");
    // A constructor that throws runs no destructor: release what exists here.
    try {
      // Losses 0, 1 and 3 read the CSC arrays (for 3 after MultiCoreSolver.cpp:80-105
      // turned the samples into rows), the SVM dual the CSR by sample
      // (MulticoreEngineExecutor.h:32-58).  For loss 3 without the CSC arrays the
      // sample rows (A_csr_*, m = samples) are transposed on the device.
      const int64_t n = (int64_t)inst.n;
      const bool rows = loss_ == ACDC_LOSS_LOGISTIC && inst.A_csc_col_ptr.empty();
      const bool csc = loss_ != ACDC_LOSS_SVM_DUAL && !rows;
      const std::vector<L>& ptr = csc ? inst.A_csc_col_ptr : inst.A_csr_row_ptr;
      const std::vector<L>& idx = csc ? inst.A_csc_row_idx : inst.A_csr_col_idx;
      const std::vector<D>& val = csc ? inst.A_csc_values : inst.A_csr_values;
      const int64_t ptr_len = rows ? (int64_t)inst.m + 1 : n + 1;
      if ((int64_t)ptr.size() != ptr_len) throw std::runtime_error("pointer array does not match the sizes");
      std::vector<int64_t> cp(ptr.begin(), ptr.end());
      std::vector<int32_t> ri(idx.begin(), idx.end());
      std::vector<double> va(val.begin(), val.end());
      std::vector<double> rhs(inst.b.begin(), inst.b.end());
      if (rows)
        check(acdc_problem_create_rows(ctx_, loss_, (int64_t)inst.m, n, cp.data(),
                                       ri.empty() ? nullptr : ri.data(),
                                       va.empty() ? nullptr : va.data(), rhs.data(),
                                       (double)inst.lambda, &prob_),
              "acdc_problem_create_rows");
      else
        check(acdc_problem_create(ctx_, loss_, (int64_t)inst.m, n, cp.data(),
                                  ri.empty() ? nullptr : ri.data(), va.empty() ? nullptr : va.data(),
                                  rhs.data(), (double)inst.lambda, &prob_),
              "acdc_problem_create");
      check(acdc_problem_set_settings(prob_, &st), "acdc_problem_set_settings");
    } catch (...) {
      if (prob_) acdc_problem_destroy(prob_);
      prob_ = nullptr;
      acdc_ctx_destroy(ctx_);
      ctx_ = nullptr;
      throw;
    }
    inst.x.assign((size_t)inst.n, (D)0);
  }

  ~CudaEngineExecutor() {
    if (prob_) {
      sync_x();
      acdc_problem_destroy(prob_);
    }
    if (ctx_) acdc_ctx_destroy(ctx_);
  }

  void executeBulkOfIterations() override {
    check(acdc_run_updates(prob_, (uint64_t)this->settings->innerIterations), "acdc_run_updates");
  }

  void recomputeResiduals() override {
    check(acdc_recompute_residuals(prob_), "acdc_recompute_residuals");
  }

  D getObjectiveValue() override {
    check(acdc_evaluate(prob_, &last_), "acdc_evaluate");
    sync_x();
    if (loss_ == ACDC_LOSS_SVM_DUAL) {
      instance.primalObjective = (D)last_.primal;
      instance.dualObjective = (D)last_.dual;
      instance.oneZeroAccuracy = (D)last_.zero_one_accuracy;
      return (D)last_.gap;
    }
    return (D)last_.primal;
  }

  std::string getResultLogHeaders() override {
    if (loss_ == ACDC_LOSS_SVM_DUAL)
      return "Elapsed iterations, Current duality gap, Primal objective, Dual objective, 0-1 loss, "
             "Pure computation time, Total time, Test 0-1";
    if (loss_ == ACDC_LOSS_LOGISTIC)  // LogisticLoss.h:30-40
      return "Elapsed iterations, Current objective value, Pure computation time, Total time, "
             "Train 0-1 loss, Test 0-1 loss";
    return "Elapsed iterations, Current objective value, Pure computation time, Total time";
  }

  std::string getResultLogRow(OptimizationStatistics& statistics) override {
    std::stringstream ss;
    if (loss_ == ACDC_LOSS_SVM_DUAL) {
      ss << statistics.elapsedIterations << "," << std::setprecision(16) << last_.gap << ","
         << last_.primal << "," << last_.dual << "," << last_.zero_one_accuracy << ","
         << statistics.elapsedPureComputationTime << "," << statistics.elapsed_time << "," << 0;
    } else {
      ss << statistics.elapsedIterations << "," << std::setprecision(16) << last_.primal << ","
         << statistics.elapsedPureComputationTime << "," << statistics.elapsed_time;
      if (loss_ == ACDC_LOSS_LOGISTIC) ss << "," << last_.zero_one_accuracy << "," << 0;
    }
    return ss.str();
  }

  // Solves to the gap target (refresh and FP64 gap every refresh_every epochs).
  acdc_solve_result solve() {
    acdc_solve_result r;
    check(acdc_solve(prob_, &r), "acdc_solve");
    last_ = r.eval;
    sync_x();
    return r;
  }

  const acdc_eval& lastEvaluation() const { return last_; }
  acdc_problem* problem() { return prob_; }

 private:
  void check(int rc, const char* what) {
    if (rc != ACDC_OK)
      throw std::runtime_error(std::string(what) + ": " + acdc_status_string(rc) + " (" +
                               (ctx_ ? acdc_last_error(ctx_) : "") + ")");
  }
  void sync_x() {
    std::vector<double> x((size_t)instance.n);
    if (acdc_get_x(prob_, x.data()) == ACDC_OK)
      for (size_t j = 0; j < x.size(); ++j) instance.x[j] = (D)x[j];
  }

  CudaEngineOptions opt_;
  int loss_ = 0;
  acdc_ctx* ctx_ = nullptr;
  acdc_problem* prob_ = nullptr;
  acdc_eval last_{};
};

#endif

// The bulk driver of the reference's cpp/src/solver/Solver.h:13-79: optional
// initial objective, iters_bulkIterations_count bulks timed as "pure
// computation", optional residual recomputation and objective after each bulk,
// the last objective at the end; log rows to stdout and the optional log file.
#ifndef ACDC_CPP_SOLVER_H_
#define ACDC_CPP_SOLVER_H_

#include <sys/time.h>

#include <iomanip>
#include <iostream>

#include "AbstractEngineExecutor.h"
#include "settingsAndStatistics.h"

inline double acdc_wall_seconds() {
  struct timeval t;
  gettimeofday(&t, nullptr);
  return (double)t.tv_sec + 1e-6 * (double)t.tv_usec;
}

template <typename L, typename D>
class Solver {
 public:
  AbstractEngineExecutor<L, D>& executor;
  OptimizationSettings* settings;
  explicit Solver(AbstractEngineExecutor<L, D>& e) : executor(e), settings(e.settings) {}

  void log(const std::string& row) {
    std::cout << row << std::endl;
    if (settings->logToFile && settings->logFile) (*settings->logFile) << row << std::endl;
  }

  void runSolver() {
    if (settings->verbose)
      std::cout << "Number of large iterations: " << settings->iters_bulkIterations_count << std::endl;
    OptimizationStatistics statistics;
    if (settings->showInitialObjectiveValue) {
      executor.getObjectiveValue();
      if (settings->verbose) {
        std::cout << executor.getResultLogHeaders() << std::endl;
        log(executor.getResultLogRow(statistics));
      }
    }
    const double total_start = acdc_wall_seconds();
    for (unsigned long i = 0; i < settings->iters_bulkIterations_count; ++i) {
      const double start = acdc_wall_seconds();
      executor.executeBulkOfIterations();
      const double end = acdc_wall_seconds();
      statistics.elapsedPureComputationTime += end - start;
      statistics.elapsed_time = end - total_start;
      statistics.elapsedIterations++;
      if (settings->recomputeResidualAfterEachBulkIteration) executor.recomputeResiduals();
      if (settings->showIntermediateObjectiveValue) {
        executor.getObjectiveValue();
        if (settings->verbose) log(executor.getResultLogRow(statistics));
      }
    }
    if (settings->showLastObjectiveValue) {
      const D obj = executor.getObjectiveValue();
      if (settings->verbose)
        std::cout << "Last objective value: " << std::setprecision(16) << obj << std::endl;
    }
  }
};

#endif

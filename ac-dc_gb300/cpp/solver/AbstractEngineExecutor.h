// The engine interface the driver calls, as in the reference's
// cpp/src/solver/AbstractEngineExecutor.h:14-37: bulks of coordinate updates,
// residual recomputation, the objective and the log-row pair.
#ifndef ACDC_CPP_ABSTRACT_ENGINE_H_
#define ACDC_CPP_ABSTRACT_ENGINE_H_

#include <string>

#include "settingsAndStatistics.h"

template <typename L, typename D>
class AbstractEngineExecutor {
 public:
  OptimizationSettings* settings = nullptr;
  virtual ~AbstractEngineExecutor() {}
  virtual std::string getResultLogHeaders() { return "Function is not implemented"; }
  virtual std::string getResultLogRow(OptimizationStatistics& statistics) {
    (void)statistics;
    return "Function is not implemented";
  }
  virtual void executeBulkOfIterations() {}
  virtual void recomputeResiduals() {}
  virtual D getObjectiveValue() { return 0; }
};

#endif

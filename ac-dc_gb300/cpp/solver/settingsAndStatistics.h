// OptimizationSettings and OptimizationStatistics with the field names and
// defaults of the reference's cpp/src/solver/settingsAndStatistics.h:11-149
// that this path reads, plus the device knobs of the GPU engine.
#ifndef ACDC_CPP_SETTINGS_H_
#define ACDC_CPP_SETTINGS_H_

#include <fstream>
#include <string>

class OptimizationSettings {
 public:
  int lossFunction = 0;           // 0: L1-regularised square loss, 2: SVM dual
  bool showInitialObjectiveValue = false;
  bool showIntermediateObjectiveValue = true;
  bool showLastObjectiveValue = true;
  bool verbose = false;
  bool logToFile = false;
  std::ofstream* logFile = nullptr;
  bool recomputeResidualAfterEachBulkIteration = false;
  int totalThreads = 8;           // tau: updates in flight
  double forcedSigma = -1;        // > 0 overrides the ESO parameter
  unsigned long iters_bulkIterations_count = 10;
  unsigned long innerIterations = 100;
  // q-shrinking (settings fields of the reference; implemented here)
  bool use_shrinking = false;
  double shrinking_probability = 0.9;
  int shrinking_starting_iter = 2;
};

class OptimizationStatistics {
 public:
  double elapsed_time = 0;
  double elapsedPureComputationTime = 0;
  unsigned long elapsedIterations = 0;
};

#endif

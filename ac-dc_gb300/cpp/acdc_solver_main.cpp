// acdc_solver: the console solver of the reference's
// cpp/src/frontends/solvers/MultiCoreSolver.cpp:18-115 on the GPU engine.
//
// Same flags and flow: -A matrix (CSC text prefix for -f 0 and 1, LIBSVM file
// for -f 2 and 3), -b vector file (-f 0, 1), -l lambda, -t threads (tau), -f loss, -I inner
// iterations per bulk, -i show objectives; omega is the largest number of
// entries in one residual row and sigma = 1 + (omega-1)(tau-1)/(n-1); the
// Solver driver runs the bulks.  Flags the reference lacks:
//   -B bulks (iters_bulkIterations_count)   -d device   -s seed
//   -G gap  : solve to this duality gap instead of running bulks
//   -S q    : q-shrinking with probability q
// The reference's -I also falls through into LocalMethods and -T is disabled;
// here -I sets innerIterations only and -T names a test LIBSVM file that is
// parsed but not used by this path.
#include <getopt.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "acdc_gpu.h"
#include "acdc_host.h"
#include "solver/AbstractEngineExecutor.h"
#include "solver/Solver.h"
#include "solver/settingsAndStatistics.h"
#include "solver/structures.h"
#include "solver/CudaEngineExecutor.h"

namespace {

void usage() {
  std::cout << "usage: acdc_solver -A <matrix> [-b <vector>] -l <lambda> [-t tau] [-f 0|1|2|3]\n"
               "                   [-I inner] [-B bulks] [-i 0|1] [-d device] [-s seed]\n"
               "                   [-G gap] [-S q]\n";
}

bool load(int loss, const std::string& a, const std::string& b, double lambda,
          ProblemData<int, double>& inst) {
  if (loss == 0 || loss == 1) {
    int64_t m = 0, n = 0, nnz = 0;
    if (acdc_load_csc_text_sizes(a.c_str(), b.c_str(), &m, &n, &nnz) != ACDC_OK) return false;
    std::vector<int64_t> cp((size_t)n + 1);
    std::vector<int32_t> ri((size_t)nnz);
    inst.A_csc_values.resize((size_t)nnz);
    inst.b.resize((size_t)m);
    if (acdc_load_csc_text(a.c_str(), b.c_str(), cp.data(), ri.data(), inst.A_csc_values.data(),
                           inst.b.data()) != ACDC_OK)
      return false;
    inst.A_csc_col_ptr.assign(cp.begin(), cp.end());
    inst.A_csc_row_idx.assign(ri.begin(), ri.end());
    inst.m = (int)m;
    inst.n = (int)n;
  } else {
    int64_t n = 0, d = 0, nnz = 0;
    if (acdc_load_libsvm_sizes(a.c_str(), &n, &d, &nnz) != ACDC_OK) return false;
    std::vector<int64_t> rp((size_t)n + 1);
    std::vector<int32_t> ci((size_t)nnz);
    inst.A_csr_values.resize((size_t)nnz);
    inst.b.resize((size_t)n);
    if (acdc_load_libsvm(a.c_str(), rp.data(), ci.data(), inst.A_csr_values.data(),
                         inst.b.data()) != ACDC_OK)
      return false;
    inst.A_csr_row_ptr.assign(rp.begin(), rp.end());
    inst.A_csr_col_idx.assign(ci.begin(), ci.end());
    inst.m = (int)d;
    inst.n = (int)n;
    if (loss == 3) {
      // MultiCoreSolver.cpp:80-105 turns the samples into the rows of a CSC
      // matrix over the features (m = samples, n = features).  Here the sample
      // rows stay as read: the engine transposes them on the device
      // (acdc_problem_create_rows) instead of getCSR_from_CSC on the host.
      inst.m = (int)n;
      inst.n = (int)d;
    }
  }
  inst.lambda = lambda;
  return true;
}

}  // namespace

int main(int argc, char* argv[]) {
  OptimizationSettings settings;
  settings.verbose = true;
  CudaEngineOptions eng;
  std::string matrix, vector_file;
  double lambda = 0, gap = 0, q = 0;
  int c;
  while ((c = getopt(argc, argv, "x:y:z:r:e:A:b:l:t:c:f:i:I:T:B:d:s:G:S:h")) != -1) {
    switch (c) {
      case 'A': matrix = optarg; break;
      case 'b': vector_file = optarg; break;
      case 'l': lambda = std::atof(optarg); break;
      case 't': settings.totalThreads = std::atoi(optarg); break;
      case 'f': settings.lossFunction = std::atoi(optarg); break;
      case 'I': settings.innerIterations = std::strtoul(optarg, nullptr, 10); break;
      case 'i':
        settings.showIntermediateObjectiveValue = std::atoi(optarg) != 0;
        settings.showInitialObjectiveValue = std::atoi(optarg) != 0;
        settings.showLastObjectiveValue = std::atoi(optarg) != 0;
        break;
      case 'B': settings.iters_bulkIterations_count = std::strtoul(optarg, nullptr, 10); break;
      case 'd': eng.device = std::atoi(optarg); break;
      case 's': eng.seed = std::strtoull(optarg, nullptr, 10); break;
      case 'G': gap = std::atof(optarg); break;
      case 'S': q = std::atof(optarg); break;
      case 'h': usage(); return 0;
      default: break;  // -x -y -z -r -e -c -T: accepted for compatibility
    }
  }
  const int loss = settings.lossFunction;
  if (matrix.empty() || ((loss == 0 || loss == 1) && vector_file.empty()) || !(lambda > 0) ||
      loss < 0 || loss > 3) {
    usage();
    return 2;
  }
  ProblemData<int, double> instance;
  if (!load(settings.lossFunction, matrix, vector_file, lambda, instance)) {
    std::cerr << "cannot read the input files" << std::endl;
    return 1;
  }
  std::cout << "Data loaded with size: " << instance.m << " x " << instance.n << std::endl;
  // omega = largest number of entries in one residual row (MultiCoreSolver.cpp:32-38, 55-62;
  // for -f 3 the longest sample, :98-103)
  double omega = 1;
  if (settings.lossFunction == 3) {
    for (int i = 0; i < instance.m; ++i)
      omega = std::max<double>(omega, instance.A_csr_row_ptr[(size_t)i + 1] - instance.A_csr_row_ptr[(size_t)i]);
  } else {
    const std::vector<int>& idx =
        settings.lossFunction == 2 ? instance.A_csr_col_idx : instance.A_csc_row_idx;
    std::vector<int> rows((size_t)instance.m, 0);
    for (int r : idx)
      if (++rows[(size_t)r] > omega) omega = rows[(size_t)r];
  }
  instance.omega = omega;
  // (one column: the reference's formula divides by zero; beta is then 1)
  instance.sigma = instance.n > 1 ? 1 + (omega - 1) * (settings.totalThreads - 1) / (instance.n - 1.0) : 1.0;
  std::cout << "Omega: " << omega << std::endl;
  if (q > 0) {
    settings.use_shrinking = true;
    settings.shrinking_probability = q;
  }
  try {
    if (gap > 0) eng.gap_target = gap;
    CudaEngineExecutor<int, double> executor(instance, &settings, eng);
    if (gap > 0) {
      acdc_solve_result r = executor.solve();
      std::cout << "converged," << r.converged << ",epochs," << r.epochs << ",primal,"
                << std::setprecision(16) << r.eval.primal << ",dual," << r.eval.dual << ",gap,"
                << r.eval.gap << ",seconds," << r.seconds << std::endl;
    } else {
      Solver<int, double> solver(executor);
      solver.runSolver();
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}

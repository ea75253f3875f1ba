// ProblemData<L,D>: the problem container the engine reads, with the field
// names and meanings of the reference's cpp/src/solver/structures.h:31-97
// (CSC of A for the Lasso, CSR by sample for the SVM dual, b / labels, x, Li,
// m = residual length, n = coordinates, lambda, omega, sigma).  Only the
// fields this path reads or writes are declared.
#ifndef ACDC_CPP_STRUCTURES_H_
#define ACDC_CPP_STRUCTURES_H_

#include <string>
#include <vector>

template <typename L, typename D>
class ProblemData {
 public:
  std::vector<D> A_csc_values;
  std::vector<L> A_csc_row_idx;
  std::vector<L> A_csc_col_ptr;

  std::vector<D> A_csr_values;
  std::vector<L> A_csr_col_idx;
  std::vector<L> A_csr_row_ptr;

  std::vector<D> A_test_csr_values;
  std::vector<L> A_test_csr_col_idx;
  std::vector<L> A_test_csr_row_ptr;
  std::vector<D> test_b;

  std::vector<D> Li;
  std::vector<D> b;
  std::vector<D> x;

  std::string experimentName;

  L m = 0;
  L n = 0;
  D lambda = 0;
  D omega = 1;
  D sigma = 1;
  D omegaMin = 0;
  D omegaAvg = 0;

  D oneZeroAccuracy = 0;
  D dualObjective = 0;
  D primalObjective = 0;
};

#endif

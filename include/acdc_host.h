/*
 * acdc_host.h - host-side C-ABI of the GB300 PCDM library: seeded synthetic
 * problem generators and the on-disk loaders.  Plain pointers and sizes only.
 *
 * All functions return 0 on success and a negative ACDC_E* code (acdc_gpu.h)
 * on failure.  Caller owns every array; sizes are given by the *_sizes /
 * *_colptr calls first (two-phase: count, then fill).
 */
#ifndef ACDC_HOST_H_
#define ACDC_HOST_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Column-length distributions of the Lasso generator. */
enum {
  ACDC_NNZ_FIXED = 0,   /* every column has nnz_per_col entries                */
  ACDC_NNZ_ZIPF = 1,    /* Zipf(zipf_s) on [1, nnz_max], rescaled to nnz_mean  */
  ACDC_NNZ_UNIFORM = 2  /* uniform integer in [nnz_min, nnz_max]               */
};

/* Seeded Lasso instance: A (m x n, CSC) with distinct uniform rows per column,
 * N(0,1) values (columns scaled to unit L2 norm when normalize_columns),
 * x* with n_star entries +-1, b = A x* + N(0, noise_sigma^2),
 * lambda = lambda_frac * ||A^T b||_inf.
 * Replaces the reference's synthetic generators
 * (cpp/src/problem_generator/generator_nesterov.h:24-186 and relatives) with a
 * counter-based (Philox) stream so any machine regenerates the same data. */
typedef struct acdc_lasso_gen {
  int64_t m;
  int64_t n;
  int32_t nnz_mode;
  int32_t nnz_per_col;
  double zipf_s;
  int32_t nnz_min;
  int32_t nnz_max;
  double nnz_mean;
  int64_t n_star;
  double noise_sigma;
  double lambda_frac;
  uint64_t seed;
  int32_t normalize_columns;
  int32_t threads; /* OpenMP threads; <= 0 means all */
} acdc_lasso_gen;

/* Phase 1: column pointers (n+1 entries).  col_ptr[n] is the nnz. */
int acdc_gen_lasso_colptr(const acdc_lasso_gen* g, int64_t* col_ptr);
/* Phase 2: rows (sorted ascending within a column), values, b, x* (n entries,
 * may be NULL) and the resulting lambda. */
int acdc_gen_lasso_fill(const acdc_lasso_gen* g, const int64_t* col_ptr, int32_t* row_idx,
                        double* vals, double* b, double* x_star, double* lambda_out);

/* Seeded hinge-loss SVM instance, stored by sample (CSR of X = CSC of X^T,
 * the layout of ProblemData::A_csr_* in cpp/src/solver/structures.h:37-39):
 * per-sample nnz ~ LogNormal(ln nnz_median, nnz_sigma) clipped to [1, d],
 * distinct uniform features, Exp(1) values, rows scaled to unit L2 norm;
 * labels y_i = sign(x_i^T w*) for w* with w_star_nnz N(0,1) entries, each label
 * flipped with probability flip_prob. */
typedef struct acdc_svm_gen {
  int64_t n_samples;
  int64_t d;
  double nnz_median;
  double nnz_sigma;
  int64_t w_star_nnz;
  double flip_prob;
  uint64_t seed;
  int32_t threads;
} acdc_svm_gen;

int acdc_gen_svm_rowptr(const acdc_svm_gen* g, int64_t* row_ptr);
int acdc_gen_svm_fill(const acdc_svm_gen* g, const int64_t* row_ptr, int32_t* col_idx,
                      double* vals, double* y);

/* Known-optimum Lasso instance (the construction of
 * cpp/src/problem_generator/generator_nesterov.h:24-186, with the support
 * chosen per column): A has p uniform(-1,1) entries per column at distinct rows,
 * y* is a random unit-direction vector, the n_nonzero columns with the largest
 * |a_j^T y*| are scaled so a_j^T y* = +-lambda and all others so that
 * |a_j^T y*| <= 0.9 lambda; x*_j = sign(a_j^T y*) * U(0,1) * rho on the
 * support; b = y* + A x*.  Then x* is the unique minimiser of
 * 0.5||Ax-b||^2 + lambda ||x||_1 and f_star its value.
 * col_ptr must hold n+1 entries (filled with j*p), row_idx/vals n*p, b m, x_star n. */
int acdc_gen_nesterov(int64_t m, int64_t n, int32_t p, int64_t n_nonzero, double lambda,
                      double rho, uint64_t seed, int64_t* col_ptr, int32_t* row_idx,
                      double* vals, double* b, double* x_star, double* f_star);

/* Sizes of instance `index` of the batched Lasso mix: m log-uniform in
 * [m_lo, m_hi], n log-uniform in [n_lo, n_hi]; the caller then generates it
 * with acdc_gen_lasso_* (nnz per column uniform in [nnz_lo, nnz_hi]). */
int acdc_gen_mix_sizes(uint64_t seed, int64_t index, int64_t m_lo, int64_t m_hi, int64_t n_lo,
                       int64_t n_hi, int64_t* m_out, int64_t* n_out);

/* Row counts and omega = max_i |{j : A_ij != 0}| (the ESO parameter of
 * cpp/src/frontends/solvers/MultiCoreSolver.cpp:32-38, 55-62). */
int acdc_host_omega(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                    int64_t* omega_out);

/* Philox4x32-10 block and the coordinate sampler exactly as the device uses
 * them (acdc_philox.h): update k of a solve with key `seed` draws coordinate
 * acdc_sample_coordinate(seed, k, n).  Replaces gsl_rng_uniform_int(gsl_rng_r, n)
 * (cpp/src/solver/MulticoreEngineExecutor.h:86). */
void acdc_philox4x32_10_host(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t acdc_sample_coordinate(uint64_t seed, uint64_t k, uint64_t n);

/* ---- On-disk formats ---------------------------------------------------- */

/* Text CSC triple <prefix>_values.txt, <prefix>_colPtr.txt, <prefix>_rowIdx.txt
 * plus the vector file, whitespace separated, 0-based rows: the format read by
 * InputOuputHelper::loadCSCData (cpp/src/utils/file_reader.h:108-137, values via
 * loadVectorData :32-48).  Phase 1 returns the sizes, phase 2 fills. */
int acdc_load_csc_text_sizes(const char* prefix, const char* vector_file, int64_t* m, int64_t* n,
                             int64_t* nnz);
int acdc_load_csc_text(const char* prefix, const char* vector_file, int64_t* col_ptr,
                       int32_t* row_idx, double* vals, double* b);

/* Binary per-rank CSC: <prefix>_colptr_<rank><suffix> (local_n + 1 text
 * offsets), <prefix>_rowid_<rank><suffix> (raw int32 rows) and
 * <prefix>_values_<rank><suffix> (raw doubles, native byte order) plus the text
 * vector file: the format read by loadANSCIAndBinaryData
 * (cpp/src/utils/file_reader.h:50-106), whose column count local_n the caller
 * gives.  Phase 1 returns the sizes, phase 2 fills. */
int acdc_load_csc_binary_sizes(const char* prefix, const char* suffix, int32_t rank,
                               const char* vector_file, int64_t local_n, int64_t* m, int64_t* n,
                               int64_t* nnz);
int acdc_load_csc_binary(const char* prefix, const char* suffix, int32_t rank,
                         const char* vector_file, int64_t local_n, int64_t* col_ptr,
                         int32_t* row_idx, double* vals, double* b);

/* Writes a CSC matrix (n columns) in that per-rank format, the three files
 * <prefix>_colptr_<rank><suffix> (text), _rowid_ (raw int32) and _values_
 * (raw doubles), so that text or generated inputs can be converted once and
 * then loaded without parsing.  The vector file stays text. */
int acdc_save_csc_binary(const char* prefix, const char* suffix, int32_t rank, int64_t n,
                         const int64_t* col_ptr, const int32_t* row_idx, const double* vals);

/* Host threads of the text loaders (acdc_load_csc_text*, the offsets file of
 * acdc_load_csc_binary*, acdc_load_libsvm*): > 0 cuts every text into that
 * many pieces, each parsed on its own thread; 0 (the default) uses one piece
 * per MiB of text, up to the hardware threads.  The loaded arrays do not
 * depend on it.  Returns the previous setting.  The reference's readers
 * (file_reader.h, distributed_instances_loader.h) parse on one thread. */
int acdc_host_threads(int32_t threads);

/* LIBSVM text (label index:value ...), 1-based feature indices mapped to
 * 0-based, labels 0 mapped to -1 for two classes: the reader
 * loadDistributedSparseSVMRowData (cpp/src/utils/distributed_instances_loader.h:68-193,
 * sizes by parse_LIB_SVM_data_get_size, cpp/src/svm/svm_parser.h:11-77). */
int acdc_load_libsvm_sizes(const char* path, int64_t* n_samples, int64_t* d, int64_t* nnz);
int acdc_load_libsvm(const char* path, int64_t* row_ptr, int32_t* col_idx, double* vals,
                     double* y);

#ifdef __cplusplus
}
#endif
#endif /* ACDC_HOST_H_ */

/*
 * Minimal stand-in for the CBLAS subset the reference's
 * cpp/src/utils/my_cblas_wrapper.h calls, written from the standard CBLAS
 * interface (plain loops, reference operation order for sums).
 * TEST INFRASTRUCTURE ONLY (used when building oracle/_ref).
 *
 * Norms are sqrt(sum x_i^2), not GSL's scaled nrm2, so objective values may
 * differ from a GSL build in the last bits; iterates are unaffected.
 */
#ifndef ACDC_GSL_SHIM_CBLAS_H_
#define ACDC_GSL_SHIM_CBLAS_H_

#include <math.h>
#include <stddef.h>

#define CBLAS_INDEX size_t
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

static inline void cblas_dscal(const int N, const double alpha, double* X, const int incX) {
  for (int i = 0; i < N; ++i) X[(size_t)i * incX] *= alpha;
}
static inline void cblas_sscal(const int N, const float alpha, float* X, const int incX) {
  for (int i = 0; i < N; ++i) X[(size_t)i * incX] *= alpha;
}
static inline void cblas_daxpy(const int N, const double alpha, const double* X, const int incX,
                               double* Y, const int incY) {
  for (int i = 0; i < N; ++i) Y[(size_t)i * incY] += alpha * X[(size_t)i * incX];
}
static inline void cblas_saxpy(const int N, const float alpha, const float* X, const int incX,
                               float* Y, const int incY) {
  for (int i = 0; i < N; ++i) Y[(size_t)i * incY] += alpha * X[(size_t)i * incX];
}
static inline void cblas_dcopy(const int N, const double* X, const int incX, double* Y,
                               const int incY) {
  for (int i = 0; i < N; ++i) Y[(size_t)i * incY] = X[(size_t)i * incX];
}
static inline void cblas_scopy(const int N, const float* X, const int incX, float* Y,
                               const int incY) {
  for (int i = 0; i < N; ++i) Y[(size_t)i * incY] = X[(size_t)i * incX];
}
static inline double cblas_dasum(const int N, const double* X, const int incX) {
  double s = 0;
  for (int i = 0; i < N; ++i) s += fabs(X[(size_t)i * incX]);
  return s;
}
static inline float cblas_sasum(const int N, const float* X, const int incX) {
  float s = 0;
  for (int i = 0; i < N; ++i) s += fabsf(X[(size_t)i * incX]);
  return s;
}
static inline double cblas_dnrm2(const int N, const double* X, const int incX) {
  double s = 0;
  for (int i = 0; i < N; ++i) s += X[(size_t)i * incX] * X[(size_t)i * incX];
  return sqrt(s);
}
static inline float cblas_snrm2(const int N, const float* X, const int incX) {
  float s = 0;
  for (int i = 0; i < N; ++i) s += X[(size_t)i * incX] * X[(size_t)i * incX];
  return sqrtf(s);
}
static inline CBLAS_INDEX cblas_idamax(const int N, const double* X, const int incX) {
  CBLAS_INDEX best = 0;
  double v = -1;
  for (int i = 0; i < N; ++i)
    if (fabs(X[(size_t)i * incX]) > v) {
      v = fabs(X[(size_t)i * incX]);
      best = (CBLAS_INDEX)i;
    }
  return best;
}
static inline CBLAS_INDEX cblas_isamax(const int N, const float* X, const int incX) {
  CBLAS_INDEX best = 0;
  float v = -1;
  for (int i = 0; i < N; ++i)
    if (fabsf(X[(size_t)i * incX]) > v) {
      v = fabsf(X[(size_t)i * incX]);
      best = (CBLAS_INDEX)i;
    }
  return best;
}

#define ACDC_SHIM_GEMM(NAME, T)                                                              \
  static inline void NAME(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA,   \
                          const enum CBLAS_TRANSPOSE TransB, const int M, const int N,       \
                          const int K, const T alpha, const T* A, const int lda, const T* B, \
                          const int ldb, const T beta, T* C, const int ldc) {                \
    for (int i = 0; i < M; ++i)                                                              \
      for (int j = 0; j < N; ++j) {                                                          \
        T acc = 0;                                                                           \
        for (int k = 0; k < K; ++k) {                                                        \
          size_t ia, ib;                                                                     \
          if (Order == CblasRowMajor) {                                                      \
            ia = TransA == CblasNoTrans ? (size_t)i * lda + k : (size_t)k * lda + i;         \
            ib = TransB == CblasNoTrans ? (size_t)k * ldb + j : (size_t)j * ldb + k;         \
          } else {                                                                           \
            ia = TransA == CblasNoTrans ? (size_t)k * lda + i : (size_t)i * lda + k;         \
            ib = TransB == CblasNoTrans ? (size_t)j * ldb + k : (size_t)k * ldb + j;         \
          }                                                                                  \
          acc += A[ia] * B[ib];                                                              \
        }                                                                                    \
        size_t ic = Order == CblasRowMajor ? (size_t)i * ldc + j : (size_t)j * ldc + i;      \
        C[ic] = alpha * acc + (beta == 0 ? 0 : beta * C[ic]);                                \
      }                                                                                      \
  }
ACDC_SHIM_GEMM(cblas_dgemm, double)
ACDC_SHIM_GEMM(cblas_sgemm, float)
#undef ACDC_SHIM_GEMM

#endif

/*
 * pcdm_oracle.c - CPU restatement of optml/ac-dc's PCDM hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library (tests, smoke
 * check, CPU-baseline leg of the benchmark).  Never part of the product path.
 *
 * Each function restates a reference routine, cited by file:line relative to
 * the reference project root.  The arithmetic keeps the reference's operation
 * order so that the serial trajectory is bit-identical to the reference's
 * engine run with one thread and the same coordinate sequence (compile with
 * -ffp-contract=off so no multiply-add is fused).
 */
#include "pcdm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- sampler ---- */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; ++round) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

uint64_t orc_sample(uint64_t seed, uint64_t k, uint64_t n) {
  uint32_t ctr[4] = {(uint32_t)k, (uint32_t)(k >> 32), 0x5A3D0001u, 0u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  uint64_t u = ((uint64_t)o[0] << 32) | o[1];
  return (uint64_t)(((unsigned __int128)u * n) >> 64);
}

/* sgn(X) (|X| - T)_+ : cpp/src/solver/treshhold_functions.h:27-33 with
 * sgn from cpp/src/helpers/utils.h:29-32 (an int promoted to double). */
static double soft_threshold(double T, double X) {
  double a = fabs(X) - T;
  if (a < 0) a = 0;
  int s = (X > 0) - (X < 0);
  return s * a;
}

/* ---- Lasso ---- */

/* MulticoreSquareLoss::computeReciprocalLipConstants
 * (cpp/src/solver/lossFunctions/squareLoss/MulticoreSquareLoss.h:27-40);
 * beta = 1 reproduces the reference, which applies no ESO factor here. */
void orc_lasso_lipschitz(int64_t n, const int64_t* col_ptr, const double* vals, double beta,
                         double* Li) {
  for (int64_t i = 0; i < n; ++i) {
    double s = 0;
    for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j) s += vals[j] * vals[j];
    Li[i] = s > 0 ? 1 / (beta * s) : 0;
  }
}

/* MulticoreSquareLoss::recomputeResiduals (MulticoreSquareLoss.h:42-53): r = -b + A x. */
void orc_lasso_residuals(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, const double* b, const double* x, double* r) {
  for (int64_t i = 0; i < m; ++i) r[i] = -b[i];
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j) r[row_idx[j]] += vals[j] * x[i];
}

/* One serial update: MulticoreL1RegSquareLoss::compute_update and
 * performOneCoordinateUpdate (MulticoreL1RegSquareLoss.h:41-63). */
static void lasso_update(int64_t idx, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, double lambda, const double* Li, double* x,
                         double* r) {
  double tmp = 0;
  for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j) tmp += vals[j] * r[row_idx[j]];
  tmp = soft_threshold(Li[idx] * lambda, x[idx] - Li[idx] * tmp) - x[idx];
  x[idx] = x[idx] + tmp;
  for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
    r[row_idx[j]] = r[row_idx[j]] + tmp * vals[j];
}

/* MulticoreEngineExecutor::executeBulkOfIterations (MulticoreEngineExecutor.h:83-89)
 * with one thread: update k draws its coordinate from the counter-based sampler. */
void orc_lasso_updates(int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                       const double* vals, double lambda, const double* Li, double* x, double* r,
                       uint64_t seed, uint64_t k0, uint64_t count) {
  for (uint64_t k = 0; k < count; ++k) {
    int64_t idx = (int64_t)orc_sample(seed, k0 + k, (uint64_t)n);
    lasso_update(idx, col_ptr, row_idx, vals, lambda, Li, x, r);
  }
}

/* Primal as MulticoreL1RegSquareLoss::computeObjectiveValue
 * (MulticoreL1RegSquareLoss.h:30-39); the dual point u = s r with
 * s = min(1, lambda/||A^T r||_inf) gives D = -s b^T r - s^2 ||r||^2 / 2. */
void orc_lasso_eval(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                    const double* vals, const double* b, double lambda, const double* x,
                    const double* r, int threads, double* out) {
  double rr = 0, br = 0, l1 = 0, gmax = 0;
  int64_t support = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
#pragma omp parallel for schedule(static) reduction(+ : rr, br)
  for (int64_t i = 0; i < m; ++i) {
    rr += r[i] * r[i];
    br += b[i] * r[i];
  }
#pragma omp parallel for schedule(static) reduction(+ : l1, support) reduction(max : gmax)
  for (int64_t j = 0; j < n; ++j) {
    double g = 0;
    for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) g += vals[e] * r[row_idx[e]];
    g = fabs(g);
    if (g > gmax) gmax = g;
    l1 += fabs(x[j]);
    support += x[j] != 0;
  }
  double P = 0.5 * rr + lambda * l1;
  double s = (gmax > lambda) ? lambda / gmax : 1.0;
  double D = -s * br - 0.5 * s * s * rr;
  out[0] = P;
  out[1] = D;
  out[2] = P - D;
  out[3] = (P - D) / (fabs(P) > 1 ? fabs(P) : 1);
  out[4] = 0;
  out[5] = l1;
  out[6] = rr;
  out[7] = gmax;
  out[8] = (double)support;
}

int64_t orc_lasso_solve(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                        const double* vals, const double* b, double lambda, double beta,
                        uint64_t seed, double target, int rel, int64_t max_epochs,
                        int64_t check_every, double* x, double* r, double* out) {
  double* Li = (double*)malloc(sizeof(double) * (size_t)n);
  orc_lasso_lipschitz(n, col_ptr, vals, beta, Li);
  orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
  orc_lasso_eval(m, n, col_ptr, row_idx, vals, b, lambda, x, r, 0, out);
  int64_t epochs = 0;
  uint64_t k = 0;
  if (check_every < 1) check_every = 1;
  while ((rel ? out[3] : out[2]) > target && epochs < max_epochs) {
    orc_lasso_updates(n, col_ptr, row_idx, vals, lambda, Li, x, r, seed, k,
                      (uint64_t)(check_every * n));
    k += (uint64_t)(check_every * n);
    epochs += check_every;
    orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
    orc_lasso_eval(m, n, col_ptr, row_idx, vals, b, lambda, x, r, 0, out);
  }
  free(Li);
  return epochs;
}

/* Active list in column order: x_j != 0 or |a_j^T r| > (1 - eps) lambda. */
static int64_t build_active(int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                            const double* vals, double lambda, double eps, const double* x,
                            const double* r, int32_t* active) {
  int64_t cnt = 0;
  for (int64_t j = 0; j < n; ++j) {
    double g = 0;
    for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) g += vals[e] * r[row_idx[e]];
    if (x[j] != 0 || fabs(g) > (1 - eps) * lambda) active[cnt++] = (int32_t)j;
  }
  return cnt;
}

int64_t orc_lasso_solve_shrink(int64_t m, int64_t n, const int64_t* col_ptr,
                               const int32_t* row_idx, const double* vals, const double* b,
                               double lambda, double beta, uint64_t seed, double target, int rel,
                               int64_t max_epochs, int64_t check_every, double q, double eps,
                               int64_t start_epoch, double step_scale, double* x, double* r,
                               double* out, double* gap_trace) {
  double* Li = (double*)malloc(sizeof(double) * (size_t)n);
  int32_t* active = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  orc_lasso_lipschitz(n, col_ptr, vals, beta, Li);
  orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
  orc_lasso_eval(m, n, col_ptr, row_idx, vals, b, lambda, x, r, 0, out);
  int64_t n_active = 0;
  int64_t epochs = 0, checks = 0;
  uint64_t k = 0;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  const uint32_t q32 = q >= 1 ? 0xffffffffu : (uint32_t)(q * 4294967296.0);
  if (check_every < 1) check_every = 1;
  while ((rel ? out[3] : out[2]) > target && epochs < max_epochs) {
    const int shrink = epochs >= start_epoch && n_active > 0 && q > 0;
    for (uint64_t t = 0; t < (uint64_t)(check_every * n); ++t, ++k) {
      uint32_t ctr[4] = {(uint32_t)k, (uint32_t)(k >> 32), 0x5A3D0001u, 0u}, o[4];
      orc_philox4x32_10(ctr, key, o);
      int64_t idx;
      double scale = 1.0;
      if (shrink && o[2] < q32) {
        idx = active[(uint32_t)(((uint64_t)o[3] * (uint64_t)n_active) >> 32)];
        scale = step_scale;
      } else {
        uint64_t u = ((uint64_t)o[0] << 32) | o[1];
        idx = (int64_t)(((unsigned __int128)u * (uint64_t)n) >> 64);
      }
      double tmp = 0;
      for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j) tmp += vals[j] * r[row_idx[j]];
      const double li = Li[idx] * scale;
      tmp = soft_threshold(li * lambda, x[idx] - li * tmp) - x[idx];
      x[idx] = x[idx] + tmp;
      for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
        r[row_idx[j]] = r[row_idx[j]] + tmp * vals[j];
    }
    epochs += check_every;
    orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
    orc_lasso_eval(m, n, col_ptr, row_idx, vals, b, lambda, x, r, 0, out);
    n_active = build_active(n, col_ptr, row_idx, vals, lambda, eps, x, r, active);
    if (gap_trace) gap_trace[checks] = out[3];
    checks++;
  }
  free(Li);
  free(active);
  return epochs;
}

/* Working-set solve for the fixtures of the large configurations: it finds the
 * optimum to a certified gap; it does not follow a sampler trajectory.  The
 * coordinate step is the reference's serial update with the exact Lipschitz
 * constant (MulticoreL1RegSquareLoss.h:41-63, MulticoreSquareLoss.h:27-40 with
 * beta = 1), applied in cyclic sweeps over the working set
 * W = {j : x_j != 0 or |a_j^T r| > (1 - eps) lambda}.  Each check recomputes
 * r = A x - b exactly (MulticoreSquareLoss.h:42-53), takes a_j^T r over every
 * column (OpenMP over `threads`, read-only), evaluates the gap as
 * orc_lasso_eval does and rebuilds W in column order.  `sweeps` sweeps run
 * between checks; the solve stops when the (relative if rel) gap is <= target
 * or after max_checks checks.  With anderson = K > 1 (at most 16), every K + 1
 * sweeps are followed by an Anderson extrapolation step.  Returns the sweeps
 * made; *checks_out gets the checks. */
int64_t orc_lasso_solve_ws(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                           const double* vals, const double* b, double lambda, double target,
                           int rel, int64_t max_checks, int64_t sweeps, double eps, int threads,
                           int anderson, double* x, double* r, double* out, int64_t* checks_out) {
  double* g = (double*)malloc(sizeof(double) * (size_t)n);
  const int K = anderson > 1 ? (anderson < 16 ? anderson : 16) : 0;
  double* snap = NULL;     /* K + 1 snapshots of x over the working set */
  double* xe = NULL;       /* extrapolated x over the working set */
  double* re = K ? (double*)malloc(sizeof(double) * (size_t)m) : NULL;
  int64_t snap_cap = 0;
  int32_t* ws = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  int64_t* wptr = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
  int32_t* wrow = NULL;
  double* wval = NULL;
  double* wli = (double*)malloc(sizeof(double) * (size_t)n);
  int64_t wcap = 0, total_sweeps = 0, checks = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  for (;;) {
    orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
    double rr = 0, br = 0, l1 = 0, gmax = 0;
    int64_t support = 0;
#pragma omp parallel for schedule(static) reduction(+ : rr, br)
    for (int64_t i = 0; i < m; ++i) {
      rr += r[i] * r[i];
      br += b[i] * r[i];
    }
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : l1, support) reduction(max : gmax)
    for (int64_t j = 0; j < n; ++j) {
      double s = 0;
      for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) s += vals[e] * r[row_idx[e]];
      g[j] = s;
      s = fabs(s);
      if (s > gmax) gmax = s;
      l1 += fabs(x[j]);
      support += x[j] != 0;
    }
    const double P = 0.5 * rr + lambda * l1;
    const double sc = (gmax > lambda) ? lambda / gmax : 1.0;
    const double D = -sc * br - 0.5 * sc * sc * rr;
    out[0] = P;
    out[1] = D;
    out[2] = P - D;
    out[3] = (P - D) / (fabs(P) > 1 ? fabs(P) : 1);
    out[4] = 0;
    out[5] = l1;
    out[6] = rr;
    out[7] = gmax;
    out[8] = (double)support;
    checks++;
    if ((rel ? out[3] : out[2]) <= target || checks >= max_checks) break;
    /* working set in column order, packed for the sweeps */
    int64_t nw = 0, entries = 0;
    for (int64_t j = 0; j < n; ++j)
      if (x[j] != 0 || fabs(g[j]) > (1 - eps) * lambda) {
        ws[nw++] = (int32_t)j;
        entries += col_ptr[j + 1] - col_ptr[j];
      }
    if (entries > wcap) {
      free(wrow);
      free(wval);
      wcap = entries;
      wrow = (int32_t*)malloc(sizeof(int32_t) * (size_t)(wcap > 0 ? wcap : 1));
      wval = (double*)malloc(sizeof(double) * (size_t)(wcap > 0 ? wcap : 1));
    }
    wptr[0] = 0;
    for (int64_t t = 0; t < nw; ++t) {
      const int64_t j = ws[t];
      int64_t o = wptr[t];
      double s = 0;
      for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e, ++o) {
        wrow[o] = row_idx[e];
        wval[o] = vals[e];
        s += vals[e] * vals[e];
      }
      wptr[t + 1] = o;
      wli[t] = s > 0 ? 1 / s : 0;
    }
    if (K && nw * (K + 1) > snap_cap) {
      free(snap);
      free(xe);
      snap_cap = nw * (K + 1);
      snap = (double*)malloc(sizeof(double) * (size_t)snap_cap);
      xe = (double*)malloc(sizeof(double) * (size_t)(nw > 0 ? nw : 1));
    }
    for (int64_t sw = 0; sw < sweeps; ++sw) {
      for (int64_t t = 0; t < nw; ++t) {
        const int64_t j = ws[t];
        double tmp = 0;
        for (int64_t e = wptr[t]; e < wptr[t + 1]; ++e) tmp += wval[e] * r[wrow[e]];
        tmp = soft_threshold(wli[t] * lambda, x[j] - wli[t] * tmp) - x[j];
        if (tmp == 0) continue;
        x[j] = x[j] + tmp;
        for (int64_t e = wptr[t]; e < wptr[t + 1]; ++e) r[wrow[e]] = r[wrow[e]] + tmp * wval[e];
      }
      if (!K || nw == 0) continue;
      /* Anderson extrapolation of the sweeps (Bertrand and Massias, "Anderson
       * acceleration of coordinate descent", AISTATS 2021): after K + 1
       * snapshots, the combination of the last K iterates whose weights
       * (summing to 1) minimise the norm of the combined differences, kept
       * only if it lowers the objective. */
      const int slot = (int)(sw % (K + 1));
      for (int64_t t = 0; t < nw; ++t) snap[(size_t)slot * nw + t] = x[ws[t]];
      if (slot != K) continue;
      double G[16 * 16], z[16];
      for (int a = 0; a < K; ++a)
        for (int c = 0; c <= a; ++c) {
          double acc = 0;
          const double* ua1 = snap + (size_t)(a + 1) * nw;
          const double* ua0 = snap + (size_t)a * nw;
          const double* uc1 = snap + (size_t)(c + 1) * nw;
          const double* uc0 = snap + (size_t)c * nw;
          for (int64_t t = 0; t < nw; ++t) acc += (ua1[t] - ua0[t]) * (uc1[t] - uc0[t]);
          G[a * K + c] = G[c * K + a] = acc;
        }
      double tr = 0;
      for (int a = 0; a < K; ++a) tr += G[a * K + a];
      if (!(tr > 0)) continue;
      for (int a = 0; a < K; ++a) {
        G[a * K + a] += 1e-12 * tr;
        z[a] = 1;
      }
      /* Cholesky solve of G z = 1 */
      int ok = 1;
      for (int a = 0; a < K && ok; ++a) {
        double d = G[a * K + a];
        for (int c = 0; c < a; ++c) d -= G[a * K + c] * G[a * K + c];
        if (!(d > 0)) {
          ok = 0;
          break;
        }
        G[a * K + a] = sqrt(d);
        for (int e = a + 1; e < K; ++e) {
          double v = G[e * K + a];
          for (int c = 0; c < a; ++c) v -= G[e * K + c] * G[a * K + c];
          G[e * K + a] = v / G[a * K + a];
        }
      }
      if (!ok) continue;
      for (int a = 0; a < K; ++a) {
        double v = z[a];
        for (int c = 0; c < a; ++c) v -= G[a * K + c] * z[c];
        z[a] = v / G[a * K + a];
      }
      for (int a = K - 1; a >= 0; --a) {
        double v = z[a];
        for (int c = a + 1; c < K; ++c) v -= G[c * K + a] * z[c];
        z[a] = v / G[a * K + a];
      }
      double zs = 0;
      for (int a = 0; a < K; ++a) zs += z[a];
      if (!(fabs(zs) > 0)) continue;
      double l1_cur = 0, l1_e = 0;
      for (int64_t t = 0; t < nw; ++t) {
        double v = 0;
        for (int a = 0; a < K; ++a) v += z[a] / zs * snap[(size_t)(a + 1) * nw + t];
        xe[t] = v;
        l1_cur += fabs(x[ws[t]]);
        l1_e += fabs(v);
      }
      memcpy(re, r, sizeof(double) * (size_t)m);
      for (int64_t t = 0; t < nw; ++t) {
        const double dlt = xe[t] - x[ws[t]];
        if (dlt == 0) continue;
        for (int64_t e = wptr[t]; e < wptr[t + 1]; ++e) re[wrow[e]] += dlt * wval[e];
      }
      double rr_cur = 0, rr_e = 0;
      for (int64_t i = 0; i < m; ++i) {
        rr_cur += r[i] * r[i];
        rr_e += re[i] * re[i];
      }
      if (0.5 * rr_e + lambda * l1_e < 0.5 * rr_cur + lambda * l1_cur) {
        for (int64_t t = 0; t < nw; ++t) x[ws[t]] = xe[t];
        memcpy(r, re, sizeof(double) * (size_t)m);
      }
    }
    total_sweeps += sweeps;
  }
  free(g);
  free(ws);
  free(wptr);
  free(wrow);
  free(wval);
  free(wli);
  free(snap);
  free(xe);
  free(re);
  if (checks_out) *checks_out = checks;
  return total_sweeps;
}

/* ---- L2-regularised square loss (lossFunction 1) and L2-regularised
 *      logistic loss (lossFunction 3): the "smooth" losses ---- */

/* MulticoreL2SquareRegSquareLoss::computeReciprocalLipConstants
 * (cpp/src/solver/lossFunctions/squareLoss/MulticoreL2SquareRegSquareLoss.h:30-43):
 * Li = 1/(lambda + ||a_j||^2), summed from lambda in column order.
 * MulticoreL2SquareRegLogisticLoss::computeReciprocalLipConstants
 * (cpp/src/solver/lossFunctions/logisticLoss/MulticoreL2SquareRegLogisticLoss.h:30-44):
 * Li = 1/(sigma (lambda + ||a_j||^2 / 4)).  beta scales the ||a_j||^2 term of the
 * square loss (1 reproduces the reference, which applies none there). */
void orc_smooth_lipschitz(int loss, int64_t n, const int64_t* col_ptr, const double* vals,
                          double lambda, double beta, double sigma, double* Li) {
  for (int64_t i = 0; i < n; ++i) {
    double acc = lambda;
    if (loss == ORC_LOSS_RIDGE) {
      if (beta == 1) {
        for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j) acc += vals[j] * vals[j];
      } else {
        double s = 0;
        for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j) s += vals[j] * vals[j];
        acc = lambda + beta * s;
      }
    } else {
      for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j) acc += 0.25 * vals[j] * vals[j];
      acc = acc * sigma;
    }
    Li[i] = acc > 0 ? 1 / acc : acc;
  }
}

/* Residuals: MulticoreSquareLoss::recomputeResiduals (MulticoreSquareLoss.h:42-53),
 * r = -b + A x, for loss 1; MulticoreLogisticLoss::recomputeResiduals
 * (cpp/src/solver/lossFunctions/logisticLoss/MulticoreLogisticLoss.h:42-55),
 * r_i = -b_i (A x)_i, for loss 3. */
void orc_smooth_residuals(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                          const int32_t* row_idx, const double* vals, const double* b,
                          const double* x, double* r) {
  if (loss == ORC_LOSS_RIDGE) {
    orc_lasso_residuals(m, n, col_ptr, row_idx, vals, b, x, r);
    return;
  }
  for (int64_t i = 0; i < m; ++i) r[i] = 0;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = col_ptr[i]; j < col_ptr[i + 1]; ++j)
      r[row_idx[j]] += -b[row_idx[j]] * vals[j] * x[i];
}

/* One serial update: MulticoreL2SquareRegSquareLoss::compute_update and
 * performOneCoordinateUpdate (MulticoreL2SquareRegSquareLoss.h:56-78), or
 * MulticoreL2SquareRegLogisticLoss::compute_update and
 * performOneCoordinateUpdate (MulticoreL2SquareRegLogisticLoss.h:88-115), whose
 * step is halved. */
static void smooth_update(int loss, int64_t idx, const int64_t* col_ptr, const int32_t* row_idx,
                          const double* vals, const double* b, double lambda, const double* Li,
                          double* x, double* r) {
  double tmp = 0;
  if (loss == ORC_LOSS_RIDGE) {
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j) tmp += vals[j] * r[row_idx[j]];
    tmp += lambda * x[idx];
    tmp = -Li[idx] * tmp;
    x[idx] = x[idx] + tmp;
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
      r[row_idx[j]] = r[row_idx[j]] + tmp * vals[j];
  } else {
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j) {
      double tt = exp(r[row_idx[j]]);
      tmp += -b[row_idx[j]] * vals[j] * tt / (1 + tt);
    }
    tmp += lambda * x[idx];
    tmp = -Li[idx] * tmp;
    tmp = tmp / 2;
    x[idx] = x[idx] + tmp;
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
      r[row_idx[j]] = r[row_idx[j]] + -b[row_idx[j]] * tmp * vals[j];
  }
}

void orc_smooth_updates(int loss, int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                        const double* vals, const double* b, double lambda, const double* Li,
                        double* x, double* r, uint64_t seed, uint64_t k0, uint64_t count) {
  for (uint64_t k = 0; k < count; ++k) {
    int64_t idx = (int64_t)orc_sample(seed, k0 + k, (uint64_t)n);
    smooth_update(loss, idx, col_ptr, row_idx, vals, b, lambda, Li, x, r);
  }
}

/* Primal as computeObjectiveValue (MulticoreL2SquareRegSquareLoss.h:45-54:
 * ||r||^2/2 + lambda ||x||^2/2; MulticoreL2SquareRegLogisticLoss.h:46-86:
 * sum log(1 + exp(r_i)) + lambda ||x||^2/2, training accuracy = fraction of
 * r_i < 0).  The duality gaps are this build's (the reference reports none):
 *   loss 1: P - D = (1/(2 lambda)) sum_j (a_j^T r + lambda x_j)^2 with the
 *           dual point u = r of D(u) = -||u||^2/2 - b^T u - ||A^T u||^2/(2 lambda);
 *   loss 3: D(a) = -sum_i [a_i log a_i + (1-a_i) log(1-a_i)]
 *                  - ||sum_i a_i b_i A_i.||^2/(2 lambda) at a_i = 1/(1+exp(-r_i)).
 * out: [0] P [1] D [2] gap [3] rel_gap [4] accuracy (loss 3) [5] ||x||^2
 *      [6] ||r||^2 (loss 1) or sum log(1+exp(r)) (loss 3) [7] 0 [8] support. */
static double sigmoid(double z) {
  if (z >= 0) return 1 / (1 + exp(-z));
  double e = exp(z);
  return e / (1 + e);
}

static double neg_entropy(double a) {
  double s = 0;
  if (a > 0) s += a * log(a);
  if (a < 1) s += (1 - a) * log1p(-a);
  return s;
}

void orc_smooth_eval(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                     const int32_t* row_idx, const double* vals, const double* b, double lambda,
                     const double* x, const double* r, double* out) {
  double xx = 0, rows = 0, ent = 0, good = 0, cols = 0;
  int64_t support = 0;
  double* alpha = NULL;
  if (loss == ORC_LOSS_LOGISTIC) alpha = (double*)malloc(sizeof(double) * (size_t)(m > 0 ? m : 1));
  for (int64_t i = 0; i < m; ++i) {
    if (loss == ORC_LOSS_RIDGE) {
      rows += r[i] * r[i];
    } else {
      rows += r[i] > 0 ? r[i] + log1p(exp(-r[i])) : log1p(exp(r[i]));
      alpha[i] = sigmoid(r[i]);
      ent += neg_entropy(alpha[i]);
      good += r[i] < 0;
    }
  }
  for (int64_t j = 0; j < n; ++j) {
    double g = 0;
    if (loss == ORC_LOSS_RIDGE) {
      for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) g += vals[e] * r[row_idx[e]];
      g += lambda * x[j];
    } else {
      for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e)
        g += b[row_idx[e]] * vals[e] * alpha[row_idx[e]];
    }
    cols += g * g;
    xx += x[j] * x[j];
    support += x[j] != 0;
  }
  double P, D;
  if (loss == ORC_LOSS_RIDGE) {
    P = 0.5 * rows + 0.5 * lambda * xx;
    D = P - cols / (2 * lambda);
  } else {
    P = rows + 0.5 * lambda * xx;
    D = -ent - cols / (2 * lambda);
  }
  free(alpha);
  out[0] = P;
  out[1] = D;
  out[2] = P - D;
  out[3] = (P - D) / (fabs(P) > 1 ? fabs(P) : 1);
  out[4] = loss == ORC_LOSS_LOGISTIC && m > 0 ? good / (double)m : 0;
  out[5] = xx;
  out[6] = rows;
  out[7] = 0;
  out[8] = (double)support;
}

int64_t orc_smooth_solve(int loss, int64_t m, int64_t n, const int64_t* col_ptr,
                         const int32_t* row_idx, const double* vals, const double* b,
                         double lambda, double beta, double sigma, uint64_t seed, double target,
                         int rel, int64_t max_epochs, double* x, double* r, double* out) {
  double* Li = (double*)malloc(sizeof(double) * (size_t)n);
  orc_smooth_lipschitz(loss, n, col_ptr, vals, lambda, beta, sigma, Li);
  orc_smooth_residuals(loss, m, n, col_ptr, row_idx, vals, b, x, r);
  orc_smooth_eval(loss, m, n, col_ptr, row_idx, vals, b, lambda, x, r, out);
  int64_t epochs = 0;
  uint64_t k = 0;
  while ((rel ? out[3] : out[2]) > target && epochs < max_epochs) {
    orc_smooth_updates(loss, n, col_ptr, row_idx, vals, b, lambda, Li, x, r, seed, k, (uint64_t)n);
    k += (uint64_t)n;
    epochs += 1;
    orc_smooth_residuals(loss, m, n, col_ptr, row_idx, vals, b, x, r);
    orc_smooth_eval(loss, m, n, col_ptr, row_idx, vals, b, lambda, x, r, out);
  }
  free(Li);
  return epochs;
}

/* ---- SVM dual ---- */

/* MulticoreSVMDualLoss::computeReciprocalLipConstants (MulticoreSVMDualLoss.h:48-61). */
void orc_svm_lipschitz(int64_t n, const int64_t* row_ptr, const double* vals, double sigma,
                       double* Li) {
  for (int64_t i = 0; i < n; ++i) {
    double s = 0;
    for (int64_t j = row_ptr[i]; j < row_ptr[i + 1]; ++j) s += vals[j] * vals[j];
    Li[i] = s > 0 ? 1 / (sigma * s) : 0;
  }
}

/* MulticoreSVMDualLoss::recomputeResiduals (MulticoreSVMDualLoss.h:31-46):
 * clip alpha into [0,1], then w = (1/(lambda n)) sum_i y_i alpha_i x_i. */
void orc_svm_residuals(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, double* alpha,
                       double* w) {
  for (int64_t i = 0; i < m; ++i) w[i] = 0;
  const double delta = 1 / (lambda * (double)n + 0.0);
  for (int64_t s = 0; s < n; ++s) {
    if (alpha[s] > 1) alpha[s] = 1;
    if (alpha[s] < 0) alpha[s] = 0;
    for (int64_t t = row_ptr[s]; t < row_ptr[s + 1]; ++t)
      w[col_idx[t]] += delta * y[s] * vals[t] * alpha[s];
  }
}

/* MulticoreSVMDualLoss::performOneCoordinateUpdate (MulticoreSVMDualLoss.h:119-141). */
static void svm_update(int64_t idx, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, const double* Li,
                       double* alpha, double* w) {
  double tmp = 0;
  for (int64_t i = row_ptr[idx]; i < row_ptr[idx + 1]; ++i) tmp += vals[i] * w[col_idx[i]];
  tmp = (1 - tmp * y[idx]) * lambda * (double)n * Li[idx];
  if (tmp < -alpha[idx])
    tmp = -alpha[idx];
  else if (tmp > 1 - alpha[idx])
    tmp = 1 - alpha[idx];
  alpha[idx] = alpha[idx] + tmp;
  const double delta = 1 / (lambda * (double)n);
  for (int64_t j = row_ptr[idx]; j < row_ptr[idx + 1]; ++j)
    w[col_idx[j]] = w[col_idx[j]] + tmp * vals[j] * y[idx] * delta;
}

void orc_svm_updates(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                     const double* vals, const double* y, double lambda, const double* Li,
                     double* alpha, double* w, uint64_t seed, uint64_t k0, uint64_t count) {
  for (uint64_t k = 0; k < count; ++k) {
    int64_t idx = (int64_t)orc_sample(seed, k0 + k, (uint64_t)n);
    svm_update(idx, n, row_ptr, col_idx, vals, y, lambda, Li, alpha, w);
  }
}

/* tau-nice sampling as the reference's mini-batch loop draws it
 * (cpp/src/experiments/mSDCA.cpp:60-74): each of the tau entries is drawn
 * from the uniform stream (gsl_rng_uniform_int, here orc_sample with a running
 * counter *k) and drawn again while it repeats an earlier entry of the same
 * step, so a step holds the first tau distinct values of the stream.  tau must
 * not exceed n.  Writes S[0..tau) in acceptance order; *k advances by the
 * candidates consumed. */
void orc_tau_nice(uint64_t seed, uint64_t* k, int64_t n, int64_t tau, int32_t* S) {
  for (int64_t i = 0; i < tau; ++i) {
    for (;;) {
      const int32_t c = (int32_t)orc_sample(seed, (*k)++, (uint64_t)n);
      int64_t j = 0;
      while (j < i && S[j] != c) ++j;
      if (j == i) {
        S[i] = c;
        break;
      }
    }
  }
}

/* Synchronous mini-batch SDCA for the hinge-loss dual: the structure of the
 * reference's mini-batch loop (cpp/src/experiments/mSDCA.cpp:79-105: every
 * delta of the step computed from the same w, then all applied) with the
 * hinge-dual coordinate step of MulticoreSVMDualLoss.h:119-141
 * (delta_i = clip((1 - y_i x_i^T w) lambda n Li_i, -alpha_i, 1 - alpha_i),
 * Li_i = 1/(sigma ||x_i||^2)).  Runs `steps` steps of tau-nice draws from the
 * counter *k; deltas are applied in the order of S. */
void orc_svm_minibatch(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, const double* Li,
                       double* alpha, double* w, uint64_t seed, uint64_t* k, int64_t tau,
                       int64_t steps) {
  if (tau > n) tau = n;
  int32_t* S = (int32_t*)malloc(sizeof(int32_t) * (size_t)(tau > 0 ? tau : 1));
  double* d = (double*)malloc(sizeof(double) * (size_t)(tau > 0 ? tau : 1));
  const double scaling = 1 / (lambda * (double)n);
  for (int64_t st = 0; st < steps; ++st) {
    orc_tau_nice(seed, k, n, tau, S);
    for (int64_t i = 0; i < tau; ++i) {
      const int64_t idx = S[i];
      double tmp = 0;
      for (int64_t t = row_ptr[idx]; t < row_ptr[idx + 1]; ++t) tmp += vals[t] * w[col_idx[t]];
      tmp = (1 - tmp * y[idx]) * lambda * (double)n * Li[idx];
      if (tmp < -alpha[idx])
        tmp = -alpha[idx];
      else if (tmp > 1 - alpha[idx])
        tmp = 1 - alpha[idx];
      d[i] = tmp;
    }
    for (int64_t i = 0; i < tau; ++i) {
      const int64_t idx = S[i];
      alpha[idx] = alpha[idx] + d[i];
      for (int64_t t = row_ptr[idx]; t < row_ptr[idx + 1]; ++t)
        w[col_idx[t]] = w[col_idx[t]] + d[i] * vals[t] * y[idx] * scaling;
    }
  }
  free(S);
  free(d);
}

/* Solve with the synchronous mini-batch: epochs of ceil(n / tau) steps, the
 * FP64 refresh and gap after every check_every epochs (the reference checks
 * once per n / tau steps, mSDCA.cpp:109-125), until the gap <= target or
 * max_epochs.  Returns the epochs run. */
int64_t orc_svm_minibatch_solve(int64_t m, int64_t n, const int64_t* row_ptr,
                                const int32_t* col_idx, const double* vals, const double* y,
                                double lambda, double sigma, uint64_t seed, int64_t tau,
                                double target, int64_t max_epochs, int64_t check_every,
                                double* alpha, double* w, double* out) {
  double* Li = (double*)malloc(sizeof(double) * (size_t)n);
  orc_svm_lipschitz(n, row_ptr, vals, sigma, Li);
  orc_svm_residuals(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w);
  orc_svm_eval(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w, 0, out);
  if (tau > n) tau = n;
  if (tau < 1) tau = 1;
  if (check_every < 1) check_every = 1;
  const int64_t steps_per_epoch = (n + tau - 1) / tau;
  uint64_t k = 0;
  int64_t epochs = 0;
  while (out[2] > target && epochs < max_epochs) {
    orc_svm_minibatch(n, row_ptr, col_idx, vals, y, lambda, Li, alpha, w, seed, &k, tau,
                      check_every * steps_per_epoch);
    epochs += check_every;
    orc_svm_residuals(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w);
    orc_svm_eval(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w, 0, out);
  }
  free(Li);
  return epochs;
}

/* MulticoreSVMDualLoss::computeObjectiveValue (MulticoreSVMDualLoss.h:63-117). */
void orc_svm_eval(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                  const double* vals, const double* y, double lambda, const double* alpha,
                  const double* w, int threads, double* out) {
  double ww = 0, sum_loss = 0, sum_alpha = 0;
  int64_t good = 0, support = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
#pragma omp parallel for schedule(static) reduction(+ : ww)
  for (int64_t i = 0; i < m; ++i) ww += w[i] * w[i];
#pragma omp parallel for schedule(static) reduction(+ : sum_loss, sum_alpha, good, support)
  for (int64_t j = 0; j < n; ++j) {
    double err = 0;
    for (int64_t i = row_ptr[j]; i < row_ptr[j + 1]; ++i) err += vals[i] * w[col_idx[i]];
    if (y[j] * err > 0) good++;
    err = 1 - y[j] * err;
    if (err < 0) err = 0;
    sum_loss += err;
    sum_alpha += alpha[j];
    support += alpha[j] != 0;
  }
  double P = lambda * 0.5 * ww + sum_loss / (0.0 + (double)n);
  double D = -lambda * 0.5 * ww + sum_alpha / (0.0 + (double)n);
  out[0] = P;
  out[1] = D;
  out[2] = P - D;
  out[3] = (P - D) / (fabs(P) > 1 ? fabs(P) : 1);
  out[4] = (double)good / (0.0 + (double)n);
  out[5] = sum_alpha;
  out[6] = ww;
  out[7] = 0;
  out[8] = (double)support;
}

int64_t orc_svm_solve(int64_t m, int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                      const double* vals, const double* y, double lambda, double sigma,
                      uint64_t seed, double target, int64_t max_epochs, int64_t check_every,
                      double* alpha, double* w, double* out) {
  double* Li = (double*)malloc(sizeof(double) * (size_t)n);
  orc_svm_lipschitz(n, row_ptr, vals, sigma, Li);
  orc_svm_residuals(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w);
  orc_svm_eval(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w, 0, out);
  int64_t epochs = 0;
  uint64_t k = 0;
  if (check_every < 1) check_every = 1;
  while (out[2] > target && epochs < max_epochs) {
    orc_svm_updates(n, row_ptr, col_idx, vals, y, lambda, Li, alpha, w, seed, k,
                    (uint64_t)(check_every * n));
    k += (uint64_t)(check_every * n);
    epochs += check_every;
    orc_svm_residuals(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w);
    orc_svm_eval(m, n, row_ptr, col_idx, vals, y, lambda, alpha, w, 0, out);
  }
  free(Li);
  return epochs;
}

/* ---- asynchronous OpenMP form ---- */

/* CAS-loop atomic add of cpp/src/parallel/parallel_essentials_posix.h:62-68. */
static void atomic_add_double(double* var, double add) {
  uint64_t* p = (uint64_t*)var;
  uint64_t oldbits = __atomic_load_n(p, __ATOMIC_RELAXED);
  for (;;) {
    double oldv, newv;
    memcpy(&oldv, &oldbits, sizeof oldv);
    newv = oldv + add;
    uint64_t newbits;
    memcpy(&newbits, &newv, sizeof newbits);
    if (__atomic_compare_exchange_n(p, &oldbits, newbits, 0, __ATOMIC_SEQ_CST, __ATOMIC_RELAXED))
      return;
  }
}

static double load_relaxed(const double* v) {
  uint64_t bits = __atomic_load_n((const uint64_t*)v, __ATOMIC_RELAXED);
  double d;
  memcpy(&d, &bits, sizeof d);
  return d;
}

static double wall_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double orc_lasso_hogwild(int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                         const double* vals, double lambda, const double* Li, double* x,
                         double* r, uint64_t seed, uint64_t k0, uint64_t count, int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  double t0 = wall_seconds();
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)count; ++k) {
    int64_t idx = (int64_t)orc_sample(seed, k0 + (uint64_t)k, (uint64_t)n);
    double tmp = 0;
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
      tmp += vals[j] * load_relaxed(&r[row_idx[j]]);
    double xi = load_relaxed(&x[idx]);
    tmp = soft_threshold(Li[idx] * lambda, xi - Li[idx] * tmp) - xi;
    atomic_add_double(&x[idx], tmp);
    for (int64_t j = col_ptr[idx]; j < col_ptr[idx + 1]; ++j)
      atomic_add_double(&r[row_idx[j]], tmp * vals[j]);
  }
  return wall_seconds() - t0;
}

double orc_svm_hogwild(int64_t n, const int64_t* row_ptr, const int32_t* col_idx,
                       const double* vals, const double* y, double lambda, const double* Li,
                       double* alpha, double* w, uint64_t seed, uint64_t k0, uint64_t count,
                       int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const double delta = 1 / (lambda * (double)n);
  double t0 = wall_seconds();
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)count; ++k) {
    int64_t idx = (int64_t)orc_sample(seed, k0 + (uint64_t)k, (uint64_t)n);
    double tmp = 0;
    for (int64_t i = row_ptr[idx]; i < row_ptr[idx + 1]; ++i)
      tmp += vals[i] * load_relaxed(&w[col_idx[i]]);
    double ai = load_relaxed(&alpha[idx]);
    tmp = (1 - tmp * y[idx]) * lambda * (double)n * Li[idx];
    if (tmp < -ai)
      tmp = -ai;
    else if (tmp > 1 - ai)
      tmp = 1 - ai;
    atomic_add_double(&alpha[idx], tmp);
    for (int64_t j = row_ptr[idx]; j < row_ptr[idx + 1]; ++j)
      atomic_add_double(&w[col_idx[j]], tmp * vals[j] * y[idx] * delta);
  }
  return wall_seconds() - t0;
}

int64_t orc_omega(int64_t m, int64_t n, const int64_t* col_ptr, const int32_t* row_idx) {
  int64_t* cnt = (int64_t*)calloc((size_t)m, sizeof(int64_t));
  int64_t w = 1; /* the reference starts from omega = 1 (MultiCoreSolver.cpp:24) */
  for (int64_t e = 0; e < col_ptr[n]; ++e) {
    int64_t c = ++cnt[row_idx[e]];
    if (c > w) w = c;
  }
  free(cnt);
  return w;
}

double orc_eso_beta(double omega, double tau, double n) {
  if (n <= 1) return 1.0;
  return 1 + (omega - 1) * (tau - 1) / (n - 1.0);
}

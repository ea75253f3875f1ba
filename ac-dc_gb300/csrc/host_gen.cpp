// Seeded synthetic problem generators (host, OpenMP).  Every random quantity is
// a Philox draw keyed by (seed, entity index, stream, sub-index), so the output
// depends only on the parameters, never on the thread count or schedule.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "acdc_philox.h"
#include "../../include/acdc_gpu.h"
#include "../../include/acdc_host.h"

namespace {

const double kTwoPi = 6.283185307179586476925286766559;

inline double rnd_u01(uint64_t seed, uint64_t idx, uint32_t stream, uint32_t sub) {
  return acdc_u01(acdc_rand64(seed, idx, stream, sub));
}

// Standard normal by the Box-Muller transform of two uniforms from one Philox block.
inline double rnd_normal(uint64_t seed, uint64_t idx, uint32_t stream, uint32_t sub) {
  acdc_u32x4 o = acdc_philox4x32_10((uint32_t)idx, (uint32_t)(idx >> 32), stream, sub,
                                    (uint32_t)seed, (uint32_t)(seed >> 32));
  uint64_t a = ((uint64_t)o.v[0] << 32) | o.v[1];
  uint64_t c = ((uint64_t)o.v[2] << 32) | o.v[3];
  double u1 = acdc_u01(a);
  double u2 = acdc_u01(c);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(kTwoPi * u2);
}

inline uint64_t rnd_below(uint64_t seed, uint64_t idx, uint32_t stream, uint32_t sub,
                          uint64_t bound) {
  return acdc_scale64(acdc_rand64(seed, idx, stream, sub), bound);
}

// k distinct integers from [0, range) by Floyd's algorithm, sorted ascending.
// Draw t of entity `idx` uses Philox sub-index t.
void distinct_sorted(uint64_t seed, uint64_t idx, uint32_t stream, int64_t k, int64_t range,
                     std::vector<int64_t>& out, std::vector<int64_t>& table) {
  out.clear();
  if (k <= 0) return;
  if (k >= range) {
    for (int64_t i = 0; i < range; ++i) out.push_back(i);
    return;
  }
  size_t cap = 16;
  while (cap < (size_t)(2 * k)) cap <<= 1;
  table.assign(cap, -1);
  auto insert = [&](int64_t v) -> bool {  // true if newly inserted
    size_t h = (size_t)((uint64_t)v * 0x9E3779B97F4A7C15ull >> 17) & (cap - 1);
    while (table[h] != -1) {
      if (table[h] == v) return false;
      h = (h + 1) & (cap - 1);
    }
    table[h] = v;
    return true;
  };
  uint32_t t = 0;
  for (int64_t i = range - k; i < range; ++i, ++t) {
    int64_t r = (int64_t)rnd_below(seed, idx, stream, t, (uint64_t)i + 1);
    if (insert(r))
      out.push_back(r);
    else {
      insert(i);
      out.push_back(i);
    }
  }
  std::sort(out.begin(), out.end());
}

void set_threads(int32_t t) {
  if (t > 0) omp_set_num_threads(t);
}

// Zipf(s) on [1, zmax]: cumulative table for inverse-CDF sampling.
struct Zipf {
  std::vector<double> cdf;
  Zipf(double s, int zmax) : cdf((size_t)zmax) {
    double acc = 0;
    for (int k = 1; k <= zmax; ++k) {
      acc += std::pow((double)k, -s);
      cdf[(size_t)k - 1] = acc;
    }
    for (auto& c : cdf) c /= acc;
  }
  int draw(double u) const {  // u in (0,1]
    size_t pos = (size_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    if (pos >= cdf.size()) pos = cdf.size() - 1;
    return (int)pos + 1;
  }
  double pmf(int k) const { return cdf[(size_t)k - 1] - (k > 1 ? cdf[(size_t)k - 2] : 0.0); }
};

inline int64_t clamp64(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Scale s so that E[clamp(round(s z), lo, hi)] is as close as possible to mean.
double zipf_scale(const Zipf& z, int lo, int hi, double mean) {
  auto expect = [&](double s) {
    double e = 0;
    for (int k = 1; k <= (int)z.cdf.size(); ++k)
      e += z.pmf(k) * (double)clamp64(std::llround(s * k), lo, hi);
    return e;
  };
  double a = 1e-6, b = (double)hi;
  for (int it = 0; it < 200; ++it) {
    double c = 0.5 * (a + b);
    if (expect(c) < mean)
      a = c;
    else
      b = c;
  }
  return 0.5 * (a + b);
}

int64_t column_nnz(const acdc_lasso_gen* g, const Zipf* zipf, double zscale, int64_t j) {
  int64_t k;
  switch (g->nnz_mode) {
    case ACDC_NNZ_ZIPF: {
      int z = zipf->draw(rnd_u01(g->seed, (uint64_t)j, ACDC_STREAM_GEN_NNZ, 0));
      k = clamp64(std::llround(zscale * z), g->nnz_min > 0 ? g->nnz_min : 1, g->nnz_max);
      break;
    }
    case ACDC_NNZ_UNIFORM: {
      int64_t span = (int64_t)g->nnz_max - g->nnz_min + 1;
      k = g->nnz_min + (int64_t)rnd_below(g->seed, (uint64_t)j, ACDC_STREAM_GEN_NNZ, 0, (uint64_t)span);
      break;
    }
    default:
      k = g->nnz_per_col;
  }
  if (k > g->m) k = g->m;
  if (k < 0) k = 0;
  return k;
}

int check_lasso(const acdc_lasso_gen* g) {
  if (!g || g->m <= 0 || g->n <= 0 || g->m > INT32_MAX) return ACDC_EINVAL;
  if (g->nnz_mode == ACDC_NNZ_ZIPF && (g->nnz_max < 1 || g->zipf_s <= 1.0 || g->nnz_mean <= 0))
    return ACDC_EINVAL;
  if (g->nnz_mode == ACDC_NNZ_UNIFORM && (g->nnz_min < 0 || g->nnz_max < g->nnz_min))
    return ACDC_EINVAL;
  if (g->nnz_mode == ACDC_NNZ_FIXED && g->nnz_per_col < 0) return ACDC_EINVAL;
  if (g->n_star < 0 || g->n_star > g->n) return ACDC_EINVAL;
  return ACDC_OK;
}

}  // namespace

extern "C" int acdc_gen_lasso_colptr(const acdc_lasso_gen* g, int64_t* col_ptr) {
  int rc = check_lasso(g);
  if (rc) return rc;
  if (!col_ptr) return ACDC_EINVAL;
  set_threads(g->threads);
  Zipf* zipf = nullptr;
  double zscale = 1.0;
  if (g->nnz_mode == ACDC_NNZ_ZIPF) {
    zipf = new Zipf(g->zipf_s, g->nnz_max);
    zscale = zipf_scale(*zipf, g->nnz_min > 0 ? g->nnz_min : 1, g->nnz_max, g->nnz_mean);
  }
  const int64_t n = g->n;
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < n; ++j) col_ptr[j + 1] = column_nnz(g, zipf, zscale, j);
  delete zipf;
  col_ptr[0] = 0;
  for (int64_t j = 0; j < n; ++j) col_ptr[j + 1] += col_ptr[j];
  return ACDC_OK;
}

extern "C" int acdc_gen_lasso_fill(const acdc_lasso_gen* g, const int64_t* col_ptr,
                                   int32_t* row_idx, double* vals, double* b, double* x_star,
                                   double* lambda_out) {
  int rc = check_lasso(g);
  if (rc) return rc;
  if (!col_ptr || !row_idx || !vals || !b) return ACDC_EINVAL;
  set_threads(g->threads);
  const int64_t m = g->m, n = g->n;
  const uint64_t seed = g->seed;
#pragma omp parallel
  {
    std::vector<int64_t> rows, table;
#pragma omp for schedule(dynamic, 256)
    for (int64_t j = 0; j < n; ++j) {
      const int64_t s = col_ptr[j], k = col_ptr[j + 1] - col_ptr[j];
      distinct_sorted(seed, (uint64_t)j, ACDC_STREAM_GEN_ROWS, k, m, rows, table);
      double nrm = 0;
      for (int64_t e = 0; e < k; ++e) {
        double v = rnd_normal(seed, (uint64_t)j, ACDC_STREAM_GEN_VALS, (uint32_t)e);
        row_idx[s + e] = (int32_t)rows[(size_t)e];
        vals[s + e] = v;
        nrm += v * v;
      }
      if (g->normalize_columns && nrm > 0) {
        double inv = 1.0 / std::sqrt(nrm);
        for (int64_t e = 0; e < k; ++e) vals[s + e] *= inv;
      }
    }
  }
  // x*: n_star distinct coordinates, signs +-1.
  std::vector<int64_t> support, table;
  distinct_sorted(seed, 0, ACDC_STREAM_GEN_XSTAR, g->n_star, n, support, table);
  if (x_star) std::memset(x_star, 0, sizeof(double) * (size_t)n);
  // b = A x* + noise, accumulated in support order (deterministic).
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m; ++i)
    b[i] = g->noise_sigma > 0 ? g->noise_sigma * rnd_normal(seed, (uint64_t)i, ACDC_STREAM_GEN_NOISE, 0) : 0.0;
  for (size_t t = 0; t < support.size(); ++t) {
    int64_t j = support[t];
    double xs = (acdc_rand64(seed, (uint64_t)j, ACDC_STREAM_GEN_XSTAR, 1u) >> 63) ? 1.0 : -1.0;
    if (x_star) x_star[j] = xs;
    for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) b[row_idx[e]] += vals[e] * xs;
  }
  // lambda = frac * ||A^T b||_inf
  double amax = 0;
#pragma omp parallel for schedule(static) reduction(max : amax)
  for (int64_t j = 0; j < n; ++j) {
    double d = 0;
    for (int64_t e = col_ptr[j]; e < col_ptr[j + 1]; ++e) d += vals[e] * b[row_idx[e]];
    d = std::fabs(d);
    if (d > amax) amax = d;
  }
  if (lambda_out) *lambda_out = g->lambda_frac * amax;
  return ACDC_OK;
}

namespace {
int64_t sample_nnz(const acdc_svm_gen* g, int64_t i) {
  double z = rnd_normal(g->seed, (uint64_t)i, ACDC_STREAM_GEN_NNZ, 0);
  double v = std::exp(std::log(g->nnz_median) + g->nnz_sigma * z);
  return clamp64(std::llround(v), 1, g->d);
}
int check_svm(const acdc_svm_gen* g) {
  if (!g || g->n_samples <= 0 || g->d <= 0 || g->d > INT32_MAX || g->nnz_median < 1 ||
      g->nnz_sigma < 0 || g->w_star_nnz < 0 || g->w_star_nnz > g->d || g->flip_prob < 0 ||
      g->flip_prob > 1)
    return ACDC_EINVAL;
  return ACDC_OK;
}
}  // namespace

extern "C" int acdc_gen_svm_rowptr(const acdc_svm_gen* g, int64_t* row_ptr) {
  int rc = check_svm(g);
  if (rc) return rc;
  if (!row_ptr) return ACDC_EINVAL;
  set_threads(g->threads);
  const int64_t n = g->n_samples;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) row_ptr[i + 1] = sample_nnz(g, i);
  row_ptr[0] = 0;
  for (int64_t i = 0; i < n; ++i) row_ptr[i + 1] += row_ptr[i];
  return ACDC_OK;
}

extern "C" int acdc_gen_svm_fill(const acdc_svm_gen* g, const int64_t* row_ptr, int32_t* col_idx,
                                 double* vals, double* y) {
  int rc = check_svm(g);
  if (rc) return rc;
  if (!row_ptr || !col_idx || !vals || !y) return ACDC_EINVAL;
  set_threads(g->threads);
  const int64_t n = g->n_samples, d = g->d;
  const uint64_t seed = g->seed;
  // w*: w_star_nnz N(0,1) entries at distinct features.
  std::vector<int64_t> wsup, table0;
  distinct_sorted(seed, 0, ACDC_STREAM_GEN_XSTAR, g->w_star_nnz, d, wsup, table0);
  std::vector<double> wstar((size_t)d, 0.0);
  for (size_t t = 0; t < wsup.size(); ++t)
    wstar[(size_t)wsup[t]] = rnd_normal(seed, (uint64_t)wsup[t], ACDC_STREAM_GEN_XSTAR, 1u);
#pragma omp parallel
  {
    std::vector<int64_t> feats, table;
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
      const int64_t s = row_ptr[i], k = row_ptr[i + 1] - row_ptr[i];
      distinct_sorted(seed, (uint64_t)i, ACDC_STREAM_GEN_ROWS, k, d, feats, table);
      double nrm = 0;
      for (int64_t e = 0; e < k; ++e) {
        double v = -std::log(rnd_u01(seed, (uint64_t)i, ACDC_STREAM_GEN_VALS, (uint32_t)e));
        col_idx[s + e] = (int32_t)feats[(size_t)e];
        vals[s + e] = v;
        nrm += v * v;
      }
      double inv = nrm > 0 ? 1.0 / std::sqrt(nrm) : 0.0;
      double dot = 0;
      for (int64_t e = 0; e < k; ++e) {
        vals[s + e] *= inv;
        dot += vals[s + e] * wstar[(size_t)col_idx[s + e]];
      }
      double label = dot >= 0 ? 1.0 : -1.0;
      if (rnd_u01(seed, (uint64_t)i, ACDC_STREAM_GEN_LABEL, 0) <= g->flip_prob) label = -label;
      y[i] = label;
    }
  }
  return ACDC_OK;
}

extern "C" int acdc_gen_nesterov(int64_t m, int64_t n, int32_t p, int64_t n_nonzero,
                                 double lambda, double rho, uint64_t seed, int64_t* col_ptr,
                                 int32_t* row_idx, double* vals, double* b, double* x_star,
                                 double* f_star) {
  if (m <= 0 || n <= 0 || p <= 0 || p > m || n_nonzero < 0 || n_nonzero > n || lambda <= 0 ||
      !col_ptr || !row_idx || !vals || !b || !x_star)
    return ACDC_EINVAL;
  // A: p uniform(-1,1) entries per column at distinct rows.
  std::vector<int64_t> rows, table;
  for (int64_t j = 0; j <= n; ++j) col_ptr[j] = j * p;
  for (int64_t j = 0; j < n; ++j) {
    distinct_sorted(seed, (uint64_t)j, ACDC_STREAM_GEN_ROWS, p, m, rows, table);
    for (int e = 0; e < p; ++e) {
      row_idx[j * p + e] = (int32_t)rows[(size_t)e];
      vals[j * p + e] = 2.0 * rnd_u01(seed, (uint64_t)j, ACDC_STREAM_GEN_VALS, (uint32_t)e) - 1.0;
    }
  }
  // y*: random direction, unit norm.
  std::vector<double> y((size_t)m);
  double ny = 0;
  for (int64_t i = 0; i < m; ++i) {
    y[(size_t)i] = rnd_normal(seed, (uint64_t)i, ACDC_STREAM_GEN_NOISE, 0);
    ny += y[(size_t)i] * y[(size_t)i];
  }
  ny = std::sqrt(ny);
  for (auto& v : y) v /= ny;
  // c_j = a_j^T y*; the n_nonzero largest |c_j| form the support.
  std::vector<double> c((size_t)n);
  for (int64_t j = 0; j < n; ++j) {
    double d = 0;
    for (int e = 0; e < p; ++e) d += vals[j * p + e] * y[(size_t)row_idx[j * p + e]];
    c[(size_t)j] = d;
  }
  std::vector<int64_t> order((size_t)n);
  for (int64_t j = 0; j < n; ++j) order[(size_t)j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t bb) {
    return std::fabs(c[(size_t)a]) > std::fabs(c[(size_t)bb]);
  });
  std::vector<char> in_support((size_t)n, 0);
  for (int64_t t = 0; t < n_nonzero; ++t) in_support[(size_t)order[(size_t)t]] = 1;
  double l1 = 0;
  for (int64_t j = 0; j < n; ++j) {
    double cj = c[(size_t)j];
    double alpha;
    x_star[j] = 0;
    if (cj == 0.0) {
      alpha = 1.0;  // column orthogonal to y*: optimal at zero for any scale
    } else if (in_support[(size_t)j]) {
      alpha = lambda / std::fabs(cj);
      double mag = rho * rnd_u01(seed, (uint64_t)j, ACDC_STREAM_GEN_XSTAR, 0);
      x_star[j] = cj > 0 ? mag : -mag;
      l1 += mag;
    } else {
      // |alpha c_j| <= 0.9 lambda keeps the support strict.
      alpha = 0.9 * lambda * rnd_u01(seed, (uint64_t)j, ACDC_STREAM_GEN_XSTAR, 2u) / std::fabs(cj);
    }
    for (int e = 0; e < p; ++e) vals[j * p + e] *= alpha;
  }
  // b = y* + A x*
  for (int64_t i = 0; i < m; ++i) b[i] = y[(size_t)i];
  for (int64_t j = 0; j < n; ++j)
    if (x_star[j] != 0)
      for (int e = 0; e < p; ++e) b[row_idx[j * p + e]] += vals[j * p + e] * x_star[j];
  if (f_star) *f_star = 0.5 + lambda * l1;  // 0.5 ||y*||^2 with ||y*|| = 1
  return ACDC_OK;
}

extern "C" int acdc_gen_mix_sizes(uint64_t seed, int64_t index, int64_t m_lo, int64_t m_hi,
                                  int64_t n_lo, int64_t n_hi, int64_t* m_out, int64_t* n_out) {
  if (m_lo <= 0 || m_hi < m_lo || n_lo <= 0 || n_hi < n_lo || !m_out || !n_out) return ACDC_EINVAL;
  double um = rnd_u01(seed, (uint64_t)index, ACDC_STREAM_GEN_SIZE, 0);
  double un = rnd_u01(seed, (uint64_t)index, ACDC_STREAM_GEN_SIZE, 1);
  *m_out = clamp64(std::llround(std::exp(std::log((double)m_lo) + um * std::log((double)m_hi / m_lo))), m_lo, m_hi);
  *n_out = clamp64(std::llround(std::exp(std::log((double)n_lo) + un * std::log((double)n_hi / n_lo))), n_lo, n_hi);
  return ACDC_OK;
}

extern "C" int acdc_host_omega(int64_t m, int64_t n, const int64_t* col_ptr,
                               const int32_t* row_idx, int64_t* omega_out) {
  if (m <= 0 || n < 0 || !col_ptr || !omega_out || (col_ptr[n] > 0 && !row_idx)) return ACDC_EINVAL;
  std::vector<int64_t> cnt((size_t)m, 0);
  const int64_t nnz = col_ptr[n];
  for (int64_t e = 0; e < nnz; ++e) {
    int32_t r = row_idx[e];
    if (r < 0 || r >= m) return ACDC_EINVAL;
    cnt[(size_t)r]++;
  }
  int64_t w = 0;
  for (auto v : cnt) w = v > w ? v : w;
  *omega_out = w;
  return ACDC_OK;
}

extern "C" void acdc_philox4x32_10_host(const uint32_t ctr[4], const uint32_t key[2],
                                        uint32_t out[4]) {
  acdc_u32x4 o = acdc_philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = o.v[i];
}

extern "C" uint64_t acdc_sample_coordinate(uint64_t seed, uint64_t k, uint64_t n) {
  return acdc_sample_coord(seed, k, n);
}

// On-disk formats of the reference's path, read on the host.
//
//  * Text CSC triple <prefix>_values.txt / _colPtr.txt / _rowIdx.txt plus a
//    vector file: InputOuputHelper::loadCSCData
//    (cpp/src/utils/file_reader.h:108-137), each file a whitespace-separated
//    list read by loadVectorData (:32-48).  One deliberate difference: the
//    reference drops a final value that has no trailing whitespace (its
//    read-then-test-eof loop); this reader keeps it.
//  * Binary per-rank CSC: loadANSCIAndBinaryData
//    (cpp/src/utils/file_reader.h:50-106): <prefix>_colptr_<rank><suffix> holds
//    local_n + 1 whitespace-separated column offsets, <prefix>_rowid_<rank><suffix>
//    the row indices as raw int32 and <prefix>_values_<rank><suffix> the values
//    as raw doubles (native byte order); b comes from a text vector file.
//  * LIBSVM text: loadDistributedSparseSVMRowData
//    (cpp/src/utils/distributed_instances_loader.h:68-193) with sizes from
//    parse_LIB_SVM_data_get_size (cpp/src/svm/svm_parser.h:11-77): one sample
//    per line, "label index:value ...", 1-based indices made 0-based, label 0
//    mapped to -1.
//
// Every reader refuses a value that is not finite (nan, inf, or out of double
// range), in the matrix as in the vector, with ACDC_EINVAL.
//
// The text formats are parsed by several host threads: the file is cut into
// pieces just after a separator (whitespace for number lists, a newline for
// LIBSVM), each piece is scanned on its own thread, and the pieces' counts are
// prefix-summed so that every thread writes its own part of the output.  The
// result does not depend on the number of threads.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/acdc_gpu.h"
#include "../../include/acdc_host.h"

namespace {

std::atomic<int> g_threads{0};

// Pieces a text of len bytes is cut into: the fixed count if one was set,
// else one per MiB of text up to the hardware threads.
int pieces_for(size_t len) {
  const int set = g_threads.load();
  if (set > 0) return set;
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t by_size = len / ((size_t)1 << 20) + 1;
  return (int)std::max<size_t>(1, std::min<size_t>(hw ? hw : 1, by_size));
}

bool is_space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t'; }
bool is_newline(char c) { return c == '\n'; }

// Decimal number at p with strtod's result and end pointer.  Plain decimals
// ([+-]digits[.digits][(e|E)[+-]digits]) of at most 19 significant digits whose
// digits fit a 53-bit integer w and whose decimal exponent e lies in [-22, 22]
// are converted as w * 10^e or w / 10^-e: w and 10^|e| are exact doubles, so the
// one rounded operation gives the correctly rounded value (Clinger, "How to
// read floating point numbers accurately", PLDI 1990), which is what strtod
// returns.  Every other token (more digits, larger exponents, hex, inf, nan, a
// letter right after the number) goes to strtod itself.  end bounds the fast
// path only; strtod, like before, reads the NUL-terminated text.
const char* parse_double(const char* p, const char* end, double* out) {
  static const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,
                                    1e8,  1e9,  1e10, 1e11, 1e12, 1e13, 1e14, 1e15,
                                    1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
  const char* q = p;
  bool neg = false;
  if (q < end && (*q == '+' || *q == '-')) neg = *q++ == '-';
  uint64_t w = 0;
  int sig = 0, digits = 0, frac = 0;
  for (; q < end && *q >= '0' && *q <= '9'; ++q, ++digits)
    if (sig || *q != '0') {
      if (++sig > 19) goto slow;
      w = w * 10 + (uint64_t)(*q - '0');
    }
  if (q < end && *q == '.') {
    for (++q; q < end && *q >= '0' && *q <= '9'; ++q, ++digits, ++frac)
      if (sig || *q != '0') {
        if (++sig > 19) goto slow;
        w = w * 10 + (uint64_t)(*q - '0');
      }
  }
  if (digits == 0) goto slow;
  {
    int e = 0;
    if (q < end && (*q == 'e' || *q == 'E')) {
      const char* t = q + 1;
      bool eneg = false;
      if (t < end && (*t == '+' || *t == '-')) eneg = *t++ == '-';
      if (!(t < end && *t >= '0' && *t <= '9')) goto slow;
      for (; t < end && *t >= '0' && *t <= '9'; ++t)
        if ((e = e * 10 + (*t - '0')) > 1000) goto slow;
      if (eneg) e = -e;
      q = t;
    }
    if (q < end && (*q == '.' || ((*q | 0x20) >= 'a' && (*q | 0x20) <= 'z'))) goto slow;
    e -= frac;
    if (w > ((uint64_t)1 << 53) || e < -22 || e > 22) goto slow;
    double v = (double)w;
    v = e >= 0 ? v * kPow10[e] : v / kPow10[-e];
    *out = neg ? -v : v;
    return q;
  }
slow:
  char* r = nullptr;
  *out = std::strtod(p, &r);
  return r;
}

// Cuts [0, len) into k ranges whose inner boundaries sit just after a
// separator, so that no token (or line) is split; ranges may be empty.
std::vector<size_t> cut_after(const std::string& text, int k, bool (*sep)(char)) {
  std::vector<size_t> b((size_t)k + 1, text.size());
  b[0] = 0;
  for (int i = 1; i < k; ++i) {
    size_t p = std::max(b[(size_t)i - 1], text.size() / (size_t)k * (size_t)i);
    while (p < text.size() && !sep(text[p])) ++p;
    b[(size_t)i] = p < text.size() ? p + 1 : text.size();
  }
  return b;
}

// Runs fn(i) for i in [0, k) on k threads (the calling thread takes i = 0).
template <typename F>
void run_pieces(int k, F fn) {
  std::vector<std::thread> th;
  th.reserve((size_t)k);
  for (int i = 1; i < k; ++i) th.emplace_back(fn, i);
  fn(0);
  for (auto& t : th) t.join();
}

bool read_file(const std::string& path, std::string& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long len = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (len < 0) {
    std::fclose(f);
    return false;
  }
  out.resize((size_t)len);
  size_t got = len > 0 ? std::fread(&out[0], 1, (size_t)len, f) : 0;
  std::fclose(f);
  return got == (size_t)len;
}

// Numbers of [p, end), a range that ends just after whitespace or at the end
// of the text; false on a bad token.
template <typename T>
bool parse_range(const char* p, const char* end, std::vector<T>& out) {
  while (p < end) {
    while (p < end && is_space(*p)) ++p;
    if (p >= end) break;
    errno = 0;
    double v = 0;
    const char* q = parse_double(p, end, &v);
    if (q == p || q > end || errno == ERANGE || !std::isfinite(v)) return false;
    out.push_back((T)v);
    p = q;
  }
  return true;
}

// Parses every number of a whitespace-separated file; false on a bad token.
template <typename T>
bool parse_numbers(const std::string& text, std::vector<T>& out) {
  out.clear();
  const int k = pieces_for(text.size());
  const std::vector<size_t> b = cut_after(text, k, is_space);
  std::vector<std::vector<T>> part((size_t)k);
  std::vector<char> ok((size_t)k, 0);
  const char* base = text.c_str();
  run_pieces(k, [&](int i) {
    ok[(size_t)i] = parse_range(base + b[(size_t)i], base + b[(size_t)i + 1], part[(size_t)i]);
  });
  size_t total = 0;
  for (int i = 0; i < k; ++i) {
    if (!ok[(size_t)i]) return false;
    total += part[(size_t)i].size();
  }
  out.reserve(total);
  for (auto& v : part) out.insert(out.end(), v.begin(), v.end());
  return true;
}

struct CscText {
  std::vector<double> vals, b;
  std::vector<int64_t> col_ptr;
  std::vector<int64_t> rows;
};

int read_csc_text(const char* prefix, const char* vector_file, CscText& t) {
  if (!prefix || !vector_file) return ACDC_EINVAL;
  std::string pre(prefix), s;
  if (!read_file(vector_file, s) || !parse_numbers(s, t.b)) return ACDC_EINVAL;
  if (!read_file(pre + "_values.txt", s) || !parse_numbers(s, t.vals)) return ACDC_EINVAL;
  if (!read_file(pre + "_colPtr.txt", s) || !parse_numbers(s, t.col_ptr)) return ACDC_EINVAL;
  if (!read_file(pre + "_rowIdx.txt", s) || !parse_numbers(s, t.rows)) return ACDC_EINVAL;
  if (t.col_ptr.size() < 1 || t.col_ptr[0] != 0) return ACDC_EINVAL;
  const int64_t n = (int64_t)t.col_ptr.size() - 1;
  const int64_t nnz = t.col_ptr[(size_t)n];
  if ((int64_t)t.vals.size() != nnz || (int64_t)t.rows.size() != nnz) return ACDC_EINVAL;
  for (int64_t j = 0; j < n; ++j)
    if (t.col_ptr[(size_t)j + 1] < t.col_ptr[(size_t)j]) return ACDC_EINVAL;
  const int64_t m = (int64_t)t.b.size();
  for (int64_t r : t.rows)
    if (r < 0 || r >= m) return ACDC_EINVAL;
  return ACDC_OK;
}

struct CscBinary {
  std::vector<int64_t> col_ptr;
  std::vector<double> b;
  std::string rowid, values;
};

long file_size(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return -1;
  std::fseek(f, 0, SEEK_END);
  long len = std::ftell(f);
  std::fclose(f);
  return len;
}

// Column offsets, b and the paths of the two binary files, with their sizes checked.
int read_csc_binary_head(const char* prefix, const char* suffix, int32_t rank,
                         const char* vector_file, int64_t local_n, CscBinary& t) {
  if (!prefix || !vector_file || local_n < 0) return ACDC_EINVAL;
  const std::string pre(prefix), suf(suffix ? suffix : ""), rk = std::to_string(rank);
  std::string s;
  if (!read_file(vector_file, s) || !parse_numbers(s, t.b)) return ACDC_EINVAL;
  std::vector<int64_t> ptr;
  if (!read_file(pre + "_colptr_" + rk + suf, s) || !parse_numbers(s, ptr)) return ACDC_EINVAL;
  if ((int64_t)ptr.size() < local_n + 1 || ptr[0] != 0) return ACDC_EINVAL;
  t.col_ptr.assign(ptr.begin(), ptr.begin() + local_n + 1);
  for (int64_t j = 0; j < local_n; ++j)
    if (t.col_ptr[(size_t)j + 1] < t.col_ptr[(size_t)j]) return ACDC_EINVAL;
  const int64_t nnz = t.col_ptr[(size_t)local_n];
  t.rowid = pre + "_rowid_" + rk + suf;
  t.values = pre + "_values_" + rk + suf;
  if (file_size(t.rowid) < (long)(nnz * (int64_t)sizeof(int32_t)) ||
      file_size(t.values) < (long)(nnz * (int64_t)sizeof(double)))
    return ACDC_EINVAL;
  return ACDC_OK;
}

bool read_raw(const std::string& path, void* dst, size_t bytes) {
  if (bytes == 0) return true;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  const size_t got = std::fread(dst, 1, bytes, f);
  std::fclose(f);
  return got == bytes;
}

struct LibsvmScan {
  int64_t n = 0, d = 0, nnz = 0;
};

// Walks the lines of [p, end) (a range of whole lines); when out pointers are
// given also fills them, sample n0 + i and entry nnz0 + e of the range at
// index i and e.
int walk_libsvm(const char* p, const char* end, LibsvmScan& sc, int64_t n0, int64_t nnz0,
                int64_t* row_ptr, int32_t* col_idx, double* vals, double* y) {
  int64_t n = 0, nnz = 0, d = 0;
  while (p < end) {
    const char* eol = (const char*)std::memchr(p, '\n', (size_t)(end - p));
    if (!eol) eol = end;
    const char* q = p;
    while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
    if (q < eol && *q != '#') {
      char* r = nullptr;
      double label = 0;
      const char* lq = parse_double(q, eol, &label);
      if (lq == q || lq > eol || !std::isfinite(label)) return ACDC_EINVAL;
      r = const_cast<char*>(lq);
      q = r;
      if (row_ptr) {
        row_ptr[n0 + n] = nnz0 + nnz;
        y[n0 + n] = label == 0 ? -1.0 : label;
      }
      for (;;) {
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q >= eol) break;
        long long idx = std::strtoll(q, &r, 10);
        if (r == q || r >= eol || *r != ':' || idx < 1) return ACDC_EINVAL;
        q = r + 1;
        // the value follows the colon directly (strtod would skip a line end)
        if (q >= eol || *q == ' ' || *q == '\t' || *q == '\r') return ACDC_EINVAL;
        double v = 0;
        const char* vq = parse_double(q, eol, &v);
        if (vq == q || vq > eol || !std::isfinite(v)) return ACDC_EINVAL;
        q = vq;
        if (idx > d) d = idx;
        if (idx - 1 > INT32_MAX) return ACDC_EINVAL;
        if (col_idx) {
          col_idx[nnz0 + nnz] = (int32_t)(idx - 1);
          vals[nnz0 + nnz] = v;
        }
        ++nnz;
      }
      ++n;
    }
    p = eol + 1;
  }
  sc.n = n;
  sc.d = d;
  sc.nnz = nnz;
  return ACDC_OK;
}

}  // namespace

extern "C" int acdc_load_csc_text_sizes(const char* prefix, const char* vector_file, int64_t* m,
                                        int64_t* n, int64_t* nnz) {
  if (!m || !n || !nnz) return ACDC_EINVAL;
  CscText t;
  int rc = read_csc_text(prefix, vector_file, t);
  if (rc) return rc;
  *m = (int64_t)t.b.size();
  *n = (int64_t)t.col_ptr.size() - 1;
  *nnz = (int64_t)t.vals.size();
  return ACDC_OK;
}

extern "C" int acdc_load_csc_text(const char* prefix, const char* vector_file, int64_t* col_ptr,
                                  int32_t* row_idx, double* vals, double* b) {
  if (!col_ptr || !b) return ACDC_EINVAL;
  CscText t;
  int rc = read_csc_text(prefix, vector_file, t);
  if (rc) return rc;
  if (!t.vals.empty() && (!row_idx || !vals)) return ACDC_EINVAL;
  std::memcpy(col_ptr, t.col_ptr.data(), sizeof(int64_t) * t.col_ptr.size());
  for (size_t e = 0; e < t.rows.size(); ++e) row_idx[e] = (int32_t)t.rows[e];
  if (!t.vals.empty()) std::memcpy(vals, t.vals.data(), sizeof(double) * t.vals.size());
  std::memcpy(b, t.b.data(), sizeof(double) * t.b.size());
  return ACDC_OK;
}

extern "C" int acdc_load_csc_binary_sizes(const char* prefix, const char* suffix, int32_t rank,
                                          const char* vector_file, int64_t local_n, int64_t* m,
                                          int64_t* n, int64_t* nnz) {
  if (!m || !n || !nnz) return ACDC_EINVAL;
  CscBinary t;
  int rc = read_csc_binary_head(prefix, suffix, rank, vector_file, local_n, t);
  if (rc) return rc;
  *m = (int64_t)t.b.size();
  *n = local_n;
  *nnz = t.col_ptr[(size_t)local_n];
  return ACDC_OK;
}

extern "C" int acdc_load_csc_binary(const char* prefix, const char* suffix, int32_t rank,
                                    const char* vector_file, int64_t local_n, int64_t* col_ptr,
                                    int32_t* row_idx, double* vals, double* b) {
  if (!col_ptr || !b) return ACDC_EINVAL;
  CscBinary t;
  int rc = read_csc_binary_head(prefix, suffix, rank, vector_file, local_n, t);
  if (rc) return rc;
  const int64_t nnz = t.col_ptr[(size_t)local_n];
  if (nnz > 0 && (!row_idx || !vals)) return ACDC_EINVAL;
  if (!read_raw(t.rowid, row_idx, sizeof(int32_t) * (size_t)nnz) ||
      !read_raw(t.values, vals, sizeof(double) * (size_t)nnz))
    return ACDC_EINVAL;
  const int64_t m = (int64_t)t.b.size();
  for (int64_t e = 0; e < nnz; ++e)
    if (row_idx[e] < 0 || row_idx[e] >= m || !std::isfinite(vals[e])) return ACDC_EINVAL;
  std::memcpy(col_ptr, t.col_ptr.data(), sizeof(int64_t) * t.col_ptr.size());
  std::memcpy(b, t.b.data(), sizeof(double) * t.b.size());
  return ACDC_OK;
}

namespace {

// LIBSVM in pieces of whole lines: per-piece sizes, then (when row_ptr is
// given) each piece fills its samples and entries at the prefix sums.
int scan_libsvm(const std::string& text, LibsvmScan& total, int64_t* row_ptr, int32_t* col_idx,
                double* vals, double* y) {
  const int k = pieces_for(text.size());
  const std::vector<size_t> b = cut_after(text, k, is_newline);
  const char* base = text.c_str();
  std::vector<LibsvmScan> sc((size_t)k);
  std::vector<int> rc((size_t)k, ACDC_OK);
  run_pieces(k, [&](int i) {
    rc[(size_t)i] = walk_libsvm(base + b[(size_t)i], base + b[(size_t)i + 1], sc[(size_t)i], 0, 0,
                                nullptr, nullptr, nullptr, nullptr);
  });
  std::vector<int64_t> n0((size_t)k + 1, 0), z0((size_t)k + 1, 0);
  total = LibsvmScan();
  for (int i = 0; i < k; ++i) {
    if (rc[(size_t)i]) return rc[(size_t)i];
    n0[(size_t)i + 1] = n0[(size_t)i] + sc[(size_t)i].n;
    z0[(size_t)i + 1] = z0[(size_t)i] + sc[(size_t)i].nnz;
    total.d = std::max(total.d, sc[(size_t)i].d);
  }
  total.n = n0[(size_t)k];
  total.nnz = z0[(size_t)k];
  if (!row_ptr) return ACDC_OK;
  if (total.nnz > 0 && (!col_idx || !vals)) return ACDC_EINVAL;
  run_pieces(k, [&](int i) {
    LibsvmScan again;
    rc[(size_t)i] = walk_libsvm(base + b[(size_t)i], base + b[(size_t)i + 1], again, n0[(size_t)i],
                                z0[(size_t)i], row_ptr, col_idx, vals, y);
  });
  for (int i = 0; i < k; ++i)
    if (rc[(size_t)i]) return rc[(size_t)i];
  row_ptr[total.n] = total.nnz;
  return ACDC_OK;
}

}  // namespace

extern "C" int acdc_host_threads(int32_t threads) {
  return g_threads.exchange(threads > 0 ? threads : 0);
}

extern "C" int acdc_save_csc_binary(const char* prefix, const char* suffix, int32_t rank,
                                    int64_t n, const int64_t* col_ptr, const int32_t* row_idx,
                                    const double* vals) {
  if (!prefix || n < 0 || !col_ptr || col_ptr[0] != 0) return ACDC_EINVAL;
  for (int64_t j = 0; j < n; ++j)
    if (col_ptr[j + 1] < col_ptr[j]) return ACDC_EINVAL;
  const int64_t nnz = col_ptr[n];
  if (nnz > 0 && (!row_idx || !vals)) return ACDC_EINVAL;
  const std::string pre(prefix), suf(suffix ? suffix : ""), rk = std::to_string(rank);
  FILE* f = std::fopen((pre + "_colptr_" + rk + suf).c_str(), "wb");
  if (!f) return ACDC_EINVAL;
  bool ok = true;
  for (int64_t j = 0; j <= n && ok; ++j) ok = std::fprintf(f, "%lld\n", (long long)col_ptr[j]) > 0;
  ok = (std::fclose(f) == 0) && ok;
  auto raw = [&](const std::string& path, const void* src, size_t bytes) {
    FILE* g = std::fopen(path.c_str(), "wb");
    if (!g) return false;
    const bool w = bytes == 0 || std::fwrite(src, 1, bytes, g) == bytes;
    return (std::fclose(g) == 0) && w;
  };
  ok = ok && raw(pre + "_rowid_" + rk + suf, row_idx, sizeof(int32_t) * (size_t)nnz);
  ok = ok && raw(pre + "_values_" + rk + suf, vals, sizeof(double) * (size_t)nnz);
  return ok ? ACDC_OK : ACDC_EINVAL;
}

extern "C" int acdc_load_libsvm_sizes(const char* path, int64_t* n_samples, int64_t* d,
                                      int64_t* nnz) {
  if (!path || !n_samples || !d || !nnz) return ACDC_EINVAL;
  std::string text;
  if (!read_file(path, text)) return ACDC_EINVAL;
  LibsvmScan sc;
  int rc = scan_libsvm(text, sc, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  *n_samples = sc.n;
  *d = sc.d;
  *nnz = sc.nnz;
  return ACDC_OK;
}

extern "C" int acdc_load_libsvm(const char* path, int64_t* row_ptr, int32_t* col_idx, double* vals,
                                double* y) {
  if (!path || !row_ptr || !y) return ACDC_EINVAL;
  std::string text;
  if (!read_file(path, text)) return ACDC_EINVAL;
  LibsvmScan sc;
  return scan_libsvm(text, sc, row_ptr, col_idx, vals, y);
}

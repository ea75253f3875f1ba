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
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/acdc_gpu.h"
#include "../../include/acdc_host.h"

namespace {

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

// Parses every number of a whitespace-separated file; false on a bad token.
template <typename T>
bool parse_numbers(const std::string& text, std::vector<T>& out) {
  out.clear();
  const char* p = text.c_str();
  const char* end = p + text.size();
  while (p < end) {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    if (p >= end) break;
    char* q = nullptr;
    errno = 0;
    double v = std::strtod(p, &q);
    if (q == p || errno == ERANGE) return false;
    out.push_back((T)v);
    p = q;
  }
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

// Walks the file; when out pointers are given also fills them.
int walk_libsvm(const std::string& text, LibsvmScan& sc, int64_t* row_ptr, int32_t* col_idx,
                double* vals, double* y) {
  const char* p = text.c_str();
  const char* end = p + text.size();
  int64_t n = 0, nnz = 0, d = 0;
  while (p < end) {
    const char* eol = (const char*)std::memchr(p, '\n', (size_t)(end - p));
    if (!eol) eol = end;
    const char* q = p;
    while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
    if (q < eol && *q != '#') {
      char* r = nullptr;
      double label = std::strtod(q, &r);
      if (r == q) return ACDC_EINVAL;
      q = r;
      if (row_ptr) {
        row_ptr[n] = nnz;
        y[n] = label == 0 ? -1.0 : label;
      }
      for (;;) {
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q >= eol) break;
        long long idx = std::strtoll(q, &r, 10);
        if (r == q || r >= eol || *r != ':' || idx < 1) return ACDC_EINVAL;
        q = r + 1;
        double v = std::strtod(q, &r);
        if (r == q) return ACDC_EINVAL;
        q = r;
        if (idx > d) d = idx;
        if (col_idx) {
          if (idx - 1 > INT32_MAX) return ACDC_EINVAL;
          col_idx[nnz] = (int32_t)(idx - 1);
          vals[nnz] = v;
        }
        ++nnz;
      }
      ++n;
    }
    p = eol + 1;
  }
  if (row_ptr) row_ptr[n] = nnz;
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
    if (row_idx[e] < 0 || row_idx[e] >= m) return ACDC_EINVAL;
  std::memcpy(col_ptr, t.col_ptr.data(), sizeof(int64_t) * t.col_ptr.size());
  std::memcpy(b, t.b.data(), sizeof(double) * t.b.size());
  return ACDC_OK;
}

extern "C" int acdc_load_libsvm_sizes(const char* path, int64_t* n_samples, int64_t* d,
                                      int64_t* nnz) {
  if (!path || !n_samples || !d || !nnz) return ACDC_EINVAL;
  std::string text;
  if (!read_file(path, text)) return ACDC_EINVAL;
  LibsvmScan sc;
  int rc = walk_libsvm(text, sc, nullptr, nullptr, nullptr, nullptr);
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
  int rc = walk_libsvm(text, sc, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  if (sc.nnz > 0 && (!col_idx || !vals)) return ACDC_EINVAL;
  return walk_libsvm(text, sc, row_ptr, col_idx, vals, y);
}

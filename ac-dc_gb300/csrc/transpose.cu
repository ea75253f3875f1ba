// Rows -> columns on the device: a matrix given in compressed-row form (m rows,
// n columns) becomes the compressed-column staging arrays that the layout pass
// reads, with the entries of every column in increasing row order.  This is the
// conversion the reference makes on the host for the logistic loss
// (getCSR_from_CSC, cpp/src/helpers/matrix_conversions.h:65-104, called at
// cpp/src/frontends/solvers/MultiCoreSolver.cpp:89-93 on the LIBSVM rows).
//
// Method: a least-significant-digit radix sort of the entries by column index
// (8-bit digits, as many passes as the column count needs).  Each pass is
// stable: tiles of 4096 entries count their digits, one exclusive scan over
// (digit, tile) gives every tile its output positions, and a tile scatters its
// entries in order, ranking equal digits within a warp with __match_any_sync
// and across the block's warps through shared-memory counts.  The input is in
// row order, so after the last pass the entries of each column stay in row
// order.  The column pointers come from per-column counts and a scan.
#include "acdc_internal.cuh"

namespace {

constexpr int kSortThreads = 256;   // = number of digit values
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kTileEntries = 4096;
constexpr int kScanThreadsT = 512;
constexpr int kScanItemsT = 8;
constexpr int kScanTileT = kScanThreadsT * kScanItemsT;

__device__ int64_t block_scan_excl(int64_t v, int64_t* smem, int64_t* total) {
  const int t = threadIdx.x;
  smem[t] = v;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    const int64_t a = t >= off ? smem[t - off] : 0;
    __syncthreads();
    smem[t] += a;
    __syncthreads();
  }
  const int64_t incl = smem[t];
  *total = smem[blockDim.x - 1];
  __syncthreads();
  return incl - v;
}

// Exclusive scan of in[0..len) into out[0..len] (out[len] = total), three passes.
template <typename T>
__global__ void k_tscan_tiles(const T* in, int64_t len, int64_t* tile_sums) {
  __shared__ int64_t smem[kScanThreadsT];
  const int64_t base = (int64_t)blockIdx.x * kScanTileT + (int64_t)threadIdx.x * kScanItemsT;
  int64_t s = 0;
  for (int i = 0; i < kScanItemsT; ++i)
    if (base + i < len) s += (int64_t)in[base + i];
  int64_t total;
  block_scan_excl(s, smem, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void k_tscan_offsets(int64_t* tile_sums, int64_t tiles) {
  __shared__ int64_t smem[kScanThreadsT];
  int64_t carry = 0;
  for (int64_t base = 0; base < tiles; base += kScanThreadsT) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < tiles ? tile_sums[i] : 0;
    int64_t total;
    const int64_t ex = block_scan_excl(v, smem, &total);
    if (i < tiles) tile_sums[i] = carry + ex;
    carry += total;
  }
}

template <typename T>
__global__ void k_tscan_apply(const T* in, int64_t len, const int64_t* tile_offsets,
                              int64_t* out) {
  __shared__ int64_t smem[kScanThreadsT];
  const int64_t base = (int64_t)blockIdx.x * kScanTileT + (int64_t)threadIdx.x * kScanItemsT;
  int64_t s = 0;
  for (int i = 0; i < kScanItemsT; ++i)
    if (base + i < len) s += (int64_t)in[base + i];
  int64_t total;
  int64_t ex = block_scan_excl(s, smem, &total) + tile_offsets[blockIdx.x];
  for (int i = 0; i < kScanItemsT; ++i) {
    const int64_t j = base + i;
    if (j < len) {
      out[j] = ex;
      ex += (int64_t)in[j];
    }
    if (j == len - 1) out[len] = ex;
  }
}

template <typename T>
cudaError_t scan_exclusive(const T* in, int64_t len, int64_t* out, int64_t* tile_sums,
                           cudaStream_t st) {
  if (len <= 0) return cudaMemsetAsync(out, 0, sizeof(int64_t), st);
  const int64_t tiles = (len + kScanTileT - 1) / kScanTileT;
  k_tscan_tiles<T><<<(unsigned)tiles, kScanThreadsT, 0, st>>>(in, len, tile_sums);
  k_tscan_offsets<<<1, kScanThreadsT, 0, st>>>(tile_sums, tiles);
  k_tscan_apply<T><<<(unsigned)tiles, kScanThreadsT, 0, st>>>(in, len, tile_sums, out);
  return cudaGetLastError();
}

// One warp per row: the row index of every entry, the column counts, and the
// check of the column indices (an index outside [0, n) is flagged and sorted as
// column 0 so that no access leaves the arrays).
__global__ void k_rows_expand(const int64_t* __restrict__ row_ptr, int64_t m, int32_t* col,
                              int64_t n, int32_t* __restrict__ rows_of, int32_t* __restrict__ cnt,
                              unsigned long long* status) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < m; i += warps) {
    const int64_t b = row_ptr[i], e = row_ptr[i + 1];
    for (int64_t k = b + lane; k < e; k += 32) {
      int32_t c = col[k];
      if (c < 0 || (int64_t)c >= n) {
        atomicOr(status, (unsigned long long)DEV_ERR_BAD_INDEX);
        c = 0;
        col[k] = 0;
      }
      rows_of[k] = (int32_t)i;
      atomicAdd(cnt + c, 1);
    }
  }
}

__global__ void k_radix_hist(const int32_t* __restrict__ keys, int64_t nnz, int shift,
                             uint32_t* __restrict__ hist, int64_t tiles) {
  __shared__ uint32_t h[kSortThreads];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTileEntries;
  const int64_t end = min(base + kTileEntries, nnz);
  for (int64_t e = base + threadIdx.x; e < end; e += kSortThreads)
    atomicAdd(&h[(keys[e] >> shift) & 255], 1u);
  __syncthreads();
  hist[(int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile (see the file comment).  keys_out may be null on
// the last pass.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(
    const int32_t* __restrict__ keys_in, const int32_t* __restrict__ rows_in,
    const double* __restrict__ vals_in, int64_t nnz, int shift, const int64_t* __restrict__ offsets,
    int64_t tiles, int32_t* __restrict__ keys_out, int32_t* __restrict__ rows_out,
    double* __restrict__ vals_out) {
  __shared__ int64_t base_d[kSortThreads];
  __shared__ uint32_t wcnt[kSortWarps][kSortThreads];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  base_d[t] = offsets[(int64_t)t * tiles + blockIdx.x];
  const int64_t begin = (int64_t)blockIdx.x * kTileEntries;
  const int64_t end = min(begin + kTileEntries, nnz);
  for (int64_t c = begin; c < end; c += kSortThreads) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const int64_t e = c + t;
    const bool valid = e < end;
    const int32_t key = valid ? keys_in[e] : 0;
    const int d = valid ? ((key >> shift) & 255) : 256 + lane;  // invalid lanes match no one
    const unsigned peers = __match_any_sync(ACDC_FULL_MASK, d);
    const unsigned rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    if (valid) {
      int64_t pos = base_d[d] + rank;
      for (int w = 0; w < warp; ++w) pos += wcnt[w][d];
      if (keys_out) keys_out[pos] = key;
      rows_out[pos] = rows_in[e];
      vals_out[pos] = vals_in[e];
    }
    __syncthreads();
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) tot += wcnt[w][t];
    base_d[t] += tot;
    __syncthreads();
  }
}

}  // namespace

namespace {
size_t carve_size(size_t bytes) { return (bytes + 255) & ~(size_t)255; }
int64_t scan_tiles_for(int64_t len) { return (std::max<int64_t>(len, 1) + kScanTileT - 1) / kScanTileT; }
}  // namespace

// The carve of launch_rows_to_columns, piece by piece.
int64_t rows_to_columns_scratch_bytes(int64_t m, int64_t n, int64_t nnz) {
  (void)m;
  const int64_t tiles = (nnz + kTileEntries - 1) / kTileEntries;
  const int64_t scan_tiles = std::max(scan_tiles_for(n), scan_tiles_for(256 * tiles));
  size_t b = 0;
  b += 3 * carve_size(sizeof(int32_t) * (size_t)nnz);          // rows_of, keys_b, rows_b
  b += carve_size(sizeof(double) * (size_t)nnz);               // vals_b
  b += carve_size(sizeof(uint32_t) * 256 * (size_t)tiles);     // digit counts
  b += carve_size(sizeof(int64_t) * (256 * (size_t)tiles + 1));  // their offsets
  b += carve_size(sizeof(int32_t) * (size_t)n);                // column counts
  b += sizeof(int64_t) * (size_t)scan_tiles;                   // scan tile sums
  return (int64_t)b;
}

cudaError_t launch_rows_to_columns(const int64_t* row_ptr, int32_t* col, double* val, int64_t m,
                                   int64_t n, int64_t nnz, char* scratch, int64_t* col_ptr,
                                   int32_t* rows_out, double* vals_out,
                                   unsigned long long* status, cudaStream_t st) {
  const int64_t tiles = (nnz + kTileEntries - 1) / kTileEntries;
  auto carve = [&](size_t bytes) {
    char* p = scratch;
    scratch += carve_size(bytes);
    return p;
  };
  int32_t* rows_of = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)nnz));
  int32_t* keys_b = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)nnz));
  int32_t* rows_b = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)nnz));
  double* vals_b = reinterpret_cast<double*>(carve(sizeof(double) * (size_t)nnz));
  uint32_t* hist = reinterpret_cast<uint32_t*>(carve(sizeof(uint32_t) * 256 * (size_t)tiles));
  int64_t* offs = reinterpret_cast<int64_t*>(carve(sizeof(int64_t) * (256 * (size_t)tiles + 1)));
  int32_t* cnt = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)n));
  int64_t* tsum = reinterpret_cast<int64_t*>(scratch);

  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)n, st);
  if (e != cudaSuccess) return e;
  if (m > 0) {
    const int64_t blocks = std::min<int64_t>((m + 7) / 8, 152 * 16);
    k_rows_expand<<<(unsigned)blocks, 256, 0, st>>>(row_ptr, m, col, n, rows_of, cnt, status);
  }
  e = scan_exclusive<int32_t>(cnt, n, col_ptr, tsum, st);
  if (e != cudaSuccess || nnz == 0) return e;

  int bits = 1;
  while (bits < 31 && ((int64_t)1 << bits) < n) ++bits;
  const int passes = (bits + 7) / 8;
  const int32_t* kin = col;
  const int32_t* rin = rows_of;
  const double* vin = val;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = 8 * pass;
    const bool last = pass == passes - 1;
    // even passes read the input set and write set b; odd ones the reverse
    int32_t* kout = last ? nullptr : (pass % 2 == 0 ? keys_b : col);
    int32_t* rout = last ? rows_out : (pass % 2 == 0 ? rows_b : rows_of);
    double* vout = last ? vals_out : (pass % 2 == 0 ? vals_b : val);
    k_radix_hist<<<(unsigned)tiles, kSortThreads, 0, st>>>(kin, nnz, shift, hist, tiles);
    e = scan_exclusive<uint32_t>(hist, 256 * tiles, offs, tsum, st);
    if (e != cudaSuccess) return e;
    k_radix_scatter<<<(unsigned)tiles, kSortThreads, 0, st>>>(kin, rin, vin, nnz, shift, offs,
                                                              tiles, kout, rout, vout);
    kin = kout;
    rin = rout;
    vin = vout;
  }
  return cudaGetLastError();
}

// Layout build, Lipschitz constants, FP64 residual refresh and FP64
// objective / duality-gap kernels (sm_103a).
//
// Refresh: MulticoreSquareLoss::recomputeResiduals
// (cpp/src/solver/lossFunctions/squareLoss/MulticoreSquareLoss.h:42-53) and
// MulticoreSVMDualLoss::recomputeResiduals (MulticoreSVMDualLoss.h:31-46),
// scattering only coordinates that are nonzero, in FP64.
// Objective: MulticoreL1RegSquareLoss::computeObjectiveValue
// (MulticoreL1RegSquareLoss.h:30-39) plus the Lasso dual point
// u = s r, s = min(1, lambda/||A^T r||_inf); MulticoreSVMDualLoss::computeObjectiveValue
// (MulticoreSVMDualLoss.h:63-117).  Every reduction runs on a fixed grid of
// ACDC_RED_BLOCKS blocks whose partials one block then adds in index order.
#include <algorithm>

#include "acdc_internal.cuh"

namespace {

constexpr int kScanItems = 8;
constexpr int kScanThreads = 512;
constexpr int kScanTile = kScanItems * kScanThreads;

__device__ __forceinline__ int64_t padded_units(const int64_t* col_ptr, int64_t j) {
  const int64_t len = col_ptr[j + 1] - col_ptr[j];
  return len > 0 ? (len + 3) >> 2 : 0;
}

// Block-wide exclusive scan of int64 values held kScanItems per thread.
__device__ int64_t block_exclusive_scan(int64_t v, int64_t* smem, int64_t* total) {
  const int t = threadIdx.x;
  smem[t] = v;
  __syncthreads();
  for (int off = 1; off < blockDim.x; off <<= 1) {
    int64_t a = t >= off ? smem[t - off] : 0;
    __syncthreads();
    smem[t] += a;
    __syncthreads();
  }
  int64_t incl = smem[t];
  *total = smem[blockDim.x - 1];
  __syncthreads();
  return incl - v;
}

// Pass 1: per-tile totals of padded column lengths (units of 4 entries); also
// flags decreasing column pointers.
__global__ void k_scan_tiles(const int64_t* col_ptr, int64_t n, int64_t* tile_sums,
                             unsigned long long* counters) {
  __shared__ int64_t smem[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    int64_t j = base + i;
    if (j < n) {
      if (col_ptr[j + 1] < col_ptr[j]) atomicOr(counters + CNT_STATUS, (unsigned long long)DEV_ERR_BAD_LAYOUT);
      s += padded_units(col_ptr, j);
    }
  }
  int64_t total;
  block_exclusive_scan(s, smem, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// Pass 2: exclusive scan of the tile totals (one block, sequential over chunks).
__global__ void k_scan_offsets(int64_t* tile_sums, int64_t tiles, int64_t* grand_total) {
  __shared__ int64_t smem[kScanThreads];
  int64_t carry = 0;
  for (int64_t base = 0; base < tiles; base += kScanThreads) {
    int64_t i = base + threadIdx.x;
    int64_t v = i < tiles ? tile_sums[i] : 0;
    int64_t total;
    int64_t ex = block_exclusive_scan(v, smem, &total);
    if (i < tiles) tile_sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *grand_total = carry;
}

// Pass 3: start4[j] = exclusive prefix of padded units.
__global__ void k_scan_apply(const int64_t* col_ptr, int64_t n, const int64_t* tile_offsets,
                             int64_t* start4) {
  __shared__ int64_t smem[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    int64_t j = base + i;
    if (j < n) s += padded_units(col_ptr, j);
  }
  int64_t total;
  int64_t ex = block_exclusive_scan(s, smem, &total) + tile_offsets[blockIdx.x];
  for (int i = 0; i < kScanItems; ++i) {
    int64_t j = base + i;
    if (j < n) {
      start4[j] = ex;
      ex += padded_units(col_ptr, j);
    }
  }
}

// One warp per column: copy FP64 values to FP32 and indices into the padded
// segment, zero the pad, check indices, compute ||a_j||^2 in FP64 and write meta.
// For the logistic loss the stored value is b_i A_ij (the label folded in, so
// the update never loads b); ||a_j||^2 is taken from A itself.
__global__ void k_build_columns(const int64_t* col_ptr, const int32_t* row_idx,
                                const double* vals64, const int64_t* start4, int64_t m, int64_t n,
                                DevProblem d, int32_t loss) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < n; j += warps) {
    const int64_t s = col_ptr[j];
    const int64_t len = col_ptr[j + 1] - s;
    const int64_t dst = start4[j] << 2;
    const int64_t plen = len > 0 ? ((len + 3) >> 2) << 2 : 0;
    double sq = 0;
    for (int64_t e = lane; e < plen; e += 32) {
      float v = 0.f;
      int32_t r = 0;
      if (e < len) {
        double dv = vals64[s + e];
        r = row_idx[s + e];
        if (r < 0 || r >= m) {
          atomicOr(d.counters + CNT_STATUS, (unsigned long long)DEV_ERR_BAD_INDEX);
          r = 0;
          dv = 0;
        }
        v = (float)(loss == ACDC_LOSS_LOGISTIC ? d.rhs64[r] * dv : dv);
        sq += dv * dv;
      }
      d.vals[dst + e] = v;
      d.idx[dst + e] = r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(ACDC_FULL_MASK, sq, o);
    if (lane == 0) {
      d.col_sq[j] = sq;
      d.meta[j] = make_int4((int)(uint32_t)start4[j], (int)len, 0, 0);
    }
  }
}

__global__ void k_row_counts(const int32_t* idx, int64_t nnz, int32_t* counts, int64_t m) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
    int32_t r = idx[e];
    if (r >= 0 && r < m) atomicAdd(counts + r, 1);
  }
}

__global__ void k_max_i32(const int32_t* v, int64_t len, unsigned long long* out) {
  int32_t best = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
    best = max(best, v[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(ACDC_FULL_MASK, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)best);
}

// Li = 1/(beta ||a_j||^2) (0 for an empty column); the SVM stores y_j Li.
// Li of every column, and the largest ||a_j||^2 (CNT_COLSQ_BITS; non-negative
// doubles order like their bit patterns):
//   losses 0, 2: 1/(beta ||a_j||^2)              (0 for an empty column)
//   loss 1:      1/(lambda + beta ||a_j||^2)     (MulticoreL2SquareRegSquareLoss.h:30-43)
//   loss 3:      1/(beta (lambda + ||a_j||^2/4)) (MulticoreL2SquareRegLogisticLoss.h:30-44,
//                with the engine's sigma = beta)
__global__ void k_set_li(DevProblem d, int32_t loss, double beta, double lambda) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double sq_max = 0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < d.n; j += stride) {
    double sq = d.col_sq[j];
    sq_max = fmax(sq_max, sq);
    double li;
    if (loss == ACDC_LOSS_L2_SQUARE)
      li = 1.0 / (lambda + beta * sq);
    else if (loss == ACDC_LOSS_LOGISTIC)
      li = 1.0 / (beta * (lambda + 0.25 * sq));
    else
      li = sq > 0 ? 1.0 / (beta * sq) : 0.0;
    if (loss == ACDC_LOSS_SVM_DUAL && d.rhs64[j] < 0) li = -li;
    d.meta[j].z = __float_as_int((float)li);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sq_max = fmax(sq_max, __shfl_xor_sync(ACDC_FULL_MASK, sq_max, o));
  if ((threadIdx.x & 31) == 0 && sq_max > 0)
    atomicMax(d.counters + CNT_COLSQ_BITS, (unsigned long long)__double_as_longlong(sq_max));
}

__global__ void k_widen_i32(const int32_t* src, int64_t* dst, int64_t len) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
    dst[i] = (int64_t)src[i];
}

// xbuf (FP64, caller order) -> x32 and, in polish mode, x64.
__global__ void k_set_x(DevProblem d, int fp64) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < d.n; j += stride) {
    const double v = d.xbuf[j];
    d.x32[j] = (float)v;
    if (fp64) d.x64[j] = v;
  }
}

__global__ void k_get_x(DevProblem d, int fp64) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < d.n; j += stride)
    d.xbuf[j] = fp64 ? __ldcg(d.x64 + j) : (double)__ldcg(d.x32 + j);
}

__global__ void k_x32_to_x64(DevProblem d) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < d.n; j += stride)
    d.x64[j] = (double)d.x32[j];
}

__global__ void k_x64_to_x32(DevProblem d) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < d.n; j += stride)
    d.x32[j] = (float)d.x64[j];
}

// Coordinate j as the evaluation sees it: FP64 in polish mode, else FP32.
__device__ __forceinline__ double coord(const EvalParams& p, int64_t j) {
  return p.x64 ? p.x64[j] : (double)p.x32[j];
}

// ---- refresh ----

// r64 = -b (losses 0 and 1) or 0 (losses 2 and 3).
__device__ __forceinline__ void k_refresh_init_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  const int64_t stride = (int64_t)nb * blockDim.x;
  for (int64_t i = (int64_t)rank * blockDim.x + threadIdx.x; i < p.m; i += stride)
    p.r64[i] = p.loss == ACDC_LOSS_L1_SQUARE || p.loss == ACDC_LOSS_L2_SQUARE ? -p.rhs64[i] : 0.0;
}

__global__ void k_refresh_init(EvalParams p) { k_refresh_init_body(p, blockIdx.x, gridDim.x); }

// Each warp reads 32 consecutive coordinates, then scatters the nonzero ones
// cooperatively: r64 += coef_j a_j with coef = x_j (Lasso) or
// alpha_j y_j / (lambda n) after clipping alpha_j into [0, 1] (SVM).  The
// Lasso pass also sums |x_j| and the support (slots 2 and 4).
__device__ __forceinline__ void k_refresh_scatter_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  __shared__ double s_l1[ACDC_RED_THREADS / 32], s_sp[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)nb * blockDim.x) >> 5;
  const double inv_ln = 1.0 / (p.lambda * (double)p.n);
  double l1 = 0, sp = 0;
  for (int64_t base = (((int64_t)rank * blockDim.x + threadIdx.x) >> 5) * 32; base < p.n;
       base += warps * 32) {
    const int64_t j = base + lane;
    double coef = 0;
    if (j < p.n) {
      const double xv = coord(p, j);
      if (p.loss == ACDC_LOSS_SVM_DUAL) {
        const double c = xv > 1.0 ? 1.0 : (xv < 0.0 ? 0.0 : xv);
        if (c != xv) {
          if (p.x64)
            p.x64[j] = c;
          else
            p.x32[j] = (float)c;
        }
        if (c != 0.0) coef = c * p.rhs64[j] * inv_ln;
      } else {
        // the logistic residual is r = -(b A) x with b folded into the values
        coef = p.loss == ACDC_LOSS_LOGISTIC ? -xv : xv;
        l1 += p.loss == ACDC_LOSS_L1_SQUARE ? fabs(xv) : xv * xv;
        sp += xv != 0.0 ? 1.0 : 0.0;
      }
    }
    // Columns of the nonzero coordinates, one at a time by the whole warp.  The
    // records of the live lanes are loaded together first; each column's
    // entries are loaded four 32-entry groups at a time before their atomics.
    unsigned live = __ballot_sync(ACDC_FULL_MASK, coef != 0.0);
    if (!live) continue;
    int2 sl = make_int2(0, 0);
    if (coef != 0.0) sl = *reinterpret_cast<const int2*>(p.meta + j);
    while (live) {
      const int src = __ffs(live) - 1;
      live &= live - 1;
      const double cj = __shfl_sync(ACDC_FULL_MASK, coef, src);
      const int64_t start = (int64_t)(uint32_t)__shfl_sync(ACDC_FULL_MASK, sl.x, src) << 2;
      const int32_t len = __shfl_sync(ACDC_FULL_MASK, sl.y, src);
      for (int32_t e0 = lane; e0 < len; e0 += 128) {
        int32_t row[4];
        float val[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int32_t e = e0 + 32 * k;
          row[k] = e < len ? p.idx[start + e] : -1;
          val[k] = e < len ? p.vals[start + e] : 0.f;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (row[k] >= 0) atomicAdd(p.r64 + row[k], cj * (double)val[k]);
      }
    }
  }
  if (p.loss == ACDC_LOSS_SVM_DUAL) return;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    l1 += __shfl_down_sync(ACDC_FULL_MASK, l1, o);
    sp += __shfl_down_sync(ACDC_FULL_MASK, sp, o);
  }
  if (lane == 0) {
    s_l1[threadIdx.x >> 5] = l1;
    s_sp[threadIdx.x >> 5] = sp;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t0 += s_l1[w];
      t1 += s_sp[w];
    }
    p.part[rank * ACDC_NPART + 2] = t0;
    p.part[rank * ACDC_NPART + 4] = t1;
  }
}

__global__ void k_refresh_scatter(EvalParams p) { k_refresh_scatter_body(p, blockIdx.x, gridDim.x); }

// r32 = (float) r64 and the partial sums sum r^2 (slot 0), sum b r (slot 1).
// With r_ref: a screened evaluation adds sum (r - r_ref)^2 (slot 6); a full one
// stores r64 into r_ref.  The logistic loss sums log(1 + exp(r)) (slot 0), the
// dual entropy terms (slot 1) and the rows with r < 0 (slot 6) instead.
__device__ __forceinline__ void k_refresh_finish_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  __shared__ double s0[ACDC_RED_THREADS / 32], s1[ACDC_RED_THREADS / 32],
      s2[ACDC_RED_THREADS / 32];
  double a0 = 0, a1 = 0, a2 = 0;
  const int64_t stride = (int64_t)nb * blockDim.x;
  for (int64_t i = (int64_t)rank * blockDim.x + threadIdx.x; i < p.m; i += stride) {
    double v = p.r64[i];
    p.r32[i] = (float)v;
    if (p.loss == ACDC_LOSS_LOGISTIC) {
      // sum log(1 + exp(r)), sum of a log a + (1-a) log(1-a) at a = sigma(r),
      // count of r < 0 (the training accuracy), and sigma(r) for the column pass
      a0 += v > 0.0 ? v + log1p(exp(-v)) : log1p(exp(v));
      const double a = v >= 0.0 ? 1.0 / (1.0 + exp(-v)) : exp(v) / (1.0 + exp(v));
      a1 += (a > 0.0 ? a * log(a) : 0.0) + (a < 1.0 ? (1.0 - a) * log1p(-a) : 0.0);
      a2 += v < 0.0 ? 1.0 : 0.0;
      p.roww[i] = a;
      continue;
    }
    a0 += v * v;
    if (p.loss == ACDC_LOSS_L1_SQUARE) a1 += p.rhs64[i] * v;
    if (p.r_ref) {
      if (p.screened) {
        const double dv = v - p.r_ref[i];
        a2 += dv * dv;
      } else {
        p.r_ref[i] = v;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_down_sync(ACDC_FULL_MASK, a0, o);
    a1 += __shfl_down_sync(ACDC_FULL_MASK, a1, o);
    a2 += __shfl_down_sync(ACDC_FULL_MASK, a2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s0[threadIdx.x >> 5] = a0;
    s1[threadIdx.x >> 5] = a1;
    s2[threadIdx.x >> 5] = a2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t0 += s0[w];
      t1 += s1[w];
      t2 += s2[w];
    }
    p.part[rank * ACDC_NPART + 0] = t0;
    p.part[rank * ACDC_NPART + 1] = t1;
    p.part[rank * ACDC_NPART + 6] = t2;
  }
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_refresh_finish(EvalParams p) { k_refresh_finish_body(p, blockIdx.x, gridDim.x); }

// ---- gap ----

// Lasso gap, pass 1 (segment-parallel): a warp takes 32 consecutive columns.
// Every column contributes |x_j| and the support count (slots 2 and 4).  The
// padded entries of the columns with at most kShortLen entries are contiguous,
// so the warp streams them as 4-entry units (one 128-bit load of values and one
// of row indices per lane, coalesced), gathers r, and adds each column's units
// with a segmented warp scan in a fixed order; these columns contribute
// |a_j^T r| (slot 3) and may join the active set.  Longer columns are listed in
// long_cols and handled by pass 2.
constexpr int kShortLen = 32;
constexpr int kShortUnits = kShortLen / 4;

struct ShortWarp {
  double colsum[32];
  uint32_t ustart[32];  // first unit of each column in the padded arrays
  int32_t uexcl[32];    // first unit of each column in the warp's unit stream
  uint8_t owner[32 * kShortUnits];
};

__device__ __forceinline__ void append_active(const EvalParams& p, bool join, int64_t j,
                                              int lane) {
  // One counter increment per warp for its joining columns.
  const unsigned joiners = __ballot_sync(ACDC_FULL_MASK, join);
  if (!joiners) return;
  const int leader = __ffs(joiners) - 1;
  unsigned long long first = 0;
  if (lane == leader) first = atomicAdd(p.counters + CNT_ACTIVE, (unsigned long long)__popc(joiners));
  first = __shfl_sync(ACDC_FULL_MASK, first, leader);
  if (join) {
    const unsigned long long pos = first + __popc(joiners & ((1u << lane) - 1u));
    if (pos < (unsigned long long)p.n) p.active[pos] = (int32_t)j;
  }
}

__device__ __forceinline__ void k_gap_lasso_short_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  __shared__ double s_gm[ACDC_RED_THREADS / 32], s_go[ACDC_RED_THREADS / 32];
  __shared__ ShortWarp sw_all[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  ShortWarp& sw = sw_all[threadIdx.x >> 5];
  const int64_t stride = (int64_t)nb * blockDim.x;  // a multiple of 32
  double gmax = 0, gout = 0;
  for (int64_t base = (int64_t)rank * blockDim.x + (threadIdx.x & ~31); base < p.n;
       base += stride) {
    const int64_t j = base + lane;
    const bool valid = j < p.n;
    int4 mt = make_int4(0, 0, 0, 0);
    if (valid) mt = p.meta[j];
    const double xv = valid ? coord(p, j) : 0.0;
    const bool is_short = valid && mt.y <= kShortLen;
    const int units = is_short ? (mt.y + 3) >> 2 : 0;
    // Exclusive scan of the unit counts over the 32 columns.
    int incl = units;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(ACDC_FULL_MASK, incl, o);
      if (lane >= o) incl += t;
    }
    const int excl = incl - units;
    const int total = __shfl_sync(ACDC_FULL_MASK, incl, 31);
    sw.colsum[lane] = 0.0;
    sw.ustart[lane] = (uint32_t)mt.x;
    sw.uexcl[lane] = excl;
    for (int u = 0; u < units; ++u) sw.owner[excl + u] = (uint8_t)lane;
    __syncwarp();
    for (int cb = 0; cb < total; cb += 32) {
      const int u = cb + lane;
      const bool live = u < total;
      const int own = live ? sw.owner[u] : 31;
      double v = 0.0;
      if (live) {
        const uint64_t e = ((uint64_t)sw.ustart[own] + (uint64_t)(u - sw.uexcl[own])) << 2;
        const float4 a = __ldcs(reinterpret_cast<const float4*>(p.vals + e));
        const int4 id = __ldcs(reinterpret_cast<const int4*>(p.idx + e));
        if (a.x != 0.f) v += (double)a.x * p.r64[id.x];
        if (a.y != 0.f) v += (double)a.y * p.r64[id.y];
        if (a.z != 0.f) v += (double)a.z * p.r64[id.z];
        if (a.w != 0.f) v += (double)a.w * p.r64[id.w];
      }
      // Segmented inclusive scan: lanes of one column are contiguous.
      const int prev_own = __shfl_up_sync(ACDC_FULL_MASK, own, 1);
      const bool head = lane == 0 || prev_own != own;
      const unsigned heads = __ballot_sync(ACDC_FULL_MASK, head);
      const int seg0 = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(ACDC_FULL_MASK, v, o);
        if (lane - o >= seg0) v += t;
      }
      const int next_own = __shfl_down_sync(ACDC_FULL_MASK, own, 1);
      const bool tail = live && (lane == 31 || u + 1 >= total || next_own != own);
      if (tail) sw.colsum[own] += v;  // one tail per column per chunk
      __syncwarp();
    }
    const double ag = fabs(sw.colsum[lane]);
    if (is_short) gmax = fmax(gmax, ag);
    const bool join = p.active && is_short && (xv != 0.0 || ag > p.shrink_thresh);
    if (p.active && is_short && !join) gout = fmax(gout, ag);
    append_active(p, join, j, lane);
    __syncwarp();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gmax = fmax(gmax, __shfl_down_sync(ACDC_FULL_MASK, gmax, o));
    gout = fmax(gout, __shfl_down_sync(ACDC_FULL_MASK, gout, o));
  }
  if (lane == 0) {
    s_gm[threadIdx.x >> 5] = gmax;
    s_go[threadIdx.x >> 5] = gout;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0, t3 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t1 = fmax(t1, s_gm[w]);
      t3 = fmax(t3, s_go[w]);
    }
    p.part[rank * ACDC_NPART + 3] = t1;
    p.part[rank * ACDC_NPART + 7] = t3;
  }
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_gap_lasso_short(EvalParams p) { k_gap_lasso_short_body(p, blockIdx.x, gridDim.x); }

// Lasso gap, pass 2: one warp per long column (slot 5: max |a_j^T r|).  The
// metadata of the warp's next column is loaded while the current one is summed,
// and each 128-entry chunk is loaded before the previous chunk's gathers.
__device__ __forceinline__ void k_gap_lasso_long_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  __shared__ double s_gm[ACDC_RED_THREADS / 32], s_go[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)nb * blockDim.x) >> 5;
  double gmax = 0, gout = 0;
  int64_t t = ((int64_t)rank * blockDim.x + threadIdx.x) >> 5;
  auto first_chunk = [&](const int4& m, float4& v, int4& id) {
    const int32_t off = 4 * lane;
    if (off < m.y) {
      const int64_t s = ((int64_t)(uint32_t)m.x << 2) + off;
      v = __ldcs(reinterpret_cast<const float4*>(p.vals + s));
      id = __ldcs(reinterpret_cast<const int4*>(p.idx + s));
    } else {
      v = make_float4(0.f, 0.f, 0.f, 0.f);
      id = make_int4(0, 0, 0, 0);
    }
  };
  // Two-deep pipeline: the first chunk of the next column and the record of
  // the column after it are in flight while the current column is summed.
  int64_t j = t < p.n_long ? p.long_cols[t] : 0;
  int4 mt = t < p.n_long ? p.meta[j] : make_int4(0, 0, 0, 0);
  float4 v0;
  int4 id0;
  first_chunk(mt, v0, id0);
  int64_t jn = t + warps < p.n_long ? p.long_cols[t + warps] : 0;
  int4 mtn = t + warps < p.n_long ? p.meta[jn] : make_int4(0, 0, 0, 0);
  for (; t < p.n_long; t += warps) {
    float4 v1;
    int4 id1;
    first_chunk(mtn, v1, id1);
    const int64_t tnn = t + 2 * warps;
    const int64_t jnn = tnn < p.n_long ? p.long_cols[tnn] : 0;
    const int4 mtnn = tnn < p.n_long ? p.meta[jnn] : make_int4(0, 0, 0, 0);
    const int64_t start = (int64_t)(uint32_t)mt.x << 2;
    const int32_t len = mt.y;
    double g = 0;
    int32_t off = 4 * lane;
    float4 v = v0;
    int4 id = id0;
    for (; off < len; off += 128) {
      float4 vn = make_float4(0.f, 0.f, 0.f, 0.f);
      int4 idn = make_int4(0, 0, 0, 0);
      if (off + 128 < len) {
        vn = __ldcs(reinterpret_cast<const float4*>(p.vals + start + off + 128));
        idn = __ldcs(reinterpret_cast<const int4*>(p.idx + start + off + 128));
      }
      g += (double)v.x * p.r64[id.x];
      g += (double)v.y * p.r64[id.y];
      g += (double)v.z * p.r64[id.z];
      g += (double)v.w * p.r64[id.w];
      v = vn;
      id = idn;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(ACDC_FULL_MASK, g, o);
    const double ag = fabs(g);
    gmax = fmax(gmax, ag);
    const double xv = coord(p, j);
    if (p.active) {
      if (xv != 0.0 || ag > p.shrink_thresh) {
        if (lane == 0) {
          const unsigned long long pos = atomicAdd(p.counters + CNT_ACTIVE, 1ull);
          if (pos < (unsigned long long)p.n) p.active[pos] = (int32_t)j;
        }
      } else {
        gout = fmax(gout, ag);
      }
    }
    j = jn;
    mt = mtn;
    v0 = v1;
    id0 = id1;
    jn = jnn;
    mtn = mtnn;
  }
  if (lane == 0) {
    s_gm[threadIdx.x >> 5] = gmax;
    s_go[threadIdx.x >> 5] = gout;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0, t2 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t1 = fmax(t1, s_gm[w]);
      t2 = fmax(t2, s_go[w]);
    }
    p.part[rank * ACDC_NPART + 5] = t1;
    p.part[rank * ACDC_NPART + 8] = t2;
  }
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_gap_lasso_long(EvalParams p) { k_gap_lasso_long_body(p, blockIdx.x, gridDim.x); }

// a_j^T vec for one column, one warp; every lane gets the sum.  The loads of
// four 128-entry chunks are issued before their gathers, so a long column costs
// a few memory latencies rather than one per chunk.
__device__ __forceinline__ double active_dot(const EvalParams& p, const int4 mt, int lane,
                                             const double* vec) {
  const int64_t start = (int64_t)(uint32_t)mt.x << 2;
  double g = 0;
  for (int32_t off = 4 * lane; off < mt.y; off += 512) {
    float4 v[4];
    int4 id[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int32_t e = off + 128 * k;
      if (e < mt.y) {
        v[k] = __ldcs(reinterpret_cast<const float4*>(p.vals + start + e));
        id[k] = __ldcs(reinterpret_cast<const int4*>(p.idx + start + e));
      } else {
        v[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        id[k] = make_int4(0, 0, 0, 0);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      g += (double)v[k].x * vec[id[k].x];
      g += (double)v[k].y * vec[id[k].y];
      g += (double)v[k].z * vec[id[k].z];
      g += (double)v[k].w * vec[id[k].w];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(ACDC_FULL_MASK, g, o);
  return g;
}

// KKT violation of coordinate j (value xv) with gradient g: |g + lambda sign(x_j)|
// when x_j != 0, else max(|g| - lambda, 0).
__device__ __forceinline__ double kkt_violation(const EvalParams& p, double xv, double g) {
  return xv != 0.0 ? fabs(g + (xv > 0.0 ? p.lambda : -p.lambda)) : fmax(fabs(g) - p.lambda, 0.0);
}

// Active columns of at most this many entries are summed by one lane alone.
constexpr int kLaneLen = 16;

// a_j^T vec by one lane over a short column (len <= kLaneLen, padded to 4): all
// entry loads first, then all gathers.
__device__ __forceinline__ double lane_dot(const EvalParams& p, const int4 mt,
                                           const double* vec) {
  const int64_t start = (int64_t)(uint32_t)mt.x << 2;
  float4 v[kLaneLen / 4];
  int4 id[kLaneLen / 4];
#pragma unroll
  for (int k = 0; k < kLaneLen / 4; ++k) {
    if (4 * k < mt.y) {
      v[k] = __ldcs(reinterpret_cast<const float4*>(p.vals + start + 4 * k));
      id[k] = __ldcs(reinterpret_cast<const int4*>(p.idx + start + 4 * k));
    } else {
      v[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      id[k] = make_int4(0, 0, 0, 0);
    }
  }
  double g = 0;
#pragma unroll
  for (int k = 0; k < kLaneLen / 4; ++k) {
    if (4 * k < mt.y) {
      g += (double)v[k].x * vec[id[k].x];
      g += (double)v[k].y * vec[id[k].y];
      g += (double)v[k].z * vec[id[k].z];
      g += (double)v[k].w * vec[id[k].w];
    }
  }
  return g;
}

// Pass over the active list, 32 columns per warp step.  The list holds the
// long columns together (the long gap pass appends them), so the entries are
// dealt out with a stride: in step k, lane l of warp w (of W) takes entry
// 32 W k + W l + w, and no warp is left with a run of long columns.  A lane
// sums a short column alone; the warp then sums the long ones together.  Every lane ends with g and x of its own column (valid = false
// past the end of the list).
struct ActiveCol {
  bool valid;
  int32_t j;
  int4 mt;
  double g;
  double xv;
};

__device__ __forceinline__ ActiveCol active_col(const EvalParams& p, int64_t t, int64_t cnt,
                                                int lane) {
  ActiveCol c;
  c.valid = t < cnt;
  c.j = c.valid ? p.active[t] : 0;
  c.mt = c.valid ? p.meta[c.j] : make_int4(0, 0, 0, 0);
  c.g = c.valid && c.mt.y <= kLaneLen ? lane_dot(p, c.mt, p.r64) : 0.0;
  unsigned longs = __ballot_sync(ACDC_FULL_MASK, c.valid && c.mt.y > kLaneLen);
  while (longs) {
    const int src = __ffs(longs) - 1;
    longs &= longs - 1;
    int4 m;
    m.x = __shfl_sync(ACDC_FULL_MASK, c.mt.x, src);
    m.y = __shfl_sync(ACDC_FULL_MASK, c.mt.y, src);
    m.z = m.w = 0;
    const double g = active_dot(p, m, lane, p.r64);
    if (lane == src) c.g = g;
  }
  c.xv = c.valid ? coord(p, c.j) : 0.0;
  return c;
}

// Screened Lasso gap: |a_j^T r| over the active list only (slot 3; the inactive
// columns are bounded in the finalize step, |x|_1 and the support come from the
// refresh pass), with the active columns' KKT violations (viol[], slot 9).
__device__ __forceinline__ void active_pass_body(const EvalParams& p, const int64_t rank,
                                                 const int64_t nb, bool gap_slots) {
  __shared__ double s_gm[ACDC_RED_THREADS / 32], s_vm[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  double gmax = 0, vmax = 0;
  const int64_t cnt = (int64_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
  const int64_t step = (int64_t)nb * blockDim.x;
  const int64_t nw = step >> 5, gw = ((int64_t)rank * blockDim.x + threadIdx.x) >> 5;
  for (int64_t base = 0; base < cnt; base += step) {
    const int64_t t = base + lane * nw + gw;
    const ActiveCol c = active_col(p, t, cnt, lane);
    if (c.valid) {
      gmax = fmax(gmax, fabs(c.g));
      if (p.viol) {
        const double v = kkt_violation(p, c.xv, c.g);
        p.viol[t] = (float)v;
        vmax = fmax(vmax, v);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gmax = fmax(gmax, __shfl_xor_sync(ACDC_FULL_MASK, gmax, o));
    vmax = fmax(vmax, __shfl_xor_sync(ACDC_FULL_MASK, vmax, o));
  }
  if (lane == 0) {
    s_gm[threadIdx.x >> 5] = gmax;
    s_vm[threadIdx.x >> 5] = vmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0, t2 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t1 = fmax(t1, s_gm[w]);
      t2 = fmax(t2, s_vm[w]);
    }
    double* q = p.part + rank * ACDC_NPART;
    if (gap_slots) {
      q[3] = t1;
      q[5] = 0;
      q[7] = 0;
      q[8] = 0;
    }
    q[9] = t2;
  }
}

__device__ __forceinline__ void k_gap_lasso_screened_body(const EvalParams& p, const int64_t rank,
                                                         const int64_t nb) {
  active_pass_body(p, rank, nb, true);
}

// KKT violations of the active columns after a full pass (slot 9, viol[]).
__global__ void __launch_bounds__(ACDC_RED_THREADS) k_active_viol(EvalParams p) {
  active_pass_body(p, blockIdx.x, gridDim.x, false);
}

// Hot set, pass 1: rows of the active columns whose violation exceeds
// hot_frac times the largest one (eval_out[12]) are flagged.
__global__ void k_hot_mark(EvalParams p) {
  const int lane = threadIdx.x & 31;
  const int64_t cnt = (int64_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
  const double vmax = p.eval_out[12];
  if (!(vmax > 0)) return;
  const float thresh = (float)(p.hot_frac * vmax);
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  const int64_t nw = step >> 5, gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int64_t base = 0; base < cnt; base += step) {
    const int64_t t = base + lane * nw + gw;
    unsigned hot = __ballot_sync(ACDC_FULL_MASK, t < cnt && p.viol[t] > thresh);
    while (hot) {
      const int src = __ffs(hot) - 1;
      hot &= hot - 1;
      const int4 mt = p.meta[p.active[base + src * nw + gw]];
      const int64_t start = (int64_t)(uint32_t)mt.x << 2;
      for (int32_t e = lane; e < mt.y; e += 32) p.row_flag[p.idx[start + e]] = 1;
    }
  }
}

// Hot set, pass 2: every active column with an entry in a flagged row joins the
// hot list; its rows are counted for the hot set's ESO parameter.  A lane checks
// a short column alone; the warp checks the long ones together.
__global__ void k_hot_collect(EvalParams p) {
  const int lane = threadIdx.x & 31;
  const int64_t cnt = (int64_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  const int64_t nw = step >> 5, gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int64_t base = 0; base < cnt; base += step) {
    const int64_t t = base + lane * nw + gw;
    const bool valid = t < cnt;
    const int32_t j = valid ? p.active[t] : 0;
    const int4 mt = valid ? p.meta[j] : make_int4(0, 0, 0, 0);
    const int64_t start = (int64_t)(uint32_t)mt.x << 2;
    bool touch = false;
    if (valid && mt.y <= kLaneLen) {
      int4 id[kLaneLen / 4];
#pragma unroll
      for (int k = 0; k < kLaneLen / 4; ++k)
        id[k] = 4 * k < mt.y ? __ldcs(reinterpret_cast<const int4*>(p.idx + start + 4 * k))
                             : make_int4(0, 0, 0, 0);
      // pad entries (index 0) sit past len: only the first len rows count
#pragma unroll
      for (int k = 0; k < kLaneLen / 4; ++k) {
        const int32_t e = 4 * k;
        touch |= e < mt.y && p.row_flag[id[k].x] != 0;
        touch |= e + 1 < mt.y && p.row_flag[id[k].y] != 0;
        touch |= e + 2 < mt.y && p.row_flag[id[k].z] != 0;
        touch |= e + 3 < mt.y && p.row_flag[id[k].w] != 0;
      }
    }
    unsigned longs = __ballot_sync(ACDC_FULL_MASK, valid && mt.y > kLaneLen);
    while (longs) {
      const int src = __ffs(longs) - 1;
      longs &= longs - 1;
      const int64_t s0 = (int64_t)(uint32_t)__shfl_sync(ACDC_FULL_MASK, mt.x, src) << 2;
      const int32_t len = __shfl_sync(ACDC_FULL_MASK, mt.y, src);
      bool any = false;
      for (int32_t e0 = lane; e0 < len && !any; e0 += 128) {
        int32_t row[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) row[k] = e0 + 32 * k < len ? p.idx[s0 + e0 + 32 * k] : -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) any |= row[k] >= 0 && p.row_flag[row[k]] != 0;
      }
      any = __any_sync(ACDC_FULL_MASK, any);
      if (lane == src) touch = any;
    }
    // Join: the list entry, then the rows of the column (short: by the lane;
    // long: by the warp).
    const unsigned joiners = __ballot_sync(ACDC_FULL_MASK, touch);
    if (!joiners) continue;
    const int leader = __ffs(joiners) - 1;
    unsigned long long first = 0;
    if (lane == leader) first = atomicAdd(p.counters + CNT_HOT, (unsigned long long)__popc(joiners));
    first = __shfl_sync(ACDC_FULL_MASK, first, leader);
    if (touch) {
      const unsigned long long pos = first + __popc(joiners & ((1u << lane) - 1u));
      if (pos < (unsigned long long)p.n) p.hot[pos] = j;
    }
    int32_t top = 0;
    if (touch && mt.y <= kLaneLen)
      for (int32_t e = 0; e < mt.y; ++e) top = max(top, atomicAdd(p.rowcnt + p.idx[start + e], 1) + 1);
    unsigned jl = joiners & __ballot_sync(ACDC_FULL_MASK, mt.y > kLaneLen);
    while (jl) {
      const int src = __ffs(jl) - 1;
      jl &= jl - 1;
      const int64_t s0 = (int64_t)(uint32_t)__shfl_sync(ACDC_FULL_MASK, mt.x, src) << 2;
      const int32_t len = __shfl_sync(ACDC_FULL_MASK, mt.y, src);
      for (int32_t e0 = lane; e0 < len; e0 += 128) {
        int32_t row[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) row[k] = e0 + 32 * k < len ? p.idx[s0 + e0 + 32 * k] : -1;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (row[k] >= 0) top = max(top, atomicAdd(p.rowcnt + row[k], 1) + 1);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(ACDC_FULL_MASK, top, o));
    if (lane == 0 && top > 0) atomicMax(p.counters + CNT_OMEGA_HOT, (unsigned long long)top);
  }
}

// Duality gap of losses 1 and 3, column pass (slot 3): sum_j q_j^2 with
//   loss 1: q_j = a_j^T r + lambda x_j         (gap = sum q^2 / (2 lambda))
//   loss 3: q_j = sum_i b_i A_ij sigma(r_i)    (dual term ||.||^2 / (2 lambda))
// over every column: a lane sums a short column alone, the warp the long ones.
__device__ __forceinline__ void k_gap_smooth_body(const EvalParams& p, const int64_t rank,
                                                  const int64_t nb) {
  __shared__ double s_q[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  const bool ridge = p.loss == ACDC_LOSS_L2_SQUARE;
  const double* vec = ridge ? p.r64 : p.roww;
  const int64_t step = (int64_t)nb * blockDim.x;
  double qq = 0;
  for (int64_t base = (int64_t)rank * blockDim.x + (threadIdx.x & ~31); base < p.n; base += step) {
    const int64_t j = base + lane;
    const bool valid = j < p.n;
    const int4 mt = valid ? p.meta[j] : make_int4(0, 0, 0, 0);
    double g = valid && mt.y <= kLaneLen ? lane_dot(p, mt, vec) : 0.0;
    unsigned longs = __ballot_sync(ACDC_FULL_MASK, valid && mt.y > kLaneLen);
    while (longs) {
      const int src = __ffs(longs) - 1;
      longs &= longs - 1;
      int4 m;
      m.x = __shfl_sync(ACDC_FULL_MASK, mt.x, src);
      m.y = __shfl_sync(ACDC_FULL_MASK, mt.y, src);
      m.z = m.w = 0;
      const double gl = active_dot(p, m, lane, vec);
      if (lane == src) g = gl;
    }
    if (valid) {
      if (ridge) g += p.lambda * coord(p, j);
      qq += g * g;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) qq += __shfl_down_sync(ACDC_FULL_MASK, qq, o);
  if (lane == 0) s_q[threadIdx.x >> 5] = qq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) t += s_q[w];
    p.part[rank * ACDC_NPART + 3] = t;
  }
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_gap_smooth(EvalParams p) {
  k_gap_smooth_body(p, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_gap_lasso_screened(EvalParams p) {
  k_gap_lasso_screened_body(p, blockIdx.x, gridDim.x);
}

// Columns with more than kShortLen entries, for pass 2 (order not significant).
__global__ void k_list_long(const DevProblem d, int32_t* list, unsigned long long* count) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < d.n;
       base += stride) {
    const int64_t j = base + lane;
    const bool is_long = j < d.n && d.meta[j].y > kShortLen;
    const unsigned mask = __ballot_sync(ACDC_FULL_MASK, is_long);
    if (!mask) continue;
    const int leader = __ffs(mask) - 1;
    unsigned long long first = 0;
    if (lane == leader) first = atomicAdd(count, (unsigned long long)__popc(mask));
    first = __shfl_sync(ACDC_FULL_MASK, first, leader);
    if (is_long) list[first + __popc(mask & ((1u << lane) - 1u))] = (int32_t)j;
  }
}

// SVM: one warp per sample; slots 2: sum alpha, 3: sum hinge, 4: support,
// 5: correctly classified count.  Samples that are margin-violating or have
// 0 < alpha < 1 join the active set.
__device__ __forceinline__ void k_gap_svm_body(const EvalParams& p, const int64_t rank,
                                                const int64_t nb) {
  __shared__ double s_a[ACDC_RED_THREADS / 32], s_h[ACDC_RED_THREADS / 32],
      s_sp[ACDC_RED_THREADS / 32], s_ok[ACDC_RED_THREADS / 32];
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)nb * blockDim.x) >> 5;
  double sa = 0, sh = 0, sp = 0, ok = 0;
  for (int64_t j = ((int64_t)rank * blockDim.x + threadIdx.x) >> 5; j < p.n; j += warps) {
    const int4 mt = p.meta[j];
    const int64_t start = (int64_t)(uint32_t)mt.x << 2;
    const int32_t len = mt.y;
    double g = 0;
    for (int32_t off = 4 * lane; off < len; off += 128) {
      float4 v = __ldcs(reinterpret_cast<const float4*>(p.vals + start + off));
      int4 id = __ldcs(reinterpret_cast<const int4*>(p.idx + start + off));
      g += (double)v.x * p.r64[id.x];
      g += (double)v.y * p.r64[id.y];
      g += (double)v.z * p.r64[id.z];
      g += (double)v.w * p.r64[id.w];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(ACDC_FULL_MASK, g, o);
    if (lane == 0) {
      const double y = p.rhs64[j];
      const double a = coord(p, j);
      if (y * g > 0) ok += 1.0;
      double h = 1.0 - y * g;
      if (h < 0) h = 0;
      sh += h;
      sa += a;
      sp += a != 0.0 ? 1.0 : 0.0;
      if (p.active && ((a > 0.0 && a < 1.0) || (h > 0.0 && a < 1.0) || (h == 0.0 && a > 0.0))) {
        unsigned long long pos = atomicAdd(p.counters + CNT_ACTIVE, 1ull);
        if (pos < (unsigned long long)p.n) p.active[pos] = (int32_t)j;
      }
    }
  }
  if (lane == 0) {
    s_a[threadIdx.x >> 5] = sa;
    s_h[threadIdx.x >> 5] = sh;
    s_sp[threadIdx.x >> 5] = sp;
    s_ok[threadIdx.x >> 5] = ok;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0, t2 = 0, t3 = 0;
    for (int w = 0; w < ACDC_RED_THREADS / 32; ++w) {
      t0 += s_a[w];
      t1 += s_h[w];
      t2 += s_sp[w];
      t3 += s_ok[w];
    }
    p.part[rank * ACDC_NPART + 2] = t0;
    p.part[rank * ACDC_NPART + 3] = t1;
    p.part[rank * ACDC_NPART + 4] = t2;
    p.part[rank * ACDC_NPART + 5] = t3;
  }
}

__global__ void __launch_bounds__(ACDC_RED_THREADS) k_gap_svm(EvalParams p) { k_gap_svm_body(p, blockIdx.x, gridDim.x); }

// Adds the per-block partials in block order and forms P, D and the gap.
// eval_out: [0] P [1] D [2] gap [3] rel_gap [4] 0-1 accuracy [5] reg_norm
//           [6] sq_norm [7] max_abs_grad [8] support [9] active
constexpr int kFinThreads = 32 * ACDC_NPART;

// Warp w reduces partial slot w over the blocks: lane l takes blocks l, l+32,
// ... in order, then a fixed butterfly combines the lanes, so the association
// is fixed and the result reproducible.  Maxima (Lasso slots 3, 5, 7, 8) and
// sums otherwise.
__device__ __forceinline__ void k_finalize_body(const EvalParams& p, const int64_t nparts) {
  __shared__ double red[ACDC_NPART];
  const bool lasso = p.loss == ACDC_LOSS_L1_SQUARE;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w < ACDC_NPART) {
    const bool is_max = lasso && (w == 3 || w == 5 || w == 7 || w == 8 || w == 9);
    double a = 0;
    for (int64_t b = lane; b < nparts; b += 32) {
      const double v = p.part[b * ACDC_NPART + w];
      a = is_max ? fmax(a, v) : a + v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(ACDC_FULL_MASK, a, o);
      a = is_max ? fmax(a, t) : a + t;
    }
    if (lane == 0) red[w] = a;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double rr = red[0], br = red[1], s2 = red[2], s4 = red[4];
  const double s3 = lasso ? fmax(red[3], red[5]) : red[3];
  const double s5 = red[5], s6 = red[6], s7 = fmax(red[7], red[8]);
  double P, D, acc = 0, gmax = 0;
  const double nn = (double)p.n;
  double* o = p.eval_out;
  if (p.loss == ACDC_LOSS_L1_SQUARE) {
    gmax = s3;
    if (p.screened) {
      // Inactive columns: |a_j^T r| <= |a_j^T r_ref| + ||a_j|| ||r - r_ref||.
      const double bound = o[10] + p.col_norm_max * sqrt(s6);
      o[11] = bound;
      gmax = fmax(gmax, bound);
    } else {
      o[10] = s7;
      o[11] = 0;
    }
    if (p.viol) o[12] = red[9];
    P = 0.5 * rr + p.lambda * s2;
    const double s = gmax > p.lambda ? p.lambda / gmax : 1.0;
    D = -s * br - 0.5 * s * s * rr;
  } else if (p.loss == ACDC_LOSS_L2_SQUARE) {
    P = 0.5 * rr + 0.5 * p.lambda * s2;
    D = P - s3 / (2.0 * p.lambda);
  } else if (p.loss == ACDC_LOSS_LOGISTIC) {
    P = rr + 0.5 * p.lambda * s2;
    D = -br - s3 / (2.0 * p.lambda);
    acc = p.m > 0 ? s6 / (double)p.m : 0.0;
  } else {
    P = p.lambda * 0.5 * rr + s3 / nn;
    D = -p.lambda * 0.5 * rr + s2 / nn;
    acc = s5 / nn;
  }
  const double gap = P - D;
  o[0] = P;
  o[1] = D;
  o[2] = gap;
  o[3] = gap / fmax(1.0, fabs(P));
  o[4] = acc;
  o[5] = s2;
  o[6] = rr;
  o[7] = gmax;
  o[8] = s4;
  o[9] = (double)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
}

__global__ void __launch_bounds__(kFinThreads) k_finalize(EvalParams p) {
  k_finalize_body(p, ACDC_RED_BLOCKS);
}

}  // namespace

// ---- launchers ----

// Pass 1 of the layout: padded column lengths are scanned per tile and the
// grand total (in units of 4 entries) lands in scratch[n + tiles].
// scratch must hold n + tiles + 1 int64 entries (start4[n], tile sums, total).
int64_t layout_scan_tiles(int64_t n) { return (n + kScanTile - 1) / kScanTile; }

cudaError_t launch_layout_scan(const int64_t* col_ptr, int64_t n, int64_t* scratch,
                               unsigned long long* counters, cudaStream_t st) {
  const int64_t tiles = layout_scan_tiles(n);
  int64_t* tile_sums = scratch + n;
  int64_t* total = tile_sums + tiles;
  cudaError_t e = cudaMemsetAsync(total, 0, sizeof(int64_t), st);
  if (e != cudaSuccess || n == 0) return e;
  k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, st>>>(col_ptr, n, tile_sums, counters);
  k_scan_offsets<<<1, kScanThreads, 0, st>>>(tile_sums, tiles, total);
  return cudaGetLastError();
}

// Pass 2: column starts and the padded FP32 / int32 arrays with ||a_j||^2.
cudaError_t launch_layout_fill(const int64_t* col_ptr, const int32_t* row_idx,
                               const double* vals64, int64_t m, int64_t n, int64_t* scratch,
                               DevProblem& d, int32_t loss, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int64_t tiles = layout_scan_tiles(n);
  int64_t* start4 = scratch;
  int64_t* tile_sums = scratch + n;
  k_scan_apply<<<(unsigned)tiles, kScanThreads, 0, st>>>(col_ptr, n, tile_sums, start4);
  const int64_t blocks = std::min<int64_t>((n + 7) / 8, 152 * 32);
  k_build_columns<<<(unsigned)blocks, 256, 0, st>>>(col_ptr, row_idx, vals64, start4, m, n, d,
                                                      loss);
  return cudaGetLastError();
}

cudaError_t launch_row_counts(const int32_t* idx, int64_t nnz, int32_t* counts, int64_t m,
                              unsigned long long* counters, cudaStream_t st) {
  (void)counters;
  if (nnz == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((nnz + 255) / 256, 152 * 16);
  k_row_counts<<<(unsigned)blocks, 256, 0, st>>>(idx, nnz, counts, m);
  return cudaGetLastError();
}

cudaError_t launch_max_i32(const int32_t* v, int64_t len, unsigned long long* out_slot,
                           cudaStream_t st) {
  if (len == 0) return cudaSuccess;
  const int64_t blocks = std::min<int64_t>((len + 255) / 256, 152 * 8);
  k_max_i32<<<(unsigned)blocks, 256, 0, st>>>(v, len, out_slot);
  return cudaGetLastError();
}

static unsigned grid_for(int64_t n, int threads, int64_t cap) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  return (unsigned)std::min<int64_t>(b, cap);
}

cudaError_t launch_set_li(const DevProblem& d, int32_t loss, double beta, double lambda,
                          cudaStream_t st) {
  k_set_li<<<grid_for(d.n, 256, 152 * 8), 256, 0, st>>>(d, loss, beta, lambda);
  return cudaGetLastError();
}

cudaError_t launch_widen_i32(const int32_t* src, int64_t* dst, int64_t len, cudaStream_t st) {
  k_widen_i32<<<grid_for(len, 256, 152 * 8), 256, 0, st>>>(src, dst, len);
  return cudaGetLastError();
}

cudaError_t launch_set_x(const DevProblem& d, bool fp64, cudaStream_t st) {
  k_set_x<<<grid_for(d.n, 256, 152 * 8), 256, 0, st>>>(d, fp64 ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_get_x(const DevProblem& d, bool fp64, cudaStream_t st) {
  k_get_x<<<grid_for(d.n, 256, 152 * 8), 256, 0, st>>>(d, fp64 ? 1 : 0);
  return cudaGetLastError();
}

// One warp per active column: rowcnt[row] += 1 for each of its entries.
__global__ void k_active_rowcount(EvalParams p, int32_t* rowcnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t cnt = (int64_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < cnt; t += warps) {
    const int4 mt = p.meta[p.active[t]];
    const int64_t start = (int64_t)(uint32_t)mt.x << 2;
    for (int32_t e = lane; e < mt.y; e += 32) atomicAdd(rowcnt + p.idx[start + e], 1);
  }
}

cudaError_t launch_list_long(const DevProblem& d, int32_t* list, unsigned long long* count,
                             cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::min<int64_t>((d.n + 255) / 256, 152 * 8);
  k_list_long<<<(unsigned)(blocks > 0 ? blocks : 1), 256, 0, st>>>(d, list, count);
  return cudaGetLastError();
}

cudaError_t launch_active_omega(const EvalParams& p, int32_t* rowcnt, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(rowcnt, 0, sizeof(int32_t) * p.m, st);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(p.counters + CNT_OMEGA_ACTIVE, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  k_active_rowcount<<<152 * 8, 256, 0, st>>>(p, rowcnt);
  const int64_t blocks = std::min<int64_t>((p.m + 255) / 256, 152 * 8);
  k_max_i32<<<(unsigned)blocks, 256, 0, st>>>(rowcnt, p.m, p.counters + CNT_OMEGA_ACTIVE);
  return cudaGetLastError();
}

cudaError_t launch_x32_to_x64(const DevProblem& d, cudaStream_t st) {
  k_x32_to_x64<<<grid_for(d.n, 256, 152 * 8), 256, 0, st>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_x64_to_x32(const DevProblem& d, cudaStream_t st) {
  k_x64_to_x32<<<grid_for(d.n, 256, 152 * 8), 256, 0, st>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_refresh(const EvalParams& p, cudaStream_t st) {
  k_refresh_init<<<grid_for(p.m, 256, 152 * 8), 256, 0, st>>>(p);
  k_refresh_scatter<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
  k_refresh_finish<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_gap(const EvalParams& p, cudaStream_t st) {
  if (p.loss == ACDC_LOSS_L2_SQUARE || p.loss == ACDC_LOSS_LOGISTIC) {
    k_gap_smooth<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
    k_finalize<<<1, kFinThreads, 0, st>>>(p);
    return cudaGetLastError();
  }
  if (p.loss == ACDC_LOSS_L1_SQUARE && p.screened) {
    k_gap_lasso_screened<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
    k_finalize<<<1, kFinThreads, 0, st>>>(p);
    return cudaGetLastError();
  }
  cudaError_t e = cudaMemsetAsync(p.counters + CNT_ACTIVE, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  if (p.loss == ACDC_LOSS_L1_SQUARE)
  {
    k_gap_lasso_short<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
    k_gap_lasso_long<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
    if (p.viol && p.active) k_active_viol<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
  }
  else
    k_gap_svm<<<ACDC_RED_BLOCKS, ACDC_RED_THREADS, 0, st>>>(p);
  k_finalize<<<1, kFinThreads, 0, st>>>(p);
  return cudaGetLastError();
}

// Test-set 0-1 accuracy: one warp per test sample i, margin y_i x_i^T w in FP64
// with w the weight vector (the SVM's w = r64 after a refresh, the logistic
// loss's x); features at or beyond the weights' length count as zero.  Adds the
// number of positive margins to *good.
__global__ void k_test_accuracy(int64_t n_test, const int64_t* row_ptr, const int32_t* col_idx,
                                const double* vals, const double* labels, const double* w64,
                                const float* w32, int64_t w_len, unsigned long long* good) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long mine = 0;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n_test; i += warps) {
    double s = 0;
    for (int64_t e = row_ptr[i] + lane; e < row_ptr[i + 1]; e += 32) {
      const int32_t f = col_idx[e];
      if (f >= 0 && f < w_len) s += vals[e] * (w64 ? w64[f] : (double)w32[f]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(ACDC_FULL_MASK, s, o);
    if (lane == 0 && labels[i] * s > 0.0) ++mine;
  }
  if (lane == 0 && mine) atomicAdd(good, mine);
}

cudaError_t launch_test_accuracy(int64_t n_test, const int64_t* row_ptr, const int32_t* col_idx,
                                 const double* vals, const double* labels, const double* w64,
                                 const float* w32, int64_t w_len, unsigned long long* good,
                                 cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(good, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess || n_test == 0) return e;
  const int64_t blocks = std::min<int64_t>((n_test + 7) / 8, 152 * 16);
  k_test_accuracy<<<(unsigned)blocks, 256, 0, st>>>(n_test, row_ptr, col_idx, vals, labels, w64,
                                                    w32, w_len, good);
  return cudaGetLastError();
}

cudaError_t launch_hot_set(const EvalParams& p, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(p.counters + CNT_HOT, 0, 2 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(p.rowcnt, 0, sizeof(int32_t) * p.m, st);
  if (e != cudaSuccess) return e;
  k_hot_mark<<<152 * 4, 256, 0, st>>>(p);
  k_hot_collect<<<152 * 4, 256, 0, st>>>(p);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemsetAsync(p.row_flag, 0, p.m, st);
  return e;
}

// ---- batched rounds ----
namespace {

enum {
  EV_REFRESH_INIT,
  EV_REFRESH_SCATTER,
  EV_REFRESH_FINISH,
  EV_GAP,  // the gap pass of the slot's loss (Lasso: short, then long columns)
  EV_ACTIVE_OMEGA
};

// omega_A of a slot's active list: rowcnt (zeroed by the refresh pass) counts
// the active columns per row; the largest count lands in CNT_OMEGA_ACTIVE.
__device__ __forceinline__ void active_omega_body(const EvalParams& p, const int64_t rank,
                                                  const int64_t nb) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)nb * blockDim.x) >> 5;
  const int64_t cnt = (int64_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n);
  int32_t top = 0;
  for (int64_t t = ((int64_t)rank * blockDim.x + threadIdx.x) >> 5; t < cnt; t += warps) {
    const int4 mt = p.meta[p.active[t]];
    const int64_t start = (int64_t)(uint32_t)mt.x << 2;
    for (int32_t e = lane; e < mt.y; e += 32)
      top = max(top, atomicAdd(p.rowcnt + p.idx[start + e], 1) + 1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) top = max(top, __shfl_xor_sync(ACDC_FULL_MASK, top, o));
  if (lane == 0 && top > 0) atomicMax(p.counters + CNT_OMEGA_ACTIVE, (unsigned long long)top);
}

// One evaluation kernel over every live slot; a block serves its slot at rank
// blockIdx.x - first block of the slot, out of that slot's block count.
template <int KIND>
__global__ void __launch_bounds__(ACDC_RED_THREADS) k_eval_batch(BatchDev b) {
  const int s = b.eblk_slot[blockIdx.x];
  if (!b.ctl[s].live) return;
  const EvalParams p = b.ep[s];
  const int64_t rank = (int64_t)blockIdx.x - b.eblk_first[s];
  const int64_t nb = b.eblk_count[s];
  if (KIND == EV_REFRESH_INIT) k_refresh_init_body(p, rank, nb);
  if (KIND == EV_REFRESH_INIT && p.active && p.rowcnt) {
    // The gap pass of this round rebuilds the active list and its row counts.
    if (rank == 0 && threadIdx.x == 0) {
      p.counters[CNT_ACTIVE] = 0;
      p.counters[CNT_OMEGA_ACTIVE] = 0;
    }
    const int64_t stride = nb * blockDim.x;
    for (int64_t i = rank * blockDim.x + threadIdx.x; i < p.m; i += stride) p.rowcnt[i] = 0;
  }
  if (KIND == EV_ACTIVE_OMEGA) {
    if (p.active && p.rowcnt) active_omega_body(p, rank, nb);
    return;
  }
  if (KIND == EV_REFRESH_SCATTER) k_refresh_scatter_body(p, rank, nb);
  if (KIND == EV_REFRESH_FINISH) k_refresh_finish_body(p, rank, nb);
  if (KIND == EV_GAP) {
    if (p.loss == ACDC_LOSS_L1_SQUARE) {
      k_gap_lasso_short_body(p, rank, nb);
      k_gap_lasso_long_body(p, rank, nb);
    } else {
      k_gap_svm_body(p, rank, nb);
    }
  }
}

// One block per slot: form the gap from the slot's partials, then decide.
//  * converged (relative gap <= target) or the lambda's update budget spent:
//    record the result row, move to the next lambda (warm start: x and the
//    residual carry over; FP64 coordinates are rounded back to FP32 for the next
//    bulk) or retire the slot after the last lambda;
//  * otherwise, below polish_rel_gap in FP32, or stalled near it (the gap,
//    below 1e-4, has not halved over stall_updates): continue in FP64 (x64 = x).
__global__ void __launch_bounds__(kFinThreads) k_batch_control(BatchDev b) {
  __shared__ int s_action;
  const int s = blockIdx.x;
  SlotCtl& c = b.ctl[s];
  if (!c.live) return;
  UpdateParams& up = b.up[s];
  EvalParams& ep = b.ep[s];
  const EvalParams epc = ep;
  k_finalize_body(epc, b.eblk_count[s]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double* o = epc.eval_out;
    up.k_base += up.count;
    c.updates_here += up.count;
    const bool conv = o[3] <= c.gap_target;
    if (o[3] < 0.5 * c.best_gap) {
      c.best_gap = o[3];
      c.gain_at = c.updates_here;
    }
    int action = 0;
    if (conv || c.updates_here >= c.max_updates) {
      double* row = c.results + (int64_t)c.k * ACDC_BATCH_RESULT_LEN;
      for (int i = 0; i < 10; ++i) row[i] = o[i];
      row[10] = epc.lambda;
      row[11] = conv ? 1.0 : 0.0;
      row[12] = (double)((c.updates_here + (uint64_t)epc.n - 1) / (uint64_t)epc.n);
      row[13] = (double)up.n_warps;
      c.k++;
      c.updates_here = 0;
      c.best_gap = 1e300;
      c.gain_at = 0;
      if (c.k >= c.path_len) {
        c.live = 0;
        atomicSub(b.live_count, 1);
      } else {
        const double lam = c.lambdas[c.k];
        ep.lambda = lam;
        ep.shrink_thresh = 0.9 * lam;
        if (up.loss == ACDC_LOSS_SVM_DUAL) {
          up.lambda_d = lam * (double)up.n;
          up.inv_lambda_n_d = 1.0 / (lam * (double)up.n);
        } else {
          up.lambda_d = lam;
        }
        if (up.fp64) action = 2;
      }
    } else if (!up.fp64 && (o[3] <= c.polish_rel_gap ||
                            (o[3] < 1e-4 && c.updates_here - c.gain_at >= c.stall_updates))) {
      action = 1;
    }
    // Next round: uniform right after a lambda change (the active list was built
    // for the previous lambda), else active-set draws.
    c.shrink_next = c.updates_here > 0 ? 1 : 0;
    const int64_t a = (int64_t)min(up.counters[CNT_ACTIVE], (unsigned long long)epc.n);
    if (c.shrink && c.shrink_next && a > 0) {
      const double tau = (double)up.n_warps;
      const double draws = c.q * tau;
      const double w_a = fmax(1.0, (double)up.counters[CNT_OMEGA_ACTIVE]);
      const double beta_a =
          a > 1 && draws > 1 ? 1.0 + (w_a - 1.0) * (draws - 1.0) / ((double)a - 1.0) : 1.0;
      up.li_scale = c.beta / fmax(c.beta, beta_a);
      up.shrink_q32 = c.q32;
      const double lo = fmax(32.0 * tau, 0.25 * (double)epc.n);
      const double want = (double)c.active_passes * (double)a / c.q;
      up.count = (uint64_t)fmin((double)c.round_updates, fmax(lo, want));
    } else {
      up.li_scale = 1.0;
      up.shrink_q32 = 0;
      up.count = c.round_updates;
    }
    up.counters[CNT_WORK] = 0;
    s_action = action;
  }
  __syncthreads();
  const int action = s_action;
  if (action == 1) {
    for (int64_t j = threadIdx.x; j < epc.n; j += blockDim.x)
      up.x64[j] = (double)epc.x32[j];
  } else if (action == 2) {
    for (int64_t j = threadIdx.x; j < epc.n; j += blockDim.x)
      epc.x32[j] = (float)up.x64[j];
  }
  __syncthreads();
  if (threadIdx.x == 0 && action == 1) {
    up.fp64 = 1;
    ep.x64 = up.x64;
  } else if (threadIdx.x == 0 && action == 2) {
    up.fp64 = 0;
    ep.x64 = nullptr;
  }
}

}  // namespace

cudaError_t launch_batch_eval(const BatchDev& b, int eval_blocks, cudaStream_t st) {
  if (eval_blocks <= 0) return cudaSuccess;
  k_eval_batch<EV_REFRESH_INIT><<<eval_blocks, ACDC_RED_THREADS, 0, st>>>(b);
  k_eval_batch<EV_REFRESH_SCATTER><<<eval_blocks, ACDC_RED_THREADS, 0, st>>>(b);
  k_eval_batch<EV_REFRESH_FINISH><<<eval_blocks, ACDC_RED_THREADS, 0, st>>>(b);
  k_eval_batch<EV_GAP><<<eval_blocks, ACDC_RED_THREADS, 0, st>>>(b);
  k_eval_batch<EV_ACTIVE_OMEGA><<<eval_blocks, ACDC_RED_THREADS, 0, st>>>(b);
  k_batch_control<<<b.n_slots, kFinThreads, 0, st>>>(b);
  return cudaGetLastError();
}

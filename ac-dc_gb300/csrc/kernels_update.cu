// PCDM coordinate-update kernel (sm_103a).
//
// Replaces MulticoreEngineExecutor::executeBulkOfIterations
// (cpp/src/solver/MulticoreEngineExecutor.h:83-89) and the per-coordinate
// updates MulticoreL1RegSquareLoss::performOneCoordinateUpdate
// (cpp/src/solver/lossFunctions/squareLoss/MulticoreL1RegSquareLoss.h:41-63) and
// MulticoreSVMDualLoss::performOneCoordinateUpdate
// (cpp/src/solver/lossFunctions/SVMDualLoss/MulticoreSVMDualLoss.h:119-141).
//
// tau warps run concurrently; each warp takes 128 update numbers at a time from
// a global work counter and performs those updates one after another:
//   j      = sampler(seed, k)                         (Philox, see acdc_philox.h)
//   g      = a_j^T r                                  (lanes gather, shuffle reduce)
//   delta  = Lasso: S(lambda Li, x_j - Li g) - x_j    (treshhold_functions.h:27-33)
//            SVM:   clip((1 - y_j g) lambda n Li, -a_j, 1 - a_j)
//   x_j   += delta;  r += c delta a_j                 (red.global.add)
// with Li = 1/(beta ||a_j||^2), beta the ESO parameter for tau.
//
// Memory pipeline.  The column metadata of update s + 2D + 1 and the first 128
// entries (values and row indices) of update s + D are copied into the warp's
// shared-memory ring with cp.async while update s runs: lane l copies entries
// 4l..4l+3 as one 16-byte transfer of values and one of indices (the device
// layout starts every column on a 16-byte boundary).  The warp waits only for
// the copies of update s (cp.async.wait_group D-1), so D updates' worth of DRAM
// traffic is in flight per warp while it waits on its L2 gathers of r.  x_j (in
// x32 or x64) and r are read when the update runs (ld.global.cg, L2), so the sequence of
// updates a warp performs reads exactly the state its own previous updates left.
// Entries beyond the first 128 of a long column are streamed with direct loads.
//
// Precision: T = float keeps x and r in FP32 (the bulk mode); T = double keeps
// x and r in FP64 arrays (the polish mode).  Matrix
// values are FP32 in both.
//
// Kernels of this file: k_pcdm_update (the ring kernel above, for uniform
// bulks), k_pcdm_update_lean (the same updates with a per-chunk record table,
// for the q-shrinking bulks), k_pcdm_update_grouped (8, 16 or 32 lanes per
// update, a setting), k_pcdm_update_batch (one launch over the slots of a
// batch, with the ring or lean body per slot), and the synchronous mini-batch
// SDCA kernels (k_tau_nice, k_sdca_phase1, k_sdca_phase2).
#include "acdc_internal.cuh"

namespace {

constexpr int kChunk = 128;          // updates taken from the work counter at a time
constexpr int kD = 3;                // entry copies in flight per warp
constexpr int kDS = kD + 1;          // entry slots (the slot being written is never the one read)
constexpr int kDM = 2 * kD + 1;      // metadata prefetch distance
constexpr int kMS = kDM + 1;         // metadata slots
static_assert((kDS & (kDS - 1)) == 0 && (kMS & (kMS - 1)) == 0,
              "ring slots are taken modulo a power of two");
// The entries of update s + kD are copied at step s from metadata issued at
// step s + kD - kDM, which wait_group(kD - 1) has completed only if
// kDM >= 2 kD.
static_assert(kDM >= 2 * kD && kMS > kDM, "metadata must land before its entries are copied");
constexpr int kMaxWarps = 8;         // warps per block

struct WarpRing {
  float4 vals[kDS][32];
  int4 idx[kDS][32];
  int4 meta[kMS];
  int32_t coords[kChunk];  // coordinates of the current chunk of updates
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Sum over the lanes that hold entries of a column of len entries.  Lane l
// holds entries 4l..4l+3, so a column of at most 16 entries lives in lanes
// 0..3: two butterfly steps give its sum in those lanes, which are the only
// ones that scatter (lane 0 also writes x_j); other lanes get partial sums
// that they do not use.  Longer columns take all five steps (sum in every
// lane).  No broadcast and no loop: the short case is two dependent shuffles.
template <typename T>
__device__ __forceinline__ T column_sum(T v, uint32_t len) {
  v += __shfl_xor_sync(ACDC_FULL_MASK, v, 1);
  v += __shfl_xor_sync(ACDC_FULL_MASK, v, 2);
  if (len > 16u) {
    v += __shfl_xor_sync(ACDC_FULL_MASK, v, 4);
    v += __shfl_xor_sync(ACDC_FULL_MASK, v, 8);
    v += __shfl_xor_sync(ACDC_FULL_MASK, v, 16);
  }
  return v;
}

// Coordinate of update k.  With shrinking, word 2 picks the tier (hot set below
// hot_q32, active set below shrink_q32, else all coordinates) and word 3 the
// entry of the list; a hot-set draw is returned with bit 31 set.
constexpr int32_t kHotBit = (int32_t)0x80000000u;
constexpr int32_t kCoordMask = 0x7fffffff;

__device__ __forceinline__ int32_t draw_coord(const UpdateParams& p, uint64_t k,
                                              int32_t active_cnt, int32_t hot_cnt) {
  acdc_u32x4 o = acdc_philox4x32_10((uint32_t)k, (uint32_t)(k >> 32), ACDC_STREAM_SAMPLER, 0u,
                                    (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
  if (active_cnt > 0 && o.v[2] < p.shrink_q32) {
    if (hot_cnt > 0 && o.v[2] < p.hot_q32)
      return __ldg(p.hot + __umulhi(o.v[3], (uint32_t)hot_cnt)) | kHotBit;
    uint32_t t = __umulhi(o.v[3], (uint32_t)active_cnt);
    return __ldg(p.active + t);
  }
  uint64_t u = ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
  return (int32_t)__umul64hi(u, (uint64_t)p.n);
}

struct Chunk {
  float4 v;
  int4 i;
};

__device__ __forceinline__ Chunk load_chunk(const UpdateParams& p, uint64_t start, uint32_t len,
                                            uint32_t off, int lane) {
  Chunk c;
  const uint32_t e = off + 4u * (uint32_t)lane;
  if (e < len) {
    c.v = __ldcs(reinterpret_cast<const float4*>(p.vals + start + e));
    c.i = __ldcs(reinterpret_cast<const int4*>(p.idx + start + e));
  } else {
    c.v = make_float4(0.f, 0.f, 0.f, 0.f);
    c.i = make_int4(0, 0, 0, 0);
  }
  return c;
}

// The residual entry as the gradient uses it: r itself, or for the logistic
// loss sigma(r) = 1/(1 + exp(-r)), in a form that does not overflow.
__device__ __forceinline__ float sigmoid_t(float z) {
  if (z >= 0.f) return 1.f / (1.f + expf(-z));
  const float e = expf(z);
  return e / (1.f + e);
}
__device__ __forceinline__ double sigmoid_t(double z) {
  if (z >= 0.0) return 1.0 / (1.0 + exp(-z));
  const double e = exp(z);
  return e / (1.0 + e);
}
template <int LOSS, typename T>
__device__ __forceinline__ T rval(const T* r, int32_t i) {
  const T v = __ldcg(r + i);
  if constexpr (LOSS == ACDC_LOSS_LOGISTIC) return sigmoid_t(v);
  return v;
}

template <int LOSS, typename T>
__device__ __forceinline__ T gather_dot(const T* r, const Chunk& c, bool live) {
  if (!live) return T(0);
  T a = (T)c.v.x * rval<LOSS>(r, c.i.x);
  a += (T)c.v.y * rval<LOSS>(r, c.i.y);
  a += (T)c.v.z * rval<LOSS>(r, c.i.z);
  a += (T)c.v.w * rval<LOSS>(r, c.i.w);
  return a;
}

// The same for the first chunk, skipping the pad entries of a column whose
// length is not a multiple of 4 (most columns are short: one gather, not four).
template <int LOSS, typename T>
__device__ __forceinline__ T gather_dot_head(const T* r, const Chunk& c, uint32_t e0,
                                             uint32_t len) {
  T a = T(0);
  if (e0 < len) a = (T)c.v.x * rval<LOSS>(r, c.i.x);
  if (e0 + 1u < len) a += (T)c.v.y * rval<LOSS>(r, c.i.y);
  if (e0 + 2u < len) a += (T)c.v.z * rval<LOSS>(r, c.i.z);
  if (e0 + 3u < len) a += (T)c.v.w * rval<LOSS>(r, c.i.w);
  return a;
}

// The same for the first chunk, whose lanes past the column may hold stale
// ring contents: only entries below len are written.
template <typename T>
__device__ __forceinline__ void scatter_head(T* r, const Chunk& c, T coef, uint32_t e0,
                                             uint32_t len) {
  if (e0 < len) atomicAdd(r + c.i.x, coef * (T)c.v.x);
  if (e0 + 1u < len) atomicAdd(r + c.i.y, coef * (T)c.v.y);
  if (e0 + 2u < len) atomicAdd(r + c.i.z, coef * (T)c.v.z);
  if (e0 + 3u < len) atomicAdd(r + c.i.w, coef * (T)c.v.w);
}

template <typename T>
__device__ __forceinline__ void scatter(T* r, const Chunk& c, T coef, bool live) {
  if (!live) return;
  if (c.v.x != 0.f) atomicAdd(r + c.i.x, coef * (T)c.v.x);
  if (c.v.y != 0.f) atomicAdd(r + c.i.y, coef * (T)c.v.y);
  if (c.v.z != 0.f) atomicAdd(r + c.i.z, coef * (T)c.v.z);
  if (c.v.w != 0.f) atomicAdd(r + c.i.w, coef * (T)c.v.w);
}

// The step of one coordinate from g = a_j^T r (for the logistic loss the
// gather already applied sigma), x_j and li = Li times the launch's step scale:
// delta for x_j, and coef, the factor of a_j in the residual update
// r += coef a_j.
template <int LOSS, typename T>
__device__ __forceinline__ T step_delta(T g, T xj, T li, T lam, T inv_ln, T& coef) {
  T delta;
  if (LOSS == ACDC_LOSS_L1_SQUARE) {
    const T z = xj - li * g;
    T a = fabs(z) - lam * li;
    a = a < T(0) ? T(0) : a;
    const T xn = z > T(0) ? a : (z < T(0) ? -a : T(0));
    delta = xn - xj;
    coef = delta;
  } else if (LOSS == ACDC_LOSS_L2_SQUARE) {
    // MulticoreL2SquareRegSquareLoss.h:56-78: delta = -Li (a_j^T r + lambda x_j)
    delta = -li * (g + lam * xj);
    coef = delta;
  } else if (LOSS == ACDC_LOSS_LOGISTIC) {
    // MulticoreL2SquareRegLogisticLoss.h:88-115 with the label folded into the
    // values: gradient -sum_i v_i sigma(r_i) + lambda x_j, half step, and
    // r_i += -delta v_i.
    delta = -li * (lam * xj - g) / T(2);
    coef = -delta;
  } else {
    const T y = li < T(0) ? T(-1) : T(1);
    delta = (T(1) - g * y) * lam * fabs(li);
    if (delta < -xj)
      delta = -xj;
    else if (delta > T(1) - xj)
      delta = T(1) - xj;
    coef = delta * y * inv_ln;
  }
  return delta;
}

__device__ __forceinline__ void issue_meta(WarpRing& w, const UpdateParams& p, int32_t j, int slot,
                                           int lane) {
  if (lane == 0) cp_async16(&w.meta[slot], p.meta + j);
}

__device__ __forceinline__ void issue_entries(WarpRing& w, const UpdateParams& p, int mslot,
                                              int dslot, int lane) {
  const int4 mt = w.meta[mslot];
  const uint32_t len = (uint32_t)mt.y;
  if (4u * (uint32_t)lane < len) {
    const uint64_t src = ((uint64_t)(uint32_t)mt.x << 2) + 4u * (uint32_t)lane;
    cp_async16(&w.vals[dslot][lane], p.vals + src);
    cp_async16(&w.idx[dslot][lane], p.idx + src);
  }
}

// One warp's share of an update launch; rank is the block's position among the
// blocks serving this problem (the grid for one problem, a block range for one
// slot of a batch).
template <int LOSS, typename T>
__device__ __forceinline__ void pcdm_update_body(const UpdateParams& p, uint64_t k_base,
                                                 int64_t rank, WarpRing* rings) {
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int64_t gwarp = (rank * blockDim.x + threadIdx.x) >> 5;
  if (gwarp >= p.n_warps) return;
  WarpRing& w = rings[wib];
  T* r = reinterpret_cast<T*>(sizeof(T) == 8 ? (void*)p.r64 : (void*)p.r);
  unsigned long long* work = p.counters + CNT_WORK;
  const int32_t active_cnt =
      p.shrink_q32 ? (int32_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n) : 0;
  const int32_t hot_cnt =
      p.hot_q32 ? (int32_t)min(p.counters[CNT_HOT], (unsigned long long)p.n) : 0;
  const T lam = (T)p.lambda_d;
  const T inv_ln = (T)p.inv_lambda_n_d;
  const T li_scale = (T)p.li_scale;
  const T li_scale_hot = (T)p.li_scale_hot;
  unsigned long long n_upd = 0, n_nz = 0, n_read = 0, n_scat = 0;

  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, (unsigned long long)kChunk);
    base = __shfl_sync(ACDC_FULL_MASK, base, 0);
    if (base >= p.count) break;
    const int cnt = (int)min((unsigned long long)kChunk, p.count - base);
#pragma unroll
    for (int q = 0; q < kChunk / 32; ++q) {
      const int s = 32 * q + lane;
      w.coords[s] = s < cnt ? draw_coord(p, k_base + base + (uint64_t)s, active_cnt, hot_cnt) : 0;
    }
    __syncwarp();

    // Prologue: metadata of updates 0..kDM-1, then entries of updates 0..D-1,
    // one commit group per update so that wait_group(D-1) below always means
    // "the copies of update s have landed".
    for (int t = 0; t < kDM && t < cnt; ++t) issue_meta(w, p, w.coords[t] & kCoordMask, t, lane);
    cp_async_commit();
    cp_async_wait<0>();
    __syncwarp();
#pragma unroll
    for (int t = 0; t < kD; ++t) {
      if (t < cnt) issue_entries(w, p, t, t, lane);
      cp_async_commit();
    }

    // Ring positions: update s reads meta slot s mod kMS and entry slot
    // s mod kDS; the refill writes entries of s+D into slot (s+D) mod kDS and
    // meta of s+kDM into slot (s+kDM) mod kMS, which are the slots update s-1
    // used.
    uint32_t chunk_read = 0, chunk_nz = 0, chunk_scat = 0;
    for (int s = 0; s < cnt; ++s) {
      const int ms = s & (kMS - 1), ds = s & (kDS - 1);
      const int ms_d = (s + kD) & (kMS - 1), ds_d = (s + kD) & (kDS - 1);
      const int ms_2d = (s + kDM) & (kMS - 1);
      cp_async_wait<kD - 1>();
      __syncwarp();  // copies of update s visible; every lane is done with update s-1
      const int32_t cj = w.coords[s];
      const int32_t j = cj & kCoordMask;
      const int4 mt = w.meta[ms];
      T xj;
      if constexpr (sizeof(T) == 8)
        xj = __ldcg(p.x64 + j);
      else
        xj = __ldcg(p.x32 + j);
      const uint64_t start = (uint64_t)(uint32_t)mt.x << 2;
      const uint32_t len = (uint32_t)mt.y;
      const uint32_t e0 = 4u * (uint32_t)lane;
      Chunk c0;  // lanes past the column read stale slots, never used below
      c0.v = w.vals[ds][lane];
      c0.i = w.idx[ds][lane];
      // Refill: entries of update s + D, metadata of update s + 2D.
      if (s + kD < cnt) issue_entries(w, p, ms_d, ds_d, lane);
      if (s + kDM < cnt) issue_meta(w, p, w.coords[s + kDM] & kCoordMask, ms_2d, lane);
      cp_async_commit();

      // g = a_j^T r.  (Issuing these gathers before the refill above, or
      // prefetching x_j into L2 with the record, did not shorten the launches
      // in the measurements: active-set launches, which dominate the solve,
      // got longer.)
      T acc = gather_dot_head<LOSS, T>(r, c0, e0, len);
      if (len > 128u) {
        Chunk a = load_chunk(p, start, len, 128u, lane);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk b = load_chunk(p, start, len, off + 128u, lane);
          acc += gather_dot<LOSS, T>(r, a, off + e0 < len);
          a = b;
        }
      }
      const T g = column_sum<T>(acc, len);

      const T li = (T)__int_as_float(mt.z) * (cj < 0 ? li_scale_hot : li_scale);
      T coef;
      const T delta = step_delta<LOSS, T>(g, xj, li, lam, inv_ln, coef);
      chunk_read += len;
      // lanes with entries (and lane 0, which writes x_j) hold the column's sum
      const bool holds = e0 < len || lane == 0 || len > 16u;
      if (holds && delta != T(0)) {
        chunk_nz++;
        chunk_scat += len;
        scatter_head<T>(r, c0, coef, e0, len);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk a = load_chunk(p, start, len, off, lane);
          scatter<T>(r, a, coef, off + e0 < len);
        }
        if (lane == 0) {
          if constexpr (sizeof(T) == 8)
            atomicAdd(p.x64 + j, delta);
          else
            atomicAdd(p.x32 + j, delta);
        }
      }
    }
    cp_async_wait<0>();
    __syncwarp();
    n_upd += (unsigned)cnt;
    n_read += chunk_read;
    n_nz += chunk_nz;
    n_scat += chunk_scat;
  }
  if (lane == 0) {
    atomicAdd(p.counters + CNT_UPDATES, n_upd);
    atomicAdd(p.counters + CNT_NONZERO, n_nz);
    atomicAdd(p.counters + CNT_NNZ_READ, n_read);
    atomicAdd(p.counters + CNT_NNZ_SCATTERED, n_scat);
  }
}

template <int LOSS, typename T>
__global__ void __launch_bounds__(256, 4) k_pcdm_update(UpdateParams p, uint64_t k_base) {
  __shared__ WarpRing rings[kMaxWarps];
  pcdm_update_body<LOSS, T>(p, k_base, blockIdx.x, rings);
}

// ---- lean update kernel: a record table per chunk and the entry ring only ----
//
// The same updates, draws and arithmetic as k_pcdm_update (at one update in
// flight the two give identical iterates), with a shorter path per update for
// the q-shrinking launches, whose draws mostly land on short columns (the
// active set of a Zipf-length Lasso is about 94% columns of at most 4
// entries):
// - the records of all updates of a chunk are copied into a table when the
//   chunk is drawn, and word 3 of each copy (0 in the layout) is overwritten
//   with the drawn coordinate and its hot-tier bit, so an update reads its
//   record, coordinate and tier with one 16-byte shared load, and there is no
//   record ring;
// - lane l copies, and later reads, only pieces l of the entry ring (entries
//   4l..4l+3), so an update waits on its own lane's copies with
//   cp.async.wait_group and needs no __syncwarp;
// - a column of at most 4 entries sits in lane 0 and needs no shuffles;
// - the work counter of the next chunk is taken while this one runs.
constexpr int kLeanWarps = 8;  // warps per block

struct WarpLean {
  float4 vals[kDS][32];
  int4 idx[kDS][32];
  int4 rec[kChunk];  // {start4, len, Li, drawn coordinate | hot bit} per update
};
static_assert(sizeof(WarpLean) * kLeanWarps <= 48 * 1024, "static shared memory of a block");

__device__ __forceinline__ void lean_issue(WarpLean& w, const UpdateParams& p, const int4 mt,
                                           int dslot, int lane) {
  const uint32_t len = (uint32_t)mt.y;
  if (4u * (uint32_t)lane < len) {
    const uint64_t src = ((uint64_t)(uint32_t)mt.x << 2) + 4u * (uint32_t)lane;
    cp_async16(&w.vals[dslot][lane], p.vals + src);
    cp_async16(&w.idx[dslot][lane], p.idx + src);
  }
}

// Sum over the lanes holding a column of len entries (lane l: entries
// 4l..4l+3): nothing to add for at most 4 entries (lane 0 alone), two steps up
// to 16 (lanes 0..3), five beyond.
template <typename T>
__device__ __forceinline__ T lean_sum(T v, uint32_t len) {
  if (len > 4u) {
    v += __shfl_xor_sync(ACDC_FULL_MASK, v, 1);
    v += __shfl_xor_sync(ACDC_FULL_MASK, v, 2);
    if (len > 16u) {
      v += __shfl_xor_sync(ACDC_FULL_MASK, v, 4);
      v += __shfl_xor_sync(ACDC_FULL_MASK, v, 8);
      v += __shfl_xor_sync(ACDC_FULL_MASK, v, 16);
    }
  }
  return v;
}

template <int LOSS, typename T>
__device__ __forceinline__ void pcdm_lean_body(const UpdateParams& p, uint64_t k_base,
                                               int64_t rank, WarpLean* lean) {
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = (rank * blockDim.x + threadIdx.x) >> 5;
  if (gwarp >= p.n_warps) return;
  WarpLean& w = lean[threadIdx.x >> 5];
  T* r = reinterpret_cast<T*>(sizeof(T) == 8 ? (void*)p.r64 : (void*)p.r);
  T* x = reinterpret_cast<T*>(sizeof(T) == 8 ? (void*)p.x64 : (void*)p.x32);
  unsigned long long* work = p.counters + CNT_WORK;
  const int32_t active_cnt =
      p.shrink_q32 ? (int32_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n) : 0;
  const int32_t hot_cnt =
      p.hot_q32 ? (int32_t)min(p.counters[CNT_HOT], (unsigned long long)p.n) : 0;
  const T lam = (T)p.lambda_d;
  const T inv_ln = (T)p.inv_lambda_n_d;
  const T li_scale = (T)p.li_scale;
  const T li_scale_hot = (T)p.li_scale_hot;
  const uint32_t e0 = 4u * (uint32_t)lane;
  unsigned long long n_upd = 0, n_nz = 0, n_read = 0, n_scat = 0;

  unsigned long long next = 0;
  if (lane == 0) next = atomicAdd(work, (unsigned long long)kChunk);
  for (;;) {
    const unsigned long long base = __shfl_sync(ACDC_FULL_MASK, next, 0);
    if (base >= p.count) break;
    if (lane == 0) next = atomicAdd(work, (unsigned long long)kChunk);
    const int cnt = (int)min((unsigned long long)kChunk, p.count - base);

    // Draw the chunk and copy its records; then stamp each copy with its draw.
    int32_t cj[kChunk / 32];
#pragma unroll
    for (int q = 0; q < kChunk / 32; ++q) {
      const int s = 32 * q + lane;
      cj[q] = s < cnt ? draw_coord(p, k_base + base + (uint64_t)s, active_cnt, hot_cnt) : 0;
      if (s < cnt) cp_async16(&w.rec[s], p.meta + (cj[q] & kCoordMask));
    }
    cp_async_commit();
    cp_async_wait<0>();
#pragma unroll
    for (int q = 0; q < kChunk / 32; ++q) {
      const int s = 32 * q + lane;
      if (s < cnt) w.rec[s].w = cj[q];
    }
    __syncwarp();
    // Entries of updates 0..D-1, one commit group per update, so that
    // wait_group(D-1) at update s means "this lane's copies of update s landed".
#pragma unroll
    for (int t = 0; t < kD; ++t) {
      if (t < cnt) lean_issue(w, p, w.rec[t], t, lane);
      cp_async_commit();
    }

    uint32_t chunk_read = 0, chunk_nz = 0, chunk_scat = 0;
    for (int s = 0; s < cnt; ++s) {
      const int ds = s & (kDS - 1);
      cp_async_wait<kD - 1>();
      const int4 mt = w.rec[s];
      const int32_t j = mt.w & kCoordMask;
      const T xj = __ldcg(x + j);
      const uint32_t len = (uint32_t)mt.y;
      Chunk c0;  // lanes past the column hold stale pieces, never used below
      c0.v = w.vals[ds][lane];
      c0.i = w.idx[ds][lane];
      // Refill: entries of update s + D into the slot update s - 1 used (this
      // lane's own pieces).  Issued before the gathers: the other order made the
      // active-set launches 11% slower in the measurements.
      if (s + kD < cnt) lean_issue(w, p, w.rec[s + kD], (s + kD) & (kDS - 1), lane);
      cp_async_commit();
      T acc = gather_dot_head<LOSS, T>(r, c0, e0, len);
      const uint64_t start = (uint64_t)(uint32_t)mt.x << 2;
      if (len > 128u) {
        Chunk a = load_chunk(p, start, len, 128u, lane);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk b = load_chunk(p, start, len, off + 128u, lane);
          acc += gather_dot<LOSS, T>(r, a, off + e0 < len);
          a = b;
        }
      }
      const T g = lean_sum<T>(acc, len);
      const T li = (T)__int_as_float(mt.z) * (mt.w < 0 ? li_scale_hot : li_scale);
      T coef;
      const T delta = step_delta<LOSS, T>(g, xj, li, lam, inv_ln, coef);
      chunk_read += len;
      // the lanes holding entries (and lane 0, which writes x_j) hold the sum
      const bool holds = e0 < len || lane == 0 || len > 16u;
      if (holds && delta != T(0)) {
        chunk_nz++;
        chunk_scat += len;
        scatter_head<T>(r, c0, coef, e0, len);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk a = load_chunk(p, start, len, off, lane);
          scatter<T>(r, a, coef, off + e0 < len);
        }
        if (lane == 0) atomicAdd(x + j, delta);
      }
    }
    cp_async_wait<0>();
    __syncwarp();  // every lane is done with this chunk's record table
    n_upd += (unsigned)cnt;
    n_read += chunk_read;
    n_nz += chunk_nz;
    n_scat += chunk_scat;
  }
  if (lane == 0) {
    atomicAdd(p.counters + CNT_UPDATES, n_upd);
    atomicAdd(p.counters + CNT_NONZERO, n_nz);
    atomicAdd(p.counters + CNT_NNZ_READ, n_read);
    atomicAdd(p.counters + CNT_NNZ_SCATTERED, n_scat);
  }
}

template <int LOSS, typename T>
__global__ void __launch_bounds__(256, 4) k_pcdm_update_lean(UpdateParams p, uint64_t k_base) {
  __shared__ WarpLean lean[kLeanWarps];
  pcdm_lean_body<LOSS, T>(p, k_base, blockIdx.x, lean);
}

// ---- grouped update kernel: G lanes per update, 32/G updates per warp ----
//
// A group of G lanes (G = 8, 16 or 32) performs one update at a time; a warp runs
// 32/G groups side by side on independent update numbers, so p.n_warps (tau,
// the updates in flight) needs tau G / 32 warps.  Lane l of a group holds
// entries 4l..4l+3 of a column's first 4G entries (one 128-bit load of values
// and one of row indices, the layout's 16-byte column starts); longer columns
// stream further chunks of 4G entries.  Nothing is staged in shared memory but
// the warp's drawn coordinates: the record of the group's update i+3 and the
// first entry chunk of update i+2 are loaded into registers while update i
// runs (ld.global.nc: the matrix and the records do not change during a
// launch), so one update costs the gathers of r, the group reduction (log2 G
// shuffles) and the scatter, with no copy bookkeeping.  x_j and r are read
// through L2 (ld.cg) when the update runs, as in the ring kernel.
struct GroupChunk {
  float4 v;
  int4 i;
};

template <int G>
__device__ __forceinline__ GroupChunk group_chunk(const UpdateParams& p, int4 mt, int gl,
                                                  bool stream) {
  GroupChunk c;
  const uint32_t len = (uint32_t)mt.y;
  const uint32_t e = 4u * (uint32_t)gl;
  if (e < len) {
    const uint64_t src = ((uint64_t)(uint32_t)mt.x << 2) + e;
    if (stream) {
      c.v = __ldcs(reinterpret_cast<const float4*>(p.vals + src));
      c.i = __ldcs(reinterpret_cast<const int4*>(p.idx + src));
    } else {
      c.v = __ldg(reinterpret_cast<const float4*>(p.vals + src));
      c.i = __ldg(reinterpret_cast<const int4*>(p.idx + src));
    }
  } else {
    c.v = make_float4(0.f, 0.f, 0.f, 0.f);
    c.i = make_int4(0, 0, 0, 0);
  }
  return c;
}

template <int G, typename T>
__device__ __forceinline__ T group_sum(T v, unsigned gmask) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gmask, v, o);
  return v;
}

template <int LOSS, typename T, int G>
__device__ __forceinline__ void pcdm_update_grouped_body(const UpdateParams& p, uint64_t k_base,
                                                         int64_t rank, int32_t* coords) {
  constexpr int kGroups = 32 / G;
  constexpr uint32_t kSpan = 4u * G;  // entries per chunk
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const int grp = lane / G;
  const int64_t gwarp = (rank * blockDim.x + threadIdx.x) >> 5;
  const int64_t warps = ((int64_t)p.n_warps + kGroups - 1) / kGroups;
  if (gwarp >= warps) return;
  // groups of this warp that run (tau need not fill the last warp: tau = 1
  // keeps a single update in flight)
  const int ng = (int)min((int64_t)kGroups, (int64_t)p.n_warps - gwarp * kGroups);
  T* r = reinterpret_cast<T*>(sizeof(T) == 8 ? (void*)p.r64 : (void*)p.r);
  unsigned long long* work = p.counters + CNT_WORK;
  const int32_t active_cnt =
      p.shrink_q32 ? (int32_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n) : 0;
  const int32_t hot_cnt =
      p.hot_q32 ? (int32_t)min(p.counters[CNT_HOT], (unsigned long long)p.n) : 0;
  // uniform-draw launches read each column about once: stream its entries
  // past L2 instead of evicting the residual and the active columns
  const bool stream = p.shrink_q32 == 0;
  const T lam = (T)p.lambda_d;
  const T inv_ln = (T)p.inv_lambda_n_d;
  const T li_scale = (T)p.li_scale;
  const T li_scale_hot = (T)p.li_scale_hot;
  const uint32_t e0 = 4u * (uint32_t)gl;
  unsigned long long n_upd = 0, n_nz = 0, n_read = 0, n_scat = 0;

  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, (unsigned long long)kChunk);
    base = __shfl_sync(ACDC_FULL_MASK, base, 0);
    if (base >= p.count) break;
    const int cnt = (int)min((unsigned long long)kChunk, p.count - base);
#pragma unroll
    for (int q = 0; q < kChunk / 32; ++q) {
      const int s = 32 * q + lane;
      coords[s] = s < cnt ? draw_coord(p, k_base + base + (uint64_t)s, active_cnt, hot_cnt) : 0;
    }
    __syncwarp();
    // this group's updates of the chunk: s = i * ng + grp.  Every lane of the
    // warp runs the same my_all iterations (a group past its last update, or
    // beyond ng, runs them with a zero-length record), so the group reductions
    // are full-warp shuffles of a converged warp.
    const int my = grp < ng && cnt > grp ? (cnt - grp + ng - 1) / ng : 0;
    const int my_all = (cnt + ng - 1) / ng;
    const int4 none = make_int4(0, 0, 0, 0);
    auto coord_of = [&](int i) { return coords[i * ng + grp]; };
    auto meta_of = [&](int i) {
      return i < my ? __ldg(p.meta + (coord_of(i) & kCoordMask)) : none;
    };
    // Pipeline: at update i the group holds the records of updates i..i+3 and
    // the first entry chunks of updates i and i+1; it issues the record of
    // update i+4 and the chunk of update i+2 (whose record came in two updates
    // ago) after the gathers of update i, so neither waits on the other.
    int4 m0 = meta_of(0), m1 = meta_of(1), m2 = meta_of(2), m3 = meta_of(3);
    GroupChunk c0 = group_chunk<G>(p, m0, gl, stream);
    GroupChunk c1 = group_chunk<G>(p, m1, gl, stream);
    for (int i = 0; i < my_all; ++i) {
      const bool live = i < my;
      const int32_t cj = live ? coord_of(i) : 0;
      const int32_t j = cj & kCoordMask;
      const int4 mt = m0;
      const uint64_t start = (uint64_t)(uint32_t)mt.x << 2;
      const uint32_t len = (uint32_t)mt.y;
      T xj = T(0);
      if (live) {
        if constexpr (sizeof(T) == 8)
          xj = __ldcg(p.x64 + j);
        else
          xj = __ldcg(p.x32 + j);
      }
      T r0 = T(0), r1 = T(0), r2 = T(0), r3 = T(0);
      if (e0 < len) r0 = rval<LOSS>(r, c0.i.x);
      if (e0 + 1u < len) r1 = rval<LOSS>(r, c0.i.y);
      if (e0 + 2u < len) r2 = rval<LOSS>(r, c0.i.z);
      if (e0 + 3u < len) r3 = rval<LOSS>(r, c0.i.w);
      // refill while the gathers are in flight
      const GroupChunk c2 = group_chunk<G>(p, m2, gl, stream);  // zero past the group's end
      const int4 m4 = meta_of(i + 4);
      T acc = (T)c0.v.x * r0;
      acc += (T)c0.v.y * r1;
      acc += (T)c0.v.z * r2;
      acc += (T)c0.v.w * r3;
      for (uint32_t off = kSpan; off < len; off += kSpan) {
        const uint32_t e = off + e0;
        if (e < len) {
          const float4 v = __ldcs(reinterpret_cast<const float4*>(p.vals + start + e));
          const int4 ix = __ldcs(reinterpret_cast<const int4*>(p.idx + start + e));
          acc += (T)v.x * rval<LOSS>(r, ix.x);
          if (e + 1u < len) acc += (T)v.y * rval<LOSS>(r, ix.y);
          if (e + 2u < len) acc += (T)v.z * rval<LOSS>(r, ix.z);
          if (e + 3u < len) acc += (T)v.w * rval<LOSS>(r, ix.w);
        }
      }
      const T g = group_sum<G, T>(acc, ACDC_FULL_MASK);
      if (live) {
        const T li = (T)__int_as_float(mt.z) * (cj < 0 ? li_scale_hot : li_scale);
        T coef;
        const T delta = step_delta<LOSS, T>(g, xj, li, lam, inv_ln, coef);
        n_read += len;
        if (delta != T(0)) {
          n_nz++;
          n_scat += len;
          if (e0 < len) atomicAdd(r + c0.i.x, coef * (T)c0.v.x);
          if (e0 + 1u < len) atomicAdd(r + c0.i.y, coef * (T)c0.v.y);
          if (e0 + 2u < len) atomicAdd(r + c0.i.z, coef * (T)c0.v.z);
          if (e0 + 3u < len) atomicAdd(r + c0.i.w, coef * (T)c0.v.w);
          for (uint32_t off = kSpan; off < len; off += kSpan) {
            const uint32_t e = off + e0;
            if (e < len) {
              const float4 v = __ldcs(reinterpret_cast<const float4*>(p.vals + start + e));
              const int4 ix = __ldcs(reinterpret_cast<const int4*>(p.idx + start + e));
              atomicAdd(r + ix.x, coef * (T)v.x);
              if (e + 1u < len) atomicAdd(r + ix.y, coef * (T)v.y);
              if (e + 2u < len) atomicAdd(r + ix.z, coef * (T)v.z);
              if (e + 3u < len) atomicAdd(r + ix.w, coef * (T)v.w);
            }
          }
          if (gl == 0) {
            if constexpr (sizeof(T) == 8)
              atomicAdd(p.x64 + j, delta);
            else
              atomicAdd(p.x32 + j, delta);
          }
        }
      }  // live
      m0 = m1;
      m1 = m2;
      m2 = m3;
      m3 = m4;
      c0 = c1;
      c1 = c2;
    }
    n_upd += (unsigned)my;
    __syncwarp();  // every group is done with the chunk's coordinates
  }
  if (gl == 0) {
    atomicAdd(p.counters + CNT_UPDATES, n_upd);
    atomicAdd(p.counters + CNT_NONZERO, n_nz);
    atomicAdd(p.counters + CNT_NNZ_READ, n_read);
    atomicAdd(p.counters + CNT_NNZ_SCATTERED, n_scat);
  }
}

template <int LOSS, typename T, int G>
__global__ void __launch_bounds__(256) k_pcdm_update_grouped(UpdateParams p, uint64_t k_base) {
  __shared__ int32_t coords[kMaxWarps][kChunk];
  pcdm_update_grouped_body<LOSS, T, G>(p, k_base, blockIdx.x, coords[threadIdx.x >> 5]);
}

// Batched launch: each block serves one slot at rank blockIdx.x - first block
// of that slot, with the body of that slot's loss and precision, so one launch
// covers Lasso and SVM slots in FP32 and FP64 alike.  The kernel choice is the
// single-problem launch's: the lean body for a slot's q-shrinking rounds, the
// ring body for the others.
union BatchShared {
  WarpRing ring[kMaxWarps];
  WarpLean lean[kLeanWarps];
};

template <int LOSS, typename T>
__device__ __forceinline__ void batch_body(const UpdateParams& p, int64_t rank, BatchShared& sm) {
  if (p.lanes == 1 || (p.lanes == 0 && p.shrink_q32 != 0))
    pcdm_lean_body<LOSS, T>(p, p.k_base, rank, sm.lean);
  else
    pcdm_update_body<LOSS, T>(p, p.k_base, rank, sm.ring);
}

__global__ void __launch_bounds__(256, 4) k_pcdm_update_batch(BatchDev b) {
  __shared__ BatchShared sm;
  const int s = b.ublk_slot[blockIdx.x];
  if (!b.ctl[s].live) return;
  const UpdateParams p = b.up[s];
  if (p.count == 0) return;
  const int64_t rank = (int64_t)blockIdx.x - b.ublk_first[s];
  if (p.loss == ACDC_LOSS_SVM_DUAL) {
    if (p.fp64)
      batch_body<ACDC_LOSS_SVM_DUAL, double>(p, rank, sm);
    else
      batch_body<ACDC_LOSS_SVM_DUAL, float>(p, rank, sm);
  } else {
    if (p.fp64)
      batch_body<ACDC_LOSS_L1_SQUARE, double>(p, rank, sm);
    else
      batch_body<ACDC_LOSS_L1_SQUARE, float>(p, rank, sm);
  }
}

// ---- synchronous mini-batch SDCA (hinge dual), tau-nice steps ----
//
// The structure of the reference's mini-batch loop
// (cpp/src/experiments/mSDCA.cpp:60-105): a step draws tau distinct
// coordinates, computes every delta from the same w, then applies them all.
//
// k_tau_nice: one warp draws `steps` steps.  Each step takes the first tau
// distinct values of the uniform sampler stream (counter *counter, the draw of
// acdc_debug_sample), exactly the values the reference's rejection loop
// (draw again while the value repeats an earlier one of the step) accepts:
// the warp looks at 32 consecutive stream values at a time, keeps the first
// lane of each value (match_any) if its mark bit is clear, and accepts the
// fresh lanes in lane order until the step is full; the counter advances past
// the last accepted candidate only.  The n mark bits live in shared memory
// when they fit (cleared here), else in gmark (clear on entry); a step clears
// the bits it set.
template <bool kShared>
__global__ void k_tau_nice(uint64_t seed, int64_t n, int32_t tau, int32_t steps,
                           unsigned long long* counter, int32_t* S, uint32_t* gmark) {
  extern __shared__ uint32_t smark[];
  uint32_t* mark = kShared ? smark : gmark;
  const int lane = threadIdx.x & 31;
  if (kShared) {
    for (int64_t i = lane; i < (n + 31) / 32; i += 32) smark[i] = 0u;
    __syncwarp();
  }
  uint64_t k = *counter;
  for (int st = 0; st < steps; ++st) {
    int32_t* out = S + (int64_t)st * tau;
    int count = 0;
    while (count < tau) {
      const uint64_t kk = k + (uint64_t)lane;
      acdc_u32x4 o = acdc_philox4x32_10((uint32_t)kk, (uint32_t)(kk >> 32), ACDC_STREAM_SAMPLER, 0u,
                                        (uint32_t)seed, (uint32_t)(seed >> 32));
      const uint64_t u = ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
      const int32_t c = (int32_t)__umul64hi(u, (uint64_t)n);
      const unsigned same = __match_any_sync(ACDC_FULL_MASK, c);
      const bool first = (int)(__ffs(same) - 1) == lane;
      const uint32_t word = kShared ? mark[c >> 5] : __ldcg(mark + (c >> 5));
      const bool fresh = first && ((word >> (c & 31)) & 1u) == 0u;
      const unsigned fm = __ballot_sync(ACDC_FULL_MASK, fresh);
      const int need = tau - count;
      const int rank = __popc(fm & ((1u << lane) - 1u));
      if (fresh && rank < need) {
        out[count + rank] = c;
        atomicOr(mark + (c >> 5), 1u << (c & 31));
      }
      if (__popc(fm) >= need) {
        // the step fills at the need-th fresh lane: later candidates stay unused
        const unsigned lastm = __ballot_sync(ACDC_FULL_MASK, fresh && rank == need - 1);
        k += (uint64_t)(__ffs(lastm));
        count = tau;
      } else {
        k += 32;
        count += __popc(fm);
      }
      __syncwarp();  // marks and draws visible to every lane
    }
    for (int i = lane; i < tau; i += 32) {
      const int32_t c = out[i];
      atomicAnd(mark + (c >> 5), ~(1u << (c & 31)));
    }
    __syncwarp();
  }
  if (lane == 0) *counter = k;
}

// Sum of a full warp, in every lane.
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(ACDC_FULL_MASK, v, o);
  return v;
}

// Threads per block of the mini-batch phases: one block per drawn sample,
// each thread taking 4 entries of every 4 * kPhaseThreads (one 128-bit load of
// values and one of row indices per round).
constexpr int kPhaseThreads = 128;

// Values and row indices of entries e..e+3 of a column (zero past len).
__device__ __forceinline__ Chunk entries4(const UpdateParams& p, uint64_t start, uint32_t len,
                                          uint32_t e) {
  Chunk c;
  if (e < len) {
    c.v = __ldcs(reinterpret_cast<const float4*>(p.vals + start + e));
    c.i = __ldcs(reinterpret_cast<const int4*>(p.idx + start + e));
  } else {
    c.v = make_float4(0.f, 0.f, 0.f, 0.f);
    c.i = make_int4(0, 0, 0, 0);
  }
  return c;
}

// Phase 1: block i computes delta_i = clip((1 - y g) lambda n Li, -a, 1 - a),
// g = x_i^T w, for the i-th coordinate of the step, from w as the step found
// it (MulticoreSVMDualLoss.h:119-141); the block's partial sums meet in shared
// memory.
template <typename T>
__global__ void __launch_bounds__(kPhaseThreads) k_sdca_phase1(UpdateParams p, const int32_t* S,
                                                               int32_t tau, T* dout) {
  __shared__ T part[kPhaseThreads / 32];
  const int lane = threadIdx.x & 31;
  const int32_t j = S[blockIdx.x];
  const int4 mt = __ldg(p.meta + j);
  const T* r = reinterpret_cast<const T*>(sizeof(T) == 8 ? (const void*)p.r64 : (const void*)p.r);
  T xj = T(0);  // read with the entries, used after the reduction
  if (threadIdx.x == 0) {
    if constexpr (sizeof(T) == 8)
      xj = __ldcg(p.x64 + j);
    else
      xj = __ldcg(p.x32 + j);
  }
  const uint64_t start = (uint64_t)(uint32_t)mt.x << 2;
  const uint32_t len = (uint32_t)mt.y;
  T acc = T(0);
  for (uint32_t base = 0; base < len; base += 4u * kPhaseThreads) {
    const uint32_t e = base + 4u * threadIdx.x;
    const Chunk c = entries4(p, start, len, e);
    acc += gather_dot_head<ACDC_LOSS_SVM_DUAL, T>(r, c, e, len);
  }
  acc = warp_sum(acc);
  if (lane == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    T g = T(0);
#pragma unroll
    for (int w = 0; w < kPhaseThreads / 32; ++w) g += part[w];
    const T li = (T)__int_as_float(mt.z) * (T)p.li_scale;
    const T y = li < T(0) ? T(-1) : T(1);
    T delta = (T(1) - g * y) * (T)p.lambda_d * fabs(li);
    if (delta < -xj)
      delta = -xj;
    else if (delta > T(1) - xj)
      delta = T(1) - xj;
    dout[blockIdx.x] = delta;
    atomicAdd(p.counters + CNT_NNZ_READ, (unsigned long long)len);
  }
}

// Phase 2: block i applies delta_i: alpha_i += delta_i (the coordinates of a
// step are distinct, so no other block writes it) and w += delta_i y_i/(lambda n)
// x_i with red.global.
template <typename T>
__global__ void __launch_bounds__(kPhaseThreads) k_sdca_phase2(UpdateParams p, const int32_t* S,
                                                               int32_t tau, const T* din) {
  const int32_t j = S[blockIdx.x];
  const T d = din[blockIdx.x];
  if (threadIdx.x == 0) atomicAdd(p.counters + CNT_UPDATES, 1ull);
  if (d == T(0)) return;
  T* r = reinterpret_cast<T*>(sizeof(T) == 8 ? (void*)p.r64 : (void*)p.r);
  const int4 mt = __ldg(p.meta + j);
  const uint64_t start = (uint64_t)(uint32_t)mt.x << 2;
  const uint32_t len = (uint32_t)mt.y;
  const T y = __int_as_float(mt.z) < 0.f ? T(-1) : T(1);
  const T coef = d * y * (T)p.inv_lambda_n_d;
  for (uint32_t base = 0; base < len; base += 4u * kPhaseThreads) {
    const uint32_t e = base + 4u * threadIdx.x;
    if (e < len) scatter_head<T>(r, entries4(p, start, len, e), coef, e, len);
  }
  if (threadIdx.x == 0) {
    if constexpr (sizeof(T) == 8)
      p.x64[j] = p.x64[j] + d;
    else
      p.x32[j] = p.x32[j] + d;
    atomicAdd(p.counters + CNT_NONZERO, 1ull);
    atomicAdd(p.counters + CNT_NNZ_SCATTERED, (unsigned long long)len);
  }
}

// The sampler's uniform draw with a 64-bit result, so the stream can be checked
// for any n (problems themselves hold fewer than 2^31 coordinates).
__global__ void k_debug_sample(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                               int64_t* out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t k = k0 + i;
    acdc_u32x4 o = acdc_philox4x32_10((uint32_t)k, (uint32_t)(k >> 32), ACDC_STREAM_SAMPLER, 0u,
                                      (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t u = ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
    out[i] = (int64_t)__umul64hi(u, (uint64_t)n);
  }
}

}  // namespace

cudaError_t launch_debug_sample(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                                int64_t* out, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const uint64_t blocks = (count + 255) / 256 < 1024 ? (count + 255) / 256 : 1024;
  k_debug_sample<<<(unsigned)blocks, 256, 0, st>>>(seed, k0, count, n, out);
  return cudaGetLastError();
}

template <int G>
void launch_grouped(const UpdateParams& p, uint64_t k_base, dim3 grid, dim3 block,
                    cudaStream_t st) {
#define ACDC_LAUNCH(L, T) k_pcdm_update_grouped<L, T, G><<<grid, block, 0, st>>>(p, k_base)
  if (p.fp64) {
    switch (p.loss) {
      case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, double); break;
      case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, double); break;
      case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, double); break;
      default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, double); break;
    }
  } else {
    switch (p.loss) {
      case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, float); break;
      case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, float); break;
      case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, float); break;
      default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, float); break;
    }
  }
#undef ACDC_LAUNCH
}

cudaError_t launch_update(const UpdateParams& p, uint64_t k_base, int warps_per_block,
                          cudaStream_t st) {
  if (p.count == 0 || p.n_warps <= 0) return cudaSuccess;
  if (warps_per_block < 1) warps_per_block = 1;
  if (warps_per_block > kMaxWarps) warps_per_block = kMaxWarps;
  cudaError_t e = cudaMemsetAsync(p.counters + CNT_WORK, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  if (p.lanes == 8 || p.lanes == 16 || p.lanes == 32) {
    // tau updates in flight, 32 / lanes of them per warp; the warps are spread
    // over every SM (blocks of fewer warps when there are few of them) so that
    // the SMs' load/store units and L1 miss queues all take part
    const int64_t warps = ((int64_t)p.n_warps * p.lanes + 31) / 32;
    if (p.sm_count > 0) {
      const int64_t spread = (warps + p.sm_count - 1) / p.sm_count;
      if (spread < warps_per_block) warps_per_block = (int)(spread > 0 ? spread : 1);
    }
    const int64_t blocks = (warps + warps_per_block - 1) / warps_per_block;
    const dim3 grid((unsigned)blocks), block(warps_per_block * 32);
    if (p.lanes == 8)
      launch_grouped<8>(p, k_base, grid, block, st);
    else if (p.lanes == 16)
      launch_grouped<16>(p, k_base, grid, block, st);
    else
      launch_grouped<32>(p, k_base, grid, block, st);
    return cudaGetLastError();
  }
  const int blocks = (p.n_warps + warps_per_block - 1) / warps_per_block;
  dim3 grid(blocks), block(warps_per_block * 32);
  // the lean kernel for every launch (lanes 1) or for the q-shrinking ones (0)
  const bool lean = p.lanes == 1 || (p.lanes == 0 && p.shrink_q32 != 0);
  if (lean) {
#define ACDC_LAUNCH(L, T) k_pcdm_update_lean<L, T><<<grid, block, 0, st>>>(p, k_base)
    if (p.fp64) {
      switch (p.loss) {
        case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, double); break;
        case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, double); break;
        case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, double); break;
        default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, double); break;
      }
    } else {
      switch (p.loss) {
        case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, float); break;
        case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, float); break;
        case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, float); break;
        default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, float); break;
      }
    }
#undef ACDC_LAUNCH
    return cudaGetLastError();
  }
#define ACDC_LAUNCH(L, T) k_pcdm_update<L, T><<<grid, block, 0, st>>>(p, k_base)
  if (p.fp64) {
    switch (p.loss) {
      case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, double); break;
      case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, double); break;
      case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, double); break;
      default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, double); break;
    }
  } else {
    switch (p.loss) {
      case ACDC_LOSS_L1_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L1_SQUARE, float); break;
      case ACDC_LOSS_L2_SQUARE: ACDC_LAUNCH(ACDC_LOSS_L2_SQUARE, float); break;
      case ACDC_LOSS_SVM_DUAL: ACDC_LAUNCH(ACDC_LOSS_SVM_DUAL, float); break;
      default: ACDC_LAUNCH(ACDC_LOSS_LOGISTIC, float); break;
    }
  }
#undef ACDC_LAUNCH
  return cudaGetLastError();
}

cudaError_t launch_tau_nice(uint64_t seed, int64_t n, int32_t tau, int32_t steps,
                            unsigned long long* counter, int32_t* S, uint32_t* mark,
                            cudaStream_t st) {
  if (steps <= 0 || tau <= 0) return cudaSuccess;
  const int64_t words = (n + 31) / 32;
  if (words * 4 <= 48 * 1024)
    k_tau_nice<true><<<1, 32, (size_t)words * 4, st>>>(seed, n, tau, steps, counter, S, mark);
  else
    k_tau_nice<false><<<1, 32, 0, st>>>(seed, n, tau, steps, counter, S, mark);
  return cudaGetLastError();
}

cudaError_t launch_minibatch_step(const UpdateParams& p, const int32_t* S, int32_t tau, void* delta,
                                  cudaStream_t st) {
  if (tau <= 0) return cudaSuccess;
  // one block per drawn sample
  const dim3 grid((unsigned)tau), block(kPhaseThreads);
  if (p.fp64) {
    k_sdca_phase1<double><<<grid, block, 0, st>>>(p, S, tau, static_cast<double*>(delta));
    k_sdca_phase2<double><<<grid, block, 0, st>>>(p, S, tau, static_cast<const double*>(delta));
  } else {
    k_sdca_phase1<float><<<grid, block, 0, st>>>(p, S, tau, static_cast<float*>(delta));
    k_sdca_phase2<float><<<grid, block, 0, st>>>(p, S, tau, static_cast<const float*>(delta));
  }
  return cudaGetLastError();
}

cudaError_t launch_batch_update(const BatchDev& b, int update_blocks, cudaStream_t st) {
  if (update_blocks <= 0) return cudaSuccess;
  const dim3 grid(update_blocks), block(kMaxWarps * 32);
  k_pcdm_update_batch<<<grid, block, 0, st>>>(b);
  return cudaGetLastError();
}

// Four 37 KB (ring) or 48 KB (lean) blocks per SM need the shared-memory side
// of the L1 carveout.
cudaError_t update_kernels_init() {
  const int carve = cudaSharedmemCarveoutMaxShared;
  const cudaFuncAttribute a = cudaFuncAttributePreferredSharedMemoryCarveout;
  cudaError_t e = cudaSuccess;
#define ACDC_CARVE(L, T) \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pcdm_update<L, T>, a, carve)
  ACDC_CARVE(ACDC_LOSS_L1_SQUARE, float);
  ACDC_CARVE(ACDC_LOSS_L1_SQUARE, double);
  ACDC_CARVE(ACDC_LOSS_SVM_DUAL, float);
  ACDC_CARVE(ACDC_LOSS_SVM_DUAL, double);
  ACDC_CARVE(ACDC_LOSS_L2_SQUARE, float);
  ACDC_CARVE(ACDC_LOSS_L2_SQUARE, double);
  ACDC_CARVE(ACDC_LOSS_LOGISTIC, float);
  ACDC_CARVE(ACDC_LOSS_LOGISTIC, double);
#undef ACDC_CARVE
#define ACDC_CARVE_LEAN(L, T) \
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pcdm_update_lean<L, T>, a, carve)
  ACDC_CARVE_LEAN(ACDC_LOSS_L1_SQUARE, float);
  ACDC_CARVE_LEAN(ACDC_LOSS_L1_SQUARE, double);
  ACDC_CARVE_LEAN(ACDC_LOSS_SVM_DUAL, float);
  ACDC_CARVE_LEAN(ACDC_LOSS_SVM_DUAL, double);
  ACDC_CARVE_LEAN(ACDC_LOSS_L2_SQUARE, float);
  ACDC_CARVE_LEAN(ACDC_LOSS_L2_SQUARE, double);
  ACDC_CARVE_LEAN(ACDC_LOSS_LOGISTIC, float);
  ACDC_CARVE_LEAN(ACDC_LOSS_LOGISTIC, double);
#undef ACDC_CARVE_LEAN
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pcdm_update_batch, a, carve);
  return e;
}

// PCDM coordinate-update kernel (sm_103a).
//
// Replaces MulticoreEngineExecutor::executeBulkOfIterations
// (cpp/src/solver/MulticoreEngineExecutor.h:83-89) and the per-coordinate
// updates MulticoreL1RegSquareLoss::performOneCoordinateUpdate
// (cpp/src/solver/lossFunctions/squareLoss/MulticoreL1RegSquareLoss.h:41-63) and
// MulticoreSVMDualLoss::performOneCoordinateUpdate
// (cpp/src/solver/lossFunctions/SVMDualLoss/MulticoreSVMDualLoss.h:119-141).
//
// tau warps run concurrently; each warp repeatedly takes 32 update numbers from
// a global work counter and performs those updates one after another:
//   j      = sampler(seed, k)                         (Philox, see acdc_philox.h)
//   g      = a_j^T r                                  (lanes gather, shuffle reduce)
//   delta  = Lasso: S(lambda Li, x_j - Li g) - x_j    (treshhold_functions.h:27-33)
//            SVM:   clip((1 - y_j g) lambda n Li, -a_j, 1 - a_j)
//   x_j   += delta;  r += c delta a_j                 (red.global.add.f32)
// with Li = 1/(beta ||a_j||^2), beta the ESO parameter for tau.  Reads of r and
// x go to L2 (ld.global.cg) so they observe other warps' reductions; the column
// entries are streamed with evict-first loads.  The column metadata of the
// next two updates and the first 128 entries of the next column are loaded
// while the current update waits on its gathers.
#include "acdc_internal.cuh"

namespace {

constexpr int kChunk = 32;  // updates taken from the work counter at a time

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(ACDC_FULL_MASK, v, o);
  return v;  // identical in every lane: each butterfly step adds the same pair
}

__device__ __forceinline__ int64_t draw_coord(const UpdateParams& p, uint64_t k,
                                              int32_t active_cnt) {
  acdc_u32x4 o = acdc_philox4x32_10((uint32_t)k, (uint32_t)(k >> 32), ACDC_STREAM_SAMPLER, 0u,
                                    (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
  if (active_cnt > 0 && o.v[2] < p.shrink_q32) {
    uint32_t t = __umulhi(o.v[3], (uint32_t)active_cnt);
    return (int64_t)__ldg(p.active + t);
  }
  uint64_t u = ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
  return (int64_t)__umul64hi(u, (uint64_t)p.n);
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

__device__ __forceinline__ float gather_dot(const float* r, const Chunk& c, bool live) {
  if (!live) return 0.f;
  float a = c.v.x * __ldcg(r + c.i.x);
  a = fmaf(c.v.y, __ldcg(r + c.i.y), a);
  a = fmaf(c.v.z, __ldcg(r + c.i.z), a);
  a = fmaf(c.v.w, __ldcg(r + c.i.w), a);
  return a;
}

__device__ __forceinline__ void scatter(float* r, const Chunk& c, float coef, bool live) {
  if (!live) return;
  if (c.v.x != 0.f) atomicAdd(r + c.i.x, coef * c.v.x);
  if (c.v.y != 0.f) atomicAdd(r + c.i.y, coef * c.v.y);
  if (c.v.z != 0.f) atomicAdd(r + c.i.z, coef * c.v.z);
  if (c.v.w != 0.f) atomicAdd(r + c.i.w, coef * c.v.w);
}

template <int LOSS>
__global__ void __launch_bounds__(256, 4) k_pcdm_update(UpdateParams p, uint64_t k_base) {
  const int lane = threadIdx.x & 31;
  const int64_t gwarp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gwarp >= p.n_warps) return;
  unsigned long long* work = p.counters + CNT_WORK;
  const int32_t active_cnt =
      p.shrink_q32 ? (int32_t)min(p.counters[CNT_ACTIVE], (unsigned long long)p.n) : 0;
  unsigned long long n_upd = 0, n_nz = 0, n_read = 0, n_scat = 0;

  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, (unsigned long long)kChunk);
    base = __shfl_sync(ACDC_FULL_MASK, base, 0);
    if (base >= p.count) break;
    const int cnt = (int)min((unsigned long long)kChunk, p.count - base);
    int64_t my_j = 0;
    if (lane < cnt) my_j = draw_coord(p, k_base + base + (uint64_t)lane, active_cnt);

    // Pipeline prologue: meta of updates 0 and 1, entries of update 0.
    int64_t j_c = __shfl_sync(ACDC_FULL_MASK, my_j, 0);
    int4 mt_c = __ldcg(p.meta + j_c);
    int64_t j_n = __shfl_sync(ACDC_FULL_MASK, my_j, 1 & 31);
    int4 mt_n = make_int4(0, 0, 0, 0);
    if (cnt > 1) mt_n = __ldcg(p.meta + j_n);
    Chunk c_c = load_chunk(p, (uint64_t)(uint32_t)mt_c.x << 2, (uint32_t)mt_c.y, 0u, lane);

    for (int u = 0; u < cnt; ++u) {
      // Prefetch: entries of update u+1, meta of update u+2.
      Chunk c_n = {make_float4(0.f, 0.f, 0.f, 0.f), make_int4(0, 0, 0, 0)};
      if (u + 1 < cnt)
        c_n = load_chunk(p, (uint64_t)(uint32_t)mt_n.x << 2, (uint32_t)mt_n.y, 0u, lane);
      const int64_t j_nn = __shfl_sync(ACDC_FULL_MASK, my_j, (u + 2) & 31);
      int4 mt_nn = make_int4(0, 0, 0, 0);
      if (u + 2 < cnt) mt_nn = __ldcg(p.meta + j_nn);

      // Update u: g = a_j^T r.
      const uint64_t start = (uint64_t)(uint32_t)mt_c.x << 2;
      const uint32_t len = (uint32_t)mt_c.y;
      float acc = gather_dot(p.r, c_c, 4u * (uint32_t)lane < len);
      if (len > 128u) {
        Chunk a = load_chunk(p, start, len, 128u, lane);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk b = load_chunk(p, start, len, off + 128u, lane);
          acc += gather_dot(p.r, a, off + 4u * (uint32_t)lane < len);
          a = b;
        }
      }
      const float g = warp_sum(acc);

      const float li = __int_as_float(mt_c.z);
      const float xj = __int_as_float(mt_c.w);
      float delta, coef;
      if (LOSS == ACDC_LOSS_L1_SQUARE) {
        const float z = xj - li * g;
        float a = fabsf(z) - p.lambda * li;
        a = a < 0.f ? 0.f : a;
        const float xn = z > 0.f ? a : (z < 0.f ? -a : 0.f);
        delta = xn - xj;
        coef = delta;
      } else {
        const float y = li < 0.f ? -1.f : 1.f;
        delta = (1.f - g * y) * p.lambda * fabsf(li);
        if (delta < -xj)
          delta = -xj;
        else if (delta > 1.f - xj)
          delta = 1.f - xj;
        coef = delta * y * p.inv_lambda_n;
      }
      n_upd++;
      n_read += len;
      if (delta != 0.f) {
        n_nz++;
        n_scat += len;
        scatter(p.r, c_c, coef, 4u * (uint32_t)lane < len);
        for (uint32_t off = 128u; off < len; off += 128u) {
          Chunk a = load_chunk(p, start, len, off, lane);
          scatter(p.r, a, coef, off + 4u * (uint32_t)lane < len);
        }
        if (lane == 0) atomicAdd(reinterpret_cast<float*>(&p.meta[j_c].w), delta);
        // The prefetched meta of the next two updates predates this write.
        const int xn_bits = __float_as_int(xj + delta);
        if (j_n == j_c) mt_n.w = xn_bits;
        if (j_nn == j_c) mt_nn.w = xn_bits;
      }
      j_c = j_n;
      mt_c = mt_n;
      c_c = c_n;
      j_n = j_nn;
      mt_n = mt_nn;
    }
  }
  if (lane == 0) {
    atomicAdd(p.counters + CNT_UPDATES, n_upd);
    atomicAdd(p.counters + CNT_NONZERO, n_nz);
    atomicAdd(p.counters + CNT_NNZ_READ, n_read);
    atomicAdd(p.counters + CNT_NNZ_SCATTERED, n_scat);
  }
}

__global__ void k_debug_sample(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                               int64_t* out) {
  UpdateParams p;
  p.seed = seed;
  p.n = n;
  p.shrink_q32 = 0;
  p.active = nullptr;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    out[i] = draw_coord(p, k0 + i, 0);
}

}  // namespace

cudaError_t launch_debug_sample(uint64_t seed, uint64_t k0, uint64_t count, int64_t n,
                                int64_t* out, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const uint64_t blocks = (count + 255) / 256 < 1024 ? (count + 255) / 256 : 1024;
  k_debug_sample<<<(unsigned)blocks, 256, 0, st>>>(seed, k0, count, n, out);
  return cudaGetLastError();
}

cudaError_t launch_update(const UpdateParams& p, uint64_t k_base, int warps_per_block,
                          cudaStream_t st) {
  if (p.count == 0 || p.n_warps <= 0) return cudaSuccess;
  if (warps_per_block < 1) warps_per_block = 1;
  if (warps_per_block > 8) warps_per_block = 8;
  cudaError_t e = cudaMemsetAsync(p.counters + CNT_WORK, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  const int blocks = (p.n_warps + warps_per_block - 1) / warps_per_block;
  dim3 grid(blocks), block(warps_per_block * 32);
  if (p.loss == ACDC_LOSS_SVM_DUAL)
    k_pcdm_update<ACDC_LOSS_SVM_DUAL><<<grid, block, 0, st>>>(p, k_base);
  else
    k_pcdm_update<ACDC_LOSS_L1_SQUARE><<<grid, block, 0, st>>>(p, k_base);
  return cudaGetLastError();
}

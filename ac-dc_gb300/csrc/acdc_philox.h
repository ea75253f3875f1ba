/*
 * Counter-based random numbers shared by the device sampler and the host
 * generators: Philox4x32-10 from J. Salmon, M. Moraes, R. Dror, D. Shaw,
 * "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11).  A 128-bit counter
 * and a 64-bit key give four 32-bit outputs; ten rounds of two 32x32->64
 * multiplies with a Weyl-sequence key schedule.
 *
 * The coordinate sampler replaces the reference's per-thread GSL mt19937
 * stream (`gsl_rng_uniform_int(gsl_rng_r, n)`,
 * cpp/src/solver/MulticoreEngineExecutor.h:86, seeded in
 * cpp/src/utils/randomNumbersUtil.h:83-125).  Update number k of a solve
 * draws coordinate acdc_sample_coord(seed, k, n): any warp can compute the
 * k-th draw without shared state, so the RNG state of a solve is just
 * (seed, k).
 */
#ifndef ACDC_PHILOX_H_
#define ACDC_PHILOX_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define ACDC_HD __host__ __device__ __forceinline__
#else
#define ACDC_HD static inline
#endif

#define ACDC_PHILOX_M0 0xD2511F53u
#define ACDC_PHILOX_M1 0xCD9E8D57u
#define ACDC_PHILOX_W0 0x9E3779B9u
#define ACDC_PHILOX_W1 0xBB67AE85u

/* Stream identifiers (third counter word) so that independent purposes never
 * share a counter. */
enum {
  ACDC_STREAM_SAMPLER = 0x5A3D0001u,
  ACDC_STREAM_SHRINK = 0x5A3D0002u,
  ACDC_STREAM_GEN_NNZ = 0x6E000001u,
  ACDC_STREAM_GEN_ROWS = 0x6E000002u,
  ACDC_STREAM_GEN_VALS = 0x6E000003u,
  ACDC_STREAM_GEN_XSTAR = 0x6E000004u,
  ACDC_STREAM_GEN_NOISE = 0x6E000005u,
  ACDC_STREAM_GEN_LABEL = 0x6E000006u,
  ACDC_STREAM_GEN_SIZE = 0x6E000007u
};

typedef struct acdc_u32x4 {
  uint32_t v[4];
} acdc_u32x4;

ACDC_HD void acdc_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

ACDC_HD acdc_u32x4 acdc_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                       uint32_t k0, uint32_t k1) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    acdc_mulhilo32(ACDC_PHILOX_M0, c0, &hi0, &lo0);
    acdc_mulhilo32(ACDC_PHILOX_M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += ACDC_PHILOX_W0;
    k1 += ACDC_PHILOX_W1;
  }
  acdc_u32x4 out;
  out.v[0] = c0;
  out.v[1] = c1;
  out.v[2] = c2;
  out.v[3] = c3;
  return out;
}

/* 64 random bits for (seed, index, stream, sub). */
ACDC_HD uint64_t acdc_rand64(uint64_t seed, uint64_t index, uint32_t stream, uint32_t sub) {
  acdc_u32x4 o = acdc_philox4x32_10((uint32_t)index, (uint32_t)(index >> 32), stream, sub,
                                    (uint32_t)seed, (uint32_t)(seed >> 32));
  return ((uint64_t)o.v[0] << 32) | (uint64_t)o.v[1];
}

/* floor(u * n / 2^64): maps 64 random bits onto [0, n) with bias below n/2^64. */
ACDC_HD uint64_t acdc_scale64(uint64_t u, uint64_t n) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(u, n);
#else
  return (uint64_t)(((unsigned __int128)u * (unsigned __int128)n) >> 64);
#endif
}

/* Coordinate drawn by update number k of a solve with the given seed. */
ACDC_HD uint64_t acdc_sample_coord(uint64_t seed, uint64_t k, uint64_t n) {
  return acdc_scale64(acdc_rand64(seed, k, ACDC_STREAM_SAMPLER, 0u), n);
}

/* Uniform double in (0, 1]: 53 random bits, never zero (safe for log). */
ACDC_HD double acdc_u01(uint64_t bits) {
  return ((double)(bits >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

#endif /* ACDC_PHILOX_H_ */

/*
 * Minimal stand-in for GNU GSL's random-number interface, written from the
 * GSL API contract, so the reference's multicore engine compiles here without
 * GSL.  TEST INFRASTRUCTURE ONLY (used when building oracle/_ref).
 *
 * The generator is not mt19937: gsl_rng_uniform_int(r, n) returns the
 * counter-based draw orc_sample(seed, counter++, n) of pcdm_oracle.c, so the
 * reference engine visits exactly the coordinate sequence of the oracle and
 * of the GPU sampler.
 */
#ifndef ACDC_GSL_SHIM_RNG_H_
#define ACDC_GSL_SHIM_RNG_H_

#include <stdint.h>
#include <stdlib.h>

#include "../../pcdm_oracle.h"

typedef struct gsl_rng_type {
  const char* name;
} gsl_rng_type;

typedef struct gsl_rng {
  const gsl_rng_type* type;
  uint64_t seed;
  uint64_t counter;
} gsl_rng;

static const gsl_rng_type acdc_shim_rng_type = {"philox4x32-10-shim"};
static const gsl_rng_type* gsl_rng_default = &acdc_shim_rng_type;

static inline void gsl_rng_env_setup(void) {}

static inline gsl_rng* gsl_rng_alloc(const gsl_rng_type* T) {
  gsl_rng* r = (gsl_rng*)malloc(sizeof(gsl_rng));
  r->type = T;
  r->seed = 0;
  r->counter = 0;
  return r;
}

static inline void gsl_rng_free(gsl_rng* r) { free(r); }

static inline void gsl_rng_set(const gsl_rng* r, unsigned long s) {
  gsl_rng* w = (gsl_rng*)r;
  w->seed = (uint64_t)s;
  w->counter = 0;
}

static inline unsigned long gsl_rng_uniform_int(const gsl_rng* r, unsigned long n) {
  gsl_rng* w = (gsl_rng*)r;
  return (unsigned long)orc_sample(w->seed, w->counter++, (uint64_t)n);
}

static inline double gsl_rng_uniform(const gsl_rng* r) {
  gsl_rng* w = (gsl_rng*)r;
  uint64_t u = orc_sample(w->seed, w->counter++, (uint64_t)1 << 53);
  return (double)u * (1.0 / 9007199254740992.0);
}

#endif

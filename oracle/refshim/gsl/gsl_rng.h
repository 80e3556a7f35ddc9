/* Minimal stand-in for the two GSL RNG names Tint.c uses (Tint.c:79-93:
 * allocate a generator whose shuffle is commented out, then free it).
 * Test infrastructure for oracle/_ref only; GSL is not installed. */
#ifndef WLREF_GSL_RNG_H
#define WLREF_GSL_RNG_H
#include <stdlib.h>
typedef struct { int unused; } gsl_rng_type;
typedef struct { int unused; } gsl_rng;
static const gsl_rng_type wlref_mt19937_type = {0};
#define gsl_rng_mt19937 (&wlref_mt19937_type)
static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *t) {
  (void)t;
  return (gsl_rng *)malloc(sizeof(gsl_rng));
}
#endif

/* Test-infrastructure shim: the subset of GSL's RNG interface that the
 * reference's src/common.c:133-152 calls.  Backed by the oracle's MT19937. */
#ifndef SHIM_GSL_RNG_H
#define SHIM_GSL_RNG_H
typedef struct gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct gsl_rng gsl_rng;
extern const gsl_rng_type *gsl_rng_mt19937;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int s);
double gsl_rng_uniform(const gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
#endif

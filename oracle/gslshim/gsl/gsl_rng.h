/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). Only MT19937. */
#ifndef RLF_SHIM_GSL_RNG_H
#define RLF_SHIM_GSL_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char *name; } gsl_rng_type;
typedef struct { const gsl_rng_type *type; unsigned long mt[624]; int mti; } gsl_rng;
extern const gsl_rng_type *gsl_rng_mt19937;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(gsl_rng *r, unsigned long int seed);
unsigned long int gsl_rng_get(gsl_rng *r);
double gsl_rng_uniform(gsl_rng *r);
double gsl_rng_uniform_pos(gsl_rng *r);
unsigned long int gsl_rng_max(const gsl_rng *r);
unsigned long int gsl_rng_min(const gsl_rng *r);
void gsl_rng_free(gsl_rng *r);
#ifdef __cplusplus
}
#endif
#endif

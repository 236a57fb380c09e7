/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h).
 * The minimiser struct exposes the public fields the reference reads (x, fval, size). */
#ifndef RLF_SHIM_GSL_MULTIMIN_H
#define RLF_SHIM_GSL_MULTIMIN_H
#include "gsl_vector.h"
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  double (*f)(const gsl_vector *x, void *params);
  size_t n;
  void *params;
} gsl_multimin_function;

typedef struct gsl_multimin_fminimizer_type {
  const char *name;
  size_t size;
} gsl_multimin_fminimizer_type;

typedef struct {
  const gsl_multimin_fminimizer_type *type;
  gsl_multimin_function *f;
  double fval;
  gsl_vector *x;
  double size;
  void *state;
} gsl_multimin_fminimizer;

extern const gsl_multimin_fminimizer_type *gsl_multimin_fminimizer_nmsimplex2;
gsl_multimin_fminimizer *gsl_multimin_fminimizer_alloc(const gsl_multimin_fminimizer_type *T, size_t n);
int gsl_multimin_fminimizer_set(gsl_multimin_fminimizer *s, gsl_multimin_function *f,
                                const gsl_vector *x, const gsl_vector *step_size);
int gsl_multimin_fminimizer_iterate(gsl_multimin_fminimizer *s);
double gsl_multimin_fminimizer_size(const gsl_multimin_fminimizer *s);
void gsl_multimin_fminimizer_free(gsl_multimin_fminimizer *s);
int gsl_multimin_test_size(const double size, double epsabs);
#ifdef __cplusplus
}
#endif
#endif

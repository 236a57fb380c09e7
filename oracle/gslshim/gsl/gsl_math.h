/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). */
#ifndef RLF_SHIM_GSL_MATH_H
#define RLF_SHIM_GSL_MATH_H
#include <math.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
int gsl_finite(const double x);
#ifdef __cplusplus
}
#endif
#endif

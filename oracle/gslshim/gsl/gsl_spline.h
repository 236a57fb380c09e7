/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). */
#ifndef RLF_SHIM_GSL_SPLINE_H
#define RLF_SHIM_GSL_SPLINE_H
#include <stddef.h>
#include "gsl_errno.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char *name; int kind; } gsl_interp_type;
extern const gsl_interp_type *gsl_interp_linear;
extern const gsl_interp_type *gsl_interp_cspline;
typedef struct { size_t cache; size_t miss_count; size_t hit_count; } gsl_interp_accel;
typedef struct {
  const gsl_interp_type *type;
  size_t size;
  double *x;
  double *y;
  double *c;   /* second-derivative/2 coefficients (cspline) */
} gsl_spline;
gsl_interp_accel *gsl_interp_accel_alloc(void);
int gsl_interp_accel_reset(gsl_interp_accel *a);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size);
int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size);
int gsl_spline_eval_e(const gsl_spline *spline, double x, gsl_interp_accel *a, double *y);
double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *spline);
#ifdef __cplusplus
}
#endif
#endif

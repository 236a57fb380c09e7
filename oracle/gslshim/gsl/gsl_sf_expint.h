/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). */
#ifndef RLF_SHIM_GSL_SF_EXPINT_H
#define RLF_SHIM_GSL_SF_EXPINT_H
#include "gsl_sf_result.h"
#ifdef __cplusplus
extern "C" {
#endif
int gsl_sf_expint_Ei_e(const double x, gsl_sf_result *result);
double gsl_sf_expint_Ei(const double x);
#ifdef __cplusplus
}
#endif
#endif

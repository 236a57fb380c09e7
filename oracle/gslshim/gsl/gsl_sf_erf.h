/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). */
#ifndef RLF_SHIM_GSL_SF_ERF_H
#define RLF_SHIM_GSL_SF_ERF_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_erf(const double x);
#ifdef __cplusplus
}
#endif
#endif

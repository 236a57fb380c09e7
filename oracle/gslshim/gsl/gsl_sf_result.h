/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h). */
#ifndef RLF_SHIM_GSL_SF_RESULT_H
#define RLF_SHIM_GSL_SF_RESULT_H
typedef struct { double val; double err; } gsl_sf_result;
#endif

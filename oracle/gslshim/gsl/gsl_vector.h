/* Test infrastructure only (oracle): GSL-API subset (see gsl_errno.h).
 * gsl_vector keeps GSL's public field order (size, stride, data, block, owner). */
#ifndef RLF_SHIM_GSL_VECTOR_H
#define RLF_SHIM_GSL_VECTOR_H
#include <stddef.h>
#include <stdio.h>  /* GSL's vector header brings in stdio (reference files rely on it) */
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { size_t size; double *data; } gsl_block;
typedef struct {
  size_t size;
  size_t stride;
  double *data;
  gsl_block *block;
  int owner;
} gsl_vector;
gsl_vector *gsl_vector_alloc(const size_t n);
void gsl_vector_free(gsl_vector *v);
double gsl_vector_get(const gsl_vector *v, const size_t i);
void gsl_vector_set(gsl_vector *v, const size_t i, double x);
void gsl_vector_set_all(gsl_vector *v, double x);
int gsl_vector_memcpy(gsl_vector *dest, const gsl_vector *src);
#ifdef __cplusplus
}
#endif
#endif

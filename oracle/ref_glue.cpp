/*
 * Test infrastructure only (oracle/_ref).  Compiled together with the reference's own hot-path
 * sources (read in place from the reference checkout, never copied) by oracle/Makefile's `ref`
 * target.  marginalise_r.h declares its functions without extern "C" (marginalise_r.h:24-27),
 * so they carry C++ linkage in the reference build; these wrappers give them C names that
 * ctypes can bind.
 */
#include "datatype.h"
#include "marginalise_r.h"

extern "C" {
void rlfref_set_posterior_values(int numR, double *L_r, double *rprior, double *Ro, double *xmarvals,
                                 double *ymarvals, int *numvals) {
  set_posterior_values(numR, L_r, rprior, Ro, xmarvals, ymarvals, numvals);
}
double rlfref_marginalise_posterior_r(int num_marvals, double *xmarvals, double *ymarvals) {
  return marginalise_posterior_r(num_marvals, xmarvals, ymarvals);
}
unsigned long rlfref_sizeof_likelihood_params(void) { return sizeof(likelihood_params); }
}

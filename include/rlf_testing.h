/*
 * Testing and debugging aids of librlf_gb300.so.  No counterpart in the reference and not part of
 * the production API (include/rlf_gb300.h): the parity tests call them to look inside the fit (the
 * likelihood at every evaluation, the per-node log-likelihoods, the double-float functions).
 * Plain C types only; likelihood_params is the layout of datatype.h:49-74
 * (include/rlf_reference_abi.h).
 */
#ifndef RLF_TESTING_H
#define RLF_TESTING_H

#ifdef __cplusplus
extern "C" {
#endif

/* Debugging aid: source_fitting of one facet given as likelihood_params (datatype.h:49-74) in
 * the given precision, recording (e1, e2, L, error) of every likelihood evaluation into
 * trace[cap][4]; out6 = (e1, e2, simplex max e1, max e2, maxL, evaluations). */
int rlf_debug_fit_trace(void *likelihood_params_facet, double *trace, int cap, double *out6,
                        int precision);
/* Debugging aid: one loglikelihood evaluation of a facet in the given precision; out2 = (L, error),
 * node_L[1..numr-1] = the per-scalelength-node log-likelihoods before the marginalisation. */
int rlf_debug_loglike_nodes(void *likelihood_params_facet, double e1, double e2, int precision,
                            double *out2, double *node_L);
/* Testing aid (no counterpart in the reference): the fit's double-float functions on n inputs,
 * out[i] = f(x[i]) (or x[i] / y[i]) evaluated in float pairs and returned as doubles; op 0 exp,
 * 1 log (inputs in the float range), 2 log of any positive normal double, 3 x / y, 4 sqrt,
 * 5 (1 + x)^(-3/2), 6 the integer split of a double into a float pair.  Returns nonzero on error. */
int rlf_debug_df_math(int op, int n, const double *x, const double *y, double *out);
#ifdef __cplusplus
}
#endif
#endif /* RLF_TESTING_H */

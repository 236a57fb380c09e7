/*
 * Drop-in C ABI of RadioLensfit2's per-galaxy shape-measurement hot path, GB300 build.
 *
 * Every function here keeps the name, argument list and meaning of the reference's FACET build
 * (Makefile:10 always defines FACET), so a program compiled against the reference headers
 * links against librlf_gb300.so instead of likelihood.o, galaxy_visibilities.o, marginalise_r.o,
 * source_extraction.o, evaluate_uv_grid.o, galaxy_fitting.o and data_processing.o.
 * All pointers are host pointers owned by the caller, as in the reference; each call copies
 * its inputs to the GPU, runs there and copies its outputs back.  Array-valued functions run as
 * CUDA kernels; the scalar helpers (facet_size, the two shapes, marginalise_over_position_shift,
 * marf) are the same __host__ __device__ code evaluated on the host.
 *
 * Differences a caller can observe (all documented, none on the results):
 *   - visGal is scratch: source_extraction does not leave the shifted visibilities in it
 *     (data_processing.c never reads them back);
 *   - loglikelihood does not leave the per-scalelength models in par->mod;
 *   - evaluate_uv_grid_size counts cells of this process only (the MPI reduction over ranks,
 *     evaluate_uv_grid.c:85-104, belongs to the multi-rank driver);
 *   - marginalise_posterior_r returns -1e10 where the reference exits the process
 *     (xmax <= xmin, marginalise_r.c:117-123).
 */
#ifndef RLF_REFERENCE_ABI_H
#define RLF_REFERENCE_ABI_H

#include <stdio.h>
#include <stddef.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifndef DATATYPE_H_
/* datatype.h:44-47 */
typedef struct {
  double real;
  double imag;
} complexd;

/* datatype.h:49-74, FACET branch */
typedef struct {
  int numr;
  double *ro;
  double *rprior;
  unsigned int nchannels;
  double band_factor;
  double acc_time;
  double *spec;
  double *wavenumbers;
  double *uu;
  double *vv;
  double l0;
  double m0;
  complexd *data;
  double *sigma2;
  double *mod;
  unsigned int facet;
  unsigned int ncoords;
} likelihood_params;
#endif

/* GSL's public gsl_vector layout; f_likelihood reads data[0] and data[stride]. */
struct rlf_gsl_vector_layout {
  size_t size;
  size_t stride;
  double *data;
  void *block;
  int owner;
};

#ifdef __cplusplus
extern "C" {
#endif

/* evaluate_uv_grid.h:29-33 (evaluate_uv_grid.c:50-230) */
unsigned int facet_size(double theta_med, double len);
unsigned int evaluate_uv_grid_size(int rank, int nprocs, double len, double *wavenumbers,
                                   unsigned int num_channels, unsigned int ncoords, double *u,
                                   double *v, unsigned int sizeg, bool *flag);
unsigned int evaluate_facet_coords(double *grid_u, double *grid_v, double len, unsigned int sizeg,
                                   double *count_w);
void gridding_visibilities(double *wavenumbers, unsigned int num_channels, unsigned int ncoords,
                           double *u, double *v, complexd *vis, float *sigma2, double len,
                           unsigned int sizeg, complexd *new_vis, double *new_sigma2, bool *flag,
                           double *sum_w);
void average_facets(unsigned long int size, complexd *grid_vis, double *grid_sigma2, double *sum_w);

/* galaxy_visibilities.h:31-55 (galaxy_visibilities.c:40-270) */
double gaussian_shape(double k1, double k2, double scale_factor, double wave_factor);
double sersic_shape(double k1, double k2, double scale_factor, double wave_factor);
void model_galaxy_visibilities_at_zero(double e1, double e2, double scale, unsigned int num_coords,
                                       double *grid_u, double *grid_v, const double *sigma2,
                                       double *Modvis);
void data_galaxy_visibilities(double spectra, double wavenumber, double band_factor,
                              double acc_time, double e1, double e2, double scale, double flux,
                              double l, double m, unsigned int num_coords, double *uu_metres,
                              double *vv_metres, double *ww_metres, complexd *vis);
void data_visibilities_phase_shift(double wavenumber, double l, double m, unsigned int num_coords,
                                   double *uu_metres, double *vv_metres, double *ww_metres,
                                   complexd *vis);

/* likelihood.h:32-54 (likelihood.c:87-554) */
double f_likelihood(const struct rlf_gsl_vector_layout *v, void *params);
double loglikelihood(void *params, double ee1, double ee2, int *error);
double loglikelihood_r(double ee1, double ee2, double scale, unsigned long int n_uv_coords,
                       const double *variance, double *grid_u, double *grid_v, complexd *visData,
                       double *visM);
int cross_correlation(unsigned long int n_uv_coords, double *grid_u, double *grid_v,
                      complexd *visData, double *visMod, double *ho, double *det_sigma);
double marginalise_over_position_shift(double x);
void likelihood_sampling(double *mes_e1, double *mes_e2, double maxL, void *params, int np_max,
                         double *var_e1, double *var_e2, double *oneDimvar);

/* source_extraction.h:31-34 (source_extraction.c:36-68) */
void source_extraction(int rank, unsigned int facet, likelihood_params *par, complexd *facet_vis,
                       double *facet_sigma2, double *sum_w, double l0, double m0, double flux,
                       double mu, double e1, double e2, complexd *visSkyMod, complexd *visData,
                       complexd *visGal, float *sigma2_vis, bool *flag, unsigned long int num_coords,
                       double *uu_metres, double *vv_metres, double *ww_metres, double len);

/* galaxy_fitting.h:30 (galaxy_fitting.c:41-117) */
int source_fitting(int rank, likelihood_params *par, double *mes_e1, double *mes_e2,
                   double *var_e1, double *var_e2, double *oneDimvar, double *maxL);

/* data_processing.h:43-46 (data_processing.c:47-147) */
void data_processing(bool re_fitting, unsigned int *bad_list, int nsources, double len,
                     unsigned int num_coords, FILE *pFile, likelihood_params *par, double *l,
                     double *m, double *gflux, double *gscale, double *ge1, double *ge2,
                     double *SNR_vis, double *sum_w, complexd *visGal, complexd *visSkyMod,
                     complexd *visData, float *sigma2_vis, bool *flag, double *uu_metres,
                     double *vv_metres, double *ww_metres, double *fitting_time, int *bad);

/* data_simulation.h:36-38 (data_simulation.c:131-165) */
void sky_model(double *wavenumbers, double *spec, double channel_bandwidth_hz, int time_acc,
               unsigned int num_channels, unsigned int n_gal, double *gflux, double *gscale,
               double *l, double *m, unsigned long int num_coords, double *uu_metres,
               double *vv_metres, double *ww_metres, complexd *visGal, complexd *visMod);

/* distributions.h:28-30 (distributions.c:59-87): the prior of the fit */
double rfunc(const double mu, const double sigma, double r);
double scale_mean(double flux);

/* marginalise_r.h:24-27 (marginalise_r.c:29-238) declares these without extern "C"; the
 * library exports them under C++ linkage with exactly those signatures, and under C linkage
 * with an rlf_ prefix for C and FFI callers. */
void rlf_set_posterior_values(int numR, double *L_r, double *rprior, double *Ro, double *xmarvals,
                              double *ymarvals, int *numvals);
double rlf_marginalise_posterior_r(int num_marvals, double *xmarvals, double *ymarvals);
double rlf_marf(double x, void *params);

#ifdef __cplusplus
}
void set_posterior_values(int numR, double *L_r, double *rprior, double *Ro, double *xmarvals,
                          double *ymarvals, int *numvals);
double marginalise_posterior_r(int num_marvals, double *xmarvals, double *ymarvals);
double marf(double x, void *params);
#endif

#endif /* RLF_REFERENCE_ABI_H */

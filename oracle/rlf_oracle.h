/*
 * Test infrastructure only (oracle).  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs load this library, and only as the checker or the
 * timed CPU baseline; the product never links or calls it.
 *
 * CPU restatement of RadioLensfit2's per-galaxy shape-measurement hot path (FACET build,
 * the configuration Makefile:10 always selects).  Every function names the reference
 * function (file:line) whose arithmetic it follows.  The GSL routines the reference calls
 * (Ei, natural cubic spline, QAG GK41, nmsimplex2) come from oracle/gslshim/gslshim.c.
 */
#ifndef RLF_ORACLE_H
#define RLF_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double real, imag; } orc_complex;

/* likelihood state for one galaxy (datatype.h:49-74, FACET branch, plus the profile switch
 * -DGAUSSIAN made a runtime flag and an evaluation counter) */
typedef struct {
  int numr;                 /* number of scalelength nodes incl. the unused Ro[0] */
  const double *ro;         /* [numr] scalelength nodes, arcsec */
  const double *rprior;     /* [numr] ln prior at each node */
  unsigned int ncoords;     /* non-empty facet cells N_f */
  const double *uu, *vv;    /* [N_f] facet cell centres, wavelengths */
  const orc_complex *data;  /* [N_f] facet visibilities already divided by sigma2 */
  const double *sigma2;     /* [N_f] facet variances */
  double *mod;              /* [(numr-1) * N_f] model scratch */
  int gaussian;             /* 0: exponential (Sersic n=1) profile, 1: Gaussian */
  long nevals;              /* loglikelihood() calls */
  long newton_iters;        /* Newton iterations summed over all cross-correlations */
  double *trace;            /* optional [trace_cap][4]: (e1, e2, L, error) per evaluation */
  long trace_cap;
} orc_params;

typedef struct {
  double e1, e2, var_e1, var_e2, oneDimvar, maxL;
  int error;      /* source_fitting return value */
  int iters;      /* simplex iterations */
  long nevals;    /* likelihood evaluations (simplex + sampling) */
  double max_e1, max_e2;  /* simplex maximum, before the sampling */
} orc_fit_result;

unsigned int orc_facet_size(double theta_med, double len);
unsigned int orc_uv_grid_size(double len, const double *wavenumbers, unsigned int num_channels,
                              unsigned int ncoords, const double *u, const double *v,
                              unsigned int sizeg, const unsigned char *flag);
unsigned int orc_facet_coords(double *grid_u, double *grid_v, double len, unsigned int sizeg,
                              const double *count_w);
void orc_gridding(const double *wavenumbers, unsigned int num_channels, unsigned int ncoords,
                  const double *u, const double *v, const orc_complex *vis, const float *sigma2,
                  double len, unsigned int sizeg, orc_complex *new_vis, double *new_sigma2,
                  const unsigned char *flag, double *sum_w);
void orc_average_facets(unsigned long size, orc_complex *facet_vis, double *facet_sigma2,
                        const double *sum_w);

double orc_gaussian_shape(double k1, double k2, double scale_factor, double wave_factor);
double orc_sersic_shape(double k1, double k2, double scale_factor, double wave_factor);
void orc_model_at_zero(double e1, double e2, double scale, unsigned int num_coords,
                       const double *grid_u, const double *grid_v, const double *sigma2,
                       double *modvis, int gaussian);
void orc_data_galaxy_vis(double spectra, double wavenumber, double e1, double e2, double scale,
                         double flux, double l, double m, unsigned int num_coords,
                         const double *uu, const double *vv, const double *ww, orc_complex *vis,
                         int gaussian);
void orc_phase_shift(double wavenumber, double l, double m, unsigned int num_coords,
                     const double *uu, const double *vv, const double *ww, orc_complex *vis);
void orc_source_extraction(unsigned int num_channels, const double *spec, const double *wavenumbers,
                           unsigned int facet, orc_complex *facet_vis, double *facet_sigma2,
                           double *sum_w, double l0, double m0, double flux, double mu, double e1,
                           double e2, const orc_complex *visSkyMod, const orc_complex *visData,
                           orc_complex *visGal, const float *sigma2_vis, const unsigned char *flag,
                           unsigned long num_coords, const double *uu, const double *vv,
                           const double *ww, double len, int gaussian);

int orc_cross_correlation(unsigned long n, const double *grid_u, const double *grid_v,
                          const orc_complex *visData, const double *visMod, double *ho,
                          double *det_sigma, int *iters);
double orc_ei(double x);
double orc_marginalise_over_position_shift(double x);
double orc_loglikelihood_r(double e1, double e2, double scale, unsigned long n,
                           const double *variance, const double *grid_u, const double *grid_v,
                           const orc_complex *visData, double *visM, int gaussian, int *iters);
double orc_loglikelihood(orc_params *par, double e1, double e2, int *error);
double orc_loglikelihood_nodes(orc_params *par, double e1, double e2, double *L_r);
void orc_set_posterior_values(int numR, const double *L_r, const double *rprior, const double *Ro,
                              double *xmarvals, double *ymarvals, int *numvals);
double orc_marginalise_posterior_r(int num_marvals, const double *xmarvals, double *ymarvals);
void orc_likelihood_sampling(double *mes_e1, double *mes_e2, double maxL, orc_params *par,
                             int np_max, double *var_e1, double *var_e2, double *oneDimvar);
int orc_source_fitting(orc_params *par, double start_e1, double start_e2, double step,
                       orc_fit_result *out);

double orc_scale_mean(double flux);
double orc_rfunc(double mu, double sigma, double r);
int orc_ro_grid(double *Ro, int max_nodes);

void orc_sky_model(const double *wavenumbers, const double *spec, unsigned int num_channels,
                   unsigned int n_gal, const double *gflux, const double *gscale, const double *l,
                   const double *m, unsigned long num_coords, const double *uu, const double *vv,
                   const double *ww, orc_complex *visGal, orc_complex *visMod, int gaussian);

/* data_processing.c:47-147: one pass over galaxies in catalogue order (re_fitting=0) or over
 * bad_list (re_fitting=1).  Results go to out[gal]; bad_list/nbad as in the reference. */
void orc_data_processing(int re_fitting, unsigned int *bad_list, int nsources, double len,
                         unsigned int num_coords, unsigned int num_channels, const double *spec,
                         const double *wavenumbers, int numr, const double *ro,
                         const double *l, const double *m, const double *gflux,
                         const double *gscale, double *sum_w, orc_complex *visGal,
                         orc_complex *visSkyMod, orc_complex *visData, const float *sigma2_vis,
                         const unsigned char *flag, const double *uu, const double *vv,
                         const double *ww, int gaussian, orc_fit_result *out, int *bad);

/* Measurement Set column blocks (measurement_set.cpp) */
double orc_ms_read_coords(const double *uvw, unsigned int num_coords, double *uu, double *vv, double *ww);
unsigned long orc_ms_read_flag(const unsigned char *in, unsigned int num_coords, unsigned int num_channels,
                               unsigned int num_pols, unsigned char *flag);
void orc_ms_read_vis(const float *in, unsigned int num_coords, unsigned int num_channels, unsigned int num_pols,
                     orc_complex *vis);
void orc_ms_read_sigma2(const float *in, unsigned int num_coords, unsigned int num_channels, float sigma2,
                        float *sigma2_vis);
void orc_ms_write_vis(const orc_complex *vis, unsigned int num_coords, unsigned int num_channels, float *out);

#ifdef __cplusplus
}
#endif
#endif

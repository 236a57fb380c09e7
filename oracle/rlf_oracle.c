/*
 * Test infrastructure only (oracle): see rlf_oracle.h.  The product never links this file.
 *
 * CPU restatement of the FACET hot path of RadioLensfit2.  Expressions keep the reference's
 * evaluation order and its float/double mix (likelihood.c:449-540 uses float loop variables)
 * so that, built with -ffp-contract=off, the restatement reproduces the reference build to the
 * last bit except where summation is parallel.  OpenMP is used on the same loops as the
 * reference (likelihood.c:117, source_extraction.c:46, data_processing.c:109) so the timed CPU
 * baseline has the reference's parallel structure.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gsl/gsl_errno.h"
#include "gsl/gsl_math.h"
#include "gsl/gsl_sf_expint.h"
#include "gsl/gsl_vector.h"
#include "gsl/gsl_multimin.h"
#include "gsl/gsl_spline.h"
#include "gsl/gsl_integration.h"
#include "rlf_oracle.h"

#define ORC_PI 3.14159265358979323846
#define ORC_C0 299792458.0
/* default_params.h:40-81 */
#define ORC_PSF_NAT 38
#define ORC_RMIN 0.3
#define ORC_RMAX 3.5
#define ORC_NUM_R 29
#define ORC_ADD -0.93
#define ORC_ESP 0.33
#define ORC_R_STD 0.3136
#define ORC_TOL 1.0e-3
#define ORC_NP_MAX 30
#define ORC_E_RES 3.0e-3
#define ORC_VAR 1e-4

/* evaluate_uv_grid.c:50-55; ARCS2RAD is the unparenthesised macro PI/648000.0 (datatype.h:39),
 * so the product is evaluated left to right as ((len*38*theta)*PI)/648000. */
unsigned int orc_facet_size(double theta_med, double len) {
  unsigned int f = (unsigned int)2 * ceil(len * ORC_PSF_NAT * theta_med * ORC_PI / 648000.0);
  return f;
}

/* evaluate_uv_grid.c:58-109 (single process) */
unsigned int orc_uv_grid_size(double len, const double *wavenumbers, unsigned int num_channels,
                              unsigned int ncoords, const double *u, const double *v,
                              unsigned int sizeg, const unsigned char *flag) {
  unsigned long size = (unsigned long)sizeg * sizeg;
  unsigned long *count = (unsigned long *)calloc(size + 2 * (unsigned long)sizeg + 2, sizeof(unsigned long));
  double inc = 2 * len / sizeg;
  unsigned long n = 0;
  for (unsigned int ch = 0; ch < num_channels; ch++) {
    double inv_lambda = wavenumbers[ch] / (2. * ORC_PI);
    for (unsigned int k = 0; k < ncoords; k++) {
      if (!flag[n]) {
        unsigned int pu = (unsigned int)((u[k] * inv_lambda + len) / inc);
        unsigned int pv = (unsigned int)((v[k] * inv_lambda + len) / inc);
        unsigned long pc = (unsigned long)pv * sizeg + pu;
        if (pc < size) count[pc]++;
      }
      n++;
    }
  }
  n = 0;
  for (unsigned long p = 0; p < size; p++) if (count[p]) n++;
  free(count);
  return (unsigned int)n;
}

/* evaluate_uv_grid.c:113-133 */
unsigned int orc_facet_coords(double *grid_u, double *grid_v, double len, unsigned int sizeg,
                              const double *count_w) {
  double inc = 2 * len / sizeg;
  unsigned long size = (unsigned long)sizeg * sizeg, n = 0;
  for (unsigned long p = 0; p < size; p++) {
    if (count_w[p]) {
      unsigned int j = p / sizeg, i = p % sizeg;
      grid_u[n] = (i + 0.5) * inc - len;
      grid_v[n] = (j + 0.5) * inc - len;
      n++;
    }
  }
  return (unsigned int)n;
}

/* evaluate_uv_grid.c:143-211 (non-MPI branch: weight is always 1) */
void orc_gridding(const double *wavenumbers, unsigned int num_channels, unsigned int ncoords,
                  const double *u, const double *v, const orc_complex *vis, const float *sigma2,
                  double len, unsigned int sizeg, orc_complex *new_vis, double *new_sigma2,
                  const unsigned char *flag, double *sum_w) {
  double inc = 2 * len / sizeg;
  unsigned long size = (unsigned long)sizeg * sizeg;
  for (unsigned long i = 0; i < size; i++) sum_w[i] = 0.;
  orc_complex *tv = (orc_complex *)calloc(size, sizeof(orc_complex));
  double *ts = (double *)calloc(size, sizeof(double));
  unsigned long n = 0;
  for (unsigned int ch = 0; ch < num_channels; ch++) {
    double inv_lambda = wavenumbers[ch] / (2. * ORC_PI);
    for (unsigned int k = 0; k < ncoords; k++) {
      if (!flag[n]) {
        double uu = u[k] * inv_lambda;
        double vv = v[k] * inv_lambda;
        double weight = 1.;
        unsigned int pu = (unsigned int)((uu + len) / inc);
        unsigned int pv = (unsigned int)((vv + len) / inc);
        unsigned long pc = (unsigned long)pv * sizeg + pu;
        if (pc < size) {
          tv[pc].real += weight * vis[n].real;
          tv[pc].imag += weight * vis[n].imag;
          ts[pc] += weight * weight * sigma2[n];
          sum_w[pc] += weight;
        }
      }
      n++;
    }
  }
  n = 0;
  for (unsigned long p = 0; p < size; p++) {
    if (sum_w[p]) {
      new_vis[n].real = tv[p].real * sum_w[p] / ts[p];
      new_vis[n].imag = tv[p].imag * sum_w[p] / ts[p];
      new_sigma2[n] = ts[p] / (sum_w[p] * sum_w[p]);
      n++;
    }
  }
  free(tv);
  free(ts);
}

/* evaluate_uv_grid.c:216-230 */
void orc_average_facets(unsigned long size, orc_complex *facet_vis, double *facet_sigma2,
                        const double *sum_w) {
  unsigned long n = 0;
  for (unsigned long p = 0; p < size; p++) {
    if (sum_w[p]) {
      facet_vis[n].real = facet_vis[p].real * sum_w[p] / facet_sigma2[p];
      facet_vis[n].imag = facet_vis[p].imag * sum_w[p] / facet_sigma2[p];
      facet_sigma2[n] = facet_sigma2[p] / (sum_w[p] * sum_w[p]);
      n++;
    }
  }
}

/* galaxy_visibilities.c:40-53 */
double orc_gaussian_shape(double k1, double k2, double scale_factor, double wave_factor) {
  return exp(-0.5 * scale_factor * wave_factor * (k1 * k1 + k2 * k2));
}
double orc_sersic_shape(double k1, double k2, double scale_factor, double wave_factor) {
  double den = 1. + scale_factor * wave_factor * (k1 * k1 + k2 * k2);
  return 1. / (den * sqrt(den));
}

static inline double shape_of(int gaussian, double k1, double k2, double sf, double wf) {
  return gaussian ? orc_gaussian_shape(k1, k2, sf, wf) : orc_sersic_shape(k1, k2, sf, wf);
}

/* galaxy_visibilities.c:59-91 */
void orc_model_at_zero(double e1, double e2, double scale, unsigned int num_coords,
                       const double *grid_u, const double *grid_v, const double *sigma2,
                       double *modvis, int gaussian) {
  double detA = 1. - e1 * e1 - e2 * e2;
  scale *= ORC_PI / 648000.0;
  double scale_factor = (scale * scale) / (detA * detA);
  double sum = 0.;
  double cc2 = 4 * ORC_PI * ORC_PI;
  for (unsigned int i = 0; i < num_coords; ++i) {
    double uu = grid_u[i], vv = grid_v[i];
    double k1 = (1. + e1) * uu + e2 * vv;
    double k2 = e2 * uu + (1. - e1) * vv;
    modvis[i] = shape_of(gaussian, k1, k2, scale_factor, cc2);
    sum += modvis[i] * modvis[i] / sigma2[i];
  }
  sum = sqrt(sum);
  for (unsigned int k = 0; k < num_coords; k++) modvis[k] /= sum;
}

/* galaxy_visibilities.c:154-190 */
void orc_data_galaxy_vis(double spectra, double wavenumber, double e1, double e2, double scale,
                         double flux, double l, double m, unsigned int num_coords,
                         const double *uu, const double *vv, const double *ww, orc_complex *vis,
                         int gaussian) {
  double detA = 1. - e1 * e1 - e2 * e2;
  scale *= ORC_PI / 648000.0;
  double scale_factor = (scale * scale) / (detA * detA);
  double wavenumber2 = wavenumber * wavenumber;
  double n = sqrt(1. - l * l - m * m) - 1.;
  for (unsigned int i = 0; i < num_coords; ++i) {
    double u = uu[i], v = vv[i], w = ww[i];
    double phase = u * l + v * m + w * n;
    phase = wavenumber * phase;
    double k1 = (1. + e1) * u + e2 * v;
    double k2 = e2 * u + (1. - e1) * v;
    double shape = shape_of(gaussian, k1, k2, scale_factor, wavenumber2);
    shape *= spectra * flux;
    vis[i].real = shape * cos(phase);
    vis[i].imag = shape * sin(phase);
  }
}

/* galaxy_visibilities.c:244-270 */
void orc_phase_shift(double wavenumber, double l, double m, unsigned int num_coords,
                     const double *uu, const double *vv, const double *ww, orc_complex *vis) {
  double n = sqrt(1. - l * l - m * m) - 1.;
  for (unsigned int i = 0; i < num_coords; ++i) {
    double phase = uu[i] * l + vv[i] * m + ww[i] * n;
    phase *= -wavenumber;
    double sp = sin(phase), cp = cos(phase);
    double re = vis[i].real * cp - vis[i].imag * sp;
    double im = vis[i].real * sp + vis[i].imag * cp;
    vis[i].real = re;
    vis[i].imag = im;
  }
}

/* source_extraction.c:36-68 (FACET) */
void orc_source_extraction(unsigned int num_channels, const double *spec, const double *wavenumbers,
                           unsigned int facet, orc_complex *facet_vis, double *facet_sigma2,
                           double *sum_w, double l0, double m0, double flux, double mu, double e1,
                           double e2, const orc_complex *visSkyMod, const orc_complex *visData,
                           orc_complex *visGal, const float *sigma2_vis, const unsigned char *flag,
                           unsigned long num_coords, const double *uu, const double *vv,
                           const double *ww, double len, int gaussian) {
#pragma omp parallel for
  for (unsigned int ch = 0; ch < num_channels; ch++) {
    unsigned long ch_vis = ch * num_coords;
    orc_data_galaxy_vis(spec[ch], wavenumbers[ch], e1, e2, mu, flux, l0, m0, (unsigned int)num_coords,
                        uu, vv, ww, &visGal[ch_vis], gaussian);
    for (unsigned long i = ch_vis; i < ch_vis + num_coords; i++) {
      visGal[i].real += visData[i].real - visSkyMod[i].real;
      visGal[i].imag += visData[i].imag - visSkyMod[i].imag;
    }
    orc_phase_shift(wavenumbers[ch], l0, m0, (unsigned int)num_coords, uu, vv, ww, &visGal[ch_vis]);
  }
  orc_gridding(wavenumbers, num_channels, (unsigned int)num_coords, uu, vv, visGal, sigma2_vis, len,
               facet, facet_vis, facet_sigma2, flag, sum_w);
}

/* likelihood.c:194-358 (FACET): h = conj(D) M with D already divided by sigma2; Newton search
 * for the peak of Re h(x) e^{i k.x}, at most 50 iterations, tolerance 1e-7 on the step. */
int orc_cross_correlation(unsigned long n, const double *grid_u, const double *grid_v,
                          const orc_complex *visData, const double *visMod, double *ho,
                          double *det_sigma, int *iters) {
  double a, real_part, imag_part, u, v;
  double det, d2x, d2y, dx, dy, dxy, incx, incy;
  orc_complex *h = (orc_complex *)malloc((n ? n : 1) * sizeof(orc_complex));
  d2x = d2y = dx = dy = dxy = 0.;
  double value = 0;
  double cc = 2 * ORC_PI;
  for (unsigned long i = 0; i < n; i++) {
    h[i].real = visData[i].real * visMod[i];
    h[i].imag = -visData[i].imag * visMod[i];
    value += h[i].real;
    u = cc * grid_u[i];
    v = cc * grid_v[i];
    dx -= h[i].imag * u;
    dy -= h[i].imag * v;
    d2x -= h[i].real * u * u;
    d2y -= h[i].real * v * v;
    dxy -= h[i].real * u * v;
  }
  det = d2x * d2y - dxy * dxy;
  double xo = 0., yo = 0., tolerance = 1.e-7, norm = 1.;
  int iter = 0;
  while (det > 0 && (norm > tolerance) && iter < 50) {
    iter++;
    incx = (dx * d2y - dy * dxy) / det;
    incy = (dy * d2x - dx * dxy) / det;
    xo -= incx;
    yo -= incy;
    d2x = d2y = dx = dy = dxy = 0.;
    value = 0;
    for (unsigned long i = 0; i < n; ++i) {
      u = cc * grid_u[i];
      v = cc * grid_v[i];
      a = xo * u + yo * v;
      real_part = (h[i].real * cos(a) - h[i].imag * sin(a));
      imag_part = (h[i].real * sin(a) + h[i].imag * cos(a));
      value += real_part;
      dx -= imag_part * u;
      dy -= imag_part * v;
      d2x -= real_part * u * u;
      d2y -= real_part * v * v;
      dxy -= real_part * u * v;
    }
    det = d2x * d2y - dxy * dxy;
    norm = sqrt(incx * incx + incy * incy);
  }
  *ho = value;
  *det_sigma = det;
  if (iters) *iters = iter;
  free(h);
  return (det <= 0) ? 1 : 0;
}

double orc_ei(double x) {
  gsl_sf_result r;
  gsl_sf_expint_Ei_e(x, &r);
  return r.val;
}

/* likelihood.c:376-421 */
double orc_marginalise_over_position_shift(double x) {
  double Delta = 0.5 * 5.991;
  if (x <= Delta) return -1.e+10;
  if (x > 100.) return x - log(Delta) - exp(-Delta);
  if ((x - Delta) < 0.0001) x = Delta + 0.0001;
  gsl_sf_result yc, ys;
  if (gsl_sf_expint_Ei_e(x, &yc) == 0 && gsl_sf_expint_Ei_e((x - Delta), &ys) == 0)
    return log((yc.val - ys.val) / log(x / (x - Delta)));
  return -1.e+10;
}

/* likelihood.c:156-187 (FACET) */
double orc_loglikelihood_r(double e1, double e2, double scale, unsigned long n,
                           const double *variance, const double *grid_u, const double *grid_v,
                           const orc_complex *visData, double *visM, int gaussian, int *iters) {
  double ho, det_sigma, L;
  orc_model_at_zero(e1, e2, scale, (unsigned int)n, grid_u, grid_v, variance, visM, gaussian);
  int error = orc_cross_correlation(n, grid_u, grid_v, visData, visM, &ho, &det_sigma, iters);
  if (error) return -1.e10;
  double B = (ho * ho) * 0.5;
  L = orc_marginalise_over_position_shift(B);
  if (isnan(L)) L = -1.e+10;
  else L -= 0.5 * log(det_sigma);
  return L;
}

/* marginalise_r.c:29-64 */
void orc_set_posterior_values(int numR, const double *L_r, const double *rprior, const double *Ro,
                              double *xmarvals, double *ymarvals, int *numvals) {
  int num = 0, nRo = 1;
  while (nRo < numR && (L_r[nRo] <= -1.e+10)) nRo++;
  if (nRo < numR) {
    for (nRo = 1; nRo < numR; nRo++) {
      double likelval = L_r[nRo];
      if (likelval > -1.e+10) {
        xmarvals[num] = Ro[nRo];
        ymarvals[num] = likelval + rprior[nRo];
        num++;
      }
    }
  }
  *numvals = num;
}

/* marginalise_r.c:81-238: integrand exp(spline(x)) (marf), out-of-range points give 0 */
typedef struct { gsl_spline *spline; gsl_interp_accel *acc; } marf_state;
static double orc_marf(double x, void *p) {
  marf_state *st = (marf_state *)p;
  double y;
  if (gsl_spline_eval_e(st->spline, x, st->acc, &y)) return 0.;
  return exp(y);
}

double orc_marginalise_posterior_r(int num_marvals, const double *xmarvals, double *ymarvals) {
  double sump, error;
  int status;
  double ymax = -10.0;
  int ymaxpos = 0;
  for (int ii = 0; ii < num_marvals; ii++)
    if (ymarvals[ii] > ymax) { ymax = ymarvals[ii]; ymaxpos = ii; }
  double xmin, xmax;
  xmin = xmax = xmarvals[ymaxpos];
  if (ymaxpos < num_marvals - 1) xmax = xmarvals[ymaxpos + 1];
  if (ymaxpos > 0) xmin = xmarvals[ymaxpos - 1];
  for (int ii = 0; ii < num_marvals; ii++) {
    if (xmarvals[ii] < xmin) xmin = xmarvals[ii];
    if (xmarvals[ii] > xmax) xmax = xmarvals[ii];
    ymarvals[ii] -= ymax;
  }
  if (xmax <= xmin) return -1.e10; /* the reference exits the process here */
  marf_state st;
  st.acc = gsl_interp_accel_alloc();
  gsl_integration_workspace *w = gsl_integration_workspace_alloc(1000);
  st.spline = gsl_spline_alloc(gsl_interp_cspline, num_marvals);
  gsl_spline_init(st.spline, xmarvals, ymarvals, num_marvals);
  gsl_function F;
  F.function = &orc_marf;
  F.params = &st;
  status = gsl_integration_qag(&F, xmin, xmax, 0., 1.e-3, 1000, GSL_INTEG_GAUSS41, w, &sump, &error);
  if (status) {
    gsl_spline_free(st.spline);
    st.spline = gsl_spline_alloc(gsl_interp_linear, num_marvals);
    gsl_interp_accel_reset(st.acc);
    gsl_spline_init(st.spline, xmarvals, ymarvals, num_marvals);
    status = gsl_integration_qag(&F, xmin, xmax, 0., 1.e-3, 1000, GSL_INTEG_GAUSS41, w, &sump, &error);
  }
  gsl_spline_free(st.spline);
  gsl_interp_accel_free(st.acc);
  gsl_integration_workspace_free(w);
  if (status) return -1.e10;
  return log(sump) + ymax;
}

/* likelihood.c:106-149; also returns the node values L_r[1..numr-1] when L_r != NULL */
static double loglikelihood_impl(orc_params *par, double e1, double e2, int *error, double *L_out) {
  int numR = par->numr;
  double xm[64], ym[64], L_r[64];
  int numvals;
  double L_e;
  *error = 0;
  long it_sum = 0;
#pragma omp parallel for reduction(+ : it_sum)
  for (int nRo = 1; nRo < numR; nRo++) {
    unsigned long index = (unsigned long)(nRo - 1) * par->ncoords;
    int it = 0;
    L_r[nRo] = orc_loglikelihood_r(e1, e2, par->ro[nRo], par->ncoords, par->sigma2, par->uu, par->vv,
                                   par->data, &par->mod[index], par->gaussian, &it);
    it_sum += it;
  }
  par->nevals++;
  par->newton_iters += it_sum;
  if (L_out) for (int r = 1; r < numR; r++) L_out[r] = L_r[r];
  orc_set_posterior_values(numR, L_r, par->rprior, par->ro, xm, ym, &numvals);
  if (numvals > 4) L_e = orc_marginalise_posterior_r(numvals, xm, ym);
  else { *error = 1; L_e = -1.e+10; }
  if (L_e == -1.e+10) *error = 1;
  if (par->trace && par->nevals <= par->trace_cap) {
    double *t = par->trace + 4 * (par->nevals - 1);
    t[0] = e1; t[1] = e2; t[2] = L_e; t[3] = *error;
  }
  return L_e;
}

double orc_loglikelihood(orc_params *par, double e1, double e2, int *error) {
  return loglikelihood_impl(par, e1, e2, error, NULL);
}

double orc_loglikelihood_nodes(orc_params *par, double e1, double e2, double *L_r) {
  int err;
  return loglikelihood_impl(par, e1, e2, &err, L_r);
}

/* likelihood.c:87-100 */
static double orc_f_likelihood(const gsl_vector *v, void *params) {
  int error = 0;
  double e1 = gsl_vector_get(v, 0), e2 = gsl_vector_get(v, 1), L;
  if (e1 * e1 + e2 * e2 < 0.65) L = orc_loglikelihood((orc_params *)params, e1, e2, &error);
  else L = -1.e+10;
  return -L;
}

/* likelihood.c:428-554; sampling/edim/start are float as in the reference */
void orc_likelihood_sampling(double *mes_e1, double *mes_e2, double maxL, orc_params *par,
                             int np_max, double *var_e1, double *var_e2, double *oneDimvar) {
  int error = 0;
  int ie1, ie2, np;
  double totL, L_e, average_1, average_2, cov, var1, var2, x_e1, x_e2;
  double xL1, xL2, mod2 = 0;
  double L = 1.;
  double threshold = 0.05;
  double max_e1 = *mes_e1, max_e2 = *mes_e2;
  average_1 = max_e1;
  average_2 = max_e2;
  var1 = max_e1 * max_e1;
  var2 = max_e2 * max_e2;
  cov = max_e1 * max_e2;
  totL = 1.;
  np = 1;
  float sampling = 0.05;
  if (max_e1 < 0) sampling = -0.05;
  int k1 = 0;
  x_e1 = max_e1;
  while (L > threshold && mod2 < 1. && !error) {
    x_e1 += sampling;
    mod2 = x_e1 * x_e1 + max_e2 * max_e2;
    if (mod2 < 1.) {
      L_e = orc_loglikelihood(par, x_e1, max_e2, &error);
      if (!error) { L = exp(L_e - maxL); k1++; }
    }
  }
  if (L < threshold && k1 > 1) k1--;
  L = 1.;
  int k2 = 0;
  sampling = 0.05;
  if (max_e2 < 0) sampling = -0.05;
  x_e2 = max_e2;
  while (L > threshold && mod2 < 1. && !error) {
    x_e2 += sampling;
    mod2 = x_e2 * x_e2 + max_e1 * max_e1;
    if (mod2 < 1.) {
      L_e = orc_loglikelihood(par, max_e1, x_e2, &error);
      if (!error) { L = exp(L_e - maxL); k2++; }
    }
  }
  if (L < threshold && k2 > 1) k2--;
  sampling = 0.05;
  float edim1 = k1 * sampling;
  float edim2 = k2 * sampling;
  float start1 = edim1;
  float start2 = edim2;
  while (np < np_max && sampling > ORC_E_RES) {
    for (ie1 = -start1 / sampling; ie1 <= start1 / sampling; ie1 += 2) {
      for (ie2 = -start2 / sampling; ie2 <= start2 / sampling; ie2 += 2) {
        if (ie1 != 0 || ie2 != 0) {
          x_e1 = max_e1 + ie1 * sampling;
          x_e2 = max_e2 + ie2 * sampling;
          mod2 = x_e1 * x_e1 + x_e2 * x_e2;
          if (mod2 < 1.) {
            L_e = orc_loglikelihood(par, x_e1, x_e2, &error);
            if (!error) {
              L = exp(L_e - maxL);
              if (L >= threshold && !isinf(L)) {
                np++;
                xL1 = x_e1 * L;
                xL2 = x_e2 * L;
                average_1 += xL1;
                average_2 += xL2;
                var1 += x_e1 * xL1;
                var2 += x_e2 * xL2;
                cov += x_e1 * xL2;
                totL += L;
              }
            }
          }
        }
      }
    }
    sampling *= 0.5;
    start1 = edim1 - sampling;
    start2 = edim2 - sampling;
  }
  average_1 /= totL;
  average_2 /= totL;
  var1 /= totL; var1 -= average_1 * average_1;
  var2 /= totL; var2 -= average_2 * average_2;
  cov /= totL; cov -= average_1 * average_2;
  *mes_e1 = average_1;
  *mes_e2 = average_2;
  *var_e1 = var1;
  *var_e2 = var2;
  *oneDimvar = sqrt((var1) * (var2) - cov * cov);
}

/* galaxy_fitting.c:41-117, with the start point and initial step as parameters (the reference
 * uses (0,0) and 0.1) */
int orc_source_fitting(orc_params *par, double start_e1, double start_e2, double step,
                       orc_fit_result *out) {
  gsl_multimin_function fn;
  fn.n = 2;
  fn.f = orc_f_likelihood;
  fn.params = par;
  gsl_multimin_fminimizer *s = gsl_multimin_fminimizer_alloc(gsl_multimin_fminimizer_nmsimplex2, 2);
  gsl_vector *x = gsl_vector_alloc(2), *sx = gsl_vector_alloc(2);
  long ev0 = par->nevals;
  gsl_vector_set(x, 0, start_e1);
  gsl_vector_set(x, 1, start_e2);
  gsl_vector_set_all(sx, step);
  gsl_multimin_fminimizer_set(s, &fn, x, sx);
  int iter = 0, status;
  do {
    iter++;
    status = gsl_multimin_fminimizer_iterate(s);
    if (status) break;
    double size = gsl_multimin_fminimizer_size(s);
    status = gsl_multimin_test_size(size, ORC_TOL);
  } while (status == GSL_CONTINUE && iter < 50 && s->fval < 0.);
  double e1 = gsl_vector_get(s->x, 0), e2 = gsl_vector_get(s->x, 1), maxL = -s->fval;
  out->max_e1 = e1;
  out->max_e2 = e2;
  if (e1 * e1 + e2 * e2 > 0.65) maxL = -1e+10;
  int error = 0;
  double v1 = 0., v2 = 0., od = 0.;
  if (maxL > -1.e+10) {
    orc_likelihood_sampling(&e1, &e2, maxL, par, ORC_NP_MAX, &v1, &v2, &od);
    if (v1 < ORC_VAR || v2 < ORC_VAR || od < ORC_VAR) error = 1;
  } else {
    error = 1;
  }
  gsl_vector_free(x);
  gsl_vector_free(sx);
  gsl_multimin_fminimizer_free(s);
  out->e1 = e1; out->e2 = e2; out->var_e1 = v1; out->var_e2 = v2; out->oneDimvar = od;
  out->maxL = maxL; out->error = error; out->iters = iter; out->nevals = par->nevals - ev0;
  return error;
}

/* distributions.c:59-87 */
double orc_scale_mean(double flux) { return ORC_ADD + ORC_ESP * log(flux); }
double orc_rfunc(double mu, double sigma, double r) {
  double x = (log(r) - mu) / sigma;
  return -(x * x) * 0.5 - log(r * sigma);
}

/* RadioLensfit2.cpp:371-389: Ro[0]=0, Ro[1]=RMIN, quadratic spacing until Ro >= RMAX */
int orc_ro_grid(double *Ro, int max_nodes) {
  const double Rmin = ORC_RMIN, Rmax = ORC_RMAX;
  int numR = ORC_NUM_R;
  if (max_nodes < numR) return -1;
  Ro[0] = 0.;
  Ro[1] = Rmin;
  int nRo = 2;
  while (nRo < numR && Ro[nRo - 1] < Rmax) {
    double Rinterval = 0.08 + 0.4 * pow(((Ro[nRo - 1] - Rmin) / (Rmax - Rmin)), 2);
    Ro[nRo] = Ro[nRo - 1] + Rinterval;
    nRo++;
  }
  return nRo;
}

/* data_simulation.c:131-165 (SCALELENGTH_ON: the catalogue scalelength is used) */
void orc_sky_model(const double *wavenumbers, const double *spec, unsigned int num_channels,
                   unsigned int n_gal, const double *gflux, const double *gscale, const double *l,
                   const double *m, unsigned long num_coords, const double *uu, const double *vv,
                   const double *ww, orc_complex *visGal, orc_complex *visMod, int gaussian) {
  for (unsigned int g = 0; g < n_gal; g++) {
#pragma omp parallel for
    for (unsigned int ch = 0; ch < num_channels; ch++) {
      unsigned long ch_vis = (unsigned long)ch * num_coords;
      orc_data_galaxy_vis(spec[ch], wavenumbers[ch], 0., 0., gscale[g], gflux[g], l[g], m[g],
                          (unsigned int)num_coords, uu, vv, ww, &visGal[ch_vis], gaussian);
      for (unsigned long i = ch_vis; i < ch_vis + num_coords; i++) {
        visMod[i].real += visGal[i].real;
        visMod[i].imag += visGal[i].imag;
      }
    }
  }
}

/* data_processing.c:47-147 (FACET, SCALELENGTH_ON) */
void orc_data_processing(int re_fitting, unsigned int *bad_list, int nsources, double len,
                         unsigned int num_coords, unsigned int num_channels, const double *spec,
                         const double *wavenumbers, int numr, const double *ro,
                         const double *l, const double *m, const double *gflux,
                         const double *gscale, double *sum_w, orc_complex *visGal,
                         orc_complex *visSkyMod, orc_complex *visData, const float *sigma2_vis,
                         const unsigned char *flag, const double *uu, const double *vv,
                         const double *ww, int gaussian, orc_fit_result *out, int *bad) {
  unsigned int fmax_ = orc_facet_size(ORC_RMAX, len);
  unsigned long ncells = (unsigned long)fmax_ * fmax_;
  /* facet buffers sized by facet_size(RMAX) as RadioLensfit2.cpp:421-494 */
  orc_complex *fvis = (orc_complex *)calloc(ncells, sizeof(orc_complex));
  double *fs2 = (double *)calloc(ncells, sizeof(double));
  double *fu = (double *)calloc(ncells, sizeof(double));
  double *fv = (double *)calloc(ncells, sizeof(double));
  double *mod = (double *)calloc((size_t)numr * ncells, sizeof(double));
  double rprior[64];
  int nbad = 0;
  for (int g = 0; g < nsources; g++) {
    unsigned int gal = re_fitting ? bad_list[g] : (unsigned int)g;
    double l0 = l[gal], m0 = m[gal], flux = gflux[gal];
    double mu = orc_scale_mean(flux);
    double R_mu = gscale[gal];
    for (int nRo = 1; nRo < numr; nRo++) rprior[nRo] = orc_rfunc(mu, ORC_R_STD, ro[nRo]);
    unsigned int facet = orc_facet_size(R_mu, len);
    if (facet > fmax_) facet = fmax_; /* the reference would overrun its RMAX-sized buffers */
    orc_source_extraction(num_channels, spec, wavenumbers, facet, fvis, fs2, sum_w, l0, m0, flux,
                          R_mu, 0., 0., visSkyMod, visData, visGal, sigma2_vis, flag, num_coords,
                          uu, vv, ww, len, gaussian);
    orc_params par;
    memset(&par, 0, sizeof(par));
    par.numr = numr; par.ro = ro; par.rprior = rprior;
    par.ncoords = orc_facet_coords(fu, fv, len, facet, sum_w);
    par.uu = fu; par.vv = fv; par.data = fvis; par.sigma2 = fs2; par.mod = mod;
    par.gaussian = gaussian;
    orc_fit_result r;
    int error = orc_source_fitting(&par, 0., 0., 0.1, &r);
    if (error) {
      if (re_fitting) { r.e1 = 0.; r.e2 = 0.; }
      else bad_list[nbad] = gal;
      nbad++;
    } else {
#pragma omp parallel for
      for (unsigned int ch = 0; ch < num_channels; ch++) {
        unsigned long ch_vis = (unsigned long)ch * num_coords;
        orc_data_galaxy_vis(spec[ch], wavenumbers[ch], 0., 0., R_mu, flux, l0, m0, num_coords,
                            uu, vv, ww, &visGal[ch_vis], gaussian);
        for (unsigned long i = ch_vis; i < ch_vis + num_coords; i++) {
          visSkyMod[i].real -= visGal[i].real;
          visSkyMod[i].imag -= visGal[i].imag;
        }
        orc_data_galaxy_vis(spec[ch], wavenumbers[ch], r.e1, r.e2, R_mu, flux, l0, m0, num_coords,
                            uu, vv, ww, &visGal[ch_vis], gaussian);
        for (unsigned long i = ch_vis; i < ch_vis + num_coords; i++) {
          visData[i].real -= visGal[i].real;
          visData[i].imag -= visGal[i].imag;
        }
      }
    }
    out[gal] = r;
  }
  *bad = nbad;
  free(fvis); free(fs2); free(fu); free(fv); free(mod);
}

/* ------------------------------------------------------------------ Measurement Set columns
 * The readers of measurement_set.cpp applied to column blocks already read from the table
 * (casacore is not available): block layout [row][channel][correlation], row slowest. */

/* ms_read_coords (measurement_set.cpp:224-240): UVW [rows][3] -> uu, vv, ww */
double orc_ms_read_coords(const double *uvw, unsigned int num_coords, double *uu, double *vv, double *ww) {
  double umax = 0., vmax = 0.;
  for (unsigned int i = 0; i < num_coords; ++i) {
    uu[i] = uvw[3 * (size_t)i];
    vv[i] = uvw[3 * (size_t)i + 1];
    ww[i] = uvw[3 * (size_t)i + 2];
    double ua = fabs(uu[i]), va = fabs(vv[i]);
    if (ua > umax) umax = ua;
    if (va > vmax) vmax = va;
  }
  return ceil(fmax(umax, vmax));
}

/* ms_read_Flag (measurement_set.cpp:318-332): the first correlation, or first || last of four */
unsigned long orc_ms_read_flag(const unsigned char *in, unsigned int num_coords, unsigned int num_channels,
                               unsigned int num_pols, unsigned char *flag) {
  unsigned long count = 0;
  for (unsigned int c = 0; c < num_channels; ++c)
    for (unsigned int b = 0; b < num_coords; ++b) {
      unsigned long i = (unsigned long)num_pols * ((unsigned long)b * num_channels + c);
      unsigned long j = (unsigned long)c * num_coords + b;
      flag[j] = in[i];
      if (num_pols == 4) flag[j] = (flag[j] || in[i + 3]);
      if (flag[j]) count++;
    }
  return count;
}

/* ms_read_vis (measurement_set.cpp:384-400): Stokes I in uJy, channel-major */
void orc_ms_read_vis(const float *in, unsigned int num_coords, unsigned int num_channels, unsigned int num_pols,
                     orc_complex *vis) {
  for (unsigned int c = 0; c < num_channels; ++c)
    for (unsigned int b = 0; b < num_coords; ++b) {
      unsigned long i = ((unsigned long)num_pols * ((unsigned long)b * num_channels + c)) << 1;
      unsigned long j = (unsigned long)c * num_coords + b;
      vis[j].real = in[i];
      vis[j].imag = in[i + 1];
      if (num_pols == 4) {
        i += 6;
        vis[j].real += in[i];
        vis[j].imag += in[i + 1];
        vis[j].real *= 0.5;
        vis[j].imag *= 0.5;
      }
      vis[j].real *= 1e+6;
      vis[j].imag *= 1e+6;
    }
}

/* ms_read_sigma (measurement_set.cpp:266-273) into a [num_channels * num_coords] array, then the
 * driver's replacement of non-positive values (RadioLensfit2.cpp:257-270).  The reader sets only the
 * first num_coords entries; the rest are taken as unset (0) and so receive the theoretical value. */
void orc_ms_read_sigma2(const float *in, unsigned int num_coords, unsigned int num_channels, float sigma2,
                        float *sigma2_vis) {
  unsigned long num_vis = (unsigned long)num_channels * num_coords;
  for (unsigned long i = 0; i < num_vis; ++i) sigma2_vis[i] = 0.f;
  if (in)
    for (unsigned int i = 0; i < num_coords; ++i) sigma2_vis[i] = in[i] * in[i];
  for (unsigned long i = 0; i < num_vis; ++i)
    if (sigma2_vis[i] <= 0.) sigma2_vis[i] = sigma2;
}

/* ms_write_vis (measurement_set.cpp:423-433): one correlation, Jy, row-major */
void orc_ms_write_vis(const orc_complex *vis, unsigned int num_coords, unsigned int num_channels, float *out) {
  for (unsigned int c = 0; c < num_channels; ++c)
    for (unsigned int b = 0; b < num_coords; ++b) {
      unsigned long i = (unsigned long)c * num_coords + b;
      unsigned long j = ((unsigned long)b * num_channels + c) << 1;
      out[j] = vis[i].real * 1e-6;
      out[j + 1] = vis[i].imag * 1e-6;
    }
}

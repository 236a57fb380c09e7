/*
 * Test infrastructure only (oracle). Nothing in the product links this file.
 *
 * A project-written implementation of the subset of the GSL 2.5 API that the reference's
 * hot-path sources call (likelihood.c, marginalise_r.c, galaxy_fitting.c, distributions.c,
 * utils.c, data_simulation.c).  GSL itself is not installed here, so each routine restates the
 * published algorithm GSL documents for it:
 *
 *   gsl_sf_expint_Ei_e      Ei(x): power series  gamma + ln x + sum x^k/(k k!)  for 0<x<=40,
 *                           asymptotic series  e^x/x sum k!/x^k  for x>40 (truncated at the
 *                           smallest term), -E1(-x) for x<0 (series / Lentz continued fraction).
 *   gsl_interp_cspline      natural cubic spline: second derivatives from the symmetric
 *                           tridiagonal system, solved by LDL^T; evaluated in GSL's
 *                           y_i + dx (b_i + dx (c_i + dx d_i)) form.
 *   gsl_interp_linear       piecewise linear.
 *   gsl_integration_qag     QUADPACK QAG (Piessens et al. 1983) with the 41-point Gauss-Kronrod
 *                           rule, QUADPACK's error rescaling and round-off detection.
 *   nmsimplex2              Nelder-Mead as GSL documents "nmsimplex2": simplex from x0 and
 *                           x0+step_i, reflection (-1), expansion (-2), 1-D contraction (0.5),
 *                           contraction about the best vertex, incrementally updated centre
 *                           and squared RMS size.
 *   gsl_rng_mt19937         Matsumoto-Nishimura MT19937 with GSL's seeding convention.
 *
 * Bit-exact agreement with a real GSL build is not pinned (no GSL here); agreement with scipy
 * (expi, CubicSpline natural, quad) is checked by tests/test_oracle_gslshim.py.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#include "gsl/gsl_errno.h"
#include "gsl/gsl_math.h"
#include "gsl/gsl_sf_expint.h"
#include "gsl/gsl_sf_erf.h"
#include "gsl/gsl_vector.h"
#include "gsl/gsl_multimin.h"
#include "gsl/gsl_spline.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_rng.h"

/* ------------------------------------------------------------------ errors */
gsl_error_handler_t *gsl_set_error_handler_off(void) { return NULL; }

const char *gsl_strerror(const int e) {
  switch (e) {
    case GSL_SUCCESS: return "success";
    case GSL_FAILURE: return "failure";
    case GSL_CONTINUE: return "the iteration has not converged yet";
    case GSL_EDOM: return "input domain error";
    case GSL_EBADFUNC: return "problem with user-supplied function";
    case GSL_EMAXITER: return "exceeded max number of iterations";
    case GSL_EROUND: return "cannot reach the specified tolerance";
    case GSL_ESING: return "apparent singularity detected";
    case GSL_EBADTOL: return "invalid tolerance specified";
    case GSL_ENOMEM: return "malloc failed";
    default: return "unknown error code";
  }
}

int gsl_finite(const double x) { return isfinite(x) ? 1 : 0; }

/* --------------------------------------------------------------------- Ei */
static const double EULER_GAMMA = 0.57721566490153286060651209008240243;

static double ei_series(double x) { /* x > 0 */
  double term = 1.0, sum = 0.0;
  for (int k = 1; k < 1000; ++k) {
    term *= x / k;
    double t = term / k;
    sum += t;
    if (t < 1e-18 * sum) break;
  }
  return EULER_GAMMA + log(x) + sum;
}

static double ei_asymptotic(double x) { /* x large and positive */
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 200; ++k) {
    double next = term * k / x;
    if (next >= term || next < 1e-18 * sum) break;
    term = next;
    sum += term;
  }
  return exp(x) / x * sum;
}

static double e1_positive(double x) { /* E1(x), x > 0 */
  if (x <= 1.0) {
    double sum = 0.0, term = 1.0;
    for (int k = 1; k < 200; ++k) {
      term *= -x / k;
      double t = -term / k;
      sum += t;
      if (fabs(t) < 1e-18 * fabs(sum)) break;
    }
    return -EULER_GAMMA - log(x) + sum;
  }
  /* modified Lentz evaluation of the continued fraction for E1 */
  double b = x + 1.0, c = 1.0 / DBL_MIN, d = 1.0 / b, h = d;
  for (int i = 1; i < 1000; ++i) {
    double an = -(double)i * i;
    b += 2.0;
    d = 1.0 / (an * d + b);
    c = b + an / c;
    double del = c * d;
    h *= del;
    if (fabs(del - 1.0) < 1e-16) break;
  }
  return h * exp(-x);
}

int gsl_sf_expint_Ei_e(const double x, gsl_sf_result *result) {
  if (x == 0.0) { result->val = NAN; result->err = NAN; return GSL_EDOM; }
  double v;
  if (x < 0.0) v = -e1_positive(-x);
  else if (x <= 40.0) v = ei_series(x);
  else {
    if (x > 709.0) { result->val = INFINITY; result->err = INFINITY; return GSL_EOVRFLW; }
    v = ei_asymptotic(x);
  }
  result->val = v;
  result->err = 2.0 * DBL_EPSILON * fabs(v);
  return GSL_SUCCESS;
}

double gsl_sf_expint_Ei(const double x) {
  gsl_sf_result r;
  gsl_sf_expint_Ei_e(x, &r);
  return r.val;
}

double gsl_sf_erf(const double x) { return erf(x); }

/* ----------------------------------------------------------------- vector */
gsl_vector *gsl_vector_alloc(const size_t n) {
  gsl_vector *v = (gsl_vector *)calloc(1, sizeof(gsl_vector));
  v->size = n;
  v->stride = 1;
  v->data = (double *)calloc(n ? n : 1, sizeof(double));
  v->block = NULL;
  v->owner = 1;
  return v;
}
void gsl_vector_free(gsl_vector *v) { if (v) { free(v->data); free(v); } }
double gsl_vector_get(const gsl_vector *v, const size_t i) { return v->data[i * v->stride]; }
void gsl_vector_set(gsl_vector *v, const size_t i, double x) { v->data[i * v->stride] = x; }
void gsl_vector_set_all(gsl_vector *v, double x) {
  for (size_t i = 0; i < v->size; ++i) v->data[i * v->stride] = x;
}
int gsl_vector_memcpy(gsl_vector *dest, const gsl_vector *src) {
  for (size_t i = 0; i < src->size; ++i) dest->data[i * dest->stride] = src->data[i * src->stride];
  return GSL_SUCCESS;
}

/* ------------------------------------------------------------ nmsimplex2 */
typedef struct {
  size_t n;      /* dimension */
  size_t P;      /* vertices = n + 1 */
  double *x1;    /* P x n vertices, row-major */
  double *y1;    /* P function values */
  double *center;
  double *ws1, *ws2, *xc, *xc2;
  double S2;     /* squared RMS distance of vertices from the centre */
} nm_state;

static const gsl_multimin_fminimizer_type nmsimplex2_type = {"nmsimplex2rand-free", sizeof(nm_state)};
const gsl_multimin_fminimizer_type *gsl_multimin_fminimizer_nmsimplex2 = &nmsimplex2_type;

static double nm_eval(gsl_multimin_function *f, const double *x, size_t n) {
  gsl_vector v;
  v.size = n; v.stride = 1; v.data = (double *)x; v.block = NULL; v.owner = 0;
  return f->f(&v, f->params);
}

static void nm_compute_center(nm_state *s) {
  for (size_t j = 0; j < s->n; ++j) s->center[j] = 0.0;
  for (size_t i = 0; i < s->P; ++i)
    for (size_t j = 0; j < s->n; ++j) s->center[j] += s->x1[i * s->n + j];
  for (size_t j = 0; j < s->n; ++j) s->center[j] *= 1.0 / (double)s->P;
}

static double nm_compute_size(nm_state *s) {
  double ss = 0.0;
  for (size_t i = 0; i < s->P; ++i) {
    double t2 = 0.0;
    for (size_t j = 0; j < s->n; ++j) {
      double d = s->x1[i * s->n + j] - s->center[j];
      t2 += d * d;
    }
    ss += t2;
  }
  s->S2 = ss / (double)s->P;
  return sqrt(s->S2);
}

/* xc = alpha*centre + beta*x_corner with alpha=(1-coeff)P/(P-1), beta=(P coeff-1)/(P-1) */
static double nm_try_corner_move(double coeff, nm_state *s, size_t corner, double *xc,
                                 gsl_multimin_function *f) {
  const double P = (double)s->P;
  const double alpha = (1.0 - coeff) * P / (P - 1.0);
  const double beta = (P * coeff - 1.0) / (P - 1.0);
  for (size_t j = 0; j < s->n; ++j) {
    xc[j] = alpha * s->center[j];
    xc[j] += beta * s->x1[corner * s->n + j];
  }
  return nm_eval(f, xc, s->n);
}

static void nm_update_point(nm_state *s, size_t i, const double *x, double val) {
  const double P = (double)s->P;
  double dd = 0.0, xmcd = 0.0;
  for (size_t j = 0; j < s->n; ++j) {
    s->ws1[j] = x[j] - s->x1[i * s->n + j];         /* delta = x - x_orig */
    s->ws2[j] = s->x1[i * s->n + j] - s->center[j]; /* xmc = x_orig - c   */
    dd += s->ws1[j] * s->ws1[j];
    xmcd += s->ws2[j] * s->ws1[j];
  }
  const double d = sqrt(dd);
  s->S2 += (2.0 / P) * xmcd + ((P - 1.0) / P) * (d * d / P);
  for (size_t j = 0; j < s->n; ++j) s->center[j] += (1.0 / P) * s->ws1[j];
  for (size_t j = 0; j < s->n; ++j) s->x1[i * s->n + j] = x[j];
  s->y1[i] = val;
}

static int nm_contract_by_best(nm_state *s, size_t best, double *xc, gsl_multimin_function *f) {
  int status = GSL_SUCCESS;
  for (size_t i = 0; i < s->P; ++i) {
    if (i == best) continue;
    for (size_t j = 0; j < s->n; ++j)
      s->x1[i * s->n + j] = 0.5 * (s->x1[i * s->n + j] + s->x1[best * s->n + j]);
    for (size_t j = 0; j < s->n; ++j) xc[j] = s->x1[i * s->n + j];
    double v = nm_eval(f, xc, s->n);
    s->y1[i] = v;
    if (!gsl_finite(v)) status = GSL_EBADFUNC;
  }
  nm_compute_center(s);
  nm_compute_size(s);
  return status;
}

gsl_multimin_fminimizer *gsl_multimin_fminimizer_alloc(const gsl_multimin_fminimizer_type *T, size_t n) {
  gsl_multimin_fminimizer *m = (gsl_multimin_fminimizer *)calloc(1, sizeof(*m));
  nm_state *s = (nm_state *)calloc(1, sizeof(nm_state));
  s->n = n;
  s->P = n + 1;
  s->x1 = (double *)calloc(s->P * n, sizeof(double));
  s->y1 = (double *)calloc(s->P, sizeof(double));
  s->center = (double *)calloc(n, sizeof(double));
  s->ws1 = (double *)calloc(n, sizeof(double));
  s->ws2 = (double *)calloc(n, sizeof(double));
  s->xc = (double *)calloc(n, sizeof(double));
  s->xc2 = (double *)calloc(n, sizeof(double));
  m->type = T;
  m->x = gsl_vector_alloc(n);
  m->state = s;
  return m;
}

int gsl_multimin_fminimizer_set(gsl_multimin_fminimizer *m, gsl_multimin_function *f,
                                const gsl_vector *x, const gsl_vector *step_size) {
  nm_state *s = (nm_state *)m->state;
  m->f = f;
  gsl_vector_memcpy(m->x, x);
  double *xt = s->xc;
  for (size_t j = 0; j < s->n; ++j) xt[j] = gsl_vector_get(x, j);
  double v = nm_eval(f, xt, s->n);
  if (!gsl_finite(v)) return GSL_EBADFUNC;
  for (size_t j = 0; j < s->n; ++j) s->x1[j] = xt[j];
  s->y1[0] = v;
  for (size_t i = 0; i < s->n; ++i) {
    for (size_t j = 0; j < s->n; ++j) xt[j] = gsl_vector_get(x, j);
    xt[i] = gsl_vector_get(x, i) + gsl_vector_get(step_size, i);
    v = nm_eval(f, xt, s->n);
    if (!gsl_finite(v)) return GSL_EBADFUNC;
    for (size_t j = 0; j < s->n; ++j) s->x1[(i + 1) * s->n + j] = xt[j];
    s->y1[i + 1] = v;
  }
  nm_compute_center(s);
  m->size = nm_compute_size(s);
  m->fval = s->y1[0];
  return GSL_SUCCESS;
}

int gsl_multimin_fminimizer_iterate(gsl_multimin_fminimizer *m) {
  nm_state *s = (nm_state *)m->state;
  gsl_multimin_function *f = m->f;
  double *y1 = s->y1, *xc = s->xc, *xc2 = s->xc2;
  size_t hi, s_hi, lo;
  double dhi, ds_hi, dlo, val, val2;
  int status;

  /* highest, second highest and lowest vertex */
  dhi = dlo = y1[0];
  hi = 0; lo = 0;
  ds_hi = y1[1]; s_hi = 1;
  for (size_t i = 1; i < s->P; ++i) {
    val = y1[i];
    if (val < dlo) { dlo = val; lo = i; }
    else if (val > dhi) { ds_hi = dhi; s_hi = hi; dhi = val; hi = i; }
    else if (val > ds_hi) { ds_hi = val; s_hi = i; }
  }

  val = nm_try_corner_move(-1.0, s, hi, xc, f); /* reflection */
  if (gsl_finite(val) && val < y1[lo]) {
    val2 = nm_try_corner_move(-2.0, s, hi, xc2, f); /* expansion */
    if (gsl_finite(val2) && val2 < y1[lo]) nm_update_point(s, hi, xc2, val2);
    else nm_update_point(s, hi, xc, val);
  } else if (!gsl_finite(val) || val > y1[s_hi]) {
    if (gsl_finite(val) && val <= y1[hi]) nm_update_point(s, hi, xc, val);
    val2 = nm_try_corner_move(0.5, s, hi, xc2, f); /* 1-D contraction */
    if (gsl_finite(val2) && val2 <= y1[hi]) {
      nm_update_point(s, hi, xc2, val2);
    } else {
      status = nm_contract_by_best(s, lo, xc, f);
      if (status != GSL_SUCCESS) return GSL_EFAILED;
    }
  } else {
    nm_update_point(s, hi, xc, val);
  }

  /* lowest vertex is the current estimate */
  lo = 0;
  for (size_t i = 1; i < s->P; ++i) if (y1[i] < y1[lo]) lo = i;
  for (size_t j = 0; j < s->n; ++j) gsl_vector_set(m->x, j, s->x1[lo * s->n + j]);
  m->fval = y1[lo];
  if (s->S2 > 0) m->size = sqrt(s->S2);
  else m->size = nm_compute_size(s);
  return GSL_SUCCESS;
}

double gsl_multimin_fminimizer_size(const gsl_multimin_fminimizer *m) { return m->size; }

void gsl_multimin_fminimizer_free(gsl_multimin_fminimizer *m) {
  if (!m) return;
  nm_state *s = (nm_state *)m->state;
  free(s->x1); free(s->y1); free(s->center); free(s->ws1); free(s->ws2); free(s->xc); free(s->xc2);
  free(s);
  gsl_vector_free(m->x);
  free(m);
}

int gsl_multimin_test_size(const double size, double epsabs) {
  if (epsabs < 0.0) return GSL_EBADTOL;
  return (size < epsabs) ? GSL_SUCCESS : GSL_CONTINUE;
}

/* ----------------------------------------------------------------- spline */
static const gsl_interp_type linear_type = {"linear", 0};
static const gsl_interp_type cspline_type = {"cspline", 1};
const gsl_interp_type *gsl_interp_linear = &linear_type;
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
int gsl_interp_accel_reset(gsl_interp_accel *a) { a->cache = 0; a->miss_count = 0; a->hit_count = 0; return GSL_SUCCESS; }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size) {
  if (size < (T->kind == 1 ? 3u : 2u)) return NULL;
  gsl_spline *s = (gsl_spline *)calloc(1, sizeof(gsl_spline));
  s->type = T;
  s->size = size;
  s->x = (double *)calloc(size, sizeof(double));
  s->y = (double *)calloc(size, sizeof(double));
  s->c = (double *)calloc(size, sizeof(double));
  return s;
}

void gsl_spline_free(gsl_spline *s) { if (s) { free(s->x); free(s->y); free(s->c); free(s); } }

/* natural spline: c_0 = c_{n-1} = 0; interior c from the symmetric tridiagonal system
 *   h_{i+1} c_{i} + 2(h_i + h_{i+1}) c_{i+1} + h_{i+1} c_{i+2} = 3 (dy_{i+1}/h_{i+1} - dy_i/h_i)
 * solved by an LDL^T factorisation. */
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t size) {
  if (size != s->size) return GSL_EINVAL;
  for (size_t i = 0; i < size; ++i) { s->x[i] = xa[i]; s->y[i] = ya[i]; s->c[i] = 0.0; }
  for (size_t i = 1; i < size; ++i) if (!(xa[i] > xa[i - 1])) return GSL_EINVAL;
  if (s->type->kind != 1) return GSL_SUCCESS;
  if (size < 3) return GSL_EINVAL;
  const size_t m = size - 2;
  double *diag = (double *)malloc(m * sizeof(double));
  double *off = (double *)malloc(m * sizeof(double));
  double *g = (double *)malloc(m * sizeof(double));
  double *alpha = (double *)malloc(m * sizeof(double));
  double *gamma = (double *)malloc(m * sizeof(double));
  double *z = (double *)malloc(m * sizeof(double));
  for (size_t i = 0; i < m; ++i) {
    const double h_i = xa[i + 1] - xa[i];
    const double h_ip1 = xa[i + 2] - xa[i + 1];
    const double dy_i = ya[i + 1] - ya[i];
    const double dy_ip1 = ya[i + 2] - ya[i + 1];
    const double g_i = (h_i != 0.0) ? 1.0 / h_i : 0.0;
    const double g_ip1 = (h_ip1 != 0.0) ? 1.0 / h_ip1 : 0.0;
    off[i] = h_ip1;
    diag[i] = 2.0 * (h_ip1 + h_i);
    g[i] = 3.0 * (dy_ip1 * g_ip1 - dy_i * g_i);
  }
  if (m == 1) {
    s->c[1] = g[0] / diag[0];
  } else {
    alpha[0] = diag[0];
    gamma[0] = off[0] / alpha[0];
    for (size_t i = 1; i < m - 1; ++i) {
      alpha[i] = diag[i] - off[i - 1] * gamma[i - 1];
      gamma[i] = off[i] / alpha[i];
    }
    alpha[m - 1] = diag[m - 1] - off[m - 2] * gamma[m - 2];
    z[0] = g[0];
    for (size_t i = 1; i < m; ++i) z[i] = g[i] - gamma[i - 1] * z[i - 1];
    for (size_t i = 0; i < m; ++i) z[i] = z[i] / alpha[i];
    s->c[m] = z[m - 1];
    for (size_t k = m - 1; k-- > 0;) s->c[k + 1] = z[k] - gamma[k] * s->c[k + 2];
  }
  free(diag); free(off); free(g); free(alpha); free(gamma); free(z);
  return GSL_SUCCESS;
}

static size_t interval_index(const double *xa, size_t n, double x) {
  size_t lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    size_t mid = (lo + hi) / 2;
    if (xa[mid] > x) hi = mid; else lo = mid;
  }
  return lo;
}

int gsl_spline_eval_e(const gsl_spline *s, double x, gsl_interp_accel *a, double *y) {
  (void)a;
  if (x < s->x[0] || x > s->x[s->size - 1]) { *y = NAN; return GSL_EDOM; }
  size_t i = interval_index(s->x, s->size, x);
  const double x_lo = s->x[i], x_hi = s->x[i + 1];
  const double y_lo = s->y[i], y_hi = s->y[i + 1];
  const double dx = x_hi - x_lo, dy = y_hi - y_lo;
  const double delx = x - x_lo;
  if (s->type->kind == 1) {
    const double c_i = s->c[i], c_ip1 = s->c[i + 1];
    const double b_i = (dy / dx) - dx * (c_ip1 + 2.0 * c_i) / 3.0;
    const double d_i = (c_ip1 - c_i) / (3.0 * dx);
    *y = y_lo + delx * (b_i + delx * (c_i + delx * d_i));
  } else {
    *y = y_lo + delx / dx * dy;
  }
  return GSL_SUCCESS;
}

double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) {
  double y;
  gsl_spline_eval_e(s, x, a, &y);
  return y;
}

/* ----------------------------------------------------------- integration */
/* 41-point Gauss-Kronrod rule (QUADPACK qk41): Kronrod abscissae, Kronrod weights,
 * and weights of the embedded 20-point Gauss rule (abscissae xgk[1], xgk[3], ...). */
static const double xgk41[21] = {
  0.998859031588277663838315576545863, 0.993128599185094924786122388471320,
  0.981507877450250259193342994720217, 0.963971927277913791267666131197277,
  0.940822633831754753519982722212443, 0.912234428251325905867752441203298,
  0.878276811252281976077442995113078, 0.839116971822218823394529061701521,
  0.795041428837551198350638833272788, 0.746331906460150792614305070355642,
  0.693237656334751384805490711845932, 0.636053680726515025452836696226286,
  0.575140446819710315342946036586425, 0.510867001950827098004364050955251,
  0.443593175238725103199992213492640, 0.373706088715419560672548177024927,
  0.301627868114913004320555356858592, 0.227785851141645078080496195368575,
  0.152605465240922675505220241022678, 0.076526521133497333754640409398838,
  0.000000000000000000000000000000000};
static const double wgk41[21] = {
  0.003073583718520531501218293246031, 0.008600269855642942198661787950102,
  0.014626169256971252983787960308868, 0.020388373461266523598010231432755,
  0.025882133604951158834505067096153, 0.031287306777032798958543119323801,
  0.036600169758200798030557240707211, 0.041668873327973686263788305936895,
  0.046434821867497674720231880926108, 0.050944573923728691932707670050345,
  0.055195105348285994744832372419777, 0.059111400880639572374967220648594,
  0.062653237554781168025870122174255, 0.065834597133618422111563556969398,
  0.068648672928521619345623411885368, 0.071054423553444068305790361723210,
  0.073030690332786667495189417658913, 0.074582875400499188986581418362488,
  0.075704497684556674659542775376617, 0.076377867672080736705502835038061,
  0.076600711917999656445049901530102};
static const double wg20[10] = {
  0.017614007139152118311861962351853, 0.040601429800386941331039952274932,
  0.062672048334109063569506535187042, 0.083276741576704748724758143222046,
  0.101930119817240435036750135480350, 0.118194531961518417312377377711382,
  0.131688638449176626898494499748163, 0.142096109318382051329298325067165,
  0.149172986472603746787828737001969, 0.152753387130725850698084331955098};

static double rescale_error(double err, const double result_abs, const double result_asc) {
  err = fabs(err);
  if (result_asc != 0 && err != 0) {
    double scale = pow((200 * err / result_asc), 1.5);
    err = (scale < 1) ? result_asc * scale : result_asc;
  }
  if (result_abs > DBL_MIN / (50 * DBL_EPSILON)) {
    double min_err = 50 * DBL_EPSILON * result_abs;
    if (min_err > err) err = min_err;
  }
  return err;
}

static void qk41(const gsl_function *f, double a, double b, double *result, double *abserr,
                 double *resabs, double *resasc) {
  double fv1[21], fv2[21];
  const double center = 0.5 * (a + b);
  const double half_length = 0.5 * (b - a);
  const double abs_half_length = fabs(half_length);
  const double f_center = GSL_FN_EVAL(f, center);
  double result_gauss = 0;
  double result_kronrod = f_center * wgk41[20];
  double result_abs = fabs(result_kronrod);
  for (int j = 0; j < 10; ++j) {
    const int jtw = 2 * j + 1;
    const double absc = half_length * xgk41[jtw];
    const double fval1 = GSL_FN_EVAL(f, center - absc);
    const double fval2 = GSL_FN_EVAL(f, center + absc);
    const double fsum = fval1 + fval2;
    fv1[jtw] = fval1; fv2[jtw] = fval2;
    result_gauss += wg20[j] * fsum;
    result_kronrod += wgk41[jtw] * fsum;
    result_abs += wgk41[jtw] * (fabs(fval1) + fabs(fval2));
  }
  for (int j = 0; j < 10; ++j) {
    const int jtwm1 = 2 * j;
    const double absc = half_length * xgk41[jtwm1];
    const double fval1 = GSL_FN_EVAL(f, center - absc);
    const double fval2 = GSL_FN_EVAL(f, center + absc);
    fv1[jtwm1] = fval1; fv2[jtwm1] = fval2;
    result_kronrod += wgk41[jtwm1] * (fval1 + fval2);
    result_abs += wgk41[jtwm1] * (fabs(fval1) + fabs(fval2));
  }
  const double mean = result_kronrod * 0.5;
  double result_asc = wgk41[20] * fabs(f_center - mean);
  for (int j = 0; j < 20; ++j) result_asc += wgk41[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
  const double err = (result_kronrod - result_gauss) * half_length;
  result_kronrod *= half_length;
  result_abs *= abs_half_length;
  result_asc *= abs_half_length;
  *result = result_kronrod;
  *resabs = result_abs;
  *resasc = result_asc;
  *abserr = rescale_error(err, result_abs, result_asc);
}

gsl_integration_workspace *gsl_integration_workspace_alloc(const size_t n) {
  gsl_integration_workspace *w = (gsl_integration_workspace *)calloc(1, sizeof(*w));
  w->limit = n;
  w->alist = (double *)calloc(n, sizeof(double));
  w->blist = (double *)calloc(n, sizeof(double));
  w->rlist = (double *)calloc(n, sizeof(double));
  w->elist = (double *)calloc(n, sizeof(double));
  w->order = (size_t *)calloc(n, sizeof(size_t));
  w->level = (size_t *)calloc(n, sizeof(size_t));
  return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w) {
  if (!w) return;
  free(w->alist); free(w->blist); free(w->rlist); free(w->elist); free(w->order); free(w->level);
  free(w);
}

/* QUADPACK qag: global adaptive bisection of the interval with the largest error estimate.
 * Intervals are kept in arrays; the one to bisect is found by a linear scan for the largest
 * error (ties resolved towards the lowest index), which selects the same interval as
 * QUADPACK's sorted error list. */
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        size_t limit, int key, gsl_integration_workspace *w, double *result,
                        double *abserr) {
  (void)key; /* only the 41-point rule is used by the reference (GSL_INTEG_GAUSS41) */
  double area, errsum, result0, abserr0, resabs0, resasc0, tolerance;
  size_t iteration = 0;
  int roundoff_type1 = 0, roundoff_type2 = 0, error_type = 0;
  *result = 0; *abserr = 0;
  if (limit > w->limit) return GSL_EINVAL;
  if (epsabs <= 0 && (epsrel < 50 * DBL_EPSILON || epsrel < 0.5e-28)) return GSL_EBADTOL;

  qk41(f, a, b, &result0, &abserr0, &resabs0, &resasc0);
  size_t n = 1;
  w->alist[0] = a; w->blist[0] = b; w->rlist[0] = result0; w->elist[0] = abserr0; w->level[0] = 0;

  tolerance = fmax(epsabs, epsrel * fabs(result0));
  const double round_off = 50 * DBL_EPSILON * resabs0;
  if (abserr0 <= round_off && abserr0 > tolerance) {
    *result = result0; *abserr = abserr0;
    return GSL_EROUND;
  } else if ((abserr0 <= tolerance && abserr0 != resasc0) || abserr0 == 0.0) {
    *result = result0; *abserr = abserr0;
    return GSL_SUCCESS;
  } else if (limit == 1) {
    *result = result0; *abserr = abserr0;
    return GSL_EMAXITER;
  }

  area = result0;
  errsum = abserr0;
  iteration = 1;
  do {
    size_t imax = 0;
    for (size_t k = 1; k < n; ++k) if (w->elist[k] > w->elist[imax]) imax = k;
    const double a_i = w->alist[imax], b_i = w->blist[imax];
    const double r_i = w->rlist[imax], e_i = w->elist[imax];
    const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
    double area1, area2, error1, error2, resabs1, resabs2, resasc1, resasc2;
    qk41(f, a1, b1, &area1, &error1, &resabs1, &resasc1);
    qk41(f, a2, b2, &area2, &error2, &resabs2, &resasc2);
    const double area12 = area1 + area2;
    const double error12 = error1 + error2;
    errsum += (error12 - e_i);
    area += area12 - r_i;
    if (resasc1 != error1 && resasc2 != error2) {
      const double delta = r_i - area12;
      if (fabs(delta) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i) roundoff_type1++;
      if (iteration >= 10 && error12 > e_i) roundoff_type2++;
    }
    tolerance = fmax(epsabs, epsrel * fabs(area));
    if (errsum > tolerance) {
      if (roundoff_type1 >= 6 || roundoff_type2 >= 20) error_type = 2;
      const double tmp = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
      if (fabs(a1) <= tmp && fabs(b2) <= tmp) error_type = 3;
    }
    const size_t lev = w->level[imax] + 1;
    w->alist[imax] = a1; w->blist[imax] = b1; w->rlist[imax] = area1; w->elist[imax] = error1; w->level[imax] = lev;
    w->alist[n] = a2; w->blist[n] = b2; w->rlist[n] = area2; w->elist[n] = error2; w->level[n] = lev;
    n++;
    iteration++;
  } while (iteration < limit && !error_type && errsum > tolerance);

  double sum = 0;
  for (size_t k = 0; k < n; ++k) sum += w->rlist[k];
  *result = sum;
  *abserr = errsum;
  if (errsum <= tolerance) return GSL_SUCCESS;
  if (error_type == 2) return GSL_EROUND;
  if (error_type == 3) return GSL_ESING;
  if (iteration == limit) return GSL_EMAXITER;
  return GSL_EFAILED;
}

/* -------------------------------------------------------------------- rng */
static const gsl_rng_type mt_type = {"mt19937"};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  r->type = T;
  gsl_rng_set(r, 0);
  return r;
}

void gsl_rng_set(gsl_rng *r, unsigned long int s) {
  if (s == 0) s = 4357; /* GSL's default seed */
  r->mt[0] = s & 0xffffffffUL;
  for (int i = 1; i < 624; ++i)
    r->mt[i] = (1812433253UL * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (unsigned long)i) & 0xffffffffUL;
  r->mti = 624;
}

unsigned long int gsl_rng_get(gsl_rng *r) {
  static const unsigned long UPPER = 0x80000000UL, LOWER = 0x7fffffffUL, MATRIX_A = 0x9908b0dfUL;
  unsigned long k;
  if (r->mti >= 624) {
    int kk;
    for (kk = 0; kk < 624 - 397; ++kk) {
      unsigned long y = (r->mt[kk] & UPPER) | (r->mt[kk + 1] & LOWER);
      r->mt[kk] = r->mt[kk + 397] ^ (y >> 1) ^ ((y & 1) ? MATRIX_A : 0UL);
    }
    for (; kk < 623; ++kk) {
      unsigned long y = (r->mt[kk] & UPPER) | (r->mt[kk + 1] & LOWER);
      r->mt[kk] = r->mt[kk + (397 - 624)] ^ (y >> 1) ^ ((y & 1) ? MATRIX_A : 0UL);
    }
    {
      unsigned long y = (r->mt[623] & UPPER) | (r->mt[0] & LOWER);
      r->mt[623] = r->mt[396] ^ (y >> 1) ^ ((y & 1) ? MATRIX_A : 0UL);
    }
    r->mti = 0;
  }
  k = r->mt[r->mti++];
  k ^= (k >> 11);
  k ^= (k << 7) & 0x9d2c5680UL;
  k ^= (k << 15) & 0xefc60000UL;
  k ^= (k >> 18);
  return k & 0xffffffffUL;
}

double gsl_rng_uniform(gsl_rng *r) { return (double)gsl_rng_get(r) / 4294967296.0; }
double gsl_rng_uniform_pos(gsl_rng *r) {
  double x;
  do { x = gsl_rng_uniform(r); } while (x == 0);
  return x;
}
unsigned long int gsl_rng_max(const gsl_rng *r) { (void)r; return 0xffffffffUL; }
unsigned long int gsl_rng_min(const gsl_rng *r) { (void)r; return 0; }
void gsl_rng_free(gsl_rng *r) { free(r); }

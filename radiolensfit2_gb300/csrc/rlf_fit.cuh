// Facet likelihood and ellipticity fit on the GPU: declarations shared by the kernels file and
// the host layer.
#pragma once
#include "rlf_device.cuh"

namespace rlf {

// Per-galaxy fit result (the outputs of source_fitting, galaxy_fitting.c:41-117, plus counters).
struct FitOut {
  double e1, e2, var_e1, var_e2, oneDimvar, maxL;
  int error;         // source_fitting's return value: 1 = bad measurement
  int iters;         // simplex iterations
  int nevals;        // likelihood evaluations (simplex + sampling)
  int newton_iters;  // Newton iterations summed over scalelength nodes and evaluations
  int status;        // 0 ok; bit 1: QAG interval capacity reached; bit 2: non-finite simplex start
  int ncoords;       // facet cells used
  double max_e1, max_e2;  // simplex maximum (before the sampling of likelihood.c:428-554)
};

enum Precision { kF64 = 0, kMixed = 1 };

// A batch of facets packed back to back.  Cell arrays hold either double (kF64) or float
// (kMixed) values; rprior and start are always double.
struct FacetBatch {
  int n_gal;
  int max_cells;           // largest facet in the batch (sizes the shared memory)
  const int* offset;       // [n_gal] first cell of each facet
  const int* count;        // [n_gal] cells of each facet
  const void* gu;          // cell centres, wavelengths
  const void* gv;
  const void* dre;         // facet visibilities divided by their variance (likelihood.c:219)
  const void* dim;
  const void* sig2;        // facet variances
  const double* rprior;    // [n_gal * kMaxNodes] ln prior at each node
  const double* start;     // [n_gal * 3] (e1, e2, step) or nullptr for (0, 0, 0.1)
  const int* active;       // [n_gal] nonzero = fit this galaxy, or nullptr for all
  FitOut* out;             // [n_gal]
  int* queue;              // work counter, zeroed before launch
  double* trace;           // optional [n_gal][trace_cap][4]: (e1, e2, L, error) per evaluation
  int trace_cap;
};

struct FitConfigHost {
  int numr;                // nodes including the unused Ro[0]
  double ro[kMaxNodes];
  int gaussian;
  int np_max;
};

// host launchers (rlf_fit.cu)
int fit_set_config(const FitConfigHost& cfg, cudaStream_t st);
int fit_launch(const FacetBatch& b, Precision p, int grid, cudaStream_t st);
int fit_max_grid(Precision p);

// single-purpose kernels behind the reference's per-function C entry points
int launch_loglikelihood_r(double e1, double e2, double scale, int n, const double* variance,
                           const double* gu, const double* gv, const double* dre, const double* dim,
                           double* visM, double* out_L, int gaussian, cudaStream_t st);
int launch_cross_correlation(int n, const double* gu, const double* gv, const double* dre,
                             const double* dim, const double* visMod, double* out3, cudaStream_t st);
int launch_loglikelihood(const FacetBatch& b, double e1, double e2, double* out2, double* node_L,
                         cudaStream_t st);
// the same evaluation in either arithmetic policy (the facet cells must be of that policy's type)
int launch_loglikelihood_prec(const FacetBatch& b, double e1, double e2, double* out2, double* node_L,
                              Precision prec, cudaStream_t st);
int launch_likelihood_sampling(const FacetBatch& b, double e1, double e2, double maxL, int np_max,
                               double* out5, cudaStream_t st);
int launch_marginalise_posterior_r(int n, const double* x, double* y, double* out1, cudaStream_t st);
int launch_set_posterior_values(int numR, const double* Lr, const double* rprior, const double* ro,
                                double* x, double* y, int* numvals, cudaStream_t st);
int launch_position_marginal(int n, const double* x, double* y, cudaStream_t st);

}  // namespace rlf

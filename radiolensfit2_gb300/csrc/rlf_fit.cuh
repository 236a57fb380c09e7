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
  int status;        // 0 ok; bit 1: QAG interval capacity reached; bit 2: non-finite simplex start;
                     // bit 3: a sampling-grid point not delivered within the board wait limit
  int ncoords;       // facet cells used
  double max_e1, max_e2;  // simplex maximum (before the sampling of likelihood.c:428-554)
};

enum Precision { kF64 = 0, kMixed = 1 };

// Sampling board of one fit launch.  The grid of the likelihood sampling (likelihood.c:502-532)
// holds independent evaluations; the CTA fitting a galaxy publishes them a chunk at a time, and
// CTAs whose galaxy queue is empty claim points and evaluate them (the bright galaxies with a
// narrow posterior need hundreds of grid points and would otherwise hold a launch alone).  The
// owner accumulates the results in the reference's loop order, so the outcome does not depend on
// which CTA evaluated a point.  Results are double-buffered by the chunk sequence's parity.
constexpr int kBoardCap = 512;  // points per published chunk
struct SampleSlot {
  unsigned long long claim;     // (chunk sequence << 32) | next point index
  int npts;                     // points in the chunk
  int p0;                       // index of the chunk's first point in its grid level
  int lo1, lo2, n2;             // grid: ie1 = lo1 + 2 (p / n2), ie2 = lo2 + 2 (p % n2)
  float sampling;
  double me1, me2;              // grid centre
  unsigned long long pad;
};
struct SampleBoard {
  SampleSlot* slot;             // [n_gal]
  double* L;                    // [n_gal][2][kBoardCap] log-likelihood of each point
  int* err;                     // [n_gal][2][kBoardCap] error flag; -1: point outside the grid's domain
  int* flag;                    // [n_gal][2][kBoardCap] sequence of the chunk the result belongs to
  int* newton;                  // [n_gal] Newton iterations of the helpers' evaluations
  int* done_gal;                // galaxies finished in this launch
  unsigned long long wait_ns;   // an owner's limit on waiting for the helpers' points (0: kBoardWaitNs)
};

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
  SampleBoard board;       // sampling board (slot == nullptr: each CTA samples its galaxy alone)
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
// the double-float functions of the fit on device arrays (rlf_debug_df_math)
int launch_df_math(int op, int n, const double* x, const double* y, double* out, cudaStream_t st);
int launch_set_posterior_values(int numR, const double* Lr, const double* rprior, const double* ro,
                                double* x, double* y, int* numvals, cudaStream_t st);
int launch_position_marginal(int n, const double* x, double* y, cudaStream_t st);

}  // namespace rlf

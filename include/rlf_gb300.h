/*
 * Batched and device-resident API of the GB300 shape-measurement library (librlf_gb300.so).
 * These entry points have no counterpart in the reference: they replace the per-galaxy loop of
 * data_processing.c:61-138 by a pipeline that keeps the observation in GPU memory and fits many
 * galaxies concurrently.  Plain C types only.
 */
#ifndef RLF_GB300_H
#define RLF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { RLF_F64 = 0, RLF_MIXED = 1 };

/* per-galaxy result: the outputs of source_fitting (galaxy_fitting.c:41-117) plus counters */
typedef struct {
  double e1, e2, var_e1, var_e2, oneDimvar, maxL;
  int error;         /* 1 = bad measurement (the reference's bad list) */
  int iters;         /* simplex iterations */
  int nevals;        /* likelihood evaluations */
  int newton_iters;  /* Newton iterations over all nodes and evaluations */
  int status;        /* 0, or device-side limits reached (2: QAG intervals, 4: bad simplex start,
                        8: a sampling-grid point not delivered within rlf_options.board_wait_us) */
  int ncoords;       /* facet cells */
  double max_e1, max_e2;  /* simplex maximum, before the likelihood sampling */
} rlf_fit_result;

typedef struct {
  int precision;     /* visibility passes (extraction, removal): RLF_F64 (reference arithmetic) or
                        RLF_MIXED (FP32 visibilities, FP64 phase argument) */
  int batch;         /* galaxies extracted/fitted/removed together; 1 = the reference's order */
  int gaussian;      /* 0 exponential profile (default), 1 Gaussian (the -DGAUSSIAN build) */
  int refit;         /* rlf_obs_process: 1 = run the re-fit pass over bad galaxies */
  int verbose;
  const double *start;  /* optional [n_gal*3] simplex start (e1, e2, step); NULL = (0, 0, 0.1) */
  int fit_precision; /* the fit: RLF_F64 (default; the reference's fit arithmetic, so the fitted
                        ellipticities follow the reference's simplex path) or RLF_MIXED (FP32 cell
                        arithmetic: faster, log-likelihood within ~2e-7 relative, but rounding
                        noise can change simplex decisions, moving e by up to ~1e-3) */
  int rounds;        /* batched mode: extraction + fit rounds per batch (0 = default 3).  Round 1
                        extracts every galaxy of the batch from the same data; each further round
                        removes the previous round's fitted models of the earlier galaxies of the
                        batch from each facet, converging to the one-galaxy-at-a-time result. */
  int reuse_obs;     /* data_processing: 0 (default) uploads uvw, sigma2_vis and flag and builds the
                        facet tables on every call, as the reference reads them fresh on every call.
                        1 keeps them on the device between calls that pass the same arrays (same
                        addresses and sizes, same sampled contents), as the reference driver's two
                        passes do: the caller promises not to change uvw, sigma2_vis or flag in place
                        between such calls (a change at an unsampled position is not seen).
                        Visibilities and sky model are uploaded on every call either way. */
  int board_wait_us; /* the fit's limit, in microseconds, on a galaxy's wait for sampling-grid points
                        that other thread blocks claimed (0 = default 2 s); a point not delivered in
                        time counts as a failed evaluation and sets status bit 8 */
  int proposal;      /* 1: start each galaxy's simplex at the learned proposal (rlf_proposal_set_params)
                        instead of (0, 0) with step 0.1; ignored when `start` is given or no network is
                        loaded */
  int seq_facet_kb;  /* batched mode: shared memory (KB, 16..200) for the facet accumulators of one
                        sub-batch, which bounds the galaxies extracted per pass (0 = 128) */
  int fit_ctas_per_sm; /* persistent fit thread blocks per SM (1..3, 0 = 3) */
  int graphs;        /* batched mode: 1 = each sub-batch's rounds (round control, extraction,
                        finalisation, proposal, fit) and its removal are captured from the stream into
                        one CUDA graph and launched as such; 0 = launched one by one.  Either way
                        the host does not wait between rounds (the round control runs on the GPU). */
} rlf_options;

/* Mode of the reference-named drop-in entry points (data_processing, source_fitting, ...).
 * Defaults: RLF_F64, batch 1, exponential profile. Returns 0. */
int rlf_configure(const rlf_options *opt);
const char *rlf_version(void);
/* No counterpart in the reference.  Frees the observation data_processing keeps between calls. */
void rlf_release(void);
/* No counterpart in the reference.  Host<->device bytes this library has copied since it was
 * loaded (visibilities, arrays, results; not the small constant tables). */
void rlf_transfer_bytes(unsigned long long *h2d, unsigned long long *d2h);
int rlf_device_count(void);
/* number of CUDA kernels this library has launched since it was loaded */
long long rlf_launch_count(void);
/* measured FP32 FMA throughput of the current GPU, GFLOP/s (an FMA counts 2), for rooflines */
double rlf_fp32_peak_gflops(void);

/* -------- device-resident observation -------- */
typedef struct rlf_observation rlf_observation;

/* Upload an observation.  uu/vv/ww: [n_rows] metres; wavenumbers/spec: [n_ch];
 * sigma2/flag: [n_ch * n_rows] channel-major (the reference's layout), flag may be NULL.
 * len: facet half-extent in wavelengths (RadioLensfit2.cpp:406).  Returns NULL on error. */
rlf_observation *rlf_obs_create(int n_rows, int n_ch, const double *uu, const double *vv,
                                const double *ww, const double *wavenumbers, const double *spec,
                                double len, const float *sigma2, const uint8_t *flag,
                                int precision);
void rlf_obs_destroy(rlf_observation *obs);
/* data / sky model from host complex128 [n_ch*n_rows] (NULL = zero) */
int rlf_obs_set_vis(rlf_observation *obs, const double *data_c128, const double *sky_c128);
/* data from host complex64 [n_ch*n_rows] */
int rlf_obs_set_data_c64(rlf_observation *obs, const float *data_c64);
/* No counterpart in the reference: data straight from a Measurement Set DATA block
 * [n_rows][n_ch][num_pols] complex64 in Jy (num_pols 1 or 4), converted on the GPU as
 * ms_read_vis does (measurement_set.cpp:345-400): Stokes I, uJy, channel-major. */
int rlf_obs_set_data_ms(rlf_observation *obs, const float *data_block, unsigned int num_pols);

/* -------- Measurement Set columns (measurement_set.cpp:203-453) --------
 * The reference's readers take a casacore table; these take the column blocks the caller read
 * from it, row-major ([row][channel][correlation], complex64 interleaved), and produce the same
 * arrays on the GPU.  No counterpart names in the reference (its ms_* functions need casacore). */
/* ms_read_coords (measurement_set.cpp:203-241): UVW [num_coords][3] -> uu, vv, ww; returns
 * ceil(max(max|u|, max|v|)) */
double rlf_ms_read_coords(const double *uvw_block, unsigned int num_coords, double *uu, double *vv,
                          double *ww);
/* ms_read_Flag (measurement_set.cpp:280-334): FLAG [num_coords][num_channels][num_pols] (bytes)
 * -> flag [num_channels * num_coords], correlation 0, or 0 || 3 with four; returns the number
 * flagged */
unsigned long rlf_ms_read_flag(const uint8_t *flag_block, unsigned int num_coords,
                               unsigned int num_channels, unsigned int num_pols, uint8_t *flag);
/* ms_read_vis (measurement_set.cpp:345-400): DATA -> vis complex128 [num_channels * num_coords],
 * Stokes I ((0 + 3) / 2 with four correlations) in uJy */
int rlf_ms_read_vis(const float *data_block, unsigned int num_coords, unsigned int num_channels,
                    unsigned int num_pols, double *vis_c128);
/* ms_read_sigma (measurement_set.cpp:246-274) and the driver's fallback (RadioLensfit2.cpp:257-270):
 * sigma2_vis[num_channels * num_coords] = sigma[i]^2 for i < num_coords (the column read flat, as the
 * reference does), every entry <= 0 or not set by the reader = sigma2_theory; sigma_block NULL: all
 * entries sigma2_theory */
int rlf_ms_read_sigma2(const float *sigma_block, unsigned int num_coords, unsigned int num_channels,
                       float sigma2_theory, float *sigma2_vis);
/* ms_write_vis (measurement_set.cpp:409-453): vis complex128 [num_channels * num_coords] in uJy ->
 * DATA block [num_coords][num_channels] complex64 in Jy (one correlation) */
int rlf_ms_write_vis(const double *vis_c128, unsigned int num_coords, unsigned int num_channels,
                     float *data_block);
int rlf_obs_get_vis(rlf_observation *obs, double *data_c128, double *sky_c128);
/* data = sum of sheared galaxy models + complex Gaussian noise (sigma per component), on the GPU */
int rlf_obs_simulate(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                     const double *e1, const double *e2, const double *l, const double *m,
                     double noise_sigma, uint64_t seed, int gaussian);
/* sky model = sum of round models (data_simulation.c:131-165) */
int rlf_obs_sky_model(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                      const double *l, const double *m, int gaussian);
/* keep / restore copies of data and sky model on the device */
int rlf_obs_snapshot(rlf_observation *obs);
int rlf_obs_restore(rlf_observation *obs);
/* extraction -> fit -> removal for galaxies in catalogue order, then (opt->refit) the re-fit
 * pass over bad galaxies (RadioLensfit2.cpp:597-606).  out: [n_gal]; n_bad: galaxies still bad. */
int rlf_obs_process(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                    const double *l, const double *m, int numr, const double *ro,
                    const rlf_options *opt, rlf_fit_result *out, int *n_bad);
/* extraction only (source_extraction + evaluate_facet_coords of every galaxy against the current
 * data and sky model, `batch` galaxies per pass): facets[g][5][stride] receives the cell centres
 * (u, v), the facet visibilities divided by their variances (re, im) and the variances;
 * ncoords[g] the number of cells */
int rlf_obs_extract(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                    const double *l, const double *m, int batch, double *facets, int stride,
                    int *ncoords);
/* CUDA events around the last rlf_obs_process: total and per-stage milliseconds
 * [total, extract, fit, remove] */
int rlf_obs_last_timing(rlf_observation *obs, double *ms4);

/* Work counters of the last rlf_obs_process (both passes), for throughput and roofline figures:
 * stats[RLF_STAT_EXTRACT_PASSES]  sequential batch extraction passes over all visibilities,
 * stats[RLF_STAT_EXTRACT_SINGLE]  one-galaxy extraction passes,
 * stats[RLF_STAT_REMOVE_BATCHES]  batched removal passes (one per sub-batch),
 * stats[RLF_STAT_REMOVE_SINGLE]   one-galaxy removal passes,
 * stats[RLF_STAT_FITTED]          galaxy fits (every round counts),
 * stats[RLF_STAT_EXTRACT_GAL]     galaxies extracted by the batch passes, summed over passes
 *                                 (x visibilities = galaxy-visibility pairs),
 * stats[RLF_STAT_CHANGED]         galaxies whose fit still changed in the last round of their
 *                                 sub-batch (ellipticity by more than 1e-9 or the error flag),
 * stats[RLF_STAT_EXTRACT_GAL_FIRST] the part of RLF_STAT_EXTRACT_GAL in first rounds (no model
 *                                 differences removed),
 * stats[RLF_STAT_SKIPPED_GAL]     galaxy rounds not run because they could not change: the galaxies
 *                                 of a sub-batch up to the first good fit of the round before, and
 *                                 every later round of a sub-batch without good fits,
 * stats[RLF_STAT_EXTRACT_SEQ_US]  device time of the sequential batch extraction kernel's launches
 *                                 (RLF_STAT_EXTRACT_PASSES of them), microseconds, CUDA events,
 * stats[RLF_STAT_GRAPHS]          sub-batches launched as CUDA graphs (rlf_options.graphs). */
enum {
  RLF_STAT_EXTRACT_PASSES = 0,
  RLF_STAT_EXTRACT_SINGLE = 1,
  RLF_STAT_REMOVE_BATCHES = 2,
  RLF_STAT_REMOVE_SINGLE = 3,
  RLF_STAT_FITTED = 4,
  RLF_STAT_EXTRACT_GAL = 5,
  RLF_STAT_CHANGED = 6,
  RLF_STAT_EXTRACT_GAL_FIRST = 7,
  RLF_STAT_SKIPPED_GAL = 8,
  RLF_STAT_EXTRACT_SEQ_US = 9,
  RLF_STAT_GRAPHS = 10,
  RLF_NSTATS = 11
};
int rlf_obs_last_stats(rlf_observation *obs, long long *stats);

/* -------- channel shards --------
 * No counterpart names in the reference; the steps of its MPI decomposition
 * (data_processing-mpi.c:65-216), one process per GPU holding its own channels:
 * rlf_obs_facet_partials: every galaxy's facet sums over this observation's channels, un-averaged,
 *   out[g][4][stride] = sum of vis re, sum of vis im, sum of sigma^2, sum of weights per cell of the
 *   galaxy's F x F facet (row-major, F^2 <= stride; the rest zero), every galaxy extracted against
 *   the current data and sky model as source_extraction does (evaluate_uv_grid.c:143-195 before
 *   averaging); FP32 observations in batches (the sequential extraction's first round);
 * rlf_fit_partials: the facets of the summed partials of all shards (average_facets,
 *   evaluate_facet_coords), fitted together by the persistent fit kernel: source_fitting's results;
 * rlf_obs_remove: removal of the given fits from this observation's data and sky model, in order,
 *   bad fits (error != 0) skipped (data_processing.c:109-135). */
int rlf_obs_facet_partials(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                           const double *l, const double *m, double *out, int stride);
int rlf_fit_partials(int n_gal, const double *partials, int stride, const double *flux,
                     const double *scale, double len, int numr, const double *ro,
                     const rlf_options *opt, rlf_fit_result *out);
int rlf_obs_remove(rlf_observation *obs, int n_gal, const double *flux, const double *scale,
                   const double *l, const double *m, const rlf_fit_result *fits);

/* -------- learned proposal of the simplex start --------
 * No counterpart in the reference (whose simplex starts at (0, 0) with step 0.1,
 * galaxy_fitting.c:59-65).  A convolutional network (4 convolutions 3x3 stride 2 of 32 channels on
 * bf16 tensor cores, FP32 accumulation, a dense head) reads a 64 x 64 x 4 resampling of a galaxy's
 * facet (visibility / flux re and im, cell mask, cell SNR) and proposes (e1, e2, ln r, ln sigma);
 * a galaxy with sigma <= max_sigma (rlf_proposal_set_max_sigma, default 0.05) starts its fit at
 * (e1, e2) with step 2 sigma (at least 0.02), the others at the reference's (0, 0) with step 0.1;
 * the fit keeps the last word.  Parameters:
 * rlf_cnn_param_count() floats, per convolution W[32][9 cin] (k = (3 ky + kx) cin + ci) and b[32],
 * then the head's W[4][512] (feature (4 y + x) 32 + c) and b[4]. */
typedef struct rlf_cnn rlf_cnn;
int rlf_cnn_param_count(void);
/* a network for training and prediction: batches of up to max_batch images, a device store of
 * `capacity` images and their targets (e1, e2, ln r) */
rlf_cnn *rlf_cnn_create(int max_batch, int capacity);
void rlf_cnn_destroy(rlf_cnn *cnn);
int rlf_cnn_set_params(rlf_cnn *cnn, const float *params);
int rlf_cnn_get_params(rlf_cnn *cnn, float *params);
/* resample n facets (host, rlf_obs_extract's layout facets[g][5][stride], ncoords[g], facet side
 * facet[g], flux[g]) into the store at [first, first + n) */
int rlf_cnn_store_facets(rlf_cnn *cnn, int first, int n, const double *facets, int stride,
                         const int *ncoords, const int *facet, const double *flux, double len);
int rlf_cnn_set_targets(rlf_cnn *cnn, int first, int n, const float *targets);
/* the store's images [n][64][64][4] as bf16 bit patterns: write, read */
int rlf_cnn_set_images(rlf_cnn *cnn, int first, int n, const uint16_t *images);
int rlf_cnn_read_images(rlf_cnn *cnn, int first, int n, uint16_t *images);
/* forward and backward of the store images idx[0 .. n): gradient of the mean loss (Gaussian
 * negative log-likelihood of (e1, e2) with the predicted sigma, plus half the squared error of
 * ln r) in the parameter layout, the loss, the head's outputs [n][4]; any output may be NULL */
int rlf_cnn_grads(rlf_cnn *cnn, const int *idx, int n, float *grads, float *loss, float *out);
/* one Adam step (learning rate lr) on the batch idx[0 .. n); loss may be NULL */
int rlf_cnn_train_step(rlf_cnn *cnn, const int *idx, int n, float lr, float *loss);
/* head outputs [n][4] of the store images [first, first + n) */
int rlf_cnn_predict(rlf_cnn *cnn, int first, int n, float *out);
/* the network rlf_obs_process / data_processing use with rlf_options.proposal (NULL unloads) */
int rlf_proposal_set_params(const float *params);
/* the gate of the loaded network: galaxies whose predicted sigma exceeds max_sigma (default 0.05)
 * keep the reference's start */
int rlf_proposal_set_max_sigma(float max_sigma);

/* -------- gridding without device allocation --------
 * No counterpart in the reference.  The gridding of gridding_visibilities (evaluate_uv_grid.c),
 * for callers that cannot allocate device memory: code inside a framework that owns the device
 * heap (a caching allocator or a fixed pool) and real-time callers that forbid allocation after
 * start-up.  It calls no cudaMalloc/cudaFree and no allocating library routine.
 *   u, v [ncoords], vis [num_channels*ncoords] complex128 (channel-major), sigma2, flag (may be
 *   NULL): DEVICE pointers; wavenumbers [num_channels]: a host array.  Outputs (DEVICE pointers,
 *   the layout of gridding_visibilities): new_vis [sizeg^2] complex128 and new_sigma2 [sizeg^2],
 *   both compacted to the non-empty cells in row-major order; sum_w [sizeg^2].
 *   stream: a cudaStream_t (NULL = the legacy default stream); the call waits for that stream.
 * Limits: sizeg <= RLF_NOALLOC_MAX_FACET, 1 <= num_channels <= 512; other sizes return an error.
 * The partial sums live in one fixed 4.6 MiB array of this library's device memory that every
 * GPU loading the library holds until exit.  The first call on a device looks up that array's
 * device address and caches it for the process (not valid across cudaDeviceReset).  The call
 * synchronises `stream` and cannot be captured into a CUDA graph.  Every call rewrites the
 * library's constant channel table and the gridding kernel's shared-memory attribute, which all
 * entry points of this library share: a call that overlaps any other call of the library (other
 * threads or streams, no-allocation or not) races with it, so the caller serialises all calls.
 * Returns 0, or non-zero with a message on stderr. */
#define RLF_NOALLOC_MAX_FACET 48
int rlf_gridding_visibilities_noalloc(const double *wavenumbers, unsigned int num_channels,
                                      unsigned int ncoords, const double *u, const double *v,
                                      const double *vis, const float *sigma2, const uint8_t *flag,
                                      double len, unsigned int sizeg, double *new_vis,
                                      double *new_sigma2, double *sum_w, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RLF_GB300_H */

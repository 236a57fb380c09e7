// Visibility-domain kernels: galaxy model visibilities, phase shift, sky model, source
// extraction with facet gridding, removal of fitted sources.  Declarations for the host layer.
#pragma once
#include "rlf_device.cuh"

namespace rlf {

constexpr int kMaxCh = 512;
constexpr unsigned kMaxExtractFacet = 118;  // 2 * F^2 doubles of shared memory per CTA
constexpr unsigned kMaxGridFacet = 84;      // 4 * F^2 doubles

// Element strides of a visibility array: index = row * s_row + ch * s_ch.  The reference's
// arrays are channel-major (s_row = 1, s_ch = n_rows, measurement_set.cpp:394-403).
struct VisLayout {
  long long s_row;
  long long s_ch;
};

struct Observation {
  int n_rows;
  int n_ch;
  VisLayout lay;
  const double* uu;   // [n_rows] metres
  const double* vv;
  const double* ww;
  double len;         // facet half-extent, wavelengths
};

// One galaxy of an extraction or removal batch.
struct GalaxyParams {
  double l, m;        // direction cosines
  double flux;        // uJy
  double scale;       // arcsec (R_mu, the catalogue scalelength under SCALELENGTH_ON)
  double e1, e2;      // ellipticity of the model to subtract (removal)
  int facet;          // facet cells per side
  int pad;
};

double fp32_probe_gflops(int blocks, int iters, cudaStream_t st);

int set_channels(int n_ch, const double* wavenumbers, const double* spec, cudaStream_t st);

// cell index of every visibility for facet size F (0xFFFF = flagged or outside the grid),
// evaluate_uv_grid.c:160-177 arithmetic in FP64
int launch_cell_index(const Observation& o, const uint8_t* flag, unsigned F, uint16_t* cell,
                      cudaStream_t st);
// sum of variances and of weights per cell for facet size F (the galaxy-independent half of
// gridding_visibilities), deterministic FP64
int launch_grid_weights(const Observation& o, const uint16_t* cell, const float* sigma2,
                        unsigned F, double* partial, int n_part, double* sum_sigma2,
                        double* sum_w, cudaStream_t st);
int grid_partial_blocks(int n_rows);
// partial [n_part][len] -> sums [len] (fixed-order reduction, one CTA per element)
int launch_reduce_partials(const double* partial, int n_part, int len, double* sums, cudaStream_t st);

// source extraction of one galaxy into per-CTA facet partials (F64 or mixed data)
int launch_extract_f64(const Observation& o, const double2* data, const double2* sky,
                       const uint16_t* cell, const GalaxyParams* gal, unsigned F, int gaussian,
                       double* partial, int n_part, cudaStream_t st);
int launch_extract_mixed(const Observation& o, const float2* data, const float2* sky,
                         const uint16_t* cell, const GalaxyParams* gal, unsigned F, int gaussian,
                         double* partial, int n_part, cudaStream_t st);
// gridding of a given visibility array (gridding_visibilities): cell computed on the fly
int launch_grid_vis_f64(const Observation& o, const double2* vis, const float* sigma2,
                        const uint8_t* flag, unsigned F, double* partial, int n_part,
                        cudaStream_t st);
// reduce the gridding partials and compact like gridding_visibilities' non-MPI tail
int launch_grid_vis_finalize(const double* partial, int n_part, unsigned F, double2* new_vis,
                             double* new_sigma2, double* sum_w, cudaStream_t st);

// Facet finalisation for galaxies g in [0, n): sums the partials in a fixed order, divides by
// the variances and compacts the non-empty cells in row-major order (evaluate_uv_grid.c:196-209,
// 113-133).  Writes packed cells at offset[g] (double or float) and ncoords[g]; optionally the
// full-grid sums (facet_vis/facet_sigma2/sum_w of the reference before compaction).
struct FacetOut {
  const int* offset;
  int* ncoords;
  void* gu; void* gv; void* dre; void* dim; void* sig2;
  int as_float;
};
int launch_facet_finalize(int n, const int* facets, const double* partial, int n_part,
                          long long partial_stride, const double* const* sum_sigma2,
                          const double* const* sum_w, double len, FacetOut out, cudaStream_t st);

// removal of one galaxy's round model from the sky model and fitted model from the data
// (data_processing.c:109-135); skipped when *error != 0
int launch_remove_f64(const Observation& o, double2* data, double2* sky, const GalaxyParams* gal,
                      const double* fit_e1e2, const int* fit_error, int gaussian, cudaStream_t st);
int launch_remove_mixed(const Observation& o, float2* data, float2* sky, const GalaxyParams* gal,
                        const double* fit_e1e2, const int* fit_error, int gaussian, cudaStream_t st);

// sky model: sky += sum over galaxies of round models (data_simulation.c:131-165); with
// sheared e and noise it is also the visibility simulator's model term
int launch_sky_model_f64(const Observation& o, double2* sky, const GalaxyParams* gals, int n_gal,
                         int use_e, int gaussian, cudaStream_t st);
int launch_sky_model_mixed(const Observation& o, float2* sky, const GalaxyParams* gals, int n_gal,
                           int use_e, int gaussian, cudaStream_t st);

// single-channel kernels behind data_galaxy_visibilities / data_visibilities_phase_shift
int launch_galaxy_vis_channel(int n, double spectra, double wavenumber, double e1, double e2,
                              double scale, double flux, double l, double m, const double* uu,
                              const double* vv, const double* ww, double2* vis, int gaussian,
                              cudaStream_t st);
int launch_phase_shift_channel(int n, double wavenumber, double l, double m, const double* uu,
                               const double* vv, const double* ww, double2* vis, cudaStream_t st);
// model_galaxy_visibilities_at_zero
int launch_model_at_zero(double e1, double e2, double scale, int n, const double* gu,
                         const double* gv, const double* sigma2, double* mod, int gaussian,
                         cudaStream_t st);
// evaluate_uv_grid_size: number of non-empty cells
int launch_count_cells(const Observation& o, const uint16_t* cell, unsigned F, unsigned* count_out,
                       cudaStream_t st);
// evaluate_facet_coords / average_facets on a full grid
int launch_facet_coords(double* gu, double* gv, double len, unsigned F, const double* count_w,
                        unsigned* n_out, cudaStream_t st);
int launch_average_facets(long long size, double2* vis, double* sigma2, const double* sum_w,
                          cudaStream_t st);
// visibility conversion float2 [ch][row] -> double2 [ch][row]
int launch_convert_f32_to_c64(long long n, const float2* in, double2* out, cudaStream_t st);
// Conversions between the caller's visibility order ([ch][row], index ch * n_rows + row) and an
// observation stored with its rows permuted (position inv[row]; launch_row_order): the caller's
// elements [i0, i0 + count) from / to a buffer holding just those elements, so that the host side
// is read or written in order and the device side is scattered or gathered.
int launch_c64_to_f32_scatter(long long i0, long long count, int n_rows, const double2* in, const int* inv,
                              float2* out, cudaStream_t st);
int launch_f32_to_c64_gather(long long i0, long long count, int n_rows, const float2* in, const int* inv,
                             double2* out, cudaStream_t st);
template <class T>
int launch_scatter_rows(long long i0, long long count, int n_rows, const T* in, const int* inv, T* out,
                        cudaStream_t st);
// out[p] = in[perm[p]] for p < n (the per-row arrays of a permuted observation)
int launch_gather_rows_f64(int n, const double* in, const int* perm, double* out, cudaStream_t st);
// inv[perm[p]] = p
int launch_invert_perm(int n, const int* perm, int* inv, cudaStream_t st);

}  // namespace rlf

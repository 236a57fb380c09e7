// Batched mixed-precision extraction and removal (rlf_batch.cu): declarations for the host layer.
#pragma once
#include "rlf_vis.cuh"
#include "rlf_fit.cuh"

namespace rlf {

constexpr int kBatchWarps = 8;                    // warps per extraction CTA (32 galaxies each)
constexpr size_t kBatchSmemMax = 227 * 1024;      // shared memory of one extraction CTA
constexpr unsigned kBatchMaxFacet = 28;           // largest facet the batched extraction holds
constexpr int kRemCh = 16;                        // channels per removal thread
constexpr int kRemTile = 64;                      // galaxies staged per shared-memory tile

// per-row FP32 table: u, v, w as double-float, u^2+v^2 and u*v
struct RowF {
  float u_hi, u_lo, v_hi, v_lo, w_hi, w_lo, q, uv;
};

// channel constants of the batched kernels; returns -1 when the channels are not evenly spaced
// closely enough for the T0 + ch*dT phase recurrence (the caller then uses per-galaxy kernels)
int batch_set_channels(int n_ch, const double* wavenumbers, const double* spec, double max_delay_m,
                       cudaStream_t st);
int launch_row_table(int n_rows, const double* uu, const double* vv, const double* ww, RowF* rows,
                     cudaStream_t st);
// visibilities are channel-major [ch][row]; gidx[group*32 + lane] = galaxy/slot index or -1
int launch_extract_batch(int n_rows, const RowF* rows, const float2* data, const float2* sky,
                         const uint16_t* cell, const GalaxyParams* gals, const int* gidx,
                         int n_groups, int F, int ctas, int gaussian, float2* partial,
                         cudaStream_t st);
int launch_finalize_batch(int n_groups, int ctas, int F, const float2* partial, const int* gidx,
                          const double* ss, const double* sw, double len, FacetOut out,
                          cudaStream_t st);
int launch_remove_batch(int n_rows, const RowF* rows, float2* data, float2* sky,
                        const GalaxyParams* gals, const FitOut* fit, int n_gal, int gaussian,
                        cudaStream_t st);

}  // namespace rlf

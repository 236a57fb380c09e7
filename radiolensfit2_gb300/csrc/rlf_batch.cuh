// Batched mixed-precision extraction and removal (rlf_batch.cu): declarations for the host layer.
#pragma once
#include "rlf_vis.cuh"
#include "rlf_fit.cuh"

namespace rlf {

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
// ---- sequential batch extraction (exact in-batch removal order)
#ifndef RLF_SEQ_THREADS
#define RLF_SEQ_THREADS 1024
#endif
#ifndef RLF_SEQ_CTAS_PER_SM
#define RLF_SEQ_CTAS_PER_SM 1
#endif
#ifndef RLF_SEQ_FACET_KB
#define RLF_SEQ_FACET_KB 128
#endif
constexpr int kSeqThreads = RLF_SEQ_THREADS;      // threads of a sequential extraction CTA
constexpr int kSeqCtasPerSm = RLF_SEQ_CTAS_PER_SM;  // CTAs per SM (register budget of the kernel)
constexpr int kSeqMaxSizes = 16;                  // distinct facet sizes in one batch
constexpr int kSeqMaxGal = 512;                   // galaxies in one batch
constexpr size_t kSeqFacetBudget = (size_t)RLF_SEQ_FACET_KB * 1024;  // shared facet accumulators of one batch
// shared memory per facet cell of the sequential extraction: compensated (hi, lo) FP32 pairs of the
// real and imaginary sums
constexpr size_t kSeqCellBytes = 2 * sizeof(float2);
constexpr size_t kSeqMaxSmem = 227 * 1024;  // shared memory of one sequential extraction CTA

// Run descriptor of one 16-channel chunk of one row for one facet size: the cell of the chunk's
// first channel in bits 0-15, bit 16+k set when channel k of the chunk is flagged, beyond the last
// channel or in another cell (so 0 in the high half = one run over all 16 channels).
// desc: [chunk][row]; cell: [ch][row] (launch_cell_index).
// desc1: [chunk][row] the cell of channels s..15 when the chunk is two runs, channels 0..s-1 in the
// first cell and s..15 (all within the observation) in one second cell (kNoCell: flagged), with
// s the first set mask bit; kNotTwoRun otherwise.
constexpr uint16_t kNotTwoRun = 0xFFFE;
int launch_cell_desc(int n_rows, int n_ch, const uint16_t* cell, uint32_t* desc, uint16_t* desc1, cudaStream_t st);

// Rows in the order of their uv points on a kOrderBins x kOrderBins grid over the facets' extent
// (v bin major, u bin minor; rows of one bin in any order): order[p] = the row at position p.
// Mixed-precision observations store their rows in this order, so that consecutive work items of
// the sequential extraction fall in the same facet cell for every facet size (a thin strip of
// constant v bin crosses a facet row's cells in increasing u).  bins: [kOrderBins^2] scratch.
constexpr int kOrderBins = 1024;
int launch_row_order(int n_rows, const double* uu, const double* vv, double inv_lambda0, double len, int* order,
                     int* bins, cudaStream_t st);

struct SeqBatch {
  int n_gal;
  const int* ctl;             // device round control of the unit, or nullptr: ctl[0] = j0, the first
                              // galaxy taking part in this round (the earlier ones keep their
                              // facets and fits); ctl[1] != 0: the unit has converged, skip
  const GalaxyParams* gals;   // [n_gal] in catalogue order
  const FitOut* fit;          // [n_gal] fits of the previous round, whose model differences
                              // (fitted - round) are removed from every later galaxy's facet; or
                              // nullptr in the first round
  const int* fidx;            // [n_gal] index of the galaxy's facet size in desc / cells
  const int* foff;            // [n_gal] offset of the galaxy's facet in the batch's cell buffer
  const int* facet;           // [n_gal] facet size
  int total_cells;            // sum of facet^2 over the batch
  int n_sizes;
  const uint32_t* desc[kSeqMaxSizes];
  const uint16_t* desc1[kSeqMaxSizes];
  const uint16_t* cells[kSeqMaxSizes];
  const int* items;           // work items (row, 16-channel chunk) = chunk * n_rows + row: the
  const int* n_simple;        // *n_simple single-run ones first, then the general ones
  const int* items2;          // work items of at most two runs per facet size, count *n_two
  const int* n_two;
  int* queue;                 // [3] work counters of the extraction (single-run items, chunks of 32
                              // general items, two-run items), zeroed by launch_extract_seq
};
size_t seq_smem_bytes(int n_gal, int total_cells, int n_sizes);
// split the batch's work items into single-run ones (front of items), general ones (back of items)
// and ones of at most two runs for every facet size (items2; only with chunk polynomials), for
// launch_extract_seq; items, items2: [n_rows * chunks], counters: [3] (simple, general, two-run).
// Each class keeps the items' order within a block of 256 items.
int launch_classify_items(long long total, const SeqBatch& b, int* items, int* items2, int* counters,
                          cudaStream_t st);
// partial: [ctas][total_cells] double2, each CTA's compensated sums
int launch_extract_seq(int n_rows, const RowF* rows, const float2* data, const float2* sky, const SeqBatch& b,
                       int gaussian, int ctas, double2* partial, cudaStream_t st);
// partial sums of every CTA -> facet of each galaxy (FP64 sums in CTA order), evaluate_uv_grid.c
// finalisation and compaction into out (slot = galaxy index in the batch)
int launch_finalize_seq(const SeqBatch& b, int ctas, const double2* partial, const double* const* ss,
                        const double* const* sw, double len, FacetOut out, cudaStream_t st);
// the un-averaged facet sums of every galaxy of the batch (channel shards): out[slot][4][stride] =
// sum of vis re, sum of vis im, sum of sigma^2, sum of weights per cell, zero beyond F^2
int launch_partials_seq(const SeqBatch& b, int ctas, const double2* partial, const double* const* ss,
                        const double* const* sw, double* out, int stride, cudaStream_t st);
// vis += the round models (sheared = 0: the sky model) or the sheared models (sheared = 1: the
// simulator) of n_gal galaxies, FP32 visibilities, evenly spaced channels (batch_set_channels)
int launch_model_sum_batch(int n_rows, const RowF* rows, float2* vis, const GalaxyParams* gals, int n_gal,
                           int sheared, int gaussian, cudaStream_t st);
int launch_remove_batch(int n_rows, const RowF* rows, float2* data, float2* sky,
                        const GalaxyParams* gals, const FitOut* fit, int n_gal, int gaussian,
                        cudaStream_t st);

}  // namespace rlf

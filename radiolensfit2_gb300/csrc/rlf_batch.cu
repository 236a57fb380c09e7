// Batched FP32 visibility passes: many galaxies per pass over the visibilities.
//
// A one-galaxy pass over the data is HBM-bound (one read of data and sky model per galaxy);
// taking a batch of galaxies per pass reads the data once per batch and turns the pass into
// FP32/SFU work.  Every kernel forms, per (row, galaxy), the delay p = u l + v m + w n in
// double-float arithmetic from an FP32 row table, the phase turns T(ch) = p * inv_lambda(ch) =
// T0 + ch * dT (channels evenly spaced) reduced modulo 1, and rotates through the channels of a
// 16-channel chunk by a recurrence in exp(-+2 pi i dT).
//
//   k_extract_seq      source extraction of a sub-batch in the reference's removal order
//                      (source_extraction.c:46-68, evaluate_uv_grid.c:143-211, data_processing.c:61-138)
//   k_finalize_seq     per-galaxy facet sums and finalisation
//   k_remove_batch     removal of a sub-batch's fitted and round models (data_processing.c:109-135)
//   k_model_sum_batch  sums of round or sheared models: sky model and simulator
#include "rlf_batch.cuh"
#include "rlf_fit.cuh"
#include <stdio.h>
#include <algorithm>

namespace rlf {

struct BatchChan {
  float spec;      // spectral factor
  float wn2;       // wavenumber^2
  float dl;        // wn2 / wn2 at the centre of the channel's 16-channel chunk - 1
  float pad;
};
// A galaxy profile P(x), x = scale factor * wn2 * (u^2 + v^2), across the channels of a 16-channel
// chunk is P(x_c (1 + dl)) with x_c at the chunk's centre and |dl| below ~1% for the usual
// channelisations; there it is the cubic  sum_j cf_j dl^j  (profile_poly) to ~1e-9 of the peak, and
// sums over the chunk's channels weighted by the spectral factors reduce to the moments
// M_j = sum_k spec_k dl_k^j.  c_chunk_poly is set when every chunk is within that range.
struct BatchChunk {
  float wn2c;      // wn2 at the chunk's centre
  float mom[4];    // M_0 .. M_3
  float pad[3];
};
constexpr int kChunks = kMaxCh / 16;
__constant__ BatchChan c_bch[kMaxCh];
__constant__ BatchChunk c_chunk[kChunks];
// moments of the channels before and from channel s of a chunk: [chunk][s][0..3] = sum_{k<s},
// [4..7] = sum_{k>=s} of spec_k dl_k^j (the two runs of a chunk crossing a cell boundary at s)
__constant__ float c_chunk_split[kChunks][17][8];
// the channels 2q and 2q + 1 side by side for the packed (two-lane FP32) channel loops:
// dl of both, then minus the spectral factor of both
__constant__ float4 c_pair[kMaxCh / 2];
__constant__ int c_chunk_poly;
static int g_chunk_poly[64];  // host copy of c_chunk_poly per device (selects the kernel variant)
static int g_nch[64];         // host copy of c_bnch per device
__constant__ float c_il0_hi, c_il0_lo, c_dil_hi, c_dil_lo;  // inv_lambda(0) and its channel step
__constant__ int c_bnch;

static int check(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf: %s: %s\n", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

int batch_set_channels(int n_ch, const double* wavenumbers, const double* spec, double max_delay_m,
                       cudaStream_t st) {
  if (n_ch < 1 || n_ch > kMaxCh) return 1;
  const double il0 = wavenumbers[0] / (2. * kPi);
  const double il1 = n_ch > 1 ? wavenumbers[n_ch - 1] / (2. * kPi) : il0;
  const double dil = n_ch > 1 ? (il1 - il0) / (n_ch - 1) : 0.0;
  // the batched kernels assume inv_lambda(ch) = il0 + ch * dil; reject layouts where that would
  // move a phase by more than 1e-9 turn at the largest delay
  double worst = 0.0;
  for (int c = 0; c < n_ch; ++c) {
    const double il = wavenumbers[c] / (2. * kPi);
    worst = fmax(worst, fabs(il - (il0 + c * dil)));
  }
  if (worst * max_delay_m > 1e-9) return -1;
  static BatchChan h[kMaxCh];
  static float4 hp[kMaxCh / 2];
  static BatchChunk hc[kChunks];
  static float hs[kChunks][17][8];
  double dmax = 0.0;
  for (int c0 = 0; c0 < n_ch; c0 += 16) {
    const int c1 = std::min(n_ch, c0 + 16);
    double lo = 1e300, hi = -1e300;
    for (int c = c0; c < c1; ++c) {
      const double w2 = wavenumbers[c] * wavenumbers[c];
      lo = std::min(lo, w2);
      hi = std::max(hi, w2);
    }
    const double wc = 0.5 * (lo + hi);
    double mom[4] = {0, 0, 0, 0};
    for (int c = c0; c < c1; ++c) {
      const double d = wavenumbers[c] * wavenumbers[c] / wc - 1.0;
      dmax = std::max(dmax, fabs(d));
      h[c].spec = (float)spec[c];
      h[c].wn2 = (float)(wavenumbers[c] * wavenumbers[c]);
      h[c].dl = (float)d;
      h[c].pad = 0.f;
      double dp = 1.0;
      for (int j = 0; j < 4; ++j) { mom[j] += spec[c] * dp; dp *= d; }
    }
    BatchChunk& k = hc[c0 / 16];
    k.wn2c = (float)wc;
    for (int j = 0; j < 4; ++j) k.mom[j] = (float)mom[j];
    for (int sp = 0; sp <= 16; ++sp) {
      double pre[4] = {0, 0, 0, 0}, suf[4] = {0, 0, 0, 0};
      for (int c = c0; c < c1; ++c) {
        const double d = wavenumbers[c] * wavenumbers[c] / wc - 1.0;
        double dp = 1.0;
        for (int j = 0; j < 4; ++j) {
          if (c - c0 < sp) pre[j] += spec[c] * dp;
          else suf[j] += spec[c] * dp;
          dp *= d;
        }
      }
      for (int j = 0; j < 4; ++j) { hs[c0 / 16][sp][j] = (float)pre[j]; hs[c0 / 16][sp][4 + j] = (float)suf[j]; }
    }
    k.pad[0] = k.pad[1] = k.pad[2] = 0.f;
  }
  for (int q = 0; 2 * q < n_ch; ++q) {
    const int c1 = std::min(2 * q + 1, n_ch - 1);
    hp[q] = make_float4(h[2 * q].dl, h[c1].dl, -h[2 * q].spec, 2 * q + 1 < n_ch ? -h[c1].spec : 0.f);
  }
  // truncation of the cubic: below 2.5 dl^4 of the peak (exponential profile; less for the
  // Gaussian one over the range where it is not negligible)
  const int poly = 2.5 * dmax * dmax * dmax * dmax <= 1e-8 ? 1 : 0;
  const float il0_hi = (float)il0, il0_lo = (float)(il0 - (double)il0_hi);
  const float dil_hi = (float)dil, dil_lo = (float)(dil - (double)dil_hi);
  cudaError_t e = cudaMemcpyToSymbolAsync(c_bch, h, sizeof(BatchChan) * n_ch, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_il0_hi, &il0_hi, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_il0_lo, &il0_lo, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_dil_hi, &dil_hi, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_dil_lo, &dil_lo, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_bnch, &n_ch, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_chunk, hc, sizeof(BatchChunk) * ((n_ch + 15) / 16), 0,
                                                     cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_chunk_poly, &poly, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_pair, hp, sizeof(float4) * ((n_ch + 1) / 2), 0,
                                                     cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_chunk_split, hs, sizeof(float) * 17 * 8 * ((n_ch + 15) / 16), 0,
                                                     cudaMemcpyHostToDevice, st);
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    g_chunk_poly[dev] = poly;
    g_nch[dev] = n_ch;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { fprintf(stderr, "rlf: batch channels: %s\n", cudaGetErrorString(e)); return (int)e; }
  return 0;
}

// --------------------------------------------------------------- row table
__global__ void k_row_table(int n_rows, const double* uu, const double* vv, const double* ww, RowF* rows) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x) {
    const double u = uu[r], v = vv[r], w = ww[r];
    RowF o;
    f2 a = df_from_double(u), b = df_from_double(v), c = df_from_double(w);
    o.u_hi = a.hi; o.u_lo = a.lo; o.v_hi = b.hi; o.v_lo = b.lo; o.w_hi = c.hi; o.w_lo = c.lo;
    o.q = (float)(u * u + v * v);
    o.uv = (float)(u * v);
    rows[r] = o;
  }
}

int launch_row_table(int n_rows, const double* uu, const double* vv, const double* ww, RowF* rows,
                     cudaStream_t st) {
  int b = (n_rows + 255) / 256;
  if (b > 8192) b = 8192;
  k_row_table<<<b, 256, 0, st>>>(n_rows, uu, vv, ww, rows);
  return check("k_row_table");
}

// per-galaxy FP32 parameters of the batched kernels
struct GalF {
  f2 l, m, n;    // direction cosines, n = sqrt(1-l^2-m^2)-1
  float sf0;     // round model: (scale[rad])^2
  float flux;
  float sf1;     // fitted model: (scale[rad])^2 / detA^2
  float A, B, Cc;  // |k'|^2 = A u^2 + B uv + C v^2 for the sheared model
  int active;
};

__device__ __forceinline__ GalF load_gal(const GalaxyParams& g, const double* e12, const int* err) {
  GalF o;
  o.l = df_from_double(g.l);
  o.m = df_from_double(g.m);
  o.n = df_from_double(sqrt(1. - g.l * g.l - g.m * g.m) - 1.);
  o.flux = (float)g.flux;
  o.sf0 = (float)scale_factor(0., 0., g.scale);
  const double e1 = e12 ? e12[0] : g.e1, e2 = e12 ? e12[1] : g.e2;
  o.sf1 = (float)scale_factor(e1, e2, g.scale);
  // k1 = (1+e1)u + e2 v, k2 = e2 u + (1-e1) v  ->  k1^2 + k2^2
  o.A = (float)((1. + e1) * (1. + e1) + e2 * e2);
  o.B = (float)(2. * e2 * (1. + e1) + 2. * e2 * (1. - e1));
  o.Cc = (float)(e2 * e2 + (1. - e1) * (1. - e1));
  o.active = err ? (*err == 0) : 1;
  return o;
}

// delay p = u l + v m + w n in double-float
__device__ __forceinline__ f2 delay_df(const RowF& r, const GalF& g) {
  f2 a = two_prod(r.u_hi, g.l.hi);
  a.lo = fmaf(r.u_hi, g.l.lo, fmaf(r.u_lo, g.l.hi, a.lo));
  f2 b = two_prod(r.v_hi, g.m.hi);
  b.lo = fmaf(r.v_hi, g.m.lo, fmaf(r.v_lo, g.m.hi, b.lo));
  f2 c = two_prod(r.w_hi, g.n.hi);
  c.lo = fmaf(r.w_hi, g.n.lo, fmaf(r.w_lo, g.n.hi, c.lo));
  f2 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  s = quick_two_sum(s.hi, s.lo);
  f2 t = two_sum(s.hi, c.hi);
  t.lo += s.lo + c.lo;
  return quick_two_sum(t.hi, t.lo);
}

// (hi, lo) * (y_hi, y_lo) reduced modulo 1 to [-1/2, 1/2] as double-float
__device__ __forceinline__ f2 turns_mod1(f2 p, float y_hi, float y_lo) {
  f2 t = two_prod(p.hi, y_hi);
  t.lo = fmaf(p.hi, y_lo, fmaf(p.lo, y_hi, t.lo));
  const float k = rintf(t.hi);
  return quick_two_sum(t.hi - k, t.lo);
}

// T0 + ch * dT reduced to [-1/2, 1/2] (float)
__device__ __forceinline__ float turns_at(f2 T0, f2 dT, int ch) {
  const float c = (float)ch;
  f2 p = two_prod(c, dT.hi);
  p.lo = fmaf(c, dT.lo, p.lo);
  const float k = rintf(p.hi);
  f2 s = two_sum(T0.hi, p.hi - k);
  const float t = s.hi + (s.lo + T0.lo + p.lo);
  return t - rintf(t);
}

__device__ __forceinline__ float round_shape(float sfq) {
  // exponential profile (galaxy_visibilities.c:48-53): (1 + x)^-3/2
  const float y = rsqrtf(1.f + sfq);
  return y * y * y;
}

// ------------------------------------------------------------- extraction
// Sequential batch extraction: the facets of a batch of galaxies in catalogue order, each one
// extracted as data_processing.c:61-138 would extract it after fitting and removing every earlier
// galaxy of the batch.  One thread holds the residual data - sky of one row and 16 channels in
// registers and walks the batch's galaxies in order; for galaxy j it
//   * adds the residual, phase-shifted to the galaxy (exp(-2 pi i T_j)), plus the galaxy's own
//     round model (real after the shift) into the galaxy's facet cell: source_extraction.c:46-68
//     and the gridding of evaluate_uv_grid.c:143-211;
//   * subtracts the galaxy's model difference fitted - round of the previous round's fit from the
//     residual (data_processing.c:109-135 removes the fitted model from the data and the round
//     model from the sky model), so every later galaxy sees it removed.
// The first round (no fits yet) is the plain batched extraction; each further round uses the fits
// of the round before, and the rounds converge to the sequential result (a galaxy's facet depends
// on earlier galaxies' fits only through their weak, smooth model differences).
// The phase of each (row, galaxy) is formed once: delay p = u l + v m + w n in double-float, phase
// turns T(ch) = p * inv_lambda(ch) = T0 + ch * dT, reduced modulo 1.  Within a 16-channel chunk the
// rotation is a recurrence in w = exp(-2 pi i dT) anchored with an accurate sincospi at the first
// channel of the chunk (Horner's rule when nothing is removed).
// Facets of all batch galaxies are accumulated in shared memory (FP32 atomics); every CTA writes
// its partial facets, reduced in FP64 in CTA order by k_finalize_seq.
constexpr int kChunk = 16;

struct __align__(16) SeqGal {
  GalF g;
  int fidx;      // facet size index
  int off;       // facet offset in the shared buffer (float2 units)
  int apply;     // subtract fitted - round (good fit in the previous round)
};

__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

size_t seq_smem_bytes(int n_gal, int total_cells, int n_sizes) {
  return align16((size_t)total_cells * kSeqCellBytes) + align16((size_t)n_gal * sizeof(SeqGal)) +
         (size_t)n_sizes * kSeqThreads * (sizeof(uint32_t) + sizeof(uint16_t));
}

__global__ void k_cell_desc(int n_rows, int nch, const uint16_t* __restrict__ cell, uint32_t* __restrict__ desc,
                            uint16_t* __restrict__ desc1) {
  const int nchunk = (nch + kChunk - 1) / kChunk;
  const long long total = (long long)n_rows * nchunk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t % n_rows);
    const int c0 = (int)(t / n_rows) * kChunk;
    const uint16_t c = cell[(size_t)c0 * n_rows + r];
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
      const int ch = c0 + k;
      if (ch >= nch || c == kNoCell || cell[(size_t)ch * n_rows + r] != c) mask |= 1u << k;
    }
    desc[t] = (uint32_t)c | (mask << 16);
    // two runs: the first cell valid, the other channels a suffix s..15 inside the observation,
    // all in one cell
    uint16_t c1 = kNotTwoRun;
    if (mask && c != kNoCell) {
      const int sp = __ffs(mask) - 1;
      const uint32_t suffix = (0xFFFFu << sp) & 0xFFFFu;
      if (mask == suffix && c0 + kChunk <= nch) {
        const uint16_t cs = cell[(size_t)(c0 + sp) * n_rows + r];
        bool same = true;
        for (int k = sp + 1; k < kChunk; ++k) same = same && cell[(size_t)(c0 + k) * n_rows + r] == cs;
        if (same) c1 = cs;
      }
    }
    desc1[t] = c1;
  }
}

int launch_cell_desc(int n_rows, int n_ch, const uint16_t* cell, uint32_t* desc, uint16_t* desc1, cudaStream_t st) {
  const long long total = (long long)n_rows * ((n_ch + kChunk - 1) / kChunk);
  const int blocks = (int)std::min<long long>((total + 255) / 256, 8192);
  k_cell_desc<<<blocks, 256, 0, st>>>(n_rows, n_ch, cell, desc, desc1);
  return check("k_cell_desc");
}

__device__ __forceinline__ int order_bin(double u, double v, double il0, double scale, double len) {
  int bu = (int)floor((u * il0 + len) * scale), bv = (int)floor((v * il0 + len) * scale);
  bu = min(max(bu, 0), kOrderBins - 1);
  bv = min(max(bv, 0), kOrderBins - 1);
  return bv * kOrderBins + bu;
}
__global__ void k_order_count(int n_rows, const double* __restrict__ uu, const double* __restrict__ vv, double il0,
                              double scale, double len, int* __restrict__ bins) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x)
    atomicAdd(&bins[order_bin(uu[r], vv[r], il0, scale, len)], 1);
}
// exclusive prefix sum of the kOrderBins^2 bin counts in place: one block of kOrderBins threads, each
// over kOrderBins consecutive bins
__global__ void __launch_bounds__(kOrderBins) k_order_scan(int* __restrict__ bins) {
  __shared__ int sums[kOrderBins];
  int* mine = bins + (size_t)threadIdx.x * kOrderBins;
  int s = 0;
  for (int k = 0; k < kOrderBins; ++k) s += mine[k];
  sums[threadIdx.x] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan of the per-thread sums
  for (int o = 1; o < kOrderBins; o <<= 1) {
    const int x = threadIdx.x >= o ? sums[threadIdx.x - o] : 0;
    __syncthreads();
    sums[threadIdx.x] += x;
    __syncthreads();
  }
  int run = sums[threadIdx.x] - s;
  for (int k = 0; k < kOrderBins; ++k) {
    const int c = mine[k];
    mine[k] = run;
    run += c;
  }
}
__global__ void k_order_place(int n_rows, const double* __restrict__ uu, const double* __restrict__ vv, double il0,
                              double scale, double len, int* __restrict__ bins, int* __restrict__ order) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rows; r += gridDim.x * blockDim.x)
    order[atomicAdd(&bins[order_bin(uu[r], vv[r], il0, scale, len)], 1)] = r;
}

int launch_row_order(int n_rows, const double* uu, const double* vv, double inv_lambda0, double len, int* order,
                     int* bins, cudaStream_t st) {
  if (n_rows <= 0) return 0;
  const double scale = len > 0 ? kOrderBins / (2 * len) : 0.0;
  const cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(int) * kOrderBins * kOrderBins, st);
  if (e != cudaSuccess) { fprintf(stderr, "rlf: row order: %s\n", cudaGetErrorString(e)); return (int)e; }
  const int blocks = std::min((n_rows + 255) / 256, 4096);
  k_order_count<<<blocks, 256, 0, st>>>(n_rows, uu, vv, inv_lambda0, scale, len, bins);
  int r = check("k_order_count");
  if (r) return r;
  k_order_scan<<<1, kOrderBins, 0, st>>>(bins);
  r = check("k_order_scan");
  if (r) return r;
  k_order_place<<<blocks, 256, 0, st>>>(n_rows, uu, vv, inv_lambda0, scale, len, bins, order);
  return check("k_order_place");
}

// Work items (row, chunk) of a batch split into "simple" ones, one run of 16 valid channels for
// every facet size of the batch (front of items, count in counters[0]), "two-run" ones, at most
// two runs for every facet size (items2, counters[2]; only when two_run), and the general others
// (back of items, counters[1]), so that the extraction runs each kind without divergence between
// the lanes of a warp.  A block takes 256 consecutive items and places each class's items
// contiguously, in that order, with one counter update per class (the rows are stored in uv
// order, so neighbouring items stay neighbours in uv).
constexpr int kClassifyThreads = 256;
__global__ void __launch_bounds__(kClassifyThreads) k_classify_items(long long total, SeqBatch b,
                                                                     int two_run, int* __restrict__ items,
                                                                     int* __restrict__ items2,
                                                                     int* __restrict__ counters) {
  constexpr int kWarps = kClassifyThreads / 32;
  __shared__ int wcount[3][kWarps];
  __shared__ int bbase[3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long p0 = (long long)blockIdx.x * kClassifyThreads; p0 < total; p0 += (long long)gridDim.x * kClassifyThreads) {
    const long long t = p0 + threadIdx.x;
    const bool live = t < total;
    bool simple = live, two = live && two_run;
    if (live)
      for (int f = 0; f < b.n_sizes; ++f) {
        const bool one = (b.desc[f][t] >> 16) == 0;
        simple = simple && one;
        two = two && (one || b.desc1[f][t] != kNotTwoRun);
      }
    two = two && !simple;
    const bool general = live && !simple && !two;
    const unsigned m[3] = {__ballot_sync(0xffffffffu, simple), __ballot_sync(0xffffffffu, general),
                           __ballot_sync(0xffffffffu, two)};
    if (lane == 0)
      for (int k = 0; k < 3; ++k) wcount[k][warp] = __popc(m[k]);
    __syncthreads();
    if (threadIdx.x < 3) {
      int n = 0;
      for (int w = 0; w < kWarps; ++w) n += wcount[threadIdx.x][w];
      bbase[threadIdx.x] = n ? atomicAdd(&counters[threadIdx.x], n) : 0;
    }
    __syncthreads();
    const int k = simple ? 0 : (general ? 1 : 2);
    if (live) {
      int pos = bbase[k] + __popc(m[k] & ((1u << lane) - 1u));
      for (int w = 0; w < warp; ++w) pos += wcount[k][w];
      if (k == 0) items[pos] = (int)t;
      else if (k == 2) items2[pos] = (int)t;
      else items[total - 1 - pos] = (int)t;
    }
    __syncthreads();
  }
}

int launch_classify_items(long long total, const SeqBatch& b, int* items, int* items2, int* counters,
                          cudaStream_t st) {
  const cudaError_t e = cudaMemsetAsync(counters, 0, 3 * sizeof(int), st);
  if (e != cudaSuccess) { fprintf(stderr, "rlf: classify: %s\n", cudaGetErrorString(e)); return (int)e; }
  int dev = 0;
  cudaGetDevice(&dev);
  const int two_run = (dev >= 0 && dev < 64) ? g_chunk_poly[dev] : 0;
  const int blocks = (int)std::min<long long>((total + kClassifyThreads - 1) / kClassifyThreads, 4096);
  k_classify_items<<<blocks, kClassifyThreads, 0, st>>>(total, b, two_run, items, items2, counters);
  return check("k_classify_items");
}

// Compensated deposit into a facet cell: the FP32 accumulator pair (hi, lo) of the cell's real and
// imaginary sums, hi at fac[k] and lo at fac[k + lo_off].  The atomic add to hi returns the value it
// replaced, so the depositing thread knows the sum hi took, RN(old + v), and adds that addition's
// rounding error (Knuth's TwoSum, exact in FP32) to lo: hi + lo carries the cell's sum to about
// 2^-48 relative, independent of the order and number of deposits.
__device__ __forceinline__ void comp_add(float* hi, float* lo, float v) {
  const float old = atomicAdd(hi, v);
  const float s = old + v;
  const float bv = s - old;
  const float err = (old - (s - bv)) + (v - bv);
  atomicAdd(lo, err);
}
__device__ __forceinline__ void comp_add2(float2* fac, int k, int lo_off, float vr, float vi) {
  comp_add(&fac[k].x, &fac[k + lo_off].x, vr);
  comp_add(&fac[k].y, &fac[k + lo_off].y, vi);
}

// The deposits of a warp's lanes into one galaxy's facet (key: the lane's cell, negative for none).
// Float atomic adds to shared memory from several lanes of an instruction to one address are
// retried lane by lane, and with the rows in uv order a warp's lanes mostly fall in one cell of
// the small facets, or in two at a cell boundary.  So the lanes of each cell (up to four cells)
// are summed exactly as integers (redux.sync) on the fixed-point grid of 2^-24 .. 2^-25 of the
// group's largest magnitude (a power of two, so the scaling is exact; the sum stays below 2^30)
// and the group's first lane adds the sum; lanes of further cells, or of groups with non-finite or
// tiny values, add their own.  Every addition is compensated (comp_add2, lo_off: the offset of the
// lo accumulators).  All 32 lanes must call it.
__device__ __forceinline__ void warp_deposit(float2* fac, int lo_off, int key, float vr, float vi, int lane) {
  const unsigned mag = max(__float_as_uint(fabsf(vr)), __float_as_uint(fabsf(vi)));  // NaN above inf
  // the common case, every lane in one cell: the first group of the loop below without its
  // bookkeeping (the same sums and the same deposit)
  const int k0 = __shfl_sync(0xffffffffu, key, 0);
  if (__all_sync(0xffffffffu, key == k0) && k0 >= 0) {
    const int e = (int)(__reduce_max_sync(0xffffffffu, mag) >> 23);
    if (e >= 24 && e < 255) {
      const float sc = __uint_as_float((unsigned)(278 - e) << 23);
      const float inv = __uint_as_float((unsigned)(e - 24) << 23);
      const int sr = __reduce_add_sync(0xffffffffu, __float2int_rn(vr * sc));
      const int si = __reduce_add_sync(0xffffffffu, __float2int_rn(vi * sc));
      if (lane == 0) comp_add2(fac, k0, lo_off, (float)sr * inv, (float)si * inv);
    } else {
      comp_add2(fac, key, lo_off, vr, vi);
    }
    return;
  }
  unsigned todo = __ballot_sync(0xffffffffu, key >= 0), rest = 0;
#pragma unroll 1
  for (int it = 0; it < 4 && todo; ++it) {
    const int src = __ffs(todo) - 1;
    const int k = __shfl_sync(0xffffffffu, key, src);
    const bool in = key == k;
    const unsigned m = __ballot_sync(0xffffffffu, in);
    const int e = (int)(__reduce_max_sync(0xffffffffu, in ? mag : 0u) >> 23);  // biased exponent
    if (e >= 24 && e < 255) {
      const float sc = __uint_as_float((unsigned)(278 - e) << 23);  // 2^(151 - e)
      const float inv = __uint_as_float((unsigned)(e - 24) << 23);  // 2^(e - 151)
      const int sr = __reduce_add_sync(0xffffffffu, in ? __float2int_rn(vr * sc) : 0);
      const int si = __reduce_add_sync(0xffffffffu, in ? __float2int_rn(vi * sc) : 0);
      if (lane == src) comp_add2(fac, k, lo_off, (float)sr * inv, (float)si * inv);
    } else {
      rest |= m;
    }
    todo &= ~m;
  }
  if (((todo | rest) >> lane) & 1u) comp_add2(fac, key, lo_off, vr, vi);
}

// sin(2 pi t) and cos(2 pi t) for a phase in turns: quadrant q = rint(4t), remainder
// r = t - q/4 in [-1/8, 1/8] (an angle within pi/4), Taylor series of sin and cos in r with the
// coefficients (2 pi)^n / n! rounded to float (terms below 2e-9 dropped); ~1.3 ulp.
__device__ __forceinline__ void sincos_turn(float t, float* s, float* c) {
  const float q = rintf(4.f * t);
  const float r = fmaf(q, -0.25f, t);
  const float r2 = r * r;
  float sp = 42.058692932128906f;
  sp = fmaf(sp, r2, -76.70585632324219f);
  sp = fmaf(sp, r2, 81.6052474975586f);
  sp = fmaf(sp, r2, -41.34170150756836f);
  sp = fmaf(sp, r2, 6.2831854820251465f);
  sp *= r;
  float cp = 7.903536319732666f;
  cp = fmaf(cp, r2, -26.42625617980957f);
  cp = fmaf(cp, r2, 60.2446403503418f);
  cp = fmaf(cp, r2, -85.45681762695312f);
  cp = fmaf(cp, r2, 64.93939208984375f);
  cp = fmaf(cp, r2, -19.739208221435547f);
  cp = fmaf(cp, r2, 1.f);
  const int qi = (int)q & 3;
  const float s1 = (qi & 1) ? cp : sp, c1 = (qi & 1) ? -sp : cp;
  *s = (qi & 2) ? -s1 : s1;
  *c = (qi & 2) ? -c1 : c1;
}

// sin and cos of 2 pi t for |t| <= 1/2 from the SFU (__sincosf: absolute error below 2^-21.4 on
// [-pi, pi]), for a phase that no recurrence amplifies: the first channel of a chunk, or of a
// chunk's second run.  The channel step exp(-2 pi i dT), raised to the 15th power by the
// recurrence, keeps sincos_turn.
__device__ __forceinline__ void sincos_turn_sfu(float t, float* s, float* c) {
  __sincosf(6.28318530717958647692f * t, s, c);
}

__device__ __forceinline__ float profile(float x, int gauss) {
  return gauss ? __expf(-0.5f * x) : round_shape(x);
}

// P(x_c (1 + dl)) = cf0 + cf1 dl + cf2 dl^2 + cf3 dl^3 around the chunk centre x_c: the exponential
// profile (1 + x)^(-3/2) = P_c (1 + r dl)^(-3/2), r = x_c / (1 + x_c), from the binomial series;
// the Gaussian exp(-x/2) = P_c exp(-(x_c/2) dl) from the exponential series.
template <int GAUSS>
__device__ __forceinline__ void profile_poly(float xc, float cf[4]) {
  if (GAUSS) {
    const float h = -0.5f * xc;
    cf[0] = __expf(h);
    cf[1] = cf[0] * h;
    cf[2] = cf[1] * h * 0.5f;
    cf[3] = cf[2] * h * (1.f / 3.f);
  } else {
    const float y = rsqrtf(1.f + xc);
    const float P = y * y * y, r = xc * y * y;
    cf[0] = P;
    cf[1] = -1.5f * P * r;
    cf[2] = 1.875f * P * r * r;
    cf[3] = -2.1875f * P * r * r * r;
  }
}
__device__ __forceinline__ float poly3(const float c[4], float d) { return fmaf(fmaf(fmaf(c[3], d, c[2]), d, c[1]), d, c[0]); }

// Packed FP32 pairs (the two-lane FMA of this GPU: one instruction for both lanes, each lane
// rounded as fmaf).  The channel loops below run channels 2q and 2q + 1 side by side, the phase
// stepping by w^2 from exp(-2 pi i T) at the first two channels.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// one work item (row r, channels c0 .. c0 + 15) against every galaxy of the batch, in order.
// MODE 0: exact per-channel profiles; 1: the profiles from the chunk polynomial, one profile
// evaluation per galaxy and chunk; 2: as 1 for an observation of exactly one 16-channel chunk, so
// that the channel constants are compile-time operands; 3: as 1 for 2-4 full 16-channel chunks,
// the item's chunk CI a compile-time constant when the caller knows it (CI >= 0: the channel
// constants are then operands of the arithmetic instructions, not loads of a dynamic index), CI =
// -1 for any chunk.  Single-run items (SIMPLE) are called by all lanes of a warp (run_deposit), a
// lane without an item with live = false and any valid t.
template <int GAUSS, bool SIMPLE, int MODE, bool FIT, int CI = -1>
__device__ __forceinline__ void seq_item(int t, bool live, int n_rows, int nch, int ng, const RowF* __restrict__ rows,
                                         const float2* __restrict__ data, const float2* __restrict__ sky,
                                         const SeqBatch& b, const SeqGal* sg, uint32_t* dcache, float2* acc) {
  constexpr bool POLY = MODE > 0;
  constexpr bool ONE = MODE == 2;
  constexpr bool FIXED = CI >= 0;
  const int tid = threadIdx.x;
  const int r = ONE ? t : (FIXED ? t - CI * n_rows : t % n_rows);
  const int c0 = ONE ? 0 : (FIXED ? CI * kChunk : (t / n_rows) * kChunk);
  const int nk = (ONE || FIXED) ? kChunk : min(kChunk, nch - c0);
  const RowF rw = rows[r];
  // the residual of channel c0 + k: real part in rp[k / 2], imaginary part in ip[k / 2] (lane k % 2)
  float2 rp[kChunk / 2], ip[kChunk / 2];
#define PR(k) (((k) & 1) ? rp[(k) >> 1].y : rp[(k) >> 1].x)
#define PI(k) (((k) & 1) ? ip[(k) >> 1].y : ip[(k) >> 1].x)
#pragma unroll
  for (int k = 0; k < kChunk; ++k) {
    PR(k) = PI(k) = 0.f;
    if (SIMPLE || k < nk) {
      const size_t idx = (size_t)(c0 + k) * n_rows + r;
      const float2 d = data[idx], s = sky[idx];
      PR(k) = d.x - s.x;
      PI(k) = d.y - s.y;
    }
  }
  for (int f = 0; f < b.n_sizes; ++f) dcache[f * kSeqThreads + tid] = b.desc[f][t];
  const float uu = rw.u_hi * rw.u_hi, vv = rw.v_hi * rw.v_hi;
  const float invq = rw.q > 0.f ? 1.f / rw.q : 0.f;
  // wn^2 (u^2 + v^2) of channel c0 + k
#define XB(k) (c_bch[c0 + (k)].wn2 * rw.q)
  for (int j = 0; j < ng; ++j) {
    const SeqGal s = sg[j];
    const GalF& g = s.g;
    const bool apply = FIT && s.apply;
    const f2 p = delay_df(rw, g);
    const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
    const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
    float ws, wc, zs, zc;
    sincos_turn(dT.hi + dT.lo, &ws, &wc);
    const float ta = c0 == 0 ? (T0.hi + T0.lo) : turns_at(T0, dT, c0);
    sincos_turn_sfu(ta, &zs, &zc);
    const float wr = wc, wi = -ws;    // w = exp(-2 pi i dT)
    const float zr0 = zc, zi0 = -zs;  // exp(-2 pi i T(c0))
    const uint32_t d = dcache[s.fidx * kSeqThreads + tid];
    float2* fac = acc + s.off;
    // fitted model: |k'|^2 = A u^2 + B uv + C v^2 (sheared), as a factor on wn^2 (u^2 + v^2)
    const float f1 = apply ? g.sf1 * (g.A * uu + g.B * rw.uv + g.Cc * vv) * invq : 0.f;
    // chunk polynomials of the round model (c0p) and of flux * (fitted - round) (dfp)
    float c0p[4], dfp[4];
    if (POLY) {
      const float xq = c_chunk[c0 / kChunk].wn2c * rw.q;
      profile_poly<GAUSS>(g.sf0 * xq, c0p);
      if (apply) {
        float c1p[4];
        profile_poly<GAUSS>(f1 * xq, c1p);
#pragma unroll
        for (int j = 0; j < 4; ++j) dfp[j] = g.flux * (c1p[j] - c0p[j]);
      }
    }
    if (SIMPLE) {
      // one run: all 16 channels valid and in the cell d & 0xffff
      float cr, ci;
      if (!apply && POLY) {
        // sum_k residual_k w^k as two Horner sums in w^2, channels 2q (lane x) and 2q + 1 (lane y),
        // then the odd one times w
        const float w2r = fmaf(wr, wr, -wi * wi), w2i = 2.f * wr * wi;
        const float2 W2R = dup2(w2r), W2I = dup2(w2i), NW2I = dup2(-w2i);
        float2 SR = make_float2(0.f, 0.f), SI = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = kChunk / 2 - 1; q >= 0; --q) {
          const float2 nr_ = ffma2(SR, W2R, ffma2(SI, NW2I, rp[q]));
          const float2 ni_ = ffma2(SR, W2I, ffma2(SI, W2R, ip[q]));
          SR = nr_;
          SI = ni_;
        }
        const float sr = fmaf(SR.y, wr, fmaf(-SI.y, wi, SR.x));
        const float si = fmaf(SR.y, wi, fmaf(SI.y, wr, SI.x));
        const BatchChunk& ck = c_chunk[c0 / kChunk];
        const float rs = fmaf(c0p[3], ck.mom[3], fmaf(c0p[2], ck.mom[2], fmaf(c0p[1], ck.mom[1], c0p[0] * ck.mom[0])));
        cr = fmaf(sr, zr0, fmaf(-si, zi0, rs * g.flux));
        ci = fmaf(sr, zi0, si * zr0);
      } else if (!apply) {
        float sr = 0.f, si = 0.f, rs = 0.f;
#pragma unroll
        for (int k = kChunk - 1; k >= 0; --k) {
          const float nr_ = fmaf(sr, wr, fmaf(-si, wi, PR(k)));
          const float ni_ = fmaf(sr, wi, fmaf(si, wr, PI(k)));
          sr = nr_;
          si = ni_;
          rs = fmaf(profile(g.sf0 * XB(k), GAUSS), c_bch[c0 + k].spec, rs);
        }
        cr = fmaf(sr, zr0, fmaf(-si, zi0, rs * g.flux));
        ci = fmaf(sr, zi0, si * zr0);
      } else if (POLY) {
        // channels 2q and 2q + 1 side by side: z = exp(-2 pi i T) as (ZR, NZI = -Im z), stepped by w^2;
        // the residual rotated and summed (ar, ai), then the galaxy's model difference
        // a = spec * poly3(dfp, dl) removed from it: residual -= a exp(+2 pi i T)
        const float w2r = fmaf(wr, wr, -wi * wi), w2i = 2.f * wr * wi;
        const float2 W2R = dup2(w2r), W2I = dup2(w2i), NW2I = dup2(-w2i);
        const float z1r = fmaf(zr0, wr, -zi0 * wi), z1i = fmaf(zr0, wi, zi0 * wr);
        float2 ZR = make_float2(zr0, z1r), NZI = make_float2(-zi0, -z1i);
        const float2 D0 = dup2(dfp[0]), D1 = dup2(dfp[1]), D2 = dup2(dfp[2]), D3 = dup2(dfp[3]);
        float2 AR = make_float2(0.f, 0.f), AI = make_float2(0.f, 0.f), BI = make_float2(0.f, 0.f);
#pragma unroll
        for (int q = 0; q < kChunk / 2; ++q) {
          AR = ffma2(ip[q], NZI, ffma2(rp[q], ZR, AR));  // + re z re - im z im
          AI = ffma2(ip[q], ZR, AI);                     // + res im * re z
          BI = ffma2(rp[q], NZI, BI);                    // - res re * im z
          const float4 cp = c_pair[c0 / 2 + q];
          const float2 DL = make_float2(cp.x, cp.y);
          const float2 AN = fmul2(make_float2(cp.z, cp.w), ffma2(ffma2(ffma2(D3, DL, D2), DL, D1), DL, D0));
          rp[q] = ffma2(AN, ZR, rp[q]);
          ip[q] = ffma2(AN, NZI, ip[q]);
          const float2 nzr = ffma2(NZI, W2I, fmul2(ZR, W2R));
          const float2 nzi = ffma2(ZR, NW2I, fmul2(NZI, W2R));
          ZR = nzr;
          NZI = nzi;
        }
        const BatchChunk& ck = c_chunk[c0 / kChunk];
        const float rs = fmaf(c0p[3], ck.mom[3], fmaf(c0p[2], ck.mom[2], fmaf(c0p[1], ck.mom[1], c0p[0] * ck.mom[0])));
        cr = fmaf(rs, g.flux, AR.x + AR.y);
        ci = (AI.x + AI.y) - (BI.x + BI.y);
      } else {
        float ar = 0.f, ai = 0.f, rs = 0.f, zr = zr0, zi = zi0;
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
          ar = fmaf(PR(k), zr, fmaf(-PI(k), zi, ar));
          ai = fmaf(PR(k), zi, fmaf(PI(k), zr, ai));
          const float spec = c_bch[c0 + k].spec;
          const float xbk = XB(k);
          const float s0 = profile(g.sf0 * xbk, GAUSS);
          const float s1 = profile(f1 * xbk, GAUSS);
          rs = fmaf(s0, spec, rs);
          const float a = g.flux * spec * (s1 - s0);
          // residual -= a * exp(+2 pi i T)
          PR(k) = fmaf(-a, zr, PR(k));
          PI(k) = fmaf(a, zi, PI(k));
          const float nzr = fmaf(zr, wr, -zi * wi);
          const float nzi = fmaf(zr, wi, zi * wr);
          zr = nzr;
          zi = nzi;
        }
        cr = fmaf(rs, g.flux, ar);
        ci = ai;
      }
      warp_deposit(fac, b.total_cells, live ? (int)(d & 0xffffu) : -1, cr, ci, tid & 31);
    } else {
      // flagged channels, several cells or a short chunk: channel by channel, each run of
      // channels in one cell summed before its deposit
      const uint16_t* cl = b.cells[s.fidx];
      const uint16_t cell0 = (uint16_t)(d & 0xffffu);
      const uint32_t mask = d >> 16;
      float zr = zr0, zi = zi0;
      int cur = kNoCell;
      float ur = 0.f, ui = 0.f;
#pragma unroll
      for (int k = 0; k < kChunk; ++k) {
        if (k < nk) {
          const float spec = c_bch[c0 + k].spec;
          const float xbk = XB(k);
          const float s0 = POLY ? poly3(c0p, c_bch[c0 + k].dl) : profile(g.sf0 * xbk, GAUSS);
          const int c = (mask & (1u << k)) ? (int)cl[(size_t)(c0 + k) * n_rows + r] : (int)cell0;
          if (c != kNoCell) {
            const float cr = fmaf(PR(k), zr, fmaf(-PI(k), zi, s0 * spec * g.flux));
            const float ci = fmaf(PR(k), zi, PI(k) * zr);
            if (c != cur) {
              if (cur != kNoCell) comp_add2(fac, cur, b.total_cells, ur, ui);
              cur = c;
              ur = cr;
              ui = ci;
            } else {
              ur += cr;
              ui += ci;
            }
          }
          if (apply) {
            const float a = POLY ? spec * poly3(dfp, c_bch[c0 + k].dl)
                                 : g.flux * spec * (profile(f1 * xbk, GAUSS) - s0);
            PR(k) = fmaf(-a, zr, PR(k));
            PI(k) = fmaf(a, zi, PI(k));
          }
          const float nzr = fmaf(zr, wr, -zi * wi);
          const float nzi = fmaf(zr, wi, zi * wr);
          zr = nzr;
          zi = nzi;
        }
      }
      if (cur != kNoCell) comp_add2(fac, cur, b.total_cells, ur, ui);
    }
  }
#undef XB
#undef PR
#undef PI
}

// one work item whose chunk is, for every facet size of the batch, one run or two runs: channels
// 0..s-1 in the chunk's first cell, s..15 in a second cell (a row's uv point crossing a cell
// boundary within the chunk).  As the single-run path with a deposit per run: in the first round
// two Horner sums split at s, the second one rotated by the phase at channel s; in the correction
// rounds the phase recurrence with the rotated residual summed per run; the round model of each
// run from the moments of its channels.  Needs the chunk polynomials (MODE 1 or 2).  Called by all
// lanes of a warp, as seq_item's single-run items.
template <int GAUSS, int MODE, bool FIT, int CI = -1>
__device__ __forceinline__ void seq_item2(int t, bool live, int n_rows, int ng, const RowF* __restrict__ rows,
                                          const float2* __restrict__ data, const float2* __restrict__ sky,
                                          const SeqBatch& b, const SeqGal* sg, uint32_t* dcache, uint16_t* d1cache,
                                          float2* acc) {
  constexpr bool ONE = MODE == 2;
  constexpr bool FIXED = CI >= 0;
  const int tid = threadIdx.x;
  const int r = ONE ? t : (FIXED ? t - CI * n_rows : t % n_rows);
  const int c0 = ONE ? 0 : (FIXED ? CI * kChunk : (t / n_rows) * kChunk);
  const int ci = c0 / kChunk;
  const RowF rw = rows[r];
  float pr[kChunk], pi[kChunk];
#pragma unroll
  for (int k = 0; k < kChunk; ++k) {
    const size_t idx = (size_t)(c0 + k) * n_rows + r;
    const float2 d = data[idx], sk = sky[idx];
    pr[k] = d.x - sk.x;
    pi[k] = d.y - sk.y;
  }
  for (int f = 0; f < b.n_sizes; ++f) {
    dcache[f * kSeqThreads + tid] = b.desc[f][t];
    d1cache[f * kSeqThreads + tid] = b.desc1[f][t];
  }
  const float uu = rw.u_hi * rw.u_hi, vv = rw.v_hi * rw.v_hi;
  const float invq = rw.q > 0.f ? 1.f / rw.q : 0.f;
  const float xq = c_chunk[ci].wn2c * rw.q;
  for (int j = 0; j < ng; ++j) {
    const SeqGal s = sg[j];
    const GalF& g = s.g;
    const bool apply = FIT && s.apply;
    const f2 p = delay_df(rw, g);
    const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
    const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
    float ws, wc, zs, zc;
    sincos_turn(dT.hi + dT.lo, &ws, &wc);
    sincos_turn_sfu(c0 == 0 ? (T0.hi + T0.lo) : turns_at(T0, dT, c0), &zs, &zc);
    const float wr = wc, wi = -ws;    // w = exp(-2 pi i dT)
    const float zr0 = zc, zi0 = -zs;  // exp(-2 pi i T(c0))
    const uint32_t d = dcache[s.fidx * kSeqThreads + tid];
    const uint32_t mask = d >> 16;
    const int split = mask ? __ffs(mask) - 1 : kChunk;
    const int cell_a = (int)(d & 0xffffu);
    const uint16_t cell_b = d1cache[s.fidx * kSeqThreads + tid];
    float2* fac = acc + s.off;
    const float f1 = apply ? g.sf1 * (g.A * uu + g.B * rw.uv + g.Cc * vv) * invq : 0.f;
    float c0p[4], dfp[4];
    profile_poly<GAUSS>(g.sf0 * xq, c0p);
    if (apply) {
      float c1p[4];
      profile_poly<GAUSS>(f1 * xq, c1p);
#pragma unroll
      for (int q = 0; q < 4; ++q) dfp[q] = g.flux * (c1p[q] - c0p[q]);
    }
    const float* ms = c_chunk_split[ci][split];
    const float rs_a = fmaf(c0p[3], ms[3], fmaf(c0p[2], ms[2], fmaf(c0p[1], ms[1], c0p[0] * ms[0])));
    const float rs_b = fmaf(c0p[3], ms[7], fmaf(c0p[2], ms[6], fmaf(c0p[1], ms[5], c0p[0] * ms[4])));
    float ar, ai, br, bi;  // the rotated residual of each run
    if (!apply) {
      // Horner from channel 15 down: run B (from s) relative to channel s, then run A from channel 0
      float sr = 0.f, si = 0.f, hr = 0.f, hi = 0.f;
#pragma unroll
      for (int k = kChunk - 1; k >= 0; --k) {
        if (k == split - 1) { hr = sr; hi = si; sr = 0.f; si = 0.f; }
        const float nr_ = fmaf(sr, wr, fmaf(-si, wi, pr[k]));
        const float ni_ = fmaf(sr, wi, fmaf(si, wr, pi[k]));
        sr = nr_;
        si = ni_;
      }
      ar = fmaf(sr, zr0, -si * zi0);
      ai = fmaf(sr, zi0, si * zr0);
      br = bi = 0.f;
      if (split < kChunk) {
        float ys, yc;
        sincos_turn_sfu(turns_at(T0, dT, c0 + split), &ys, &yc);  // exp(-2 pi i T(c0 + s)) = yc - i ys
        br = fmaf(hr, yc, hi * ys);
        bi = fmaf(hi, yc, -hr * ys);
      }
    } else {
      float zr = zr0, zi = zi0;
      ar = ai = br = bi = 0.f;
#pragma unroll
      for (int k = 0; k < kChunk; ++k) {
        const float tr = fmaf(pr[k], zr, -pi[k] * zi);
        const float ti = fmaf(pr[k], zi, pi[k] * zr);
        if (k < split) { ar += tr; ai += ti; }
        else { br += tr; bi += ti; }
        const float a = c_bch[c0 + k].spec * poly3(dfp, c_bch[c0 + k].dl);
        pr[k] = fmaf(-a, zr, pr[k]);
        pi[k] = fmaf(a, zi, pi[k]);
        const float nzr = fmaf(zr, wr, -zi * wi);
        const float nzi = fmaf(zr, wi, zi * wr);
        zr = nzr;
        zi = nzi;
      }
    }
    const int lane = tid & 31;
    warp_deposit(fac, b.total_cells, live ? cell_a : -1, fmaf(rs_a, g.flux, ar), ai, lane);
    warp_deposit(fac, b.total_cells, live && split < kChunk && cell_b != kNoCell ? (int)cell_b : -1,
                 fmaf(rs_b, g.flux, br), bi, lane);
  }
}

// the chunk of item t if every lane of the warp has an item of that chunk, else -1 (all lanes call)
__device__ __forceinline__ int uniform_chunk(int t, int n_rows) {
  const int ci = t / n_rows;
  const int c0 = __shfl_sync(0xffffffffu, ci, 0);
  return __all_sync(0xffffffffu, ci == c0) ? c0 : -1;
}

template <int GAUSS, int MODE, bool FIT>
__global__ void __launch_bounds__(kSeqThreads, kSeqCtasPerSm) k_extract_seq(int n_rows, const RowF* __restrict__ rows,
                                                                const float2* __restrict__ data,
                                                                const float2* __restrict__ sky, SeqBatch b,
                                                                double2* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* acc = reinterpret_cast<float2*>(smem_raw);  // [total_cells] hi, then [total_cells] lo
  SeqGal* sg = reinterpret_cast<SeqGal*>(smem_raw + align16((size_t)b.total_cells * kSeqCellBytes));
  uint32_t* dcache = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(sg) +
                                                 align16((size_t)b.n_gal * sizeof(SeqGal)));
  uint16_t* d1cache = reinterpret_cast<uint16_t*>(dcache + (size_t)b.n_sizes * kSeqThreads);
  const int tid = threadIdx.x;
  // galaxies [j0, n_gal) of the unit take part (device round control)
  if (b.ctl && b.ctl[1]) return;
  const int j0 = b.ctl ? b.ctl[0] : 0;
  const int ng = b.n_gal - j0;
  for (int i = tid; i < 2 * b.total_cells; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);
  for (int i = tid; i < ng; i += blockDim.x) {
    SeqGal s;
    const int gi = j0 + i;
    const bool has_fit = b.fit != nullptr;
    s.g = load_gal(b.gals[gi], has_fit ? &b.fit[gi].e1 : nullptr, has_fit ? &b.fit[gi].error : nullptr);
    s.fidx = b.fidx[gi];
    s.off = b.foff[gi];
    s.apply = has_fit && b.fit[gi].error == 0;
    sg[i] = s;
  }
  __syncthreads();
  const int nch = c_bnch;
  const int total = (int)((long long)n_rows * ((nch + kChunk - 1) / kChunk));
  const int ns = *b.n_simple;
  const int lane = tid & 31;
  // Work comes from device counters, the costliest items first so that the cheap single-run ones
  // even out the end of the launch.  The general items (rare; a deposit per run of channels each)
  // come in chunks of 32 whose lane l takes item l * chunks + c of the list, so that the rows of a
  // warp lie far apart in uv and their deposits rarely meet in a cell.
  const int ngen = b.n_simple[1];
  const int gch = (ngen + 31) / 32;
  while (true) {
    int c = 0;
    if (lane == 0) c = atomicAdd(&b.queue[1], 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= gch) break;
    const int k = lane * gch + c;
    if (k < ngen) seq_item<GAUSS, false, MODE, FIT>(b.items[total - ngen + k], true, n_rows, nch, ng, rows, data, sky, b, sg, dcache, acc);
  }
  // the two-run and single-run items: 32 consecutive items of the list (neighbours in uv) at a time
  // MODE 3: the items of a block of the list come from one chunk (the list is in chunk-major
  // order), so a warp's 32 items almost always share it; such a warp runs the item code compiled
  // for that chunk, the rare mixed warp the code for any chunk
  if (MODE > 0) {
    const int nt = *b.n_two;
    while (true) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&b.queue[2], 32);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= nt) break;
      const int q = base + lane;
      const int t = b.items2[min(q, nt - 1)];
      const int ci = MODE == 3 ? uniform_chunk(t, n_rows) : -1;
#define RLF_ITEM2(C) seq_item2<GAUSS, MODE, FIT, C>(t, q < nt, n_rows, ng, rows, data, sky, b, sg, dcache, d1cache, acc)
      switch (ci) {
        case 0: RLF_ITEM2(0); break;
        case 1: RLF_ITEM2(1); break;
        case 2: RLF_ITEM2(2); break;
        case 3: RLF_ITEM2(3); break;
        default: RLF_ITEM2(-1);
      }
#undef RLF_ITEM2
    }
  }
  while (true) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&b.queue[0], 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= ns) break;
    const int q = base + lane;
    const int t = b.items[min(q, ns - 1)];
    const int ci = MODE == 3 ? uniform_chunk(t, n_rows) : -1;
#define RLF_ITEM(C) seq_item<GAUSS, true, MODE, FIT, C>(t, q < ns, n_rows, nch, ng, rows, data, sky, b, sg, dcache, acc)
    switch (ci) {
      case 0: RLF_ITEM(0); break;
      case 1: RLF_ITEM(1); break;
      case 2: RLF_ITEM(2); break;
      case 3: RLF_ITEM(3); break;
      default: RLF_ITEM(-1);
    }
#undef RLF_ITEM
  }
  __syncthreads();
  double2* out = partial + (size_t)blockIdx.x * b.total_cells;
  for (int i = tid; i < b.total_cells; i += blockDim.x) {
    const float2 hi = acc[i], lo = acc[i + b.total_cells];
    out[i] = make_double2((double)hi.x + (double)lo.x, (double)hi.y + (double)lo.y);
  }
}

int launch_extract_seq(int n_rows, const RowF* rows, const float2* data, const float2* sky, const SeqBatch& b,
                       int gaussian, int ctas, double2* partial, cudaStream_t st) {
  if (b.n_gal < 1 || b.n_gal > kSeqMaxGal || b.n_sizes < 1 || b.n_sizes > kSeqMaxSizes) {
    fprintf(stderr, "rlf: sequential extraction batch of %d galaxies / %d facet sizes unsupported\n", b.n_gal,
            b.n_sizes);
    return 1;
  }
  const size_t smem = seq_smem_bytes(b.n_gal, b.total_cells, b.n_sizes);
  if (smem > 227 * 1024) { fprintf(stderr, "rlf: sequential extraction batch too large (%zu B)\n", smem); return 1; }
  const cudaError_t qe = cudaMemsetAsync(b.queue, 0, 3 * sizeof(int), st);
  if (qe != cudaSuccess) { fprintf(stderr, "rlf: extraction queue: %s\n", cudaGetErrorString(qe)); return (int)qe; }
  int dev = 0;
  cudaGetDevice(&dev);
  const bool known = dev >= 0 && dev < 64;
  int mode = known && g_chunk_poly[dev] ? (g_nch[dev] == kChunk ? 2 : 1) : 0;
  if (mode == 1 && g_nch[dev] % kChunk == 0 && g_nch[dev] <= 4 * kChunk) mode = 3;
  // FIT: a correction round (fitted - round model differences to remove); the first round's kernel
  // leaves that path out
  const void* kernels[2][2][4] = {
      {{(const void*)k_extract_seq<0, 0, false>, (const void*)k_extract_seq<0, 1, false>,
        (const void*)k_extract_seq<0, 2, false>, (const void*)k_extract_seq<0, 3, false>},
       {(const void*)k_extract_seq<1, 0, false>, (const void*)k_extract_seq<1, 1, false>,
        (const void*)k_extract_seq<1, 2, false>, (const void*)k_extract_seq<1, 3, false>}},
      {{(const void*)k_extract_seq<0, 0, true>, (const void*)k_extract_seq<0, 1, true>,
        (const void*)k_extract_seq<0, 2, true>, (const void*)k_extract_seq<0, 3, true>},
       {(const void*)k_extract_seq<1, 0, true>, (const void*)k_extract_seq<1, 1, true>,
        (const void*)k_extract_seq<1, 2, true>, (const void*)k_extract_seq<1, 3, true>}}};
  const void* kern = kernels[b.fit ? 1 : 0][gaussian ? 1 : 0][mode];
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  void* args[] = {(void*)&n_rows, (void*)&rows, (void*)&data, (void*)&sky, (void*)&b, (void*)&partial};
  const cudaError_t le = cudaLaunchKernel(kern, dim3(ctas), dim3(kSeqThreads), args, smem, st);
  if (le != cudaSuccess) { fprintf(stderr, "rlf: k_extract_seq: %s\n", cudaGetErrorString(le)); return (int)le; }
  return check("k_extract_seq");
}

// one block per galaxy of the batch: FP64 sums of the CTA partials, then the facet finalisation of
// evaluate_uv_grid.c:196-209 / 113-133 with compaction to the non-empty cells in row-major order
__global__ void k_finalize_seq(SeqBatch b, int ctas, const double2* __restrict__ partial,
                               const double* const* __restrict__ ss_of, const double* const* __restrict__ sw_of,
                               double len, FacetOut out) {
  const int slot = blockIdx.x;
  if (slot >= b.n_gal) return;
  if (b.ctl && (b.ctl[1] || slot < b.ctl[0])) return;  // converged, or a galaxy before this round's first
  const int F = b.facet[slot], off = b.foff[slot];
  const int nc = F * F;
  const double inc = 2 * len / F;
  const double* ss = ss_of[slot];
  const double* sw = sw_of[slot];
  __shared__ int warp_tot[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int dst = out.offset[slot];
  for (int cbase = 0; cbase < nc; cbase += blockDim.x) {
    const int c = cbase + threadIdx.x;
    int flagc = 0;
    double vre = 0, vim = 0, sg = 0;
    if (c < nc) {
      const double w = sw[c];
      if (w != 0.0) {
        double sre = 0.0, sim = 0.0;
        for (int p = 0; p < ctas; ++p) {
          const double2 v = partial[(size_t)p * b.total_cells + off + c];
          sre += v.x;
          sim += v.y;
        }
        const double s2 = ss[c];
        vre = sre * w / s2;
        vim = sim * w / s2;
        sg = s2 / (w * w);
        flagc = 1;
      }
    }
    const int ln = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, flagc);
    const int inwarp = __popc(bal & ((1u << ln) - 1u));
    if (ln == 0) warp_tot[wp] = __popc(bal);
    __syncthreads();
    int before = base;
    for (int w = 0; w < wp; ++w) before += warp_tot[w];
    if (flagc) {
      const int pos = dst + before + inwarp;
      const int i = c % F, jj = c / F;
      // evaluate_uv_grid.c:125-126 without a fused multiply-add
      const double gu = __dsub_rn(__dmul_rn(i + 0.5, inc), len), gv = __dsub_rn(__dmul_rn(jj + 0.5, inc), len);
      if (out.as_float) {
        ((float*)out.gu)[pos] = (float)gu; ((float*)out.gv)[pos] = (float)gv;
        ((float*)out.dre)[pos] = (float)vre; ((float*)out.dim)[pos] = (float)vim;
        ((float*)out.sig2)[pos] = (float)sg;
      } else {
        ((double*)out.gu)[pos] = gu; ((double*)out.gv)[pos] = gv;
        ((double*)out.dre)[pos] = vre; ((double*)out.dim)[pos] = vim;
        ((double*)out.sig2)[pos] = sg;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_tot[w];
      base += t;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out.ncoords[slot] = base;
}

// one block per galaxy of the batch: the un-averaged facet sums of a channel shard, out[slot][4][stride]
// = (sum of vis re, sum of vis im, sum of sigma^2, sum of weights) per cell of the galaxy's F x F
// facet in row-major order (evaluate_uv_grid.c:143-195 before the averaging of :196-209), FP64 sums
// of the CTA partials in CTA order; cells F^2 .. stride - 1 zero
__global__ void k_partials_seq(SeqBatch b, int ctas, const double2* __restrict__ partial,
                               const double* const* __restrict__ ss_of, const double* const* __restrict__ sw_of,
                               double* __restrict__ out, int stride) {
  const int slot = blockIdx.x;
  if (slot >= b.n_gal) return;
  const int F = b.facet[slot], off = b.foff[slot];
  const int nc = F * F;
  const double* ss = ss_of[slot];
  const double* sw = sw_of[slot];
  double* row = out + (size_t)slot * 4 * stride;
  for (int c = threadIdx.x; c < stride; c += blockDim.x) {
    double sre = 0.0, sim = 0.0, s2 = 0.0, w = 0.0;
    if (c < nc) {
      for (int p = 0; p < ctas; ++p) {
        const double2 v = partial[(size_t)p * b.total_cells + off + c];
        sre += v.x;
        sim += v.y;
      }
      s2 = ss[c];
      w = sw[c];
    }
    row[c] = sre;
    row[stride + c] = sim;
    row[2 * stride + c] = s2;
    row[3 * stride + c] = w;
  }
}

int launch_partials_seq(const SeqBatch& b, int ctas, const double2* partial, const double* const* ss,
                        const double* const* sw, double* out, int stride, cudaStream_t st) {
  k_partials_seq<<<b.n_gal, 256, 0, st>>>(b, ctas, partial, ss, sw, out, stride);
  return check("k_partials_seq");
}

int launch_finalize_seq(const SeqBatch& b, int ctas, const double2* partial, const double* const* ss,
                        const double* const* sw, double len, FacetOut out, cudaStream_t st) {
  k_finalize_seq<<<b.n_gal, 256, 0, st>>>(b, ctas, partial, ss, sw, len, out);
  return check("k_finalize_seq");
}

// ---------------------------------------------------------------- removal
// The models of the galaxies sg[0..gn) at one (row, chunk): ar, ai += the round models, br, bi +=
// the fitted models (flux times profile times the phase exp(+2 pi i T), before the spectral
// factor), channel c0 + k in lane k % 2 of element k / 2.  CI >= 0: the chunk CI (compile-time
// channel constants, MODE 3); -1: the chunk of ch0.  With the chunk polynomials the channels 2q and
// 2q + 1 run side by side in packed FP32 pairs, the phase stepping by w^2.
template <int GAUSS, int MODE, int CI>
__device__ __forceinline__ void remove_models(const RowF& rw, int ch0, int nch, const GalF* sg, int gn,
                                              float2 (&ar)[kRemCh / 2], float2 (&ai)[kRemCh / 2],
                                              float2 (&br)[kRemCh / 2], float2 (&bi)[kRemCh / 2]) {
  constexpr bool POLY = MODE > 0;
  if (CI >= 0) ch0 = CI * kChunk;
  for (int i = 0; i < gn; ++i) {
    const GalF g = sg[i];
    if (!g.active) continue;
    const f2 p = delay_df(rw, g);
    const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
    const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
    float zs, zc, ws, wc;
    sincos_turn_sfu(ch0 == 0 ? T0.hi + T0.lo : turns_at(T0, dT, ch0), &zs, &zc);
    sincos_turn(dT.hi + dT.lo, &ws, &wc);
    const float k1q = g.A * (rw.u_hi * rw.u_hi) + g.B * rw.uv + g.Cc * (rw.v_hi * rw.v_hi);
    if (POLY) {
      float c0p[4], c1p[4];
      const float wc2 = c_chunk[ch0 / kChunk].wn2c;
      profile_poly<GAUSS>(g.sf0 * wc2 * rw.q, c0p);
      profile_poly<GAUSS>(g.sf1 * wc2 * k1q, c1p);
      const float2 E0 = dup2(c0p[0] * g.flux), E1 = dup2(c0p[1] * g.flux), E2 = dup2(c0p[2] * g.flux),
                   E3 = dup2(c0p[3] * g.flux);
      const float2 F0 = dup2(c1p[0] * g.flux), F1 = dup2(c1p[1] * g.flux), F2 = dup2(c1p[2] * g.flux),
                   F3 = dup2(c1p[3] * g.flux);
      // z = exp(+2 pi i T) at channels ch0 + 2q (lane x) and ch0 + 2q + 1 (lane y), stepped by w^2
      const float w2r = fmaf(wc, wc, -ws * ws), w2i = 2.f * wc * ws;
      const float2 W2R = dup2(w2r), W2I = dup2(w2i), NW2I = dup2(-w2i);
      float2 ZR = make_float2(zc, fmaf(zc, wc, -zs * ws)), ZI = make_float2(zs, fmaf(zc, ws, zs * wc));
#pragma unroll
      for (int q = 0; q < kRemCh / 2; ++q) {
        if (CI >= 0 || ch0 + 2 * q < nch) {
          const float4 cp = c_pair[ch0 / 2 + q];
          const float2 DL = make_float2(cp.x, cp.y);
          const float2 a0 = ffma2(ffma2(ffma2(E3, DL, E2), DL, E1), DL, E0);
          const float2 a1 = ffma2(ffma2(ffma2(F3, DL, F2), DL, F1), DL, F0);
          ar[q] = ffma2(a0, ZR, ar[q]);
          ai[q] = ffma2(a0, ZI, ai[q]);
          br[q] = ffma2(a1, ZR, br[q]);
          bi[q] = ffma2(a1, ZI, bi[q]);
          const float2 nzr = ffma2(ZI, NW2I, fmul2(ZR, W2R));
          const float2 nzi = ffma2(ZR, W2I, fmul2(ZI, W2R));
          ZR = nzr;
          ZI = nzi;
        }
      }
    } else {
      float zr = zc, zi = zs;  // exp(+2 pi i T): the model phase
#pragma unroll
      for (int k = 0; k < kRemCh; ++k) {
        const int ch = ch0 + k;
        if (ch < nch) {
          const BatchChan bc = c_bch[ch];
          const float x0 = g.sf0 * bc.wn2 * rw.q;
          const float x1 = g.sf1 * bc.wn2 * k1q;
          const float a0 = (GAUSS ? __expf(-0.5f * x0) : round_shape(x0)) * g.flux;
          const float a1 = (GAUSS ? __expf(-0.5f * x1) : round_shape(x1)) * g.flux;
          float2& A = ar[k >> 1];
          float2& B = ai[k >> 1];
          float2& C = br[k >> 1];
          float2& D = bi[k >> 1];
          if (k & 1) {
            A.y = fmaf(a0, zr, A.y); B.y = fmaf(a0, zi, B.y); C.y = fmaf(a1, zr, C.y); D.y = fmaf(a1, zi, D.y);
          } else {
            A.x = fmaf(a0, zr, A.x); B.x = fmaf(a0, zi, B.x); C.x = fmaf(a1, zr, C.x); D.x = fmaf(a1, zi, D.x);
          }
          const float nzr = fmaf(zr, wc, -zi * ws);
          const float nzi = fmaf(zr, ws, zi * wc);
          zr = nzr;
          zi = nzi;
        }
      }
    }
  }
}

// grid-stride over (row, chunk of kRemCh channels); galaxies staged through shared memory in
// tiles of kRemTile.  Inactive galaxies (bad fits) are skipped.  The channel's spectral factor
// multiplies the sums over galaxies once, after the galaxy loop.  MODE as k_extract_seq: 0 exact
// per-channel profiles; 1 the profiles of a chunk from its cubic in dl (profile_poly), one profile
// evaluation per model, galaxy and chunk; 2 as 1 with exactly one 16-channel chunk (compile-time
// channel constants); 3 as 1 with 2-4 full chunks, a warp whose items share a chunk running the
// code compiled for that chunk.
static_assert(kRemCh == kChunk, "removal chunks must be the chunks of the channel polynomials");
template <int GAUSS, int MODE>
__global__ void __launch_bounds__(256) k_remove_batch(int n_rows, const RowF* __restrict__ rows, float2* data,
                                                      float2* sky, const GalaxyParams* __restrict__ gals,
                                                      const FitOut* __restrict__ fit, int n_gal) {
  constexpr bool ONE = MODE == 2;
  __shared__ GalF sg[kRemTile];
  const int nch = ONE ? kChunk : c_bnch;
  const int nchunk = ONE ? 1 : (nch + kRemCh - 1) / kRemCh;
  const long long total = (long long)n_rows * nchunk;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // all threads of the block iterate the same number of times so that the tiles can be shared
  const long long iters = (total + stride - 1) / stride;
  for (long long it = 0; it < iters; ++it) {
    const long long t = it * stride + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t < total;
    const int r = live ? (ONE ? (int)t : (int)(t % n_rows)) : 0;
    const int ch0 = ONE ? 0 : (live ? (int)(t / n_rows) * kRemCh : 0);
    // a warp of one chunk (its lanes without an item count as any chunk)
    int ci = ONE ? 0 : -1;
    if (MODE == 3) {
      const int mine = live ? ch0 / kChunk : -1;
      const int lead = __reduce_max_sync(0xffffffffu, mine);
      ci = __all_sync(0xffffffffu, mine == lead || mine < 0) ? lead : -1;
    }
    RowF rw = rows[r];
    float2 ar[kRemCh / 2], ai[kRemCh / 2], br[kRemCh / 2], bi[kRemCh / 2];
#pragma unroll
    for (int q = 0; q < kRemCh / 2; ++q) ar[q] = ai[q] = br[q] = bi[q] = make_float2(0.f, 0.f);
    for (int g0 = 0; g0 < n_gal; g0 += kRemTile) {
      const int gn = min(kRemTile, n_gal - g0);
      __syncthreads();
      for (int i = threadIdx.x; i < gn; i += blockDim.x)
        sg[i] = load_gal(gals[g0 + i], &fit[g0 + i].e1, &fit[g0 + i].error);
      __syncthreads();
      if (!live) continue;
      switch (MODE == 3 ? ci : -1) {
        case 0: remove_models<GAUSS, MODE, 0>(rw, ch0, nch, sg, gn, ar, ai, br, bi); break;
        case 1: remove_models<GAUSS, MODE, 1>(rw, ch0, nch, sg, gn, ar, ai, br, bi); break;
        case 2: remove_models<GAUSS, MODE, 2>(rw, ch0, nch, sg, gn, ar, ai, br, bi); break;
        case 3: remove_models<GAUSS, MODE, 3>(rw, ch0, nch, sg, gn, ar, ai, br, bi); break;
        default: remove_models<GAUSS, MODE, ONE ? 0 : -1>(rw, ch0, nch, sg, gn, ar, ai, br, bi);
      }
    }
    if (!live) continue;
#pragma unroll
    for (int k = 0; k < kRemCh; ++k) {
      const int ch = ch0 + k;
      if (ch < nch) {
        const size_t idx = (size_t)ch * n_rows + r;
        const float spec = c_bch[ch].spec;
        const int q = k >> 1;
        const float mr = (k & 1) ? ar[q].y : ar[q].x, mi = (k & 1) ? ai[q].y : ai[q].x;
        const float fr = (k & 1) ? br[q].y : br[q].x, fi = (k & 1) ? bi[q].y : bi[q].x;
        float2 s = sky[idx];
        s.x = fmaf(-spec, mr, s.x);
        s.y = fmaf(-spec, mi, s.y);
        sky[idx] = s;
        float2 d = data[idx];
        d.x = fmaf(-spec, fr, d.x);
        d.y = fmaf(-spec, fi, d.y);
        data[idx] = d;
      }
    }
  }
}

int launch_remove_batch(int n_rows, const RowF* rows, float2* data, float2* sky, const GalaxyParams* gals,
                        const FitOut* fit, int n_gal, int gaussian, cudaStream_t st) {
  if (n_gal <= 0) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4;
  const bool known = dev >= 0 && dev < 64;
  int mode = known && g_chunk_poly[dev] ? (g_nch[dev] == kChunk ? 2 : 1) : 0;
  if (mode == 1 && g_nch[dev] % kChunk == 0 && g_nch[dev] <= 4 * kChunk) mode = 3;
  const void* kernels[2][4] = {{(const void*)k_remove_batch<0, 0>, (const void*)k_remove_batch<0, 1>,
                                (const void*)k_remove_batch<0, 2>, (const void*)k_remove_batch<0, 3>},
                               {(const void*)k_remove_batch<1, 0>, (const void*)k_remove_batch<1, 1>,
                                (const void*)k_remove_batch<1, 2>, (const void*)k_remove_batch<1, 3>}};
  void* args[] = {(void*)&n_rows, (void*)&rows, (void*)&data, (void*)&sky, (void*)&gals, (void*)&fit, (void*)&n_gal};
  const cudaError_t le = cudaLaunchKernel(kernels[gaussian ? 1 : 0][mode], dim3(blocks), dim3(256), args, 0, st);
  if (le != cudaSuccess) { fprintf(stderr, "rlf: k_remove_batch: %s\n", cudaGetErrorString(le)); return (int)le; }
  return check("k_remove_batch");
}

// ------------------------------------------------------------- model sums
// vis += sum over galaxies of their model visibilities: the round models for the sky model
// (data_simulation.c:131-165, sky_model) or the sheared models for the simulator
// (data_simulation.c:41-127 with galaxy_visibilities.c:154-190).  Thread per (row, 16-channel
// chunk), galaxies staged in shared memory; per (row, galaxy) the double-float delay and two
// sin/cos of the phase, per channel a phase recurrence and the profile (MODE as k_extract_seq: 0
// exact profiles, 1 chunk polynomials, 2 chunk polynomials with one 16-channel chunk).
template <int GAUSS, int SHEARED, int MODE>
__global__ void __launch_bounds__(256) k_model_sum_batch(int n_rows, const RowF* __restrict__ rows, float2* vis,
                                                         const GalaxyParams* __restrict__ gals, int n_gal) {
  constexpr bool POLY = MODE > 0;
  constexpr bool ONE = MODE == 2;
  __shared__ GalF sg[kRemTile];
  const int nch = ONE ? kChunk : c_bnch;
  const int nchunk = ONE ? 1 : (nch + kRemCh - 1) / kRemCh;
  const long long total = (long long)n_rows * nchunk;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // all threads of the block iterate the same number of times so that the tiles can be shared
  const long long iters = (total + stride - 1) / stride;
  for (long long it = 0; it < iters; ++it) {
    const long long t = it * stride + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t < total;
    const int r = live ? (ONE ? (int)t : (int)(t % n_rows)) : 0;
    const int ch0 = ONE ? 0 : (live ? (int)(t / n_rows) * kRemCh : 0);
    const RowF rw = rows[r];
    const float uu = rw.u_hi * rw.u_hi, vv = rw.v_hi * rw.v_hi;
    float ar[kRemCh], ai[kRemCh];
#pragma unroll
    for (int k = 0; k < kRemCh; ++k) { ar[k] = ai[k] = 0.f; }
    for (int g0 = 0; g0 < n_gal; g0 += kRemTile) {
      const int gn = min(kRemTile, n_gal - g0);
      __syncthreads();
      for (int i = threadIdx.x; i < gn; i += blockDim.x) sg[i] = load_gal(gals[g0 + i], nullptr, nullptr);
      __syncthreads();
      if (!live) continue;
      for (int i = 0; i < gn; ++i) {
        const GalF g = sg[i];
        const f2 p = delay_df(rw, g);
        const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
        const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
        float zr, zi, ws, wc;
        sincos_turn(ch0 == 0 ? T0.hi + T0.lo : turns_at(T0, dT, ch0), &zi, &zr);  // exp(+2 pi i T)
        sincos_turn(dT.hi + dT.lo, &ws, &wc);
        const float q = SHEARED ? g.A * uu + g.B * rw.uv + g.Cc * vv : rw.q;
        const float sf = SHEARED ? g.sf1 : g.sf0;
        float cp[4];
        if (POLY) {
          profile_poly<GAUSS>(sf * c_chunk[ch0 / kChunk].wn2c * q, cp);
#pragma unroll
          for (int j = 0; j < 4; ++j) cp[j] *= g.flux;
        }
#pragma unroll
        for (int k = 0; k < kRemCh; ++k) {
          const int ch = ch0 + k;
          if (ch < nch) {
            const BatchChan bc = c_bch[ch];
            float a;
            if (POLY) {
              a = bc.spec * poly3(cp, bc.dl);
            } else {
              const float x = sf * bc.wn2 * q;
              a = (GAUSS ? __expf(-0.5f * x) : round_shape(x)) * bc.spec * g.flux;
            }
            ar[k] = fmaf(a, zr, ar[k]);
            ai[k] = fmaf(a, zi, ai[k]);
            const float nzr = fmaf(zr, wc, -zi * ws);
            const float nzi = fmaf(zr, ws, zi * wc);
            zr = nzr;
            zi = nzi;
          }
        }
      }
    }
    if (!live) continue;
#pragma unroll
    for (int k = 0; k < kRemCh; ++k) {
      const int ch = ch0 + k;
      if (ch < nch) {
        const size_t idx = (size_t)ch * n_rows + r;
        float2 v = vis[idx];
        v.x += ar[k];
        v.y += ai[k];
        vis[idx] = v;
      }
    }
  }
}

int launch_model_sum_batch(int n_rows, const RowF* rows, float2* vis, const GalaxyParams* gals, int n_gal,
                           int sheared, int gaussian, cudaStream_t st) {
  if (n_gal <= 0) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4;
  const bool known = dev >= 0 && dev < 64;
  const int mode = known && g_chunk_poly[dev] ? (g_nch[dev] == kChunk ? 2 : 1) : 0;
#define RLF_MS_K(G, S) {(const void*)k_model_sum_batch<G, S, 0>, (const void*)k_model_sum_batch<G, S, 1>, \
                        (const void*)k_model_sum_batch<G, S, 2>}
  const void* kernels[2][2][3] = {{RLF_MS_K(0, 0), RLF_MS_K(0, 1)}, {RLF_MS_K(1, 0), RLF_MS_K(1, 1)}};
#undef RLF_MS_K
  void* args[] = {(void*)&n_rows, (void*)&rows, (void*)&vis, (void*)&gals, (void*)&n_gal};
  const cudaError_t le = cudaLaunchKernel(kernels[gaussian ? 1 : 0][sheared ? 1 : 0][mode], dim3(blocks), dim3(256),
                                          args, 0, st);
  if (le != cudaSuccess) { fprintf(stderr, "rlf: k_model_sum_batch: %s\n", cudaGetErrorString(le)); return (int)le; }
  return check("k_model_sum_batch");
}

}  // namespace rlf

// Batched mixed-precision extraction and removal: many galaxies per pass over the visibilities.
//
// A single-galaxy pass over the data is HBM-bound (one read of data and sky model per galaxy);
// processing a batch of B galaxies per pass reads the data once per 32 galaxies and turns the
// pass into FP32/SFU work, B times less HBM traffic per galaxy.
//
// Extraction (source_extraction.c:46-68 + evaluate_uv_grid.c:143-211, batch form): a warp owns
// 32 galaxies with the same facet size; all lanes walk the same rows, so every row load is a
// broadcast and every facet update hits consecutive shared-memory words (lane = galaxy).  For a
// row and galaxy the delay p = u l + v m + w n is formed in double-float arithmetic, the phase
// turns T(ch) = p * inv_lambda(ch) = T0 + ch * dT (channels evenly spaced) are range-reduced, and
// the rotated residual sum over a run of channels in one cell is evaluated by Horner's rule in
// w = exp(-2 pi i dT), re-anchored with an accurate sincospi every 16 channels.  The galaxy's own
// round model, real after the shift, is added per visibility.  Warps accumulate FP32 facets in
// shared memory; CTAs write partial facets that are reduced in FP64, in a fixed order.
//
// Removal (data_processing.c:109-135, batch form): one thread per (row, 16-channel chunk) loops
// over the batch's galaxies held in shared memory and subtracts sum(round) from the sky model
// and sum(fitted) from the data with one read-modify-write of each.
#include "rlf_batch.cuh"
#include "rlf_fit.cuh"
#include <stdio.h>

namespace rlf {

struct BatchChan {
  float spec;      // spectral factor
  float wn2;       // wavenumber^2
};
__constant__ BatchChan c_bch[kMaxCh];
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
  for (int c = 0; c < n_ch; ++c) {
    h[c].spec = (float)spec[c];
    h[c].wn2 = (float)(wavenumbers[c] * wavenumbers[c]);
  }
  const float il0_hi = (float)il0, il0_lo = (float)(il0 - (double)il0_hi);
  const float dil_hi = (float)dil, dil_lo = (float)(dil - (double)dil_hi);
  cudaError_t e = cudaMemcpyToSymbolAsync(c_bch, h, sizeof(BatchChan) * n_ch, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_il0_hi, &il0_hi, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_il0_lo, &il0_lo, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_dil_hi, &dil_hi, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_dil_lo, &dil_lo, 4, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_bnch, &n_ch, 4, 0, cudaMemcpyHostToDevice, st);
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
// grid: (ctas_per_group, n_groups); block: up to kBatchWarps warps; galaxies of group j are
// gals[gidx[j*32 + lane]] (index < 0 = empty lane).  Shared memory: one facet per CTA,
// [F*F][32] float2 (lane = galaxy), updated with shared-memory atomics (warps of a CTA collide
// only when they hit the same cell of the same galaxy at the same time), then one staging tile
// per warp.
//
// Each warp walks its span of rows in tiles of kTileRows rows x kChunk channels.  The tile is
// staged with coalesced loads (lane -> row, half of the channels) as {data - sky, wn^2 |uv|^2,
// spec} per visibility plus the row's delay coordinates, and two 16-bit masks per row: valid
// channels and channels that start a run of one cell.  The 32 lanes (galaxies) then read every
// staged value as a shared-memory broadcast, so the per-visibility work is the Horner step and
// the round-model shape; the phase set-up is per row and the anchor + facet update per run.
// partial: [n_groups][ctas_per_group][F*F][32] float2
constexpr int kTileRows = 16;
constexpr int kChunk = 16;
constexpr uint32_t kFullRun = 0x0001FFFFu;  // all kChunk channels valid, one run from channel 0

struct __align__(16) ExtractTile {
  float4 v[kChunk][kTileRows];       // (re, im) of data - sky, wn^2 (u^2 + v^2), spec
  RowF row[kTileRows];
  uint16_t cell[kChunk][kTileRows];
  uint32_t mask[kTileRows];          // bits 0-15: valid channel; bits 16-31: run starts here
};

__host__ __device__ constexpr size_t extract_facet_bytes(int F) { return (size_t)F * F * 32 * sizeof(float2); }

template <int GAUSS>
__global__ void __launch_bounds__(kBatchWarps * 32) k_extract_batch(
    int n_rows, const RowF* __restrict__ rows, const float2* __restrict__ data, const float2* __restrict__ sky,
    const uint16_t* __restrict__ cell, const GalaxyParams* __restrict__ gals, const int* __restrict__ gidx,
    int F, float2* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* acc = reinterpret_cast<float2*>(smem_raw);  // [cell][lane]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int nc = F * F;
  ExtractTile& tile = reinterpret_cast<ExtractTile*>(smem_raw + ((extract_facet_bytes(F) + 15) & ~(size_t)15))[warp];
  const int group = blockIdx.y;
  for (int i = threadIdx.x; i < nc * 32; i += blockDim.x) acc[i] = make_float2(0.f, 0.f);
  __syncthreads();
  const int gi = gidx[group * 32 + lane];
  GalF g;
  if (gi >= 0) g = load_gal(gals[gi], nullptr, nullptr);
  else { g = load_gal(gals[gidx[group * 32]], nullptr, nullptr); g.active = 0; }
  float* my = reinterpret_cast<float*>(acc + lane);
  const int nch = c_bnch;
  // rows of this CTA, split into contiguous spans per warp
  const long long per_cta = ((long long)n_rows + gridDim.x - 1) / gridDim.x;
  const long long r_begin = blockIdx.x * per_cta;
  const long long r_end = min((long long)n_rows, r_begin + per_cta);
  const long long per_warp = (r_end - r_begin + nwarps - 1) / nwarps;
  const long long w_begin = r_begin + warp * per_warp;
  const long long w_end = min(r_end, w_begin + per_warp);
  const int srow = lane & (kTileRows - 1);   // staging: row of this lane
  const int shalf = lane >> 4;               // staging: channel half (8 channels)
  for (long long r0 = w_begin; r0 < w_end; r0 += kTileRows) {
    const int nr = (int)min((long long)kTileRows, w_end - r0);
    const long long rs_row = r0 + srow;
    const bool row_ok = srow < nr;
    if (shalf == 0 && row_ok) tile.row[srow] = rows[rs_row];
    const float q = row_ok ? rows[rs_row].q : 0.f;
    for (int c0 = 0; c0 < nch; c0 += kChunk) {
      // ---- stage kTileRows rows x kChunk channels
#pragma unroll
      for (int t = 0; t < kChunk / 2; ++t) {
        const int k = shalf * (kChunk / 2) + t;
        const int ch = c0 + k;
        uint16_t c = kNoCell;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (row_ok && ch < nch) {
          const size_t idx = (size_t)ch * n_rows + rs_row;
          c = cell[idx];
          const float2 d = data[idx], sk = sky[idx];
          const BatchChan bc = c_bch[ch];
          v = make_float4(d.x - sk.x, d.y - sk.y, bc.wn2 * q, bc.spec);
        }
        tile.v[k][srow] = v;
        tile.cell[k][srow] = c;
      }
      __syncwarp();
      if (shalf == 0) {
        uint32_t valid = 0, start = 0;
        uint16_t prev = kNoCell;
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
          const uint16_t c = tile.cell[k][srow];
          if (c != kNoCell) {
            valid |= 1u << k;
            if (c != prev) start |= 1u << k;
          }
          prev = c;
        }
        tile.mask[srow] = valid | (start << 16);
      }
      __syncwarp();
      // ---- every lane (galaxy) walks the staged rows
      for (int j = 0; j < nr; ++j) {
        const uint32_t m = tile.mask[j];
        if (m == 0) continue;
        const RowF rw = tile.row[j];
        const f2 p = delay_df(rw, g);
        const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
        const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
        float ws, wc;
        sincospif(2.f * (dT.hi + dT.lo), &ws, &wc);
        const float wr = wc, wi = -ws;  // w = exp(-2 pi i dT)
        float sr = 0.f, si = 0.f, rsum = 0.f;
        if (m == kFullRun) {
          // the common row: every channel of the chunk valid and in one cell
#pragma unroll
          for (int k = kChunk - 1; k >= 0; --k) {
            const float4 v = tile.v[k][j];
            const float nr_ = fmaf(sr, wr, fmaf(-si, wi, v.x));
            const float ni_ = fmaf(sr, wi, fmaf(si, wr, v.y));
            sr = nr_;
            si = ni_;
            const float x = g.sf0 * v.z;
            const float sh = GAUSS ? __expf(-0.5f * x) : round_shape(x);
            rsum = fmaf(sh, v.w, rsum);
          }
          float zs, zc;
          const float ta = c0 == 0 ? (T0.hi + T0.lo) : turns_at(T0, dT, c0);
          sincospif(2.f * ta, &zs, &zc);
          const float zr = zc, zi = -zs;
          const float cr = fmaf(sr, zr, fmaf(-si, zi, rsum * g.flux));
          const float ci = fmaf(sr, zi, si * zr);
          if (g.active) {
            const int c = tile.cell[0][j];
            atomicAdd(my + (size_t)c * 64, cr);
            atomicAdd(my + (size_t)c * 64 + 1, ci);
          }
          continue;
        }
        // Horner over each run, from its last channel down to its first: S = sum_k R_k w^(k - first)
#pragma unroll
        for (int k = kChunk - 1; k >= 0; --k) {
          if (m & (1u << k)) {
            const float4 v = tile.v[k][j];
            const float nr_ = fmaf(sr, wr, fmaf(-si, wi, v.x));
            const float ni_ = fmaf(sr, wi, fmaf(si, wr, v.y));
            sr = nr_;
            si = ni_;
            const float x = g.sf0 * v.z;
            const float sh = GAUSS ? __expf(-0.5f * x) : round_shape(x);
            rsum = fmaf(sh, v.w, rsum);
            if (m & (1u << (16 + k))) {
              float zs, zc;
              const float ta = (c0 + k == 0) ? (T0.hi + T0.lo) : turns_at(T0, dT, c0 + k);
              sincospif(2.f * ta, &zs, &zc);
              const float zr = zc, zi = -zs;  // exp(-2 pi i T(first channel))
              const float cr = fmaf(sr, zr, fmaf(-si, zi, rsum * g.flux));
              const float ci = fmaf(sr, zi, si * zr);
              if (g.active) {
                const int c = tile.cell[k][j];
                atomicAdd(my + (size_t)c * 64, cr);
                atomicAdd(my + (size_t)c * 64 + 1, ci);
              }
              sr = 0.f;
              si = 0.f;
              rsum = 0.f;
            }
          }
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
  float2* out = partial + ((size_t)group * gridDim.x + blockIdx.x) * (size_t)nc * 32;
  for (int i = threadIdx.x; i < nc * 32; i += blockDim.x) out[i] = acc[i];
}

// partials of one group -> per-galaxy facet sums (FP64, fixed order), then the facet
// finalisation of evaluate_uv_grid.c:196-209 / 113-133.  grid: one block per galaxy slot.
__global__ void k_finalize_batch(int ctas, int F, const float2* __restrict__ partial, const int* __restrict__ gidx,
                                 const double* __restrict__ ss, const double* __restrict__ sw, double len,
                                 FacetOut out) {
  const int group = blockIdx.y, lane = blockIdx.x;  // block = (lane, group)
  const int slot = gidx[group * 32 + lane];        // galaxy index = facet slot
  if (slot < 0) return;
  const int nc = F * F;
  const double inc = 2 * len / F;
  __shared__ int warp_tot[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int off = out.offset[slot];
  for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    int flagc = 0;
    double vre = 0, vim = 0, sg = 0;
    if (c < nc) {
      const double w = sw[c];
      if (w != 0.0) {
        double sre = 0.0, sim = 0.0;
        for (int p = 0; p < ctas; ++p) {
          const float2 v = partial[(((size_t)group * ctas + p) * nc + c) * 32 + lane];
          sre += (double)v.x;
          sim += (double)v.y;
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
      const int pos = off + before + inwarp;
      const int i = c % F, j = c / F;
      // evaluate_uv_grid.c:125-126 without a fused multiply-add
      const double gu = __dsub_rn(__dmul_rn(i + 0.5, inc), len), gv = __dsub_rn(__dmul_rn(j + 0.5, inc), len);
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

int launch_extract_batch(int n_rows, const RowF* rows, const float2* data, const float2* sky, const uint16_t* cell,
                         const GalaxyParams* gals, const int* gidx, int n_groups, int F, int ctas, int gaussian,
                         float2* partial, cudaStream_t st) {
  if (F < 1 || (unsigned)F > kBatchMaxFacet) { fprintf(stderr, "rlf: batched extraction facet %d unsupported\n", F); return 1; }
  const size_t facet = (extract_facet_bytes(F) + 15) & ~(size_t)15;
  // as many warps (each with its staging tile) as fit beside the facet, at most kBatchWarps
  int warps = (int)((kBatchSmemMax - facet) / sizeof(ExtractTile));
  if (warps > kBatchWarps) warps = kBatchWarps;
  if (warps < 1) { fprintf(stderr, "rlf: batched extraction facet %d too large\n", F); return 1; }
  const size_t smem = facet + (size_t)warps * sizeof(ExtractTile);
  const void* kern = gaussian ? (const void*)k_extract_batch<1> : (const void*)k_extract_batch<0>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(ctas, n_groups);
  if (gaussian)
    k_extract_batch<1><<<grid, warps * 32, smem, st>>>(n_rows, rows, data, sky, cell, gals, gidx, F, partial);
  else
    k_extract_batch<0><<<grid, warps * 32, smem, st>>>(n_rows, rows, data, sky, cell, gals, gidx, F, partial);
  return check("k_extract_batch");
}

int launch_finalize_batch(int n_groups, int ctas, int F, const float2* partial, const int* gidx, const double* ss,
                          const double* sw, double len, FacetOut out, cudaStream_t st) {
  dim3 grid(32, n_groups);
  k_finalize_batch<<<grid, 256, 0, st>>>(ctas, F, partial, gidx, ss, sw, len, out);
  return check("k_finalize_batch");
}

// ---------------------------------------------------------------- removal
// grid-stride over (row, chunk of kRemCh channels); galaxies staged through shared memory in
// tiles of kRemTile.  Inactive galaxies (bad fits) are skipped.
template <int GAUSS>
__global__ void __launch_bounds__(256) k_remove_batch(int n_rows, const RowF* __restrict__ rows, float2* data,
                                                      float2* sky, const GalaxyParams* __restrict__ gals,
                                                      const FitOut* __restrict__ fit, int n_gal) {
  __shared__ GalF sg[kRemTile];
  const int nch = c_bnch;
  const int nchunk = (nch + kRemCh - 1) / kRemCh;
  const long long total = (long long)n_rows * nchunk;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // all threads of the block iterate the same number of times so that the tiles can be shared
  const long long iters = (total + stride - 1) / stride;
  for (long long it = 0; it < iters; ++it) {
    const long long t = it * stride + blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool live = t < total;
    const int r = live ? (int)(t % n_rows) : 0;
    const int ch0 = live ? (int)(t / n_rows) * kRemCh : 0;
    RowF rw = rows[r];
    float ar[kRemCh], ai[kRemCh], br[kRemCh], bi[kRemCh];
#pragma unroll
    for (int k = 0; k < kRemCh; ++k) { ar[k] = ai[k] = br[k] = bi[k] = 0.f; }
    for (int g0 = 0; g0 < n_gal; g0 += kRemTile) {
      const int gn = min(kRemTile, n_gal - g0);
      __syncthreads();
      for (int i = threadIdx.x; i < gn; i += blockDim.x)
        sg[i] = load_gal(gals[g0 + i], &fit[g0 + i].e1, &fit[g0 + i].error);
      __syncthreads();
      if (!live) continue;
      for (int i = 0; i < gn; ++i) {
        const GalF g = sg[i];
        if (!g.active) continue;
        const f2 p = delay_df(rw, g);
        const f2 T0 = turns_mod1(p, c_il0_hi, c_il0_lo);
        const f2 dT = turns_mod1(p, c_dil_hi, c_dil_lo);
        float zs, zc, ws, wc;
        sincospif(2.f * turns_at(T0, dT, ch0), &zs, &zc);
        sincospif(2.f * (dT.hi + dT.lo), &ws, &wc);
        float zr = zc, zi = zs;  // exp(+2 pi i T): the model phase
        const float k1q = g.A * (rw.u_hi * rw.u_hi) + g.B * rw.uv + g.Cc * (rw.v_hi * rw.v_hi);
#pragma unroll
        for (int k = 0; k < kRemCh; ++k) {
          const int ch = ch0 + k;
          if (ch < nch) {
            const BatchChan bc = c_bch[ch];
            const float x0 = g.sf0 * bc.wn2 * rw.q;
            const float x1 = g.sf1 * bc.wn2 * k1q;
            const float a0 = (GAUSS ? __expf(-0.5f * x0) : round_shape(x0)) * bc.spec * g.flux;
            const float a1 = (GAUSS ? __expf(-0.5f * x1) : round_shape(x1)) * bc.spec * g.flux;
            ar[k] = fmaf(a0, zr, ar[k]);
            ai[k] = fmaf(a0, zi, ai[k]);
            br[k] = fmaf(a1, zr, br[k]);
            bi[k] = fmaf(a1, zi, bi[k]);
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
        float2 s = sky[idx];
        s.x -= ar[k];
        s.y -= ai[k];
        sky[idx] = s;
        float2 d = data[idx];
        d.x -= br[k];
        d.y -= bi[k];
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
  if (gaussian) k_remove_batch<1><<<blocks, 256, 0, st>>>(n_rows, rows, data, sky, gals, fit, n_gal);
  else k_remove_batch<0><<<blocks, 256, 0, st>>>(n_rows, rows, data, sky, gals, fit, n_gal);
  return check("k_remove_batch");
}

}  // namespace rlf

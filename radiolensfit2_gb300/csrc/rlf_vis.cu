// Visibility-domain kernels of the shape-measurement path.
//
// Layout: a visibility array is addressed as row * s_row + ch * s_ch (VisLayout), so the same
// kernels serve the reference's channel-major arrays and other layouts.  Every kernel walks rows
// with one thread per row and loops over that row's channels, so the per-row quantities
// (uvw, the geometric delay u l + v m + w n) are formed once and reused for all channels.
//
// F64 kernels follow the reference's FP64 arithmetic (galaxy_visibilities.c, source_extraction.c,
// evaluate_uv_grid.c, data_processing.c).  Mixed kernels read FP32 visibilities and evaluate the
// models in FP32; the phase 2 pi (u l + v m + w n)/lambda is formed as an FP64 delay per row and
// a double-float product per channel, range-reduced to [-1/2, 1/2] turn before the FP32 sincos.
#include "rlf_vis.cuh"
#include <stdio.h>
#include <algorithm>

namespace rlf {

static long long g_launches = 0;
void count_launch() { __atomic_add_fetch(&g_launches, 1, __ATOMIC_RELAXED); }
long long launch_count() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

// FP32 FMA throughput probe: 8 independent FMA chains per thread, no memory traffic in the loop
__global__ void k_fp32_probe(int iters, float* out) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
      a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

// FP32 FLOP/s (an FMA counts 2) measured with CUDA events on `blocks` x 256 threads
double fp32_probe_gflops(int blocks, int iters, cudaStream_t st) {
  float* d = nullptr;
  cudaMalloc(&d, sizeof(float));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fp32_probe<<<blocks, 256, 0, st>>>(iters / 4, d);  // warm-up
  cudaEventRecord(a, st);
  k_fp32_probe<<<blocks, 256, 0, st>>>(iters, d);
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d);
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * 256;
  return flops / (ms * 1e-3) / 1e9;
}

struct ChanConst {
  double wn;          // wavenumber 2 pi nu / c
  double spec;        // (nu / 1.4 GHz)^-0.7
  double inv_lambda;  // wavenumber / (2 pi), evaluate_uv_grid.c:159
  float il_hi, il_lo; // inv_lambda as double-float
  float wnf, specf;
};
__constant__ ChanConst c_ch[kMaxCh];
__constant__ int c_nch;

#define RLF_VIS_OK(call) do { int r_ = (call); if (r_) return r_; } while (0)
int launch_reduce_partials(const double* partial, int n_part, int len, double* sums, cudaStream_t st);

static int check(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf: %s: %s\n", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

static size_t facet_smem(unsigned F, int arrays, const void* kernel) {
  const size_t bytes = (size_t)arrays * F * F * sizeof(double);
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return bytes;
}

int set_channels(int n_ch, const double* wavenumbers, const double* spec, cudaStream_t st) {
  if (n_ch < 1 || n_ch > kMaxCh) {
    fprintf(stderr, "rlf: %d channels (1..%d supported)\n", n_ch, kMaxCh);
    return 1;
  }
  static ChanConst h[kMaxCh];
  for (int c = 0; c < n_ch; ++c) {
    h[c].wn = wavenumbers[c];
    h[c].spec = spec ? spec[c] : 1.0;
    h[c].inv_lambda = wavenumbers[c] / (2. * kPi);
    h[c].il_hi = (float)h[c].inv_lambda;
    h[c].il_lo = (float)(h[c].inv_lambda - (double)h[c].il_hi);
    h[c].wnf = (float)wavenumbers[c];
    h[c].specf = (float)h[c].spec;
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_ch, h, sizeof(ChanConst) * n_ch, 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_nch, &n_ch, sizeof(int), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // h is reused by the next call
  if (e != cudaSuccess) { fprintf(stderr, "rlf: set_channels: %s\n", cudaGetErrorString(e)); return (int)e; }
  return 0;
}

int grid_partial_blocks(int n_rows) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // ~2048 rows per CTA at most 4 CTAs per SM: few partials for small observations
  const int want = (n_rows + 2047) / 2048;
  return want < 1 ? 1 : (want > sms * 4 ? sms * 4 : want);
}

// partial [n_part][arrays * nc] -> sums [arrays * nc], one CTA per value, fixed-order tree
__global__ void k_reduce_partials(const double* __restrict__ partial, int n_part, int len, double* __restrict__ sums) {
  __shared__ double ws[8];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int p = threadIdx.x; p < n_part; p += blockDim.x) s += partial[(size_t)p * len + c];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    sums[c] = t;
  }
}

int launch_reduce_partials(const double* partial, int n_part, int len, double* sums, cudaStream_t st) {
  k_reduce_partials<<<len, 256, 0, st>>>(partial, n_part, len, sums);
  return check("k_reduce_partials");
}

// ------------------------------------------------------------- cell index
// evaluate_uv_grid.c:160-177: pu = (unsigned)((u*inv_lambda + len)/inc); explicit round-to-
// nearest intrinsics keep the compiler from fusing the multiply-add, so the cell boundaries are
// those of the reference's IEEE arithmetic.
__device__ __forceinline__ uint16_t cell_of(double u, double v, double il, double len, double inc, unsigned F) {
  const double uu = __dmul_rn(u, il);
  const double vv = __dmul_rn(v, il);
  const unsigned pu = (unsigned)__ddiv_rn(__dadd_rn(uu, len), inc);
  const unsigned pv = (unsigned)__ddiv_rn(__dadd_rn(vv, len), inc);
  const unsigned long long pc = (unsigned long long)pv * F + pu;
  return (pc < (unsigned long long)F * F) ? (uint16_t)pc : kNoCell;
}

__global__ void k_cell_index(Observation o, const uint8_t* flag, unsigned F, uint16_t* cell) {
  const double inc = 2 * o.len / F;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row];
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      cell[idx] = (flag && flag[idx]) ? kNoCell : cell_of(u, v, c_ch[ch].inv_lambda, o.len, inc, F);
    }
  }
}

int launch_cell_index(const Observation& o, const uint8_t* flag, unsigned F, uint16_t* cell, cudaStream_t st) {
  if (F == 0 || F > kMaxFacet) { fprintf(stderr, "rlf: facet size %u out of range\n", F); return 1; }
  int blocks = (o.n_rows + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_cell_index<<<blocks, 256, 0, st>>>(o, flag, F, cell);
  return check("k_cell_index");
}

// ----------------------------------------------------------- grid weights
__global__ void k_grid_weights(Observation o, const uint16_t* cell, const float* sigma2, unsigned F,
                               double* partial) {
  extern __shared__ double sm[];
  const int nc = F * F;
  double* ss = sm;
  double* ws = sm + nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) sm[i] = 0.0;
  __syncthreads();
  // a row's consecutive channels mostly fall in one cell: sum each run locally, one atomic pair per run
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    uint16_t cur = kNoCell;
    double s_run = 0.0, w_run = 0.0;
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      const uint16_t c = cell[idx];
      if (c == kNoCell) continue;
      if (c != cur) {
        if (cur != kNoCell) {
          atomicAdd(&ss[cur], s_run);
          atomicAdd(&ws[cur], w_run);
        }
        cur = c;
        s_run = 0.0;
        w_run = 0.0;
      }
      s_run += (double)sigma2[idx];
      w_run += 1.0;
    }
    if (cur != kNoCell) {
      atomicAdd(&ss[cur], s_run);
      atomicAdd(&ws[cur], w_run);
    }
  }
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * 2 * nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) out[i] = sm[i];
}

__global__ void k_reduce_pairs(const double* partial, int n_part, int nc, double* a, double* b) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    double sa = 0.0, sb = 0.0;
    for (int p = 0; p < n_part; ++p) {
      sa += partial[(size_t)p * 2 * nc + c];
      sb += partial[(size_t)p * 2 * nc + nc + c];
    }
    a[c] = sa;
    b[c] = sb;
  }
}

int launch_grid_weights(const Observation& o, const uint16_t* cell, const float* sigma2, unsigned F,
                        double* partial, int n_part, double* sum_sigma2, double* sum_w, cudaStream_t st) {
  const int nc = F * F;
  if (F == 0 || F > kMaxExtractFacet) { fprintf(stderr, "rlf: facet size %u out of range\n", F); return 1; }
  k_grid_weights<<<n_part, 256, facet_smem(F, 2, (const void*)k_grid_weights), st>>>(o, cell, sigma2, F, partial);
  int e = check("k_grid_weights");
  if (e) return e;
  double* sums = partial + (size_t)n_part * 2 * nc;
  RLF_VIS_OK(launch_reduce_partials(partial, n_part, 2 * nc, sums, st));
  cudaMemcpyAsync(sum_sigma2, sums, nc * sizeof(double), cudaMemcpyDeviceToDevice, st);
  cudaMemcpyAsync(sum_w, sums + nc, nc * sizeof(double), cudaMemcpyDeviceToDevice, st);
  return check("grid_weights copy");
}

// --------------------------------------------------------- extraction F64
// source_extraction.c:46-68 for one galaxy with e = 0: visGal = round model + data - sky model,
// phase-shifted to (l0, m0), gridded.  A thread keeps a running sum while consecutive channels of
// its row fall in the same cell and adds it to the CTA's shared-memory facet when the cell
// changes; each CTA writes its facet to partial[blockIdx] (reduced in fixed order later).
__global__ void k_extract_f64(Observation o, const double2* data, const double2* sky, const uint16_t* cell,
                              const GalaxyParams* galp, int gaussian, double* partial) {
  extern __shared__ double sm[];
  const GalaxyParams g = *galp;
  const int nc = g.facet * g.facet;
  double* fre = sm;
  double* fim = sm + nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) sm[i] = 0.0;
  __syncthreads();
  const double l = g.l, m = g.m;
  const double n = sqrt(1. - l * l - m * m) - 1.;
  const double sf = scale_factor(g.e1, g.e2, g.scale);
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    const double p = u * l + v * m + w * n;
    const double k1 = (1. + g.e1) * u + g.e2 * v;
    const double k2 = g.e2 * u + (1. - g.e1) * v;
    int cur = -1;
    double are = 0.0, aim = 0.0;
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      const uint16_t c = cell[idx];
      if (c == kNoCell) continue;
      const ChanConst cc = c_ch[ch];
      const double phase = cc.wn * p;
      double sp, cp;
      sincos(phase, &sp, &cp);
      const double sh = shape(gaussian, k1, k2, sf, cc.wn * cc.wn) * (cc.spec * g.flux);
      const double2 d = data[idx], s = sky[idx];
      const double gr = sh * cp + (d.x - s.x);
      const double gi = sh * sp + (d.y - s.y);
      // rotation by e^{-i phase} (galaxy_visibilities.c:244-270)
      const double re = gr * cp + gi * sp;
      const double im = -gr * sp + gi * cp;
      if (c != cur) {
        if (cur >= 0) { atomicAdd(&fre[cur], are); atomicAdd(&fim[cur], aim); }
        cur = c; are = 0.0; aim = 0.0;
      }
      are += re;
      aim += im;
    }
    if (cur >= 0) { atomicAdd(&fre[cur], are); atomicAdd(&fim[cur], aim); }
  }
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * 2 * nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) out[i] = sm[i];
}

int launch_extract_f64(const Observation& o, const double2* data, const double2* sky, const uint16_t* cell,
                       const GalaxyParams* gal, unsigned F, int gaussian, double* partial, int n_part,
                       cudaStream_t st) {
  if (F == 0 || F > kMaxExtractFacet) { fprintf(stderr, "rlf: facet size %u out of range\n", F); return 1; }
  k_extract_f64<<<n_part, 256, facet_smem(F, 2, (const void*)k_extract_f64), st>>>(o, data, sky, cell, gal, gaussian,
                                                                                   partial);
  return check("k_extract_f64");
}

// ------------------------------------------------------- extraction mixed
__device__ __forceinline__ float turns_reduced(f2 p, const ChanConst& cc) {
  // t = p * inv_lambda in double-float, reduced to [-1/2, 1/2]
  f2 t = two_prod(p.hi, cc.il_hi);
  t.lo = fmaf(p.hi, cc.il_lo, fmaf(p.lo, cc.il_hi, t.lo));
  const float k = rintf(t.hi);
  return (t.hi - k) + t.lo;
}

__device__ __forceinline__ float shape_f(int gaussian, float k1, float k2, float sfw) {
  const float q = sfw * (k1 * k1 + k2 * k2);
  if (gaussian) return __expf(-0.5f * q);
  const float den = 1.f + q;
  return 1.f / (den * sqrtf(den));
}

__global__ void k_extract_mixed(Observation o, const float2* data, const float2* sky, const uint16_t* cell,
                                const GalaxyParams* galp, int gaussian, double* partial) {
  extern __shared__ double sm[];
  const GalaxyParams g = *galp;
  const int nc = g.facet * g.facet;
  double* fre = sm;
  double* fim = sm + nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) sm[i] = 0.0;
  __syncthreads();
  const double l = g.l, m = g.m;
  const double n = sqrt(1. - l * l - m * m) - 1.;
  const float sf = (float)scale_factor(g.e1, g.e2, g.scale);
  const float flux = (float)g.flux;
  const float e1 = (float)g.e1, e2 = (float)g.e2;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    const f2 p = df_from_double(u * l + v * m + w * n);
    const float uf = (float)u, vf = (float)v;
    const float k1 = (1.f + e1) * uf + e2 * vf;
    const float k2 = e2 * uf + (1.f - e1) * vf;
    int cur = -1;
    float are = 0.f, aim = 0.f, cre = 0.f, cim = 0.f;  // Kahan sums of the current cell run
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      const uint16_t c = cell[idx];
      if (c == kNoCell) continue;
      const ChanConst cc = c_ch[ch];
      float sp, cp;
      sincospif(2.f * turns_reduced(p, cc), &sp, &cp);
      const float sh = shape_f(gaussian, k1, k2, sf * cc.wnf * cc.wnf) * (cc.specf * flux);
      const float2 d = data[idx], s = sky[idx];
      const float gr = fmaf(sh, cp, d.x - s.x);
      const float gi = fmaf(sh, sp, d.y - s.y);
      const float re = fmaf(gr, cp, gi * sp);
      const float im = fmaf(gi, cp, -gr * sp);
      if (c != cur) {
        if (cur >= 0) { atomicAdd(&fre[cur], (double)are - (double)cre); atomicAdd(&fim[cur], (double)aim - (double)cim); }
        cur = c; are = aim = cre = cim = 0.f;
      }
      float y = re - cre, t = are + y;
      cre = (t - are) - y; are = t;
      y = im - cim; t = aim + y;
      cim = (t - aim) - y; aim = t;
    }
    if (cur >= 0) { atomicAdd(&fre[cur], (double)are - (double)cre); atomicAdd(&fim[cur], (double)aim - (double)cim); }
  }
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * 2 * nc;
  for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) out[i] = sm[i];
}

int launch_extract_mixed(const Observation& o, const float2* data, const float2* sky, const uint16_t* cell,
                         const GalaxyParams* gal, unsigned F, int gaussian, double* partial, int n_part,
                         cudaStream_t st) {
  if (F == 0 || F > kMaxExtractFacet) { fprintf(stderr, "rlf: facet size %u out of range\n", F); return 1; }
  k_extract_mixed<<<n_part, 256, facet_smem(F, 2, (const void*)k_extract_mixed), st>>>(o, data, sky, cell, gal,
                                                                                       gaussian, partial);
  return check("k_extract_mixed");
}

// gridding_visibilities (evaluate_uv_grid.c:143-211) of a caller-given visibility array: the
// visibilities and variances are summed per cell; weights are 1.
__global__ void k_grid_vis_f64(Observation o, const double2* vis, const float* sigma2, const uint8_t* flag,
                               unsigned F, double* partial) {
  extern __shared__ double sm[];
  const int nc = F * F;
  double* fre = sm;
  double* fim = sm + nc;
  double* fs = sm + 2 * nc;
  double* fw = sm + 3 * nc;
  for (int i = threadIdx.x; i < 4 * nc; i += blockDim.x) sm[i] = 0.0;
  __syncthreads();
  const double inc = 2 * o.len / F;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row];
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      if (flag && flag[idx]) continue;
      const uint16_t c = cell_of(u, v, c_ch[ch].inv_lambda, o.len, inc, F);
      if (c == kNoCell) continue;
      const double2 x = vis[idx];
      atomicAdd(&fre[c], x.x);
      atomicAdd(&fim[c], x.y);
      atomicAdd(&fs[c], (double)sigma2[idx]);
      atomicAdd(&fw[c], 1.0);
    }
  }
  __syncthreads();
  double* out = partial + (size_t)blockIdx.x * 4 * nc;
  for (int i = threadIdx.x; i < 4 * nc; i += blockDim.x) out[i] = sm[i];
}

int launch_grid_vis_f64(const Observation& o, const double2* vis, const float* sigma2, const uint8_t* flag,
                        unsigned F, double* partial, int n_part, cudaStream_t st) {
  if (F == 0 || F > kMaxGridFacet) { fprintf(stderr, "rlf: gridding facet %u unsupported\n", F); return 1; }
  k_grid_vis_f64<<<n_part, 256, facet_smem(F, 4, (const void*)k_grid_vis_f64), st>>>(o, vis, sigma2, flag, F, partial);
  return check("k_grid_vis_f64");
}

// ------------------------------------------------------------ finalize
// partial layout per galaxy: [n_part][2][F*F] (re, im); sum tables: sum_sigma2[gi][F*F],
// sum_w[gi][F*F] indexed by the galaxy.
__global__ void k_facet_finalize(const int* facets, const double* partial, int n_part, long long pstride,
                                 const double* const* sum_sigma2, const double* const* sum_w, double len,
                                 FacetOut out) {
  const int g = blockIdx.x;
  const int F = facets[g];
  const int nc = F * F;
  const double* P = partial + (size_t)g * pstride;
  const double* SS = sum_sigma2[g];
  const double* SW = sum_w[g];
  const double inc = 2 * len / F;
  __shared__ int warp_tot[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int off = out.offset[g];
  for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    int flagc = 0;
    double vre = 0, vim = 0, sg = 0;
    if (c < nc) {
      const double sw = SW[c];
      if (sw != 0.0) {
        double sre = 0.0, sim = 0.0;
        for (int p = 0; p < n_part; ++p) {
          sre += P[(size_t)p * 2 * nc + c];
          sim += P[(size_t)p * 2 * nc + nc + c];
        }
        const double ss = SS[c];
        vre = sre * sw / ss;
        vim = sim * sw / ss;
        sg = ss / (sw * sw);
        flagc = 1;
      }
    }
    // block exclusive scan of flagc, in cell order
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, flagc);
    const int inwarp = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) warp_tot[warp] = __popc(bal);
    __syncthreads();
    int before = base;
    for (int w = 0; w < warp; ++w) before += warp_tot[w];
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
  if (threadIdx.x == 0) out.ncoords[g] = base;
}

int launch_facet_finalize(int n, const int* facets, const double* partial, int n_part, long long pstride,
                          const double* const* sum_sigma2, const double* const* sum_w, double len,
                          FacetOut out, cudaStream_t st) {
  if (n <= 0) return 0;
  k_facet_finalize<<<n, 1024, 0, st>>>(facets, partial, n_part, pstride, sum_sigma2, sum_w, len, out);
  return check("k_facet_finalize");
}

// ------------------------------------------------------------- removal
__global__ void k_remove_f64(Observation o, double2* data, double2* sky, const GalaxyParams* galp,
                             const double* fit_e1e2, const int* fit_error, int gaussian) {
  if (fit_error && *fit_error) return;
  const GalaxyParams g = *galp;
  const double e1 = fit_e1e2 ? fit_e1e2[0] : g.e1, e2 = fit_e1e2 ? fit_e1e2[1] : g.e2;
  const double l = g.l, m = g.m;
  const double n = sqrt(1. - l * l - m * m) - 1.;
  const double sf0 = scale_factor(0., 0., g.scale);
  const double sf = scale_factor(e1, e2, g.scale);
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    const double p = u * l + v * m + w * n;
    const double k1 = (1. + e1) * u + e2 * v;
    const double k2 = e2 * u + (1. - e1) * v;
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      const ChanConst cc = c_ch[ch];
      double sp, cp;
      sincos(cc.wn * p, &sp, &cp);
      const double wn2 = cc.wn * cc.wn;
      const double a0 = shape(gaussian, u, v, sf0, wn2) * (cc.spec * g.flux);
      const double a1 = shape(gaussian, k1, k2, sf, wn2) * (cc.spec * g.flux);
      double2 s = sky[idx];
      s.x -= a0 * cp;
      s.y -= a0 * sp;
      sky[idx] = s;
      double2 d = data[idx];
      d.x -= a1 * cp;
      d.y -= a1 * sp;
      data[idx] = d;
    }
  }
}

__global__ void k_remove_mixed(Observation o, float2* data, float2* sky, const GalaxyParams* galp,
                               const double* fit_e1e2, const int* fit_error, int gaussian) {
  if (fit_error && *fit_error) return;
  const GalaxyParams g = *galp;
  const double e1d = fit_e1e2 ? fit_e1e2[0] : g.e1, e2d = fit_e1e2 ? fit_e1e2[1] : g.e2;
  const double l = g.l, m = g.m;
  const double n = sqrt(1. - l * l - m * m) - 1.;
  const float sf0 = (float)scale_factor(0., 0., g.scale);
  const float sf = (float)scale_factor(e1d, e2d, g.scale);
  const float e1 = (float)e1d, e2 = (float)e2d, flux = (float)g.flux;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    const f2 p = df_from_double(u * l + v * m + w * n);
    const float uf = (float)u, vf = (float)v;
    const float k1 = (1.f + e1) * uf + e2 * vf;
    const float k2 = e2 * uf + (1.f - e1) * vf;
    for (int ch = 0; ch < c_nch; ++ch) {
      const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
      const ChanConst cc = c_ch[ch];
      float sp, cp;
      sincospif(2.f * turns_reduced(p, cc), &sp, &cp);
      const float wn2 = cc.wnf * cc.wnf;
      const float a0 = shape_f(gaussian, uf, vf, sf0 * wn2) * (cc.specf * flux);
      const float a1 = shape_f(gaussian, k1, k2, sf * wn2) * (cc.specf * flux);
      float2 s = sky[idx];
      s.x -= a0 * cp;
      s.y -= a0 * sp;
      sky[idx] = s;
      float2 d = data[idx];
      d.x -= a1 * cp;
      d.y -= a1 * sp;
      data[idx] = d;
    }
  }
}

static int row_blocks(int n_rows) {
  int b = (n_rows + 255) / 256;
  return b > 8192 ? 8192 : (b < 1 ? 1 : b);
}

int launch_remove_f64(const Observation& o, double2* data, double2* sky, const GalaxyParams* gal,
                      const double* fit_e1e2, const int* fit_error, int gaussian, cudaStream_t st) {
  k_remove_f64<<<row_blocks(o.n_rows), 256, 0, st>>>(o, data, sky, gal, fit_e1e2, fit_error, gaussian);
  return check("k_remove_f64");
}
int launch_remove_mixed(const Observation& o, float2* data, float2* sky, const GalaxyParams* gal,
                        const double* fit_e1e2, const int* fit_error, int gaussian, cudaStream_t st) {
  k_remove_mixed<<<row_blocks(o.n_rows), 256, 0, st>>>(o, data, sky, gal, fit_e1e2, fit_error, gaussian);
  return check("k_remove_mixed");
}

// ----------------------------------------------------------- sky model
__global__ void k_sky_model_f64(Observation o, double2* sky, const GalaxyParams* gals, int n_gal, int use_e,
                                int gaussian) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    for (int gi = 0; gi < n_gal; ++gi) {
      const GalaxyParams g = gals[gi];
      const double e1 = use_e ? g.e1 : 0., e2 = use_e ? g.e2 : 0.;
      const double sf = scale_factor(e1, e2, g.scale);
      const double n = sqrt(1. - g.l * g.l - g.m * g.m) - 1.;
      const double p = u * g.l + v * g.m + w * n;
      const double k1 = (1. + e1) * u + e2 * v;
      const double k2 = e2 * u + (1. - e1) * v;
      for (int ch = 0; ch < c_nch; ++ch) {
        const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
        const ChanConst cc = c_ch[ch];
        double sp, cp;
        sincos(cc.wn * p, &sp, &cp);
        const double a = shape(gaussian, k1, k2, sf, cc.wn * cc.wn) * (cc.spec * g.flux);
        double2 s = sky[idx];
        s.x += a * cp;
        s.y += a * sp;
        sky[idx] = s;
      }
    }
  }
}

// mixed: one thread per (row, 8-channel chunk), FP32 accumulation per visibility over galaxies
constexpr int kChunk = 8;
__global__ void k_sky_model_mixed(Observation o, float2* sky, const GalaxyParams* gals, int n_gal, int use_e,
                                  int gaussian) {
  const int nchunk = (c_nch + kChunk - 1) / kChunk;
  const long long total = (long long)o.n_rows * nchunk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int row = (int)(t % o.n_rows);
    const int ch0 = (int)(t / o.n_rows) * kChunk;
    const double u = o.uu[row], v = o.vv[row], w = o.ww[row];
    const float uf = (float)u, vf = (float)v;
    float ar[kChunk], ai[kChunk];
#pragma unroll
    for (int k = 0; k < kChunk; ++k) { ar[k] = 0.f; ai[k] = 0.f; }
    for (int gi = 0; gi < n_gal; ++gi) {
      const GalaxyParams g = gals[gi];
      const float e1 = use_e ? (float)g.e1 : 0.f, e2 = use_e ? (float)g.e2 : 0.f;
      const float sf = (float)scale_factor(use_e ? g.e1 : 0., use_e ? g.e2 : 0., g.scale);
      const double n = sqrt(1. - g.l * g.l - g.m * g.m) - 1.;
      const f2 p = df_from_double(u * g.l + v * g.m + w * n);
      const float k1 = (1.f + e1) * uf + e2 * vf;
      const float k2 = e2 * uf + (1.f - e1) * vf;
      const float flux = (float)g.flux;
#pragma unroll
      for (int k = 0; k < kChunk; ++k) {
        const int ch = ch0 + k;
        if (ch < c_nch) {
          const ChanConst cc = c_ch[ch];
          float sp, cp;
          sincospif(2.f * turns_reduced(p, cc), &sp, &cp);
          const float a = shape_f(gaussian, k1, k2, sf * cc.wnf * cc.wnf) * (cc.specf * flux);
          ar[k] = fmaf(a, cp, ar[k]);
          ai[k] = fmaf(a, sp, ai[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kChunk; ++k) {
      const int ch = ch0 + k;
      if (ch < c_nch) {
        const long long idx = row * o.lay.s_row + ch * o.lay.s_ch;
        float2 s = sky[idx];
        s.x += ar[k];
        s.y += ai[k];
        sky[idx] = s;
      }
    }
  }
}

int launch_sky_model_f64(const Observation& o, double2* sky, const GalaxyParams* gals, int n_gal, int use_e,
                         int gaussian, cudaStream_t st) {
  k_sky_model_f64<<<row_blocks(o.n_rows), 256, 0, st>>>(o, sky, gals, n_gal, use_e, gaussian);
  return check("k_sky_model_f64");
}
int launch_sky_model_mixed(const Observation& o, float2* sky, const GalaxyParams* gals, int n_gal, int use_e,
                           int gaussian, cudaStream_t st) {
  k_sky_model_mixed<<<row_blocks(o.n_rows * 2), 256, 0, st>>>(o, sky, gals, n_gal, use_e, gaussian);
  return check("k_sky_model_mixed");
}

// ----------------------------------------------- single-function kernels
__global__ void k_galaxy_vis_channel(int n, double spectra, double wavenumber, double e1, double e2, double scale,
                                     double flux, double l, double m, const double* uu, const double* vv,
                                     const double* ww, double2* vis, int gaussian) {
  const double sf = scale_factor(e1, e2, scale);
  const double wn2 = wavenumber * wavenumber;
  const double nn = sqrt(1. - l * l - m * m) - 1.;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double u = uu[i], v = vv[i], w = ww[i];
    double phase = u * l + v * m + w * nn;
    phase = wavenumber * phase;
    const double k1 = (1. + e1) * u + e2 * v;
    const double k2 = e2 * u + (1. - e1) * v;
    double sh = shape(gaussian, k1, k2, sf, wn2);
    sh *= spectra * flux;
    double sp, cp;
    sincos(phase, &sp, &cp);
    vis[i] = make_double2(sh * cp, sh * sp);
  }
}

__global__ void k_phase_shift_channel(int n, double wavenumber, double l, double m, const double* uu,
                                      const double* vv, const double* ww, double2* vis) {
  const double nn = sqrt(1. - l * l - m * m) - 1.;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double phase = uu[i] * l + vv[i] * m + ww[i] * nn;
    phase *= -wavenumber;
    double sp, cp;
    sincos(phase, &sp, &cp);
    const double2 x = vis[i];
    vis[i] = make_double2(x.x * cp - x.y * sp, x.x * sp + x.y * cp);
  }
}

int launch_galaxy_vis_channel(int n, double spectra, double wavenumber, double e1, double e2, double scale,
                              double flux, double l, double m, const double* uu, const double* vv,
                              const double* ww, double2* vis, int gaussian, cudaStream_t st) {
  if (n <= 0) return 0;
  k_galaxy_vis_channel<<<row_blocks(n), 256, 0, st>>>(n, spectra, wavenumber, e1, e2, scale, flux, l, m, uu, vv,
                                                      ww, vis, gaussian);
  return check("k_galaxy_vis_channel");
}
int launch_phase_shift_channel(int n, double wavenumber, double l, double m, const double* uu, const double* vv,
                               const double* ww, double2* vis, cudaStream_t st) {
  if (n <= 0) return 0;
  k_phase_shift_channel<<<row_blocks(n), 256, 0, st>>>(n, wavenumber, l, m, uu, vv, ww, vis);
  return check("k_phase_shift_channel");
}

// model_galaxy_visibilities_at_zero: one CTA, deterministic block sum of M^2/sigma^2
__global__ void k_model_at_zero(double e1, double e2, double scale, int n, const double* gu, const double* gv,
                                const double* sigma2, double* mod, int gaussian) {
  __shared__ double ws[32];
  const double sf = scale_factor(e1, e2, scale);
  const double cc2 = 4 * kPi * kPi;
  double part = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = gu[i], v = gv[i];
    const double k1 = (1. + e1) * u + e2 * v;
    const double k2 = e2 * u + (1. - e1) * v;
    const double mv = shape(gaussian, k1, k2, sf, cc2);
    mod[i] = mv;
    part += mv * mv / sigma2[i];
  }
  part = warp_sum(part);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = part;
  __syncthreads();
  double sum = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += ws[w];
  sum = sqrt(sum);
  for (int i = threadIdx.x; i < n; i += blockDim.x) mod[i] /= sum;
}

int launch_model_at_zero(double e1, double e2, double scale, int n, const double* gu, const double* gv,
                         const double* sigma2, double* mod, int gaussian, cudaStream_t st) {
  if (n <= 0) return 0;
  k_model_at_zero<<<1, 1024, 0, st>>>(e1, e2, scale, n, gu, gv, sigma2, mod, gaussian);
  return check("k_model_at_zero");
}

__global__ void k_count_cells(Observation o, const uint16_t* cell, unsigned F, unsigned* count) {
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < o.n_rows; row += gridDim.x * blockDim.x) {
    for (int ch = 0; ch < c_nch; ++ch) {
      const uint16_t c = cell[row * o.lay.s_row + ch * o.lay.s_ch];
      if (c != kNoCell) atomicOr(&count[c], 1u);
    }
  }
}
__global__ void k_count_nonzero(const unsigned* count, int nc, unsigned* out) {
  unsigned s = 0;
  for (int i = threadIdx.x; i < nc; i += blockDim.x) s += count[i] ? 1u : 0u;
  for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  __shared__ unsigned ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    *out = t;
  }
}

int launch_count_cells(const Observation& o, const uint16_t* cell, unsigned F, unsigned* count_out,
                       cudaStream_t st) {
  // count_out: [F*F + 1] scratch, last element receives the number of non-empty cells
  const int nc = F * F;
  cudaMemsetAsync(count_out, 0, (nc + 1) * sizeof(unsigned), st);
  k_count_cells<<<row_blocks(o.n_rows), 256, 0, st>>>(o, cell, F, count_out);
  k_count_nonzero<<<1, 1024, 0, st>>>(count_out, nc, count_out + nc);
  return check("k_count_cells");
}

// evaluate_facet_coords (evaluate_uv_grid.c:113-133): row-major compaction of non-empty cells
__global__ void k_facet_coords(double* gu, double* gv, double len, unsigned F, const double* count_w, unsigned* n_out) {
  if (threadIdx.x != 0) return;
  const double inc = 2 * len / F;
  unsigned n = 0;
  for (unsigned p = 0; p < F * F; ++p) {
    if (count_w[p]) {
      unsigned j = p / F, i = p % F;
      gu[n] = __dsub_rn(__dmul_rn(i + 0.5, inc), len);
      gv[n] = __dsub_rn(__dmul_rn(j + 0.5, inc), len);
      n++;
    }
  }
  *n_out = n;
}
int launch_facet_coords(double* gu, double* gv, double len, unsigned F, const double* count_w, unsigned* n_out,
                        cudaStream_t st) {
  k_facet_coords<<<1, 32, 0, st>>>(gu, gv, len, F, count_w, n_out);
  return check("k_facet_coords");
}

// average_facets (evaluate_uv_grid.c:216-230): in-place compaction, sequential like the reference
__global__ void k_average_facets(long long size, double2* vis, double* sigma2, const double* sum_w) {
  if (threadIdx.x != 0) return;
  long long n = 0;
  for (long long p = 0; p < size; p++) {
    const double sw = sum_w[p];
    if (sw) {
      const double s = sigma2[p];
      const double2 x = vis[p];
      vis[n] = make_double2(x.x * sw / s, x.y * sw / s);
      sigma2[n] = s / (sw * sw);
      n++;
    }
  }
}
int launch_average_facets(long long size, double2* vis, double* sigma2, const double* sum_w, cudaStream_t st) {
  k_average_facets<<<1, 32, 0, st>>>(size, vis, sigma2, sum_w);
  return check("k_average_facets");
}

__global__ void k_f32_to_c64(long long n, const float2* in, double2* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 x = in[i];
    out[i] = make_double2((double)x.x, (double)x.y);
  }
}
// caller index -> position in a row-permuted observation
__device__ __forceinline__ long long permuted(long long idx, int n_rows, const int* __restrict__ inv) {
  const long long ch = idx / n_rows;
  return ch * n_rows + inv[idx - ch * n_rows];
}
__global__ void k_c64_to_f32_scatter(long long i0, long long count, int n_rows, const double2* __restrict__ in,
                                     const int* __restrict__ inv, float2* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const double2 x = in[i];
    out[permuted(i0 + i, n_rows, inv)] = make_float2((float)x.x, (float)x.y);
  }
}
__global__ void k_f32_to_c64_gather(long long i0, long long count, int n_rows, const float2* __restrict__ in,
                                    const int* __restrict__ inv, double2* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float2 x = in[permuted(i0 + i, n_rows, inv)];
    out[i] = make_double2((double)x.x, (double)x.y);
  }
}
template <class T>
__global__ void k_scatter_rows(long long i0, long long count, int n_rows, const T* __restrict__ in,
                               const int* __restrict__ inv, T* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    out[permuted(i0 + i, n_rows, inv)] = in[i];
}
__global__ void k_gather_rows_f64(int n, const double* __restrict__ in, const int* __restrict__ perm,
                                  double* __restrict__ out) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) out[p] = in[perm[p]];
}
__global__ void k_invert_perm(int n, const int* __restrict__ perm, int* __restrict__ inv) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) inv[perm[p]] = p;
}
static int grid_of(long long n) { return (int)std::min<long long>((n + 255) / 256, 8192); }
int launch_c64_to_f32_scatter(long long i0, long long count, int n_rows, const double2* in, const int* inv,
                              float2* out, cudaStream_t st) {
  if (count <= 0) return 0;
  k_c64_to_f32_scatter<<<grid_of(count), 256, 0, st>>>(i0, count, n_rows, in, inv, out);
  return check("k_c64_to_f32_scatter");
}
int launch_f32_to_c64_gather(long long i0, long long count, int n_rows, const float2* in, const int* inv,
                             double2* out, cudaStream_t st) {
  if (count <= 0) return 0;
  k_f32_to_c64_gather<<<grid_of(count), 256, 0, st>>>(i0, count, n_rows, in, inv, out);
  return check("k_f32_to_c64_gather");
}
template <class T>
int launch_scatter_rows(long long i0, long long count, int n_rows, const T* in, const int* inv, T* out,
                        cudaStream_t st) {
  if (count <= 0) return 0;
  k_scatter_rows<T><<<grid_of(count), 256, 0, st>>>(i0, count, n_rows, in, inv, out);
  return check("k_scatter_rows");
}
template int launch_scatter_rows<float>(long long, long long, int, const float*, const int*, float*, cudaStream_t);
template int launch_scatter_rows<uint8_t>(long long, long long, int, const uint8_t*, const int*, uint8_t*, cudaStream_t);
template int launch_scatter_rows<float2>(long long, long long, int, const float2*, const int*, float2*, cudaStream_t);
int launch_gather_rows_f64(int n, const double* in, const int* perm, double* out, cudaStream_t st) {
  if (n <= 0) return 0;
  k_gather_rows_f64<<<grid_of(n), 256, 0, st>>>(n, in, perm, out);
  return check("k_gather_rows_f64");
}
int launch_invert_perm(int n, const int* perm, int* inv, cudaStream_t st) {
  if (n <= 0) return 0;
  k_invert_perm<<<grid_of(n), 256, 0, st>>>(n, perm, inv);
  return check("k_invert_perm");
}

int launch_convert_f32_to_c64(long long n, const float2* in, double2* out, cudaStream_t st) {
  if (n <= 0) return 0;
  k_f32_to_c64<<<4096, 256, 0, st>>>(n, in, out);
  return check("k_f32_to_c64");
}

}  // namespace rlf

namespace rlf {
// gridding_visibilities tail (evaluate_uv_grid.c:196-209): per-cell sums reduced in fixed
// partial order, then sequential row-major compaction
__global__ void k_grid_vis_reduce(const double* partial, int n_part, int nc, double* sums) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < 4 * nc; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < n_part; ++p) s += partial[(size_t)p * 4 * nc + c];
    sums[c] = s;
  }
}
__global__ void k_grid_vis_compact(const double* sums, int nc, double2* new_vis, double* new_sigma2, double* sum_w) {
  if (threadIdx.x != 0) return;
  const double* tre = sums;
  const double* tim = sums + nc;
  const double* ts = sums + 2 * nc;
  const double* tw = sums + 3 * nc;
  int n = 0;
  for (int p = 0; p < nc; ++p) {
    sum_w[p] = tw[p];
    if (tw[p]) {
      new_vis[n] = make_double2(tre[p] * tw[p] / ts[p], tim[p] * tw[p] / ts[p]);
      new_sigma2[n] = ts[p] / (tw[p] * tw[p]);
      n++;
    }
  }
}
int launch_grid_vis_finalize(const double* partial, int n_part, unsigned F, double2* new_vis, double* new_sigma2,
                             double* sum_w, cudaStream_t st) {
  const int nc = F * F;
  double* sums = const_cast<double*>(partial) + (size_t)n_part * 4 * nc;  // scratch after the partials
  RLF_VIS_OK(launch_reduce_partials(partial, n_part, 4 * nc, sums, st));
  k_grid_vis_compact<<<1, 32, 0, st>>>(sums, nc, new_vis, new_sigma2, sum_w);
  return check("k_grid_vis_finalize");
}
}  // namespace rlf

// Measurement Set column blocks to the hot path's arrays and back (measurement_set.cpp:203-453),
// without casacore: the caller reads the raw column blocks from the table (row-major, the
// correlations of a channel contiguous) and these kernels reproduce what the reference's readers
// make of them:
//   ms_read_coords  UVW [row][3] -> uu, vv, ww and ceil(max(max|u|, max|v|))
//   ms_read_sigma   SIGMA column, flattened: sigma2[i] = sigma[i]^2 for i < num_rows; the driver then
//                   replaces every entry <= 0 by the theoretical variance (RadioLensfit2.cpp:257-270)
//   ms_read_Flag    FLAG [row][ch][pol] -> [ch][row]: correlation 0, or 0 || 3 with 4 correlations
//   ms_read_vis     DATA [row][ch][pol] complex64 Jy -> [ch][row] complex uJy: correlation 0, or
//                   (0 + 3) / 2 with 4 correlations, in double as the reference computes it
//   ms_write_vis    [ch][row] complex uJy -> DATA [row][ch] complex64 Jy (one correlation)
// The transposes stage 32 x 32 (row, channel) tiles in shared memory so that both the row-major
// reads and the channel-major writes are coalesced.  All of it is HBM-bound byte work.
#include "rlf_ms.cuh"
#include <stdio.h>

namespace rlf {

static int check(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf: %s: %s\n", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

constexpr int kTile = 32;

// Stokes I of one (row, channel) in uJy, measurement_set.cpp:388-399 (double arithmetic)
__device__ __forceinline__ double2 stokes_i(const float2* in, size_t base, int npol) {
  double re = (double)in[base].x, im = (double)in[base].y;
  if (npol == 4) {
    re += (double)in[base + 3].x;
    im += (double)in[base + 3].y;
    re *= 0.5;
    im *= 0.5;
  }
  re *= 1e+6;
  im *= 1e+6;
  return make_double2(re, im);
}
__device__ __forceinline__ void put_vis(double2* out, size_t i, double2 v) { out[i] = v; }
__device__ __forceinline__ void put_vis(float2* out, size_t i, double2 v) {
  out[i] = make_float2((float)v.x, (float)v.y);
}

// DATA block [rows][nch][npol] complex64 -> out [nch][rows] (row r at position inv[r] when the
// observation stores its rows permuted); grid (row tiles, channel tiles)
template <class OUT>
__global__ void k_ms_vis(const float2* __restrict__ in, long long rows, int nch, int npol, const int* __restrict__ inv,
                         OUT* __restrict__ out) {
  __shared__ double2 tile[kTile][kTile + 1];
  const long long r0 = (long long)blockIdx.x * kTile;
  const int c0 = blockIdx.y * kTile;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  // read: consecutive threads take consecutive channels of a row
  for (int k = ty; k < kTile; k += blockDim.y) {
    const long long r = r0 + k;
    const int c = c0 + tx;
    if (r < rows && c < nch) tile[k][tx] = stokes_i(in, ((size_t)r * nch + c) * npol, npol);
  }
  __syncthreads();
  // write: consecutive threads take consecutive rows of a channel
  for (int k = ty; k < kTile; k += blockDim.y) {
    const int c = c0 + k;
    const long long r = r0 + tx;
    if (r < rows && c < nch) put_vis(out, (size_t)c * rows + (inv ? inv[r] : r), tile[tx][k]);
  }
}

// FLAG block [rows][nch][npol] -> out [nch][rows], counting the flagged (measurement_set.cpp:318-332)
__global__ void k_ms_flags(const uint8_t* __restrict__ in, long long rows, int nch, int npol, uint8_t* __restrict__ out,
                           unsigned long long* __restrict__ count) {
  __shared__ uint8_t tile[kTile][kTile + 1];
  __shared__ unsigned int cnt;
  const long long r0 = (long long)blockIdx.x * kTile;
  const int c0 = blockIdx.y * kTile;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (tx == 0 && ty == 0) cnt = 0;
  __syncthreads();
  unsigned int mine = 0;
  for (int k = ty; k < kTile; k += blockDim.y) {
    const long long r = r0 + k;
    const int c = c0 + tx;
    if (r < rows && c < nch) {
      const size_t i = ((size_t)r * nch + c) * npol;
      bool f = in[i] != 0;
      if (npol == 4) f = f || in[i + 3] != 0;
      tile[k][tx] = f;
      mine += f;
    }
  }
  if (mine) atomicAdd(&cnt, mine);
  __syncthreads();
  for (int k = ty; k < kTile; k += blockDim.y) {
    const int c = c0 + k;
    const long long r = r0 + tx;
    if (r < rows && c < nch) out[(size_t)c * rows + r] = tile[tx][k];
  }
  if (tx == 0 && ty == 0 && cnt) atomicAdd(count, (unsigned long long)cnt);
}

// vis [nch][rows] complex uJy -> DATA block [rows][nch] complex64 Jy (measurement_set.cpp:423-433)
__global__ void k_ms_write(const double2* __restrict__ vis, long long rows, int nch, float2* __restrict__ out) {
  __shared__ double2 tile[kTile][kTile + 1];
  const long long r0 = (long long)blockIdx.x * kTile;
  const int c0 = blockIdx.y * kTile;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < kTile; k += blockDim.y) {
    const int c = c0 + k;
    const long long r = r0 + tx;
    if (r < rows && c < nch) tile[k][tx] = vis[(size_t)c * rows + r];
  }
  __syncthreads();
  for (int k = ty; k < kTile; k += blockDim.y) {
    const long long r = r0 + k;
    const int c = c0 + tx;
    if (r < rows && c < nch) {
      const double2 v = tile[tx][k];
      out[(size_t)r * nch + c] = make_float2((float)(v.x * 1e-6), (float)(v.y * 1e-6));
    }
  }
}

// UVW [rows][3] -> uu, vv, ww and the per-block maxima of |u|, |v| (measurement_set.cpp:224-240)
__global__ void k_ms_coords(const double* __restrict__ uvw, long long rows, double* __restrict__ uu,
                            double* __restrict__ vv, double* __restrict__ ww, unsigned long long* __restrict__ umax) {
  double m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
    const double u = uvw[3 * i], v = uvw[3 * i + 1], w = uvw[3 * i + 2];
    uu[i] = u;
    vv[i] = v;
    ww[i] = w;
    m = fmax(m, fmax(fabs(u), fabs(v)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  // non-negative doubles order as their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(umax, (unsigned long long)__double_as_longlong(m));
}

// sigma2 [nch * rows]: sigma[i]^2 for i < rows (the SIGMA column read flat, measurement_set.cpp:
// 266-273), then entries <= 0 and the ones the reader does not set -> the theoretical variance
__global__ void k_ms_sigma2(const float* __restrict__ sigma, long long rows, long long nvis, float theory,
                            float* __restrict__ sigma2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nvis; i += (long long)gridDim.x * blockDim.x) {
    float s2 = 0.f;
    if (i < rows) {
      const float s = sigma[i];
      s2 = s * s;
    }
    sigma2[i] = s2 <= 0.f ? theory : s2;
  }
}

static dim3 tiles(long long rows, int nch) {
  return dim3((unsigned)((rows + kTile - 1) / kTile), (unsigned)((nch + kTile - 1) / kTile));
}

int launch_ms_vis_c128(const float2* in, long long rows, int nch, int npol, double2* out, cudaStream_t st) {
  if (rows <= 0 || nch <= 0) return 0;
  if (npol != 1 && npol != 4) { fprintf(stderr, "rlf: %d correlations unsupported (1 or 4)\n", npol); return 1; }
  k_ms_vis<double2><<<tiles(rows, nch), dim3(kTile, 8), 0, st>>>(in, rows, nch, npol, nullptr, out);
  return check("k_ms_vis<double2>");
}
int launch_ms_vis_f32(const float2* in, long long rows, int nch, int npol, const int* inv, float2* out,
                      cudaStream_t st) {
  if (rows <= 0 || nch <= 0) return 0;
  if (npol != 1 && npol != 4) { fprintf(stderr, "rlf: %d correlations unsupported (1 or 4)\n", npol); return 1; }
  k_ms_vis<float2><<<tiles(rows, nch), dim3(kTile, 8), 0, st>>>(in, rows, nch, npol, inv, out);
  return check("k_ms_vis<float2>");
}
int launch_ms_flags(const uint8_t* in, long long rows, int nch, int npol, uint8_t* out, unsigned long long* count,
                    cudaStream_t st) {
  if (rows <= 0 || nch <= 0) return 0;
  if (npol != 1 && npol != 4) { fprintf(stderr, "rlf: %d correlations unsupported (1 or 4)\n", npol); return 1; }
  k_ms_flags<<<tiles(rows, nch), dim3(kTile, 8), 0, st>>>(in, rows, nch, npol, out, count);
  return check("k_ms_flags");
}
int launch_ms_write(const double2* vis, long long rows, int nch, float2* out, cudaStream_t st) {
  if (rows <= 0 || nch <= 0) return 0;
  k_ms_write<<<tiles(rows, nch), dim3(kTile, 8), 0, st>>>(vis, rows, nch, out);
  return check("k_ms_write");
}
int launch_ms_coords(const double* uvw, long long rows, double* uu, double* vv, double* ww, unsigned long long* umax,
                     cudaStream_t st) {
  if (rows <= 0) return 0;
  const int blocks = (int)std::min<long long>((rows + 255) / 256, 4096);
  k_ms_coords<<<blocks, 256, 0, st>>>(uvw, rows, uu, vv, ww, umax);
  return check("k_ms_coords");
}
int launch_ms_sigma2(const float* sigma, long long rows, long long nvis, float theory, float* sigma2, cudaStream_t st) {
  if (nvis <= 0) return 0;
  const int blocks = (int)std::min<long long>((nvis + 255) / 256, 8192);
  k_ms_sigma2<<<blocks, 256, 0, st>>>(sigma, rows, nvis, theory, sigma2);
  return check("k_ms_sigma2");
}

}  // namespace rlf

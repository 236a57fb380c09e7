// Measurement Set column blocks <-> the hot path's arrays (rlf_ms.cu).
#pragma once
#include "rlf_device.cuh"
#include <algorithm>
#include <stdint.h>

namespace rlf {

// DATA block [rows][nch][npol] complex64 (Jy) -> [nch][rows] Stokes I in uJy, complex128 / complex64
int launch_ms_vis_c128(const float2* in, long long rows, int nch, int npol, double2* out, cudaStream_t st);
// inv: position of each row in an observation stored with permuted rows, or nullptr
int launch_ms_vis_f32(const float2* in, long long rows, int nch, int npol, const int* inv, float2* out,
                      cudaStream_t st);
// FLAG block [rows][nch][npol] -> [nch][rows]; *count (zeroed by the caller) += flagged
int launch_ms_flags(const uint8_t* in, long long rows, int nch, int npol, uint8_t* out, unsigned long long* count,
                    cudaStream_t st);
// [nch][rows] complex128 uJy -> DATA block [rows][nch] complex64 Jy
int launch_ms_write(const double2* vis, long long rows, int nch, float2* out, cudaStream_t st);
// UVW [rows][3] -> uu, vv, ww; *umax (zeroed by the caller, as double bits) = max(|u|, |v|)
int launch_ms_coords(const double* uvw, long long rows, double* uu, double* vv, double* ww, unsigned long long* umax,
                     cudaStream_t st);
// SIGMA (flattened) -> sigma2 [nvis]
int launch_ms_sigma2(const float* sigma, long long rows, long long nvis, float theory, float* sigma2, cudaStream_t st);

}  // namespace rlf

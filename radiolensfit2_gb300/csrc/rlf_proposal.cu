// Learned proposal of the simplex start: a small convolutional network reads a 64 x 64 resampling of
// each galaxy's facet and proposes (e1, e2, ln r) and a step scale for the fit's nmsimplex2, whose
// start the reference fixes at (0, 0) with step 0.1 (galaxy_fitting.c:59-65).  The fit keeps the
// last word: it starts from the proposal and converges to the likelihood maximum as before.  No
// counterpart in the reference.
//
// Network (NHWC bf16 activations, FP32 accumulation):
//   input  64 x 64 x 4   (facet visibility / flux: re, im; cell mask; per-cell SNR / 10)
//   conv1  3x3 stride 2 pad 1, 4 -> 32, ReLU    32 x 32 x 32
//   conv2  3x3 stride 2 pad 1, 32 -> 32, ReLU   16 x 16 x 32
//   conv3  3x3 stride 2 pad 1, 32 -> 32, ReLU    8 x  8 x 32
//   conv4  3x3 stride 2 pad 1, 32 -> 32, ReLU    4 x  4 x 32
//   head   dense 512 -> 4 (FP32): e1, e2, ln r, ln sigma
//
// The convolutions and their gradients are GEMMs on the 5th-generation tensor cores: one kernel,
// k_conv_gemm, computes D[M x 32] = A[M x K] B[32 x K]^T with tcgen05.mma (kind::f16, bf16 operands,
// FP32 accumulator in tensor memory), the operand tiles gathered by the CTA's threads into shared
// memory in the canonical no-swizzle K-major layout, and a gather/epilogue policy per use:
//   forward   A = im2col(X)          B = W           D -> bias, ReLU, bf16 Y
//   input     A = col2im gather(dY)  B = W rearranged D -> times ReLU'(X), bf16 dX
//   weights   A = im2col(X)^T        B = dY^T         D -> FP32 atomic add into dW^T (split over positions)
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "rlf_device.cuh"
#include "rlf_proposal.cuh"
#include "../../include/rlf_gb300.h"

namespace rlf {

constexpr int kImg = 64;        // proposal input side
constexpr int kInC = 4;         // input channels
constexpr int kC = 32;          // channels of every convolution
constexpr int kLayers = 4;
constexpr int kMaxResampleFacet = 48;  // facets the resampler takes (the batched fit holds up to 34)
constexpr int kHeadIn = 4 * 4 * kC;
constexpr int kHeadOut = 4;
constexpr int kTileM = 128;     // D rows per CTA (tensor-memory lanes)
constexpr int kChunkK = 64;     // K elements staged per shared-memory buffer (4 MMAs of K = 16)
constexpr int kGemmThreads = 128;
constexpr int kABytes = kTileM * kChunkK * 2;   // 16 KB
constexpr int kBBytes = kC * kChunkK * 2;       // 4 KB
// two buffers of A and B; the allocation is padded so that every address a descriptor can form
// from these layouts stays inside the CTA's shared memory
constexpr int kGemmSmem = 2 * kABytes + 2 * kBBytes + 32 * 1024;
constexpr unsigned long long kGemmWaitNs = 1000000000ull;  // bounded wait for the tensor cores (1 s)

__host__ __device__ constexpr int layer_in_side(int l) { return kImg >> l; }
__host__ __device__ constexpr int layer_out_side(int l) { return kImg >> (l + 1); }
__host__ __device__ constexpr int layer_cin(int l) { return l == 0 ? kInC : kC; }
__host__ __device__ constexpr int layer_k(int l) { return 9 * layer_cin(l); }            // 36 or 288
__host__ __device__ constexpr int layer_kpad(int l) { return (layer_k(l) + kChunkK - 1) / kChunkK * kChunkK; }

// ------------------------------------------------------------------ tcgen05 / mbarrier primitives
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading-dimension byte offset (between the two
// core matrices of a K = 16 slice), stride byte offset (between 8-row groups), descriptor version
// 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}
// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and B bf16 (bits 7-9,
// 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kC >> 3) << 17) |
                            ((uint32_t)(kTileM >> 4) << 24);

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase of the given parity to complete, at most kGemmWaitNs; false on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const unsigned long long t0 = now_ns();
  while (!mbar_test(bar, parity)) {
    if (now_ns() - t0 > kGemmWaitNs) return false;
  }
  return true;
}
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}
// 32 lanes x 32 columns of FP32 from tensor memory: this warp's 32 rows, columns col0 .. col0 + 31
__device__ __forceinline__ void tmem_load32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row, k) of a tile with `rows` rows in the no-swizzle K-major layout: core
// matrices of 8 rows x 16 bytes, the 8-row groups of one 8-element K group adjacent (stride 128 B),
// the K groups `rows` * 16 bytes apart
__device__ __forceinline__ int tile_off(int row, int kg, int rows) { return kg * rows * 16 + (row >> 3) * 128 + (row & 7) * 16; }

__device__ __forceinline__ void put8(uint8_t* tile, int row, int kg, int rows, const float* x) {
  __nv_bfloat162 h[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(x[2 * i], x[2 * i + 1]);
  *reinterpret_cast<uint4*>(tile + tile_off(row, kg, rows)) = *reinterpret_cast<uint4*>(h);
}
__device__ __forceinline__ void put8_raw(uint8_t* tile, int row, int kg, int rows, uint4 v) {
  *reinterpret_cast<uint4*>(tile + tile_off(row, kg, rows)) = v;
}

// ------------------------------------------------------------------ gather / epilogue policies
struct ConvShape {
  int n_img;        // images in the batch
  int cin;          // input channels (4 or 32)
  int in_side;      // input side (64 .. 8)
  int out_side;     // output side
  int kpad;         // K padded to kChunkK
};

// forward: A[m][k] = X[n][2 oy - 1 + ky][2 ox - 1 + kx][ci], k = (3 ky + kx) cin + ci; B = W[co][k]
struct FwdPolicy {
  ConvShape s;
  const __nv_bfloat16* x;      // [n][in][in][cin]
  const __nv_bfloat16* w;      // [32][kpad]
  const float* bias;           // [32]
  __nv_bfloat16* y;            // [n][out][out][32]
  __host__ __device__ int rows() const { return s.n_img * s.out_side * s.out_side; }
  __host__ __device__ int k_chunks() const { return s.kpad / kChunkK; }
  __device__ void fill_a(uint8_t* tile, int m0, int k0) const {
    const int row = threadIdx.x, m = m0 + row;
    const bool live = m < rows();
    const int per = s.out_side * s.out_side;
    const int n = live ? m / per : 0, r = live ? m - n * per : 0;
    const int oy = r / s.out_side, ox = r - oy * s.out_side;
    if (s.cin % 8 == 0) {
      // 8 consecutive K of one tap are 8 consecutive channels: one 16-byte load (or zero padding)
      for (int kg = 0; kg < kChunkK / 8; ++kg) {
        const int k = k0 + kg * 8;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (live && k < 9 * s.cin) {
          const int tap = k / s.cin, ci = k - tap * s.cin;
          const int iy = 2 * oy - 1 + tap / 3, ix = 2 * ox - 1 + tap % 3;
          if (iy >= 0 && iy < s.in_side && ix >= 0 && ix < s.in_side)
            v = *reinterpret_cast<const uint4*>(x + (((size_t)n * s.in_side + iy) * s.in_side + ix) * s.cin + ci);
        }
        put8_raw(tile, row, kg, kTileM, v);
      }
      return;
    }
    for (int kg = 0; kg < kChunkK / 8; ++kg) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k = k0 + kg * 8 + i;
        float val = 0.f;
        if (live && k < 9 * s.cin) {
          const int tap = k / s.cin, ci = k - tap * s.cin;
          const int iy = 2 * oy - 1 + tap / 3, ix = 2 * ox - 1 + tap % 3;
          if (iy >= 0 && iy < s.in_side && ix >= 0 && ix < s.in_side)
            val = __bfloat162float(x[(((size_t)n * s.in_side + iy) * s.in_side + ix) * s.cin + ci]);
        }
        v[i] = val;
      }
      put8(tile, row, kg, kTileM, v);
    }
  }
  __device__ void fill_b(uint8_t* tile, int k0) const {
    // 32 rows x 8 K groups: thread t takes row t / 4, groups 2 (t % 4) and 2 (t % 4) + 1
    const int row = threadIdx.x >> 2, g0 = (threadIdx.x & 3) * 2;
    for (int g = g0; g < g0 + 2; ++g)
      put8_raw(tile, row, g, kC, *reinterpret_cast<const uint4*>(w + (size_t)row * s.kpad + k0 + g * 8));
  }
  __device__ void epilogue(int m, const float* acc) const {
    if (m >= rows()) return;
    __nv_bfloat162 h[kC / 2];
#pragma unroll
    for (int c = 0; c < kC; c += 2)
      h[c / 2] = __floats2bfloat162_rn(fmaxf(acc[c] + bias[c], 0.f), fmaxf(acc[c + 1] + bias[c + 1], 0.f));
    uint4* dst = reinterpret_cast<uint4*>(y + (size_t)m * kC);
#pragma unroll
    for (int i = 0; i < kC / 8; ++i) dst[i] = reinterpret_cast<const uint4*>(h)[i];
  }
  static constexpr bool kSplit = false;
};

// gradient of the input: dX[n][iy][ix][ci] = sum over taps (ky, kx) and co of dY[n][oy][ox][co]
// W[co][(3 ky + kx) cin + ci] with 2 oy - 1 + ky = iy, 2 ox - 1 + kx = ix; A[m][k] = dY (zero where
// the tap does not land on an output), k = (3 ky + kx) 32 + co; B[ci][k] = W[co][(3 ky + kx) cin + ci].
// The result is multiplied by ReLU'(X) = (X > 0), the gradient of the previous layer's output.
struct DgradPolicy {
  ConvShape s;             // of the forward layer (cin = 32)
  const __nv_bfloat16* dy; // [n][out][out][32]
  const __nv_bfloat16* w;  // [32][kpad] forward weights
  const __nv_bfloat16* x;  // [n][in][in][32] the forward input (post-ReLU activation)
  __nv_bfloat16* dx;       // [n][in][in][32]
  __host__ __device__ int rows() const { return s.n_img * s.in_side * s.in_side; }
  // K = 9 taps x 32 output channels = 288, staged in 5 chunks of 64 (the last half zero)
  __host__ __device__ int k_chunks() const { return (9 * kC + kChunkK - 1) / kChunkK; }
  __device__ void fill_a(uint8_t* tile, int m0, int k0) const {
    const int row = threadIdx.x, m = m0 + row;
    const bool live = m < rows();
    const int per = s.in_side * s.in_side;
    const int n = live ? m / per : 0, r = live ? m - n * per : 0;
    const int iy = r / s.in_side, ix = r - iy * s.in_side;
    for (int kg = 0; kg < kChunkK / 8; ++kg) {
      const int k = k0 + kg * 8;           // 8 consecutive output channels of one tap
      const int tap = k / kC, co = k - tap * kC;
      const int ty = iy + 1 - tap / 3, tx = ix + 1 - tap % 3;  // = 2 oy, 2 ox
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (live && tap < 9 && ty >= 0 && tx >= 0 && !(ty & 1) && !(tx & 1) && (ty >> 1) < s.out_side &&
          (tx >> 1) < s.out_side)
        v = *reinterpret_cast<const uint4*>(dy + (((size_t)n * s.out_side + (ty >> 1)) * s.out_side + (tx >> 1)) * kC + co);
      put8_raw(tile, row, kg, kTileM, v);
    }
  }
  __device__ void fill_b(uint8_t* tile, int k0) const {
    const int row = threadIdx.x >> 2, g0 = (threadIdx.x & 3) * 2;  // row = ci
    for (int g = g0; g < g0 + 2; ++g) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k = k0 + g * 8 + i;
        const int tap = k / kC, co = k - tap * kC;
        v[i] = tap < 9 ? __bfloat162float(w[(size_t)co * s.kpad + tap * s.cin + row]) : 0.f;
      }
      put8(tile, row, g, kC, v);
    }
  }
  __device__ void epilogue(int m, const float* acc) const {
    if (m >= rows()) return;
    const __nv_bfloat16* xr = x + (size_t)m * kC;
    __nv_bfloat162 h[kC / 2];
#pragma unroll
    for (int c = 0; c < kC; c += 2) {
      const float a = __bfloat162float(xr[c]) > 0.f ? acc[c] : 0.f;
      const float b = __bfloat162float(xr[c + 1]) > 0.f ? acc[c + 1] : 0.f;
      h[c / 2] = __floats2bfloat162_rn(a, b);
    }
    uint4* dst = reinterpret_cast<uint4*>(dx + (size_t)m * kC);
#pragma unroll
    for (int i = 0; i < kC / 8; ++i) dst[i] = reinterpret_cast<const uint4*>(h)[i];
  }
  static constexpr bool kSplit = false;
};

// gradient of the weights: dW^T[k][co] = sum over output positions p of X_col[p][k] dY[p][co];
// D rows = k (K of the forward, padded), the MMA's K dimension = positions p, split over CTAs and
// added into dwt with FP32 atomics
struct WgradPolicy {
  ConvShape s;
  const __nv_bfloat16* x;   // [n][in][in][cin]
  const __nv_bfloat16* dy;  // [n][out][out][32], already times ReLU'(Y)
  float* dwt;               // [kpad][32]
  __host__ __device__ int rows() const { return s.kpad; }
  __host__ __device__ int positions() const { return s.n_img * s.out_side * s.out_side; }
  __host__ __device__ int k_chunks() const { return (positions() + kChunkK - 1) / kChunkK; }
  __device__ void fill_a(uint8_t* tile, int m0, int p0) const {
    const int row = threadIdx.x, k = m0 + row;  // the forward's K index
    const bool live = k < 9 * s.cin;
    const int tap = live ? k / s.cin : 0, ci = live ? k - tap * s.cin : 0;
    const int ky = tap / 3, kx = tap % 3;
    const int per = s.out_side * s.out_side;
    for (int kg = 0; kg < kChunkK / 8; ++kg) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int p = p0 + kg * 8 + i;
        float val = 0.f;
        if (live && p < positions()) {
          const int n = p / per, r = p - n * per;
          const int oy = r / s.out_side, ox = r - oy * s.out_side;
          const int iy = 2 * oy - 1 + ky, ix = 2 * ox - 1 + kx;
          if (iy >= 0 && iy < s.in_side && ix >= 0 && ix < s.in_side)
            val = __bfloat162float(x[(((size_t)n * s.in_side + iy) * s.in_side + ix) * s.cin + ci]);
        }
        v[i] = val;
      }
      put8(tile, row, kg, kTileM, v);
    }
  }
  __device__ void fill_b(uint8_t* tile, int p0) const {
    const int row = threadIdx.x >> 2, g0 = (threadIdx.x & 3) * 2;  // row = co
    for (int g = g0; g < g0 + 2; ++g) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int p = p0 + g * 8 + i;
        v[i] = p < positions() ? __bfloat162float(dy[(size_t)p * kC + row]) : 0.f;
      }
      put8(tile, row, g, kC, v);
    }
  }
  __device__ void epilogue(int m, const float* acc) const {
    if (m >= s.kpad) return;
#pragma unroll
    for (int c = 0; c < kC; ++c) atomicAdd(&dwt[(size_t)m * kC + c], acc[c]);
  }
  static constexpr bool kSplit = true;
};

// One CTA: D rows [m0, m0 + 128) over K chunks [c0, c1).  Thread t stages row t of A and a quarter
// row of B per chunk; thread 0 issues the four MMAs of a chunk and commits them to the chunk
// buffer's mbarrier, which the threads wait on before refilling that buffer two chunks later.
// Every wait is bounded: on a time-out the CTA records it in *err, waits (bounded) for the MMAs it
// issued, frees its tensor memory and leaves without writing D.
template <class P>
__global__ void __launch_bounds__(kGemmThreads) k_conv_gemm(P pol, int chunks_per_cta, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  uint8_t* abuf = smem;
  uint8_t* bbuf = smem + 2 * kABytes;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const uint32_t tmem = tmem_slot;
  const int m0 = blockIdx.x * kTileM;
  const int total = pol.k_chunks();
  const int c0 = blockIdx.y * chunks_per_cta;
  const int c1 = min(total, c0 + chunks_per_cta);
  uint32_t issued[2] = {0u, 0u};  // commits made on each buffer's barrier
  for (int c = c0; c < c1; ++c) {
    const int b = (c - c0) & 1;
    if (issued[b] > 0 && !mbar_wait(&bars[b], (issued[b] - 1) & 1)) failed = 1;
    __syncthreads();
    if (failed) break;
    pol.fill_a(abuf + b * kABytes, m0, c * kChunkK);
    pol.fill_b(bbuf + b * kBBytes, c * kChunkK);
    fence_async_shared();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
      const uint32_t a_addr = smem_addr(abuf + b * kABytes), b_addr = smem_addr(bbuf + b * kBBytes);
#pragma unroll
      for (int j = 0; j < kChunkK / 16; ++j) {
        const uint64_t ad = umma_desc(a_addr + j * 2 * (kTileM * 16), kTileM * 16, 128);
        const uint64_t bd = umma_desc(b_addr + j * 2 * (kC * 16), kC * 16, 128);
        umma_bf16(tmem, ad, bd, (c > c0 || j > 0) ? 1u : 0u);
      }
      umma_commit(&bars[b]);
    }
    issued[b] += 1;
  }
  // the last commit of each buffer: completion of every MMA issued
  for (int b = 0; b < 2; ++b)
    if (issued[b] > 0 && !mbar_wait(&bars[b], (issued[b] - 1) & 1)) failed = 1;
  __syncthreads();
  tc_after_sync();
  if (!failed && c1 > c0) {
    float acc[kC];
    tmem_load32(tmem + ((uint32_t)(warp * 32) << 16), acc);
    pol.epilogue(m0 + warp * 32 + (tid & 31), acc);
  }
  tc_before_sync();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kC) : "memory");
  if (failed && tid == 0) atomicExch(err, 1);
}

template <class P>
static int launch_gemm(const P& pol, int* err, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_conv_gemm<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
    attr = true;
  }
  const int rows = pol.rows();
  const int total = pol.k_chunks();
  if (rows <= 0 || total <= 0) return 0;
  const int mt = (rows + kTileM - 1) / kTileM;
  int split = 1, per = total;
  if (P::kSplit) {
    // positions split so that the grid fills the GPU about twice
    split = std::max(1, std::min(total, 2 * 152 * 3 / mt));
    per = (total + split - 1) / split;
    split = (total + per - 1) / per;
  }
  k_conv_gemm<P><<<dim3(mt, split), kGemmThreads, kGemmSmem, st>>>(pol, per, err);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf: k_conv_gemm: %s\n", cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

// ------------------------------------------------------------------ resampler
// Packed facets (the fit's layout: per galaxy `count` compacted cells at `offset`, centres gu, gv,
// vis / sigma^2 (dre, dim) and sigma^2 as double or float) -> 64 x 64 x 4 bf16 images: pixel
// (py, px) takes the facet cell (py F / 64, px F / 64); channels: re and im of the cell's
// visibility divided by the galaxy's flux, 1 for a non-empty cell, and the cell's flux / sigma / 10
// capped at 1.  Cell (i, j) of a facet of F cells over [-len, len] has centre ((i + 1/2) 2 len / F
// - len) (evaluate_uv_grid.c:113-133), so a compacted cell's indices come back from its centre.
template <class T>
__global__ void k_resample(int n_gal, const int* __restrict__ offset, const int* __restrict__ count,
                           const int* __restrict__ facet, const T* __restrict__ gu, const T* __restrict__ gv,
                           const T* __restrict__ dre, const T* __restrict__ dim, const T* __restrict__ sig2,
                           const double* __restrict__ flux, int flux_stride, double len,
                           __nv_bfloat16* __restrict__ img) {
  const int g = blockIdx.x;
  if (g >= n_gal) return;
  __shared__ float cell[4][kMaxResampleFacet * kMaxResampleFacet];
  const int F = facet[g];
  const int nc = min(F * F, kMaxResampleFacet * kMaxResampleFacet);
  for (int i = threadIdx.x; i < 4 * nc; i += blockDim.x) (&cell[0][0])[(i / nc) * (kMaxResampleFacet * kMaxResampleFacet) + i % nc] = 0.f;
  __syncthreads();
  const int off = offset[g], n = count[g];
  const double inc = 2.0 * len / F;
  const float fl = (float)flux[(size_t)g * flux_stride];
  const float inv_flux = fl > 0.f ? 1.f / fl : 0.f;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const int iu = (int)floor(((double)gu[off + c] + len) / inc);
    const int iv = (int)floor(((double)gv[off + c] + len) / inc);
    if (iu < 0 || iu >= F || iv < 0 || iv >= F || F > kMaxResampleFacet) continue;
    const int k = iu * F + iv;
    const float s2 = (float)sig2[off + c];
    cell[0][k] = (float)dre[off + c] * s2 * inv_flux;
    cell[1][k] = (float)dim[off + c] * s2 * inv_flux;
    cell[2][k] = 1.f;
    cell[3][k] = s2 > 0.f ? fminf(fl * rsqrtf(s2) * 0.1f, 1.f) : 0.f;
  }
  __syncthreads();
  __nv_bfloat16* out = img + (size_t)g * kImg * kImg * kInC;
  for (int p = threadIdx.x; p < kImg * kImg; p += blockDim.x) {
    const int py = p / kImg, px = p % kImg;
    const int k = F <= kMaxResampleFacet ? (py * F / kImg) * F + (px * F / kImg) : 0;
    __nv_bfloat162 a = __floats2bfloat162_rn(cell[0][k], cell[1][k]);
    __nv_bfloat162 b = __floats2bfloat162_rn(cell[2][k], cell[3][k]);
    uint2 v;
    v.x = *reinterpret_cast<uint32_t*>(&a);
    v.y = *reinterpret_cast<uint32_t*>(&b);
    *reinterpret_cast<uint2*>(out + (size_t)p * kInC) = v;
  }
}

// ------------------------------------------------------------------ head, loss, optimiser
// out[g][j] = b[j] + sum_i W[j][i] feat[g][i], FP32; one warp per (galaxy, output)
__global__ void k_head_fwd(int n, const __nv_bfloat16* __restrict__ feat, const float* __restrict__ w,
                           const float* __restrict__ b, float* __restrict__ out) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (gw >= n * kHeadOut) return;
  const int g = gw / kHeadOut, j = gw % kHeadOut;
  float s = 0.f;
  for (int i = lane; i < kHeadIn; i += 32) s = fmaf(w[j * kHeadIn + i], __bfloat162float(feat[(size_t)g * kHeadIn + i]), s);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[(size_t)g * kHeadOut + j] = s + b[j];
}

// Gaussian negative log-likelihood of (e1, e2) with the predicted ln sigma (clamped to [-5, 0.5])
// plus the squared error of ln r, averaged over the batch: gradient with respect to the head's
// outputs (dout) and the loss terms summed into loss[0]
__global__ void k_loss(int n, const float* __restrict__ out, const float* __restrict__ target, float* __restrict__ dout,
                       float* __restrict__ loss) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const float* o = out + (size_t)g * kHeadOut;
  const float* t = target + (size_t)g * 3;
  const float ls = fminf(fmaxf(o[3], -5.f), 0.5f);
  const float iv = __expf(-2.f * ls);
  const float d1 = o[0] - t[0], d2 = o[1] - t[1], d3 = o[2] - t[2];
  const float r2 = d1 * d1 + d2 * d2;
  const float inv_n = 1.f / n;
  float* d = dout + (size_t)g * kHeadOut;
  d[0] = d1 * iv * inv_n;
  d[1] = d2 * iv * inv_n;
  d[2] = d3 * inv_n;
  d[3] = (o[3] > -5.f && o[3] < 0.5f) ? (2.f - r2 * iv) * inv_n : 0.f;
  atomicAdd(loss, (0.5f * r2 * iv + 2.f * ls + 0.5f * d3 * d3) * inv_n);
}

// head backward: dW[j][i] += dout[g][j] feat[g][i], db[j] += dout[g][j]; dfeat[g][i] = sum_j dout[g][j]
// W[j][i] times ReLU'(feat) (feat is conv4's post-ReLU output), as bf16
__global__ void k_head_bwd(int n, const __nv_bfloat16* __restrict__ feat, const float* __restrict__ w,
                           const float* __restrict__ dout, float* __restrict__ dw, float* __restrict__ db,
                           __nv_bfloat16* __restrict__ dfeat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // feature index
  if (i >= kHeadIn) return;
  float acc[kHeadOut] = {0.f, 0.f, 0.f, 0.f};
  for (int g = 0; g < n; ++g) {
    const float f = __bfloat162float(feat[(size_t)g * kHeadIn + i]);
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kHeadOut; ++j) {
      const float dj = dout[(size_t)g * kHeadOut + j];
      acc[j] = fmaf(dj, f, acc[j]);
      s = fmaf(dj, w[j * kHeadIn + i], s);
    }
    dfeat[(size_t)g * kHeadIn + i] = __float2bfloat16_rn(f > 0.f ? s : 0.f);
  }
#pragma unroll
  for (int j = 0; j < kHeadOut; ++j) dw[j * kHeadIn + i] += acc[j];
  if (i < kHeadOut) {
    float s = 0.f;
    for (int g = 0; g < n; ++g) s += dout[(size_t)g * kHeadOut + i];
    db[i] += s;
  }
}

// bias gradient of a convolution: db[c] = sum over positions of dY[p][c]
__global__ void k_bias_grad(long long positions, const __nv_bfloat16* __restrict__ dy, float* __restrict__ db) {
  __shared__ float part[kC];
  if (threadIdx.x < kC) part[threadIdx.x] = 0.f;
  __syncthreads();
  const int c = threadIdx.x & (kC - 1);
  float s = 0.f;
  for (long long p = blockIdx.x * (long long)(blockDim.x / kC) + threadIdx.x / kC; p < positions;
       p += (long long)gridDim.x * (blockDim.x / kC))
    s += __bfloat162float(dy[p * kC + c]);
  atomicAdd(&part[c], s);
  __syncthreads();
  if (threadIdx.x < kC) atomicAdd(&db[threadIdx.x], part[threadIdx.x]);
}

// Adam (Kingma & Ba 2015) on FP32 parameters, bias-corrected step sizes given by the host
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr_t, float b1, float b2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

// FP32 conv weights [32][k] (dense, k = 9 cin) -> bf16 [32][kpad] zero-padded; and dW^T [kpad][32] ->
// dW [32][k] (FP32)
__global__ void k_pack_w(const float* __restrict__ w, int k, int kpad, __nv_bfloat16* __restrict__ wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kC * kpad) return;
  const int co = i / kpad, kk = i - co * kpad;
  wb[i] = __float2bfloat16_rn(kk < k ? w[co * k + kk] : 0.f);
}
__global__ void k_unpack_dw(const float* __restrict__ dwt, int k, float* __restrict__ dw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kC * k) return;
  const int co = i / k, kk = i - co * k;
  dw[i] = dwt[(size_t)kk * kC + co];
}

// proposal (e1, e2, step) for the fit from the head's outputs: e clamped to |e| <= 0.7 (the fit's
// objective is finite for |e|^2 < 0.65, likelihood.c:87-100), step 2 sigma in [0.02, 0.1].  A galaxy
// whose predicted sigma exceeds max_sigma keeps the reference's start (0, 0) with step 0.1: for
// the unresolved, noise-dominated galaxies the proposal carries no information beyond the prior,
// and a different start only moves the end of the simplex on a flat likelihood.
constexpr float kPropMaxSigma = 0.05f;  // default gate (rlf_proposal_set_max_sigma)
__global__ void k_to_start(int n, const float* __restrict__ out, float max_sigma, double* __restrict__ start) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const float* o = out + (size_t)g * kHeadOut;
  float e1 = o[0], e2 = o[1];
  const float em = sqrtf(e1 * e1 + e2 * e2);
  if (!(em <= 0.7f)) {
    const float s = em > 0.f && isfinite(em) ? 0.7f / em : 0.f;
    e1 *= s;
    e2 *= s;
  }
  const float sig = __expf(fminf(fmaxf(o[3], -5.f), 0.5f));
  const bool use = sig <= max_sigma && isfinite(e1) && isfinite(e2);
  start[3 * g + 0] = use ? (double)e1 : 0.0;
  start[3 * g + 1] = use ? (double)e2 : 0.0;
  start[3 * g + 2] = use ? (double)fminf(fmaxf(2.f * sig, 0.02f), 0.1f) : 0.1;
}

// ------------------------------------------------------------------ host side
#define RLF_P_CUDA(call)                                                                     \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      fprintf(stderr, "rlf proposal: %s: %s\n", #call, cudaGetErrorString(e_));              \
      return (int)e_;                                                                        \
    }                                                                                        \
  } while (0)
#define RLF_P_OK(call)          \
  do {                          \
    int r_ = (call);            \
    if (r_) return r_;          \
  } while (0)

static int check_p(const char* what) {
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf proposal: %s: %s\n", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

// parameter layout (FP32): per layer W [32][9 cin] (k = (3 ky + kx) cin + ci) then b [32]; head
// W [4][512] (feature (4 y + x) 32 + c) then b [4]
static int w_off(int l) {
  int o = 0;
  for (int i = 0; i < l; ++i) o += kC * layer_k(i) + kC;
  return o;
}
static int b_off(int l) { return w_off(l) + kC * layer_k(l); }
static int head_w_off() { return w_off(kLayers); }
static int head_b_off() { return head_w_off() + kHeadOut * kHeadIn; }
int cnn_param_count() { return head_b_off() + kHeadOut; }

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  int ensure(size_t count) {
    if (count <= n) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    RLF_P_CUDA(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    n = count;
    return 0;
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

struct Cnn {
  int max_batch = 0;
  int capacity = 0;
  float max_sigma = kPropMaxSigma;  // proposals with a larger predicted sigma keep the reference start
  cudaStream_t st = nullptr;
  int step = 0;
  DBuf<float> params, grads, m, v, loss, out, dout, targets, dwt;
  DBuf<__nv_bfloat16> wb[kLayers];
  DBuf<__nv_bfloat16> act[kLayers + 1];   // X0 (input batch) .. X4
  DBuf<__nv_bfloat16> dact[kLayers + 1];  // gradients of X1 .. X4 (masked: pre-activation gradients)
  DBuf<__nv_bfloat16> store;              // image store [capacity][64][64][4]
  DBuf<float> store_targets;              // [capacity][3]
  DBuf<int> err, idx;
  DBuf<double> fac[5];
  DBuf<int> foff, fcount, ffacet;
  DBuf<double> fflux;

  int init(int batch, int cap) {
    max_batch = batch;
    capacity = cap;
    RLF_P_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int np = cnn_param_count();
    RLF_P_OK(params.ensure(np));
    RLF_P_OK(grads.ensure(np));
    RLF_P_OK(m.ensure(np));
    RLF_P_OK(v.ensure(np));
    RLF_P_CUDA(cudaMemsetAsync(params.p, 0, np * sizeof(float), st));
    RLF_P_CUDA(cudaMemsetAsync(m.p, 0, np * sizeof(float), st));
    RLF_P_CUDA(cudaMemsetAsync(v.p, 0, np * sizeof(float), st));
    RLF_P_OK(loss.ensure(1));
    RLF_P_OK(out.ensure((size_t)batch * kHeadOut));
    RLF_P_OK(dout.ensure((size_t)batch * kHeadOut));
    RLF_P_OK(targets.ensure((size_t)batch * 3));
    RLF_P_OK(dwt.ensure((size_t)layer_kpad(1) * kC));
    RLF_P_OK(err.ensure(1));
    RLF_P_OK(idx.ensure(batch));
    for (int l = 0; l < kLayers; ++l) RLF_P_OK(wb[l].ensure((size_t)kC * layer_kpad(l)));
    RLF_P_OK(act[0].ensure((size_t)batch * kImg * kImg * kInC));
    for (int l = 1; l <= kLayers; ++l) {
      const int side = layer_in_side(l);
      RLF_P_OK(act[l].ensure((size_t)batch * side * side * kC));
      RLF_P_OK(dact[l].ensure((size_t)batch * side * side * kC));
    }
    if (cap > 0) {
      RLF_P_OK(store.ensure((size_t)cap * kImg * kImg * kInC));
      RLF_P_OK(store_targets.ensure((size_t)cap * 3));
    }
    RLF_P_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
    return pack();
  }
  ~Cnn() {
    if (st) cudaStreamDestroy(st);
  }
  ConvShape shape(int l, int n) const {
    ConvShape s;
    s.n_img = n;
    s.cin = layer_cin(l);
    s.in_side = layer_in_side(l);
    s.out_side = layer_out_side(l);
    s.kpad = layer_kpad(l);
    return s;
  }
  int pack() {
    for (int l = 0; l < kLayers; ++l) {
      const int tot = kC * layer_kpad(l);
      k_pack_w<<<(tot + 255) / 256, 256, 0, st>>>(params.p + w_off(l), layer_k(l), layer_kpad(l), wb[l].p);
      RLF_P_OK(check_p("k_pack_w"));
    }
    return 0;
  }
  // forward of act[0][0 .. n) into out[n][4]
  int forward(int n) {
    for (int l = 0; l < kLayers; ++l) {
      FwdPolicy f;
      f.s = shape(l, n);
      f.x = act[l].p;
      f.w = wb[l].p;
      f.bias = params.p + b_off(l);
      f.y = act[l + 1].p;
      RLF_P_OK(launch_gemm(f, err.p, st));
    }
    const int warps = n * kHeadOut;
    k_head_fwd<<<(warps * 32 + 255) / 256, 256, 0, st>>>(n, act[kLayers].p, params.p + head_w_off(),
                                                          params.p + head_b_off(), out.p);
    return check_p("k_head_fwd");
  }
  // loss and gradients of the batch in act[0] with targets[n][3]; grads overwritten
  int backward(int n) {
    RLF_P_CUDA(cudaMemsetAsync(grads.p, 0, cnn_param_count() * sizeof(float), st));
    RLF_P_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(float), st));
    k_loss<<<(n + 127) / 128, 128, 0, st>>>(n, out.p, targets.p, dout.p, loss.p);
    RLF_P_OK(check_p("k_loss"));
    k_head_bwd<<<(kHeadIn + 127) / 128, 128, 0, st>>>(n, act[kLayers].p, params.p + head_w_off(), dout.p,
                                                       grads.p + head_w_off(), grads.p + head_b_off(), dact[kLayers].p);
    RLF_P_OK(check_p("k_head_bwd"));
    for (int l = kLayers - 1; l >= 0; --l) {
      const ConvShape s = shape(l, n);
      const long long positions = (long long)n * s.out_side * s.out_side;
      k_bias_grad<<<std::min<long long>(1024, (positions + 7) / 8), 256, 0, st>>>(positions, dact[l + 1].p,
                                                                                  grads.p + b_off(l));
      RLF_P_OK(check_p("k_bias_grad"));
      RLF_P_CUDA(cudaMemsetAsync(dwt.p, 0, (size_t)s.kpad * kC * sizeof(float), st));
      WgradPolicy wg;
      wg.s = s;
      wg.x = act[l].p;
      wg.dy = dact[l + 1].p;
      wg.dwt = dwt.p;
      RLF_P_OK(launch_gemm(wg, err.p, st));
      const int tot = kC * layer_k(l);
      k_unpack_dw<<<(tot + 255) / 256, 256, 0, st>>>(dwt.p, layer_k(l), grads.p + w_off(l));
      RLF_P_OK(check_p("k_unpack_dw"));
      if (l > 0) {
        DgradPolicy dg;
        dg.s = s;
        dg.dy = dact[l + 1].p;
        dg.w = wb[l].p;
        dg.x = act[l].p;
        dg.dx = dact[l].p;
        RLF_P_OK(launch_gemm(dg, err.p, st));
      }
    }
    return 0;
  }
  int adam(float lr) {
    ++step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float lr_t = lr * sqrtf(1.f - powf(b2, (float)step)) / (1.f - powf(b1, (float)step));
    const int np = cnn_param_count();
    k_adam<<<(np + 255) / 256, 256, 0, st>>>(np, params.p, grads.p, m.p, v.p, lr_t, b1, b2, 1e-8f);
    RLF_P_OK(check_p("k_adam"));
    return pack();
  }
  int status() {
    int e = 0;
    RLF_P_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    RLF_P_CUDA(cudaStreamSynchronize(st));
    if (e) fprintf(stderr, "rlf proposal: a tensor-core GEMM did not complete within its wait limit\n");
    return e ? 1 : 0;
  }
};

__global__ void k_gather_images(int n, const int* __restrict__ idx, const __nv_bfloat16* __restrict__ store,
                                 const float* __restrict__ store_t, __nv_bfloat16* __restrict__ x, float* __restrict__ t) {
  const size_t per = (size_t)kImg * kImg * kInC / 8;  // uint4 per image
  const int g = blockIdx.x;
  if (g >= n) return;
  const uint4* src = reinterpret_cast<const uint4*>(store) + (size_t)idx[g] * per;
  uint4* dst = reinterpret_cast<uint4*>(x) + (size_t)g * per;
  for (size_t i = threadIdx.x; i < per; i += blockDim.x) dst[i] = src[i];
  if (threadIdx.x < 3) t[(size_t)g * 3 + threadIdx.x] = store_t[(size_t)idx[g] * 3 + threadIdx.x];
}

// proposals for the fit: resample the packed facets of n galaxies and run the network (in chunks
// of the network's batch), writing (e1, e2, step) to start[3 * i]
template <class T>
static int propose_t(Cnn& c, int n, const int* offset, const int* count, const int* facet, const void* gu,
                     const void* gv, const void* dre, const void* dim, const void* sig2, const double* flux,
                     int flux_stride, double len, double* start, cudaStream_t st) {
  cudaEvent_t ev;
  RLF_P_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  RLF_P_CUDA(cudaEventRecord(ev, st));
  RLF_P_CUDA(cudaStreamWaitEvent(c.st, ev, 0));
  for (int i0 = 0; i0 < n; i0 += c.max_batch) {
    const int k = std::min(c.max_batch, n - i0);
    k_resample<T><<<k, 256, 0, c.st>>>(k, offset + i0, count + i0, facet + i0, (const T*)gu, (const T*)gv,
                                        (const T*)dre, (const T*)dim, (const T*)sig2, flux + (size_t)i0 * flux_stride,
                                        flux_stride, len, c.act[0].p);
    RLF_P_OK(check_p("k_resample"));
    RLF_P_OK(c.forward(k));
    k_to_start<<<(k + 127) / 128, 128, 0, c.st>>>(k, c.out.p, c.max_sigma, start + 3 * (size_t)i0);
    RLF_P_OK(check_p("k_to_start"));
  }
  RLF_P_CUDA(cudaEventRecord(ev, c.st));
  RLF_P_CUDA(cudaStreamWaitEvent(st, ev, 0));
  RLF_P_CUDA(cudaEventDestroy(ev));
  return 0;
}

static std::mutex g_prop_mu;
static Cnn* g_prop = nullptr;

int proposal_ready() { return g_prop != nullptr; }

int propose_starts(int n, const int* offset, const int* count, const int* facet, const void* gu, const void* gv,
                   const void* dre, const void* dim, const void* sig2, int as_float, const double* flux,
                   int flux_stride, double len, double* start, cudaStream_t st) {
  std::lock_guard<std::mutex> lock(g_prop_mu);
  if (!g_prop) return 1;
  if (as_float)
    return propose_t<float>(*g_prop, n, offset, count, facet, gu, gv, dre, dim, sig2, flux, flux_stride, len, start, st);
  return propose_t<double>(*g_prop, n, offset, count, facet, gu, gv, dre, dim, sig2, flux, flux_stride, len, start, st);
}

}  // namespace rlf

using rlf::Cnn;

struct rlf_cnn {
  Cnn c;
};

extern "C" {

int rlf_cnn_param_count(void) { return rlf::cnn_param_count(); }

rlf_cnn* rlf_cnn_create(int max_batch, int capacity) {
  if (max_batch < 1 || max_batch > 4096 || capacity < 0) {
    fprintf(stderr, "rlf_cnn_create: batch %d (1..4096), capacity %d\n", max_batch, capacity);
    return nullptr;
  }
  rlf_cnn* h = new rlf_cnn();
  if (h->c.init(max_batch, capacity)) {
    delete h;
    return nullptr;
  }
  return h;
}

void rlf_cnn_destroy(rlf_cnn* h) { delete h; }

int rlf_cnn_set_params(rlf_cnn* h, const float* params) {
  if (!h || !params) return 1;
  RLF_P_CUDA(cudaMemcpyAsync(h->c.params.p, params, rlf::cnn_param_count() * sizeof(float), cudaMemcpyHostToDevice,
                             h->c.st));
  RLF_P_OK(h->c.pack());
  RLF_P_CUDA(cudaStreamSynchronize(h->c.st));
  return 0;
}

int rlf_cnn_get_params(rlf_cnn* h, float* params) {
  if (!h || !params) return 1;
  RLF_P_CUDA(cudaMemcpyAsync(params, h->c.params.p, rlf::cnn_param_count() * sizeof(float), cudaMemcpyDeviceToHost,
                             h->c.st));
  RLF_P_CUDA(cudaStreamSynchronize(h->c.st));
  return 0;
}

int rlf_cnn_store_facets(rlf_cnn* h, int first, int n, const double* facets, int stride, const int* ncoords,
                         const int* facet, const double* flux, double len) {
  if (!h || n < 0 || first < 0 || first + n > h->c.capacity) return 1;
  if (n == 0) return 0;
  Cnn& c = h->c;
  for (int a = 0; a < 5; ++a) RLF_P_OK(c.fac[a].ensure((size_t)n * stride));
  RLF_P_OK(c.foff.ensure(n));
  RLF_P_OK(c.fcount.ensure(n));
  RLF_P_OK(c.ffacet.ensure(n));
  RLF_P_OK(c.fflux.ensure(n));
  std::vector<double> plane((size_t)n * stride);
  for (int a = 0; a < 5; ++a) {
    for (int g = 0; g < n; ++g)
      std::copy(facets + ((size_t)g * 5 + a) * stride, facets + ((size_t)g * 5 + a + 1) * stride,
                plane.begin() + (size_t)g * stride);
    RLF_P_CUDA(cudaMemcpyAsync(c.fac[a].p, plane.data(), plane.size() * sizeof(double), cudaMemcpyHostToDevice, c.st));
    RLF_P_CUDA(cudaStreamSynchronize(c.st));
  }
  std::vector<int> off(n);
  for (int g = 0; g < n; ++g) off[g] = g * stride;
  RLF_P_CUDA(cudaMemcpyAsync(c.foff.p, off.data(), n * sizeof(int), cudaMemcpyHostToDevice, c.st));
  RLF_P_CUDA(cudaMemcpyAsync(c.fcount.p, ncoords, n * sizeof(int), cudaMemcpyHostToDevice, c.st));
  RLF_P_CUDA(cudaMemcpyAsync(c.ffacet.p, facet, n * sizeof(int), cudaMemcpyHostToDevice, c.st));
  RLF_P_CUDA(cudaMemcpyAsync(c.fflux.p, flux, n * sizeof(double), cudaMemcpyHostToDevice, c.st));
  rlf::k_resample<double><<<n, 256, 0, c.st>>>(n, c.foff.p, c.fcount.p, c.ffacet.p, c.fac[0].p, c.fac[1].p, c.fac[2].p,
                                              c.fac[3].p, c.fac[4].p, c.fflux.p, 1, len,
                                              c.store.p + (size_t)first * rlf::kImg * rlf::kImg * rlf::kInC);
  RLF_P_OK(rlf::check_p("k_resample"));
  RLF_P_CUDA(cudaStreamSynchronize(c.st));
  return 0;
}

int rlf_cnn_set_targets(rlf_cnn* h, int first, int n, const float* targets) {
  if (!h || n < 0 || first < 0 || first + n > h->c.capacity) return 1;
  RLF_P_CUDA(cudaMemcpyAsync(h->c.store_targets.p + (size_t)first * 3, targets, (size_t)n * 3 * sizeof(float),
                             cudaMemcpyHostToDevice, h->c.st));
  RLF_P_CUDA(cudaStreamSynchronize(h->c.st));
  return 0;
}

int rlf_cnn_set_images(rlf_cnn* h, int first, int n, const uint16_t* images) {
  if (!h || n < 0 || first < 0 || first + n > h->c.capacity || (n && !images)) return 1;
  const size_t per = (size_t)rlf::kImg * rlf::kImg * rlf::kInC;
  RLF_P_CUDA(cudaMemcpyAsync(h->c.store.p + (size_t)first * per, images, (size_t)n * per * 2, cudaMemcpyHostToDevice,
                             h->c.st));
  RLF_P_CUDA(cudaStreamSynchronize(h->c.st));
  return 0;
}

int rlf_cnn_read_images(rlf_cnn* h, int first, int n, uint16_t* out) {
  if (!h || n < 0 || first < 0 || first + n > h->c.capacity) return 1;
  const size_t per = (size_t)rlf::kImg * rlf::kImg * rlf::kInC;
  RLF_P_CUDA(cudaMemcpyAsync(out, h->c.store.p + (size_t)first * per, (size_t)n * per * 2, cudaMemcpyDeviceToHost,
                             h->c.st));
  RLF_P_CUDA(cudaStreamSynchronize(h->c.st));
  return 0;
}

// stages the batch idx[0 .. n) of the store into the network's input
static int stage_batch(Cnn& c, const int* idx, int n) {
  for (int i = 0; i < n; ++i)
    if (idx[i] < 0 || idx[i] >= c.capacity) return 1;
  RLF_P_CUDA(cudaMemcpyAsync(c.idx.p, idx, n * sizeof(int), cudaMemcpyHostToDevice, c.st));
  rlf::k_gather_images<<<n, 256, 0, c.st>>>(n, c.idx.p, c.store.p, c.store_targets.p, c.act[0].p, c.targets.p);
  return rlf::check_p("k_gather_images");
}

int rlf_cnn_grads(rlf_cnn* h, const int* idx, int n, float* grads, float* loss, float* out) {
  if (!h || n < 1 || n > h->c.max_batch) return 1;
  Cnn& c = h->c;
  RLF_P_OK(stage_batch(c, idx, n));
  RLF_P_OK(c.forward(n));
  RLF_P_OK(c.backward(n));
  if (grads)
    RLF_P_CUDA(cudaMemcpyAsync(grads, c.grads.p, rlf::cnn_param_count() * sizeof(float), cudaMemcpyDeviceToHost, c.st));
  if (loss) RLF_P_CUDA(cudaMemcpyAsync(loss, c.loss.p, sizeof(float), cudaMemcpyDeviceToHost, c.st));
  if (out) RLF_P_CUDA(cudaMemcpyAsync(out, c.out.p, (size_t)n * rlf::kHeadOut * sizeof(float), cudaMemcpyDeviceToHost, c.st));
  RLF_P_CUDA(cudaStreamSynchronize(c.st));
  return c.status();
}

int rlf_cnn_train_step(rlf_cnn* h, const int* idx, int n, float lr, float* loss) {
  if (!h || n < 1 || n > h->c.max_batch) return 1;
  Cnn& c = h->c;
  RLF_P_OK(stage_batch(c, idx, n));
  RLF_P_OK(c.forward(n));
  RLF_P_OK(c.backward(n));
  RLF_P_OK(c.adam(lr));
  if (loss) {
    RLF_P_CUDA(cudaMemcpyAsync(loss, c.loss.p, sizeof(float), cudaMemcpyDeviceToHost, c.st));
    RLF_P_CUDA(cudaStreamSynchronize(c.st));
    return c.status();
  }
  return 0;
}

int rlf_cnn_predict(rlf_cnn* h, int first, int n, float* out) {
  if (!h || n < 0 || first < 0 || first + n > h->c.capacity) return 1;
  Cnn& c = h->c;
  std::vector<int> idx(c.max_batch);
  for (int i0 = 0; i0 < n; i0 += c.max_batch) {
    const int k = std::min(c.max_batch, n - i0);
    for (int i = 0; i < k; ++i) idx[i] = first + i0 + i;
    RLF_P_OK(stage_batch(c, idx.data(), k));
    RLF_P_OK(c.forward(k));
    RLF_P_CUDA(cudaMemcpyAsync(out + (size_t)i0 * rlf::kHeadOut, c.out.p, (size_t)k * rlf::kHeadOut * sizeof(float),
                               cudaMemcpyDeviceToHost, c.st));
    RLF_P_CUDA(cudaStreamSynchronize(c.st));
  }
  return c.status();
}

int rlf_proposal_set_max_sigma(float max_sigma) {
  std::lock_guard<std::mutex> lock(rlf::g_prop_mu);
  if (!rlf::g_prop || !(max_sigma > 0.f)) return 1;
  rlf::g_prop->max_sigma = max_sigma;
  return 0;
}

int rlf_proposal_set_params(const float* params) {
  std::lock_guard<std::mutex> lock(rlf::g_prop_mu);
  if (!params) {
    delete rlf::g_prop;
    rlf::g_prop = nullptr;
    return 0;
  }
  if (!rlf::g_prop) {
    rlf::g_prop = new rlf::Cnn();
    if (rlf::g_prop->init(512, 0)) {
      delete rlf::g_prop;
      rlf::g_prop = nullptr;
      return 1;
    }
  }
  RLF_P_CUDA(cudaMemcpyAsync(rlf::g_prop->params.p, params, rlf::cnn_param_count() * sizeof(float),
                             cudaMemcpyHostToDevice, rlf::g_prop->st));
  RLF_P_OK(rlf::g_prop->pack());
  RLF_P_CUDA(cudaStreamSynchronize(rlf::g_prop->st));
  return 0;
}

}  // extern "C"

// gridding_visibilities without any device allocation.
//
// Some callers cannot allocate device memory: code running under a framework that owns the
// whole device heap (a caching allocator or a fixed memory pool), and real-time or embedded
// callers that forbid allocation after start-up.  rlf_gridding_visibilities_noalloc serves them:
// the caller passes device pointers to its inputs and outputs, and the per-block partial sums
// the gridding kernel needs live in a fixed array of this library's own device memory,
// g_noalloc_scratch below, instead of a cudaMalloc'd buffer.
//
// The scratch array holds kNoAllocParts partial facets of 4 sums (re, im, sigma^2, weight) of
// up to kNoAllocMaxFacet^2 cells, plus the reduced sums: (64 * 4 + 4) * 48^2 doubles, 4.6 MiB.
// Every GPU on which the library is loaded holds this memory until the process exits.
//
// Shared state: besides the scratch array, a call writes two things every other entry point of
// this library uses too: the __constant__ channel table (set_channels, through a static host
// staging array) and the gridding kernel's dynamic shared-memory attribute.  A call that overlaps
// ANY other call of this library on the GPU or on another host thread (data_processing,
// source_extraction, gridding_visibilities, ...) can change that call's wavenumbers, so callers
// serialise all calls into the library, not only the no-allocation ones.  The call synchronises
// the caller's stream (inside set_channels and at its end), so it cannot be captured into a CUDA
// graph.
#include <mutex>
#include <stdio.h>
#include "rlf_vis.cuh"
#include "../../include/rlf_gb300.h"

namespace rlf {

constexpr unsigned kNoAllocMaxFacet = RLF_NOALLOC_MAX_FACET;  // cells per facet side
constexpr int kNoAllocParts = 64;                             // partial facets (grid blocks)
constexpr size_t kNoAllocScratch = (size_t)(kNoAllocParts * 4 + 4) * kNoAllocMaxFacet * kNoAllocMaxFacet;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratch];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[kNoAllocMaxDevices];

// Device address of g_noalloc_scratch on the current device.  In host code the symbol itself is
// a host-side stand-in, so the address is looked up once per device (first call on that device)
// and cached for the life of the process.  The cache is not valid across cudaDeviceReset (the
// module is loaded again in the new context): a caller that resets a device does not call this
// entry point on it afterwards.
static int noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: cudaGetDevice: %s\n", cudaGetErrorString(e));
    return (int)e;
  }
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: device %d beyond %d\n", dev, kNoAllocMaxDevices);
    return 1;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "rlf_gridding_visibilities_noalloc: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
      return e != cudaSuccess ? (int)e : 1;
    }
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return 0;
}

}  // namespace rlf

extern "C" int rlf_gridding_visibilities_noalloc(const double* wavenumbers, unsigned int num_channels,
                                                 unsigned int ncoords, const double* u, const double* v,
                                                 const double* vis, const float* sigma2, const uint8_t* flag,
                                                 double len, unsigned int sizeg, double* new_vis,
                                                 double* new_sigma2, double* sum_w, void* stream) {
  using namespace rlf;
  if (sizeg == 0 || sizeg > kNoAllocMaxFacet) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: facet size %u outside 1..%u\n", sizeg, kNoAllocMaxFacet);
    return 1;
  }
  if (num_channels == 0 || num_channels > (unsigned)kMaxCh) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: %u channels outside 1..%d\n", num_channels, kMaxCh);
    return 1;
  }
  if (ncoords == 0 || !wavenumbers || !u || !v || !vis || !sigma2 || !new_vis || !new_sigma2 || !sum_w) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: empty observation or null pointer\n");
    return 1;
  }
  double* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = set_channels((int)num_channels, wavenumbers, nullptr, st);
  if (rc) return rc;
  Observation o;
  o.n_rows = (int)ncoords;
  o.n_ch = (int)num_channels;
  o.lay.s_row = 1;
  o.lay.s_ch = ncoords;
  o.uu = u;
  o.vv = v;
  o.ww = v;  // gridding reads u and v only
  o.len = len;
  int n_part = grid_partial_blocks((int)ncoords);
  if (n_part > kNoAllocParts) n_part = kNoAllocParts;
  // every block overwrites its whole partial facet and the reduction overwrites the sums, so the
  // previous call's contents need no clearing
  rc = launch_grid_vis_f64(o, reinterpret_cast<const double2*>(vis), sigma2, flag, sizeg, scratch, n_part, st);
  if (rc) return rc;
  rc = launch_grid_vis_finalize(scratch, n_part, sizeg, reinterpret_cast<double2*>(new_vis), new_sigma2, sum_w, st);
  if (rc) return rc;
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf_gridding_visibilities_noalloc: %s\n", cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

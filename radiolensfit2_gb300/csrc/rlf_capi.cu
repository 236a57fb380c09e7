// Host runtime of the GB300 shape-measurement library: the reference-named C entry points
// (host buffers in, host buffers out), the device-resident observation, and the per-galaxy
// pipeline that replaces the loop of data_processing.c:61-138.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <execinfo.h>
#include <signal.h>
#include <unistd.h>

#include <algorithm>
#include <map>
#include <vector>

#include "rlf_device.cuh"
#include "rlf_fit.cuh"
#include "rlf_vis.cuh"
#include "rlf_batch.cuh"
#include "rlf_ms.cuh"
#include "rlf_proposal.cuh"
#include "../../include/rlf_gb300.h"
#include "../../include/rlf_testing.h"

typedef struct {
  double real;
  double imag;
} complexd;

// datatype.h:49-74, FACET branch
typedef struct {
  int numr;
  double* ro;
  double* rprior;
  unsigned int nchannels;
  double band_factor;
  double acc_time;
  double* spec;
  double* wavenumbers;
  double* uu;
  double* vv;
  double l0;
  double m0;
  complexd* data;
  double* sigma2;
  double* mod;
  unsigned int facet;
  unsigned int ncoords;
} likelihood_params;

struct rlf_gsl_vector_layout {
  size_t size;
  size_t stride;
  double* data;
  void* block;
  int owner;
};

namespace rlf {

#define RLF_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      fprintf(stderr, "rlf: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_),      \
              __FILE__, __LINE__);                                                       \
      return (int)e_;                                                                    \
    }                                                                                    \
  } while (0)
#define RLF_OK(call)              \
  do {                            \
    int r_ = (call);              \
    if (r_) return r_;            \
  } while (0)

// host <-> device bytes moved by this library (rlf_transfer_bytes); every copy goes through here
static unsigned long long g_h2d_bytes = 0, g_d2h_bytes = 0;
static cudaError_t copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
  if (kind == cudaMemcpyHostToDevice) __atomic_add_fetch(&g_h2d_bytes, (unsigned long long)bytes, __ATOMIC_RELAXED);
  if (kind == cudaMemcpyDeviceToHost) __atomic_add_fetch(&g_d2h_bytes, (unsigned long long)bytes, __ATOMIC_RELAXED);
  return cudaMemcpyAsync(dst, src, bytes, kind, st);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { if (p) cudaFree(p); }
  int ensure(size_t count) {
    if (count <= n && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      fprintf(stderr, "rlf: cudaMalloc(%zu bytes): %s\n", count * sizeof(T), cudaGetErrorString(e));
      p = nullptr;
      return (int)e;
    }
    n = count;
    return 0;
  }
  int upload(const T* h, size_t count, cudaStream_t st) {
    RLF_OK(ensure(count));
    if (count) RLF_CUDA(copy_async(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
    return 0;
  }
  int download(T* h, size_t count, cudaStream_t st) const {
    if (count) RLF_CUDA(copy_async(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, st));
    return 0;
  }
};

struct Lib {
  cudaStream_t st = nullptr;
  rlf_options opt{RLF_F64, 1, 0, 1, 0, nullptr, RLF_F64, 0, 0, 0, 0, 0, 0, 0};
  // scratch for the per-function entry points
  DevBuf<double> d0, d1, d2, d3, d4, d5, d6, d7;
  DevBuf<double2> c0, c1;
  DevBuf<float> f0;
  DevBuf<uint8_t> b0;
  DevBuf<uint16_t> u16;
  DevBuf<unsigned> ucount;
  DevBuf<int> i0;
  DevBuf<FitOut> fo;
  int init() {
    if (st) return 0;
    RLF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    return 0;
  }
};
static Lib g_lib;

static int lib_stream(cudaStream_t* st) {
  RLF_OK(g_lib.init());
  *st = g_lib.st;
  return 0;
}

// ---------------------------------------------------------------- observation
struct FacetCache {
  DevBuf<uint16_t> cell;
  DevBuf<double> ss, sw;
  DevBuf<uint32_t> desc;   // run descriptors of the sequential batch extraction (built on first use)
  DevBuf<uint16_t> desc1;  // second-run cells of the two-run chunks
};

struct Timing {
  cudaEvent_t ev[8];
  bool made = false;
  double ms[4] = {0, 0, 0, 0};
};

}  // namespace rlf

struct rlf_observation {
  int n_rows = 0, n_ch = 0;
  long long n_vis = 0;
  int precision = RLF_F64;
  double len = 0;
  std::vector<double> wavenumbers, spec;
  rlf::DevBuf<double> uu, vv, ww;
  rlf::DevBuf<float> sigma2;
  rlf::DevBuf<uint8_t> flag;
  rlf::DevBuf<double2> data64, sky64, data64_0, sky64_0;
  rlf::DevBuf<float2> data32, sky32, data32_0, sky32_0;
  std::map<unsigned, rlf::FacetCache*> facets;
  rlf::DevBuf<double> partial;
  rlf::DevBuf<rlf::RowF> rows;      // FP32 row table of the batched kernels (built on first use)
  rlf::DevBuf<double2> bpartial;    // partial facets of the batched extraction
  // mixed-precision observations store their rows in uv order (launch_row_order), so that the
  // batched extraction's consecutive work items are neighbours in uv and in memory: perm[p] is the
  // caller's row at position p, inv its inverse; empty for FP64 observations (caller's order)
  rlf::DevBuf<int> perm, inv;
  rlf::DevBuf<int> items;           // work items of the sequential batch extraction
  rlf::DevBuf<int> items2;          // its two-run work items
  rlf::DevBuf<int> item_count;      // [6] simple / general / two-run work items, then the extraction's work counters
  double max_delay_m = 0;
  int n_part = 0;
  double ms[4] = {0, 0, 0, 0};
  // streaming passes over the visibilities in the last process() call (RLF_STAT_*)
  long long stats[RLF_NSTATS] = {};
  ~rlf_observation() {
    for (auto& kv : facets) delete kv.second;
  }
  rlf::Observation view() const {
    rlf::Observation o;
    o.n_rows = n_rows;
    o.n_ch = n_ch;
    o.lay.s_row = 1;
    o.lay.s_ch = n_rows;
    o.uu = uu.p;
    o.vv = vv.p;
    o.ww = ww.p;
    o.len = len;
    return o;
  }
};

namespace rlf {

static int obs_facet(rlf_observation* ob, unsigned F, FacetCache** out, cudaStream_t st) {
  auto it = ob->facets.find(F);
  if (it != ob->facets.end()) { *out = it->second; return 0; }
  if (F == 0 || F > kMaxExtractFacet) {
    fprintf(stderr, "rlf: facet size %u outside 1..%u\n", F, kMaxExtractFacet);
    return 1;
  }
  FacetCache* fc = new FacetCache();
  const Observation o = ob->view();
  int r = fc->cell.ensure((size_t)ob->n_vis);
  if (!r) r = launch_cell_index(o, ob->flag.p, F, fc->cell.p, st);
  if (!r) r = fc->ss.ensure((size_t)F * F);
  if (!r) r = fc->sw.ensure((size_t)F * F);
  if (!r) r = ob->partial.ensure((size_t)ob->n_part * 4 * F * F + 4 * F * F);
  if (!r) r = launch_grid_weights(o, fc->cell.p, ob->sigma2.p, F, ob->partial.p, ob->n_part, fc->ss.p, fc->sw.p, st);
  if (r) { delete fc; return r; }
  ob->facets[F] = fc;
  *out = fc;
  return 0;
}

// Philox4x32-10 counter-based generator (Salmon et al., SC'11) for the simulator's noise.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// Gaussian noise keyed by the visibility's index in the caller's order (perm: the caller's row of
// each stored row of a permuted observation, or nullptr)
template <class C>
__global__ void k_add_noise(long long n, C* vis, double sigma, uint64_t seed, const int* perm, int n_rows) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long key = i;
    if (perm) {
      const long long ch = i / n_rows;
      key = ch * n_rows + perm[i - ch * n_rows];
    }
    const uint4 r = philox(make_uint4((uint32_t)key, (uint32_t)(key >> 32), 0u, 0u),
                           make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const double u1 = ((double)r.x + 1.0) * (1.0 / 4294967296.0);
    const double u2 = (double)r.y * (1.0 / 4294967296.0);
    const float rad = sqrtf(-2.f * logf((float)u1));
    float s, c;
    sincospif(2.f * (float)u2, &s, &c);
    C v = vis[i];
    v.x += (decltype(v.x))(sigma * (double)(rad * c));
    v.y += (decltype(v.y))(sigma * (double)(rad * s));
    vis[i] = v;
  }
}

static std::vector<GalaxyParams> make_gals(int n, const double* flux, const double* scale, const double* e1,
                                           const double* e2, const double* l, const double* m, double len,
                                           unsigned fmax) {
  std::vector<GalaxyParams> g(n);
  for (int i = 0; i < n; ++i) {
    g[i].l = l[i];
    g[i].m = m[i];
    g[i].flux = flux[i];
    g[i].scale = scale[i];
    g[i].e1 = e1 ? e1[i] : 0.0;
    g[i].e2 = e2 ? e2[i] : 0.0;
    unsigned F = facet_size(scale[i], len);
    if (fmax && F > fmax) F = fmax;  // the reference's facet buffers hold facet_size(RMAX) cells
    if (F < 2) F = 2;
    g[i].facet = (int)F;
    g[i].pad = 0;
  }
  return g;
}

// ------------------------------------------------------------------ pipeline
enum { kPhaseExtract = 0, kPhaseFit = 1, kPhaseRemove = 2, kPhaseExtractSeq = 3 };
// CUDA-event intervals labelled extract / fit / remove (and the k_extract_seq launches within the
// extraction), summed per label
struct PhaseTimer {
  std::vector<cudaEvent_t> ev;
  std::vector<int> label;  // label of the interval that ends at ev[i]
  int mark(int lab, cudaStream_t st) {
    cudaEvent_t e;
    RLF_CUDA(cudaEventCreate(&e));
    ev.push_back(e);
    label.push_back(lab);
    // inside a stream capture the record becomes a graph node that records the event when the
    // graph runs (an external record), so the phase times stay measurable
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    RLF_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive) RLF_CUDA(cudaEventRecordWithFlags(e, st, cudaEventRecordExternal));
    else RLF_CUDA(cudaEventRecord(e, st));
    return 0;
  }
  // ms3[0..2]: extract (the k_extract_seq launches included), fit, remove; seq_ms: the
  // k_extract_seq launches alone
  void sum(double* ms3, double* seq_ms = nullptr) const {
    for (size_t i = 1; i < ev.size(); ++i) {
      float x = 0;
      cudaEventElapsedTime(&x, ev[i - 1], ev[i]);
      if (label[i] == kPhaseExtractSeq) {
        ms3[kPhaseExtract] += x;
        if (seq_ms) *seq_ms += x;
      } else if (label[i] >= 0 && label[i] < 3) {
        ms3[label[i]] += x;
      }
    }
  }
  ~PhaseTimer() { for (auto e : ev) cudaEventDestroy(e); }
};

// Device round control of a sub-batch (SeqBatch::ctl): ctl[0] = j0, the first galaxy taking part in
// the round, ctl[1] = converged.  k_round_begin marks the galaxies the round fits and counts the
// round's work; k_round_end, after a round's fit, moves j0 to the first galaxy whose facet can still
// change (a galaxy before it was good in this round or the one before) or marks the unit converged.
// The host never waits between rounds.  dstats: RLF_STAT_* counters of the pass.
__global__ void k_round_begin(int bn, int rd, const int* __restrict__ ctl, int* __restrict__ active,
                              long long* __restrict__ dstats) {
  const int done = ctl[1], j0 = ctl[0];
  for (int i = threadIdx.x; i < bn; i += blockDim.x) active[i] = !done && i >= j0;
  if (threadIdx.x == 0 && !done) {
    dstats[RLF_STAT_EXTRACT_PASSES] += 1;
    dstats[RLF_STAT_EXTRACT_GAL] += bn - j0;
    if (rd == 0) dstats[RLF_STAT_EXTRACT_GAL_FIRST] += bn - j0;
    dstats[RLF_STAT_FITTED] += bn - j0;
  }
}
__global__ void k_round_end(int bn, int rd, int nr, const FitOut* __restrict__ out, int* __restrict__ good_prev,
                            int* __restrict__ ctl, long long* __restrict__ dstats) {
  __shared__ int first;
  if (ctl[1]) return;
  const int j0 = ctl[0];
  if (threadIdx.x == 0) first = bn;
  __syncthreads();
  for (int k = j0 + threadIdx.x; k < bn; k += blockDim.x)
    if (out[k].error == 0 || good_prev[k]) atomicMin(&first, k);
  __syncthreads();
  for (int k = j0 + threadIdx.x; k < bn; k += blockDim.x) good_prev[k] = out[k].error == 0;
  if (threadIdx.x == 0) {
    if (first == bn) {
      ctl[1] = 1;
      dstats[RLF_STAT_SKIPPED_GAL] += (long long)bn * (nr - 1 - rd);
    } else {
      ctl[0] = first;
      dstats[RLF_STAT_SKIPPED_GAL] += first;
    }
  }
}

// galaxies whose fit differs between two rounds (ellipticity by more than tol, or the error flag)
__global__ void k_count_changed(int n, const FitOut* a, const FitOut* b, double tol, unsigned long long* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool changed = a[i].error != b[i].error || fabs(a[i].e1 - b[i].e1) > tol || fabs(a[i].e2 - b[i].e2) > tol;
  if (changed) atomicAdd(count, 1ull);
}

// One pass of data_processing.c:61-138 over `order` (catalogue indices).
//
// batch = 1 (or F64 visibilities, or unevenly spaced channels): each galaxy is extracted, fitted
// and removed before the next one, the reference's order.
// batch > 1 with FP32 visibilities: the galaxies are taken in sub-batches of consecutive galaxies
// (up to `batch`, and as many as the shared-memory facets of the sequential extraction hold).  Each
// sub-batch runs `rounds` times sequential extraction (k_extract_seq: every facet with the previous
// round's fitted models of the earlier galaxies of the sub-batch removed) + finalisation + one
// persistent fit launch, then one removal pass with the final fits.  Galaxies whose facet is
// larger than the batched kernels hold are processed one at a time at their place in the order.
// Everything is queued on one stream; the host waits once at the end.
static int run_pass(rlf_observation* ob, const std::vector<GalaxyParams>& gals, const std::vector<int>& order,
                    int numr, const double* ro, const rlf_options& opt, std::vector<FitOut>& out,
                    cudaStream_t st, double* ms3, double* facets_out = nullptr, int* ncoords_out = nullptr,
                    int facets_stride = 0, double* partials_out = nullptr, int partials_stride = 0) {
  const int n = (int)order.size();
  out.assign(n, FitOut{});
  if (n == 0) return 0;
  if (numr < 2 || numr > kMaxNodes) { fprintf(stderr, "rlf: %d scalelength nodes unsupported\n", numr); return 1; }
  const Precision prec = (ob->precision == RLF_F64) ? kF64 : kMixed;   // visibility passes
  const Precision fprec = (opt.fit_precision == RLF_MIXED) ? kMixed : kF64;  // the fit
  const int B = opt.batch > 0 ? opt.batch : 1;
  // extraction only (one round, no fit or removal): the packed facets (facets_out) or the
  // un-averaged facet sums of a channel shard (partials_out)
  const bool extract_only = facets_out || partials_out;
  const int rounds = extract_only ? 1 : (opt.rounds > 0 ? opt.rounds : 3);
  const Observation o = ob->view();
  unsigned fmax = 0;
  for (int i = 0; i < n; ++i) fmax = std::max<unsigned>(fmax, (unsigned)gals[order[i]].facet);
  const int max_cells = (int)(fmax * fmax);
  std::vector<FacetCache*> cache(n);
  for (int i = 0; i < n; ++i) RLF_OK(obs_facet(ob, (unsigned)gals[order[i]].facet, &cache[i], st));
  FitConfigHost fc;
  memset(&fc, 0, sizeof(fc));
  fc.numr = numr;
  fc.gaussian = opt.gaussian;
  fc.np_max = kNpMax;
  for (int i = 0; i < numr; ++i) fc.ro[i] = ro[i];
  RLF_OK(fit_set_config(fc, st));
  std::vector<GalaxyParams> hg(n);
  std::vector<double> rprior((size_t)n * kMaxNodes, 0.0);
  std::vector<int> facets(n);
  std::vector<const double*> ssp(n), swp(n);
  for (int i = 0; i < n; ++i) {
    hg[i] = gals[order[i]];
    // data_processing.c:68-76: ln prior of the scalelength at each node
    const double mu = scale_mean(hg[i].flux);
    for (int r = 1; r < numr; ++r) rprior[(size_t)i * kMaxNodes + r] = rfunc(mu, kRStd, ro[r]);
    facets[i] = hg[i].facet;
    ssp[i] = cache[i]->ss.p;
    swp[i] = cache[i]->sw.p;
  }
  // batched mode: FP32 visibilities, batch > 1, evenly spaced channels
  bool batched = prec == kMixed && B > 1;
  if (batched) {
    const int bc = batch_set_channels(ob->n_ch, ob->wavenumbers.data(), ob->spec.data(), ob->max_delay_m, st);
    if (bc < 0) batched = false;
    else if (bc > 0) return bc;
  }
  // tunables (rlf_options, chosen by the autotuner): shared-memory facet budget of a sub-batch
  const size_t facet_budget = opt.seq_facet_kb > 0
                                  ? (size_t)std::min(std::max(opt.seq_facet_kb, 16), 200) * 1024
                                  : kSeqFacetBudget;
  // units of work in order: sub-batches [u0, u1) of the sequential extraction, or single galaxies
  struct Unit { int b0, bn; bool seq; };
  std::vector<Unit> units;
  // per-galaxy index of the facet size and facet offset inside its sub-batch
  std::vector<int> fidx(n, 0), foff(n, 0);
  std::vector<std::vector<int>> unit_sizes;  // distinct facet sizes of each sequential unit
  {
    int i = 0;
    while (i < n) {
      if (!batched || (unsigned)facets[i] > kBatchMaxFacet) {
        units.push_back({i, 1, false});
        unit_sizes.push_back({});
        ++i;
        continue;
      }
      std::vector<int> sizes;
      int cells = 0, j = i;
      while (j < n && j - i < std::min(B, kSeqMaxGal) && (unsigned)facets[j] <= kBatchMaxFacet) {
        const int F = facets[j];
        const bool new_size = std::find(sizes.begin(), sizes.end(), F) == sizes.end();
        if ((size_t)(cells + F * F) * kSeqCellBytes > facet_budget) break;
        if (new_size && (int)sizes.size() == kSeqMaxSizes) break;
        if (seq_smem_bytes(j - i + 1, cells + F * F, (int)sizes.size() + (new_size ? 1 : 0)) > kSeqMaxSmem) break;
        if (new_size) sizes.push_back(F);
        fidx[j] = (int)(std::find(sizes.begin(), sizes.end(), F) - sizes.begin());
        foff[j] = cells;
        cells += F * F;
        ++j;
      }
      units.push_back({i, j - i, true});
      unit_sizes.push_back(sizes);
      i = j;
    }
  }
  // slots of the facet cell buffer: every galaxy of a unit needs its own
  int max_unit = 1;
  for (const Unit& u : units) max_unit = std::max(max_unit, u.bn);
  std::vector<int> slot_off(max_unit);
  for (int k = 0; k < max_unit; ++k) slot_off[k] = k * max_cells;
  DevBuf<GalaxyParams> dg;
  DevBuf<double> dprior, dstart;
  DevBuf<int> doff, dnc, dqueue, dfidx, dfoff, dfac;
  DevBuf<const double*> dss, dsw;
  DevBuf<FitOut> dout, dprev;
  DevBuf<unsigned long long> dchanged;
  RLF_OK(dg.upload(hg.data(), n, st));
  RLF_OK(dprior.upload(rprior.data(), rprior.size(), st));
  RLF_OK(dss.upload(ssp.data(), n, st));
  RLF_OK(dsw.upload(swp.data(), n, st));
  RLF_OK(doff.upload(slot_off.data(), max_unit, st));
  RLF_OK(dfidx.upload(fidx.data(), n, st));
  RLF_OK(dfoff.upload(foff.data(), n, st));
  RLF_OK(dfac.upload(facets.data(), n, st));
  // learned proposal of the simplex starts: computed on the device from each round's facets
  const bool learned = !opt.start && opt.proposal && proposal_ready() && !extract_only;
  if (learned) RLF_OK(dstart.ensure((size_t)3 * n));
  if (opt.start) {
    std::vector<double> sv((size_t)3 * n);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < 3; ++k) sv[3 * i + k] = opt.start[3 * order[i] + k];
    RLF_OK(dstart.upload(sv.data(), sv.size(), st));
  }
  RLF_OK(dout.ensure(n));
  RLF_CUDA(cudaMemsetAsync(dout.p, 0, n * sizeof(FitOut), st));
  RLF_OK(dnc.ensure(n));
  RLF_OK(dqueue.ensure(1));
  // sampling board of the fit launches (rows indexed by the galaxy's place in its unit)
  DevBuf<SampleSlot> bslot;
  DevBuf<double> bL;
  DevBuf<int> berr, bflag, bnewton, bdone;
  if (!extract_only) {
    RLF_OK(bslot.ensure(max_unit));
    RLF_OK(bL.ensure((size_t)max_unit * 2 * kBoardCap));
    RLF_OK(berr.ensure((size_t)max_unit * 2 * kBoardCap));
    RLF_OK(bflag.ensure((size_t)max_unit * 2 * kBoardCap));
    RLF_OK(bnewton.ensure(max_unit));
    RLF_OK(bdone.ensure(1));
  }
  // device round control of the sub-batches (k_round_begin / k_round_end)
  DevBuf<int> dctl, dactive, dgoodp;
  DevBuf<long long> dstats;
  RLF_OK(dctl.ensure(2));
  RLF_OK(dactive.ensure(max_unit));
  RLF_OK(dgoodp.ensure(max_unit));
  RLF_OK(dstats.ensure(RLF_NSTATS));
  RLF_CUDA(cudaMemsetAsync(dstats.p, 0, RLF_NSTATS * sizeof(long long), st));
  if (batched && rounds > 1) {
    RLF_OK(dprev.ensure(std::min(n, max_unit)));
    RLF_OK(dchanged.ensure(1));
    RLF_CUDA(cudaMemsetAsync(dchanged.p, 0, sizeof(unsigned long long), st));
  }
  const size_t esz = fprec == kF64 ? sizeof(double) : sizeof(float);
  DevBuf<unsigned char> cells;
  const size_t plane = (size_t)max_unit * max_cells * esz;
  RLF_OK(cells.ensure(5 * plane));
  DevBuf<double> dpart;  // [max_unit][4][partials_stride] un-averaged facet sums of a unit
  if (partials_out) RLF_OK(dpart.ensure((size_t)max_unit * 4 * partials_stride));
  void* gu = cells.p;
  void* gv = cells.p + plane;
  void* dre = cells.p + 2 * plane;
  void* dim = cells.p + 3 * plane;
  void* sg = cells.p + 4 * plane;
  RLF_OK(ob->partial.ensure((size_t)ob->n_part * 4 * fmax * fmax + 4 * fmax * fmax));
  int sms = 0, dev = 0;
  RLF_CUDA(cudaGetDevice(&dev));
  RLF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // persistent fit CTAs: per SM at most the kernel's occupancy (fit_max_grid), fewer when tuned
  const int grid_fit = opt.fit_ctas_per_sm > 0 ? std::min(fit_max_grid(fprec), sms * opt.fit_ctas_per_sm)
                                               : fit_max_grid(fprec);
  const int seq_ctas = kSeqCtasPerSm * sms;
  if (batched && !ob->rows.p) {
    RLF_OK(ob->rows.ensure(ob->n_rows));
    RLF_OK(launch_row_table(ob->n_rows, ob->uu.p, ob->vv.p, ob->ww.p, ob->rows.p, st));
  }
  PhaseTimer pt;
  // the sub-batches' executable graphs, destroyed once the stream has run them
  std::vector<cudaGraphExec_t> execs;
  struct ExecRelease {
    std::vector<cudaGraphExec_t>& v;
    cudaStream_t s;
    ~ExecRelease() {
      if (v.empty()) return;
      cudaStreamSynchronize(s);
      for (auto e : v) cudaGraphExecDestroy(e);
    }
  } exec_release{execs, st};
  RLF_OK(pt.mark(-1, st));
  for (size_t ui = 0; ui < units.size(); ++ui) {
    const Unit& u = units[ui];
    const int b0 = u.b0, bn = u.bn;
    FacetOut fo;
    fo.offset = doff.p;
    fo.ncoords = dnc.p + b0;
    fo.gu = gu; fo.gv = gv; fo.dre = dre; fo.dim = dim; fo.sig2 = sg;
    fo.as_float = fprec == kMixed;
    FacetBatch fb{};
    fb.n_gal = bn;
    fb.max_cells = max_cells;
    fb.offset = doff.p;
    fb.count = dnc.p + b0;
    fb.gu = gu; fb.gv = gv; fb.dre = dre; fb.dim = dim; fb.sig2 = sg;
    fb.rprior = dprior.p + (size_t)b0 * kMaxNodes;
    fb.start = opt.start ? dstart.p + (size_t)3 * b0 : nullptr;
    fb.active = nullptr;
    fb.out = dout.p + b0;
    fb.queue = dqueue.p;
    fb.trace = nullptr;
    fb.trace_cap = 0;
    if (bslot.p) {
      fb.board.slot = bslot.p;
      fb.board.L = bL.p;
      fb.board.err = berr.p;
      fb.board.flag = bflag.p;
      fb.board.newton = bnewton.p;
      fb.board.done_gal = bdone.p;
      fb.board.wait_ns = opt.board_wait_us > 0 ? (unsigned long long)opt.board_wait_us * 1000ull : 0ull;
    }
    SeqBatch sb{};
    if (u.seq) {
      sb.n_gal = bn;
      sb.gals = dg.p + b0;
      sb.fidx = dfidx.p + b0;
      sb.foff = dfoff.p + b0;
      sb.facet = dfac.p + b0;
      sb.total_cells = 0;
      for (int k = b0; k < b0 + bn; ++k) sb.total_cells += facets[k] * facets[k];
      sb.n_sizes = (int)unit_sizes[ui].size();
      for (int f = 0; f < sb.n_sizes; ++f) {
        FacetCache* fcF = nullptr;
        RLF_OK(obs_facet(ob, (unsigned)unit_sizes[ui][f], &fcF, st));
        if (!fcF->desc.p) {
          RLF_OK(fcF->desc.ensure((size_t)ob->n_rows * ((ob->n_ch + 15) / 16)));
          RLF_OK(fcF->desc1.ensure((size_t)ob->n_rows * ((ob->n_ch + 15) / 16)));
          RLF_OK(launch_cell_desc(ob->n_rows, ob->n_ch, fcF->cell.p, fcF->desc.p, fcF->desc1.p, st));
        }
        sb.desc[f] = fcF->desc.p;
        sb.desc1[f] = fcF->desc1.p;
        sb.cells[f] = fcF->cell.p;
      }
      RLF_OK(ob->bpartial.ensure((size_t)seq_ctas * sb.total_cells));
      const long long n_items = (long long)ob->n_rows * ((ob->n_ch + 15) / 16);
      if (n_items > 0x7fffffffLL - (1LL << 24)) { fprintf(stderr, "rlf: %lld row-chunks exceed the batched extraction\n", n_items); return 1; }
      RLF_OK(ob->items.ensure((size_t)n_items));
      RLF_OK(ob->items2.ensure((size_t)n_items));
      RLF_OK(ob->item_count.ensure(6));
      sb.items = ob->items.p;
      sb.items2 = ob->items2.p;
      sb.n_simple = ob->item_count.p;
      sb.n_two = ob->item_count.p + 2;
      sb.queue = ob->item_count.p + 3;
      RLF_OK(launch_classify_items(n_items, sb, ob->items.p, ob->items2.p, ob->item_count.p, st));
    }
    const int nr = u.seq ? rounds : 1;
    // CUDA graph of the sub-batch: every round (round control, extraction, finalisation, proposal,
    // fit) and the removal are captured from the stream and launched as one graph, the host never
    // waiting within the sub-batch (rlf_options.graphs)
    const bool graph = u.seq && opt.graphs && !extract_only;
    if (graph) RLF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    // Galaxies [j0, bn) of the unit take part in a round.  Round r+1 extracts galaxy k with the
    // fitted - round model differences of round r's good fits among the galaxies before k, round r
    // with those of round r-1 (none before round 1); a good fit's difference moves between rounds,
    // a bad fit's is zero.  So galaxy k keeps its facet and fit unless a galaxy before it was good
    // in round r or r-1: the next round starts at the first such galaxy (it is extracted again for
    // its model difference), and none means the unit has converged.
    if (u.seq) {
      RLF_CUDA(cudaMemsetAsync(dctl.p, 0, 2 * sizeof(int), st));
      RLF_CUDA(cudaMemsetAsync(dgoodp.p, 0, (size_t)bn * sizeof(int), st));
    }
    for (int rd = 0; rd < nr; ++rd) {
      // a sequential unit runs all its rounds with device round control (the galaxies before ctl[0]
      // keep their facets and fits; a converged unit's remaining rounds do nothing); a single galaxy
      // is one round
      SeqBatch sr = sb;
      FacetBatch fr = fb;
      FacetOut fq = fo;
      fq.offset = doff.p;
      fq.ncoords = dnc.p + b0;
      fr.n_gal = bn;
      fr.offset = doff.p;
      fr.count = dnc.p + b0;
      fr.rprior = dprior.p + (size_t)b0 * kMaxNodes;
      fr.start = (opt.start || learned) ? dstart.p + (size_t)3 * b0 : nullptr;
      fr.out = dout.p + b0;
      fr.active = u.seq ? dactive.p : nullptr;
      // ---- extraction
      if (u.seq) {
        sr.ctl = dctl.p;
        sr.fit = rd == 0 ? nullptr : dout.p + b0;
        k_round_begin<<<1, 256, 0, st>>>(bn, rd, dctl.p, dactive.p, dstats.p);
        count_launch();
        RLF_CUDA(cudaGetLastError());
        RLF_OK(pt.mark(kPhaseExtract, st));
        RLF_OK(launch_extract_seq(ob->n_rows, ob->rows.p, ob->data32.p, ob->sky32.p, sr, opt.gaussian, seq_ctas,
                                  ob->bpartial.p, st));
        RLF_OK(pt.mark(kPhaseExtractSeq, st));
        if (partials_out)
          RLF_OK(launch_partials_seq(sr, seq_ctas, ob->bpartial.p, dss.p + b0, dsw.p + b0, dpart.p, partials_stride,
                                     st));
        else
          RLF_OK(launch_finalize_seq(sr, seq_ctas, ob->bpartial.p, dss.p + b0, dsw.p + b0, ob->len, fq, st));
      } else {
        const int i = b0;
        const unsigned F = (unsigned)facets[i];
        ob->stats[RLF_STAT_EXTRACT_SINGLE] += 1;
        ob->stats[RLF_STAT_FITTED] += 1;
        if (prec == kF64)
          RLF_OK(launch_extract_f64(o, ob->data64.p, ob->sky64.p, cache[i]->cell.p, dg.p + i, F, opt.gaussian,
                                    ob->partial.p, ob->n_part, st));
        else
          RLF_OK(launch_extract_mixed(o, ob->data32.p, ob->sky32.p, cache[i]->cell.p, dg.p + i, F, opt.gaussian,
                                      ob->partial.p, ob->n_part, st));
        double* sums = ob->partial.p + (size_t)ob->n_part * 2 * F * F;
        RLF_OK(launch_reduce_partials(ob->partial.p, ob->n_part, 2 * F * F, sums, st));
        if (partials_out) {
          const size_t nc = (size_t)F * F;
          RLF_CUDA(cudaMemsetAsync(dpart.p, 0, (size_t)4 * partials_stride * sizeof(double), st));
          RLF_CUDA(copy_async(dpart.p, sums, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
          RLF_CUDA(copy_async(dpart.p + partials_stride, sums + nc, nc * sizeof(double), cudaMemcpyDeviceToDevice, st));
          RLF_CUDA(copy_async(dpart.p + 2 * partials_stride, cache[i]->ss.p, nc * sizeof(double),
                              cudaMemcpyDeviceToDevice, st));
          RLF_CUDA(copy_async(dpart.p + 3 * partials_stride, cache[i]->sw.p, nc * sizeof(double),
                              cudaMemcpyDeviceToDevice, st));
        } else {
          RLF_OK(launch_facet_finalize(1, dfac.p + i, sums, 1, 0, dss.p + i, dsw.p + i, ob->len, fo, st));
        }
      }
      RLF_OK(pt.mark(kPhaseExtract, st));
      if (extract_only) break;
      // ---- fit
      if (learned) {
        static_assert(sizeof(GalaxyParams) % sizeof(double) == 0, "GalaxyParams holds whole doubles");
        const double* flux = reinterpret_cast<const double*>(reinterpret_cast<const char*>(dg.p + b0) +
                                                             offsetof(GalaxyParams, flux));
        RLF_OK(propose_starts(bn, doff.p, dnc.p + b0, dfac.p + b0, gu, gv, dre, dim, sg, fprec == kMixed ? 1 : 0,
                              flux, (int)(sizeof(GalaxyParams) / sizeof(double)), ob->len, dstart.p + (size_t)3 * b0,
                              st));
      }
      const bool last = rd == nr - 1;
      if (u.seq && last && nr > 1)
        RLF_CUDA(copy_async(dprev.p, dout.p + b0, bn * sizeof(FitOut), cudaMemcpyDeviceToDevice, st));
      RLF_CUDA(cudaMemsetAsync(dqueue.p, 0, sizeof(int), st));
      if (fr.board.slot) {
        RLF_CUDA(cudaMemsetAsync(bslot.p, 0, (size_t)bn * sizeof(SampleSlot), st));
        RLF_CUDA(cudaMemsetAsync(bflag.p, 0, (size_t)bn * 2 * kBoardCap * sizeof(int), st));
        RLF_CUDA(cudaMemsetAsync(bnewton.p, 0, (size_t)bn * sizeof(int), st));
        RLF_CUDA(cudaMemsetAsync(bdone.p, 0, sizeof(int), st));
      }
      // with the board, CTAs beyond the galaxy count start as helpers of the sampling grids
      RLF_OK(fit_launch(fr, fprec, fr.board.slot ? grid_fit : std::min(grid_fit, bn), st));
      if (u.seq && last && nr > 1) {
        k_count_changed<<<(bn + 127) / 128, 128, 0, st>>>(bn, dprev.p, dout.p + b0, 1e-9, dchanged.p);
        count_launch();
        RLF_CUDA(cudaGetLastError());
      }
      if (u.seq && !last) {
        k_round_end<<<1, 256, 0, st>>>(bn, rd, nr, dout.p + b0, dgoodp.p, dctl.p, dstats.p);
        count_launch();
        RLF_CUDA(cudaGetLastError());
      }
      RLF_OK(pt.mark(kPhaseFit, st));
    }
    if (partials_out) {
      // a channel shard's un-averaged facet sums of this unit, in the caller's galaxy order
      for (int k = 0; k < bn; ++k)
        RLF_CUDA(copy_async(partials_out + (size_t)order[b0 + k] * 4 * partials_stride,
                            dpart.p + (size_t)k * 4 * partials_stride, (size_t)4 * partials_stride * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
      RLF_CUDA(cudaStreamSynchronize(st));  // dpart is reused by the next unit
      continue;
    }
    if (facets_out) {
      // extraction only: hand the packed facets of this unit back as doubles
      std::vector<int> nc(bn);
      RLF_CUDA(copy_async(nc.data(), dnc.p + b0, bn * sizeof(int), cudaMemcpyDeviceToHost, st));
      std::vector<unsigned char> h(5 * plane);
      RLF_CUDA(copy_async(h.data(), cells.p, h.size(), cudaMemcpyDeviceToHost, st));
      RLF_CUDA(cudaStreamSynchronize(st));
      for (int k = 0; k < bn; ++k) {
        ncoords_out[b0 + k] = nc[k];
        for (int a = 0; a < 5; ++a)
          for (int c = 0; c < nc[k] && c < facets_stride; ++c) {
            const size_t src = (size_t)a * plane + ((size_t)k * max_cells + c) * esz;
            const double v = esz == sizeof(double) ? *reinterpret_cast<const double*>(&h[src])
                                                   : (double)*reinterpret_cast<const float*>(&h[src]);
            facets_out[((size_t)(b0 + k) * 5 + a) * facets_stride + c] = v;
          }
      }
      continue;
    }
    // ---- removal with the final fits
    if (u.seq) {
      ob->stats[RLF_STAT_REMOVE_BATCHES] += 1;
      RLF_OK(launch_remove_batch(ob->n_rows, ob->rows.p, ob->data32.p, ob->sky32.p, dg.p + b0, dout.p + b0, bn,
                                 opt.gaussian, st));
    } else {
      ob->stats[RLF_STAT_REMOVE_SINGLE] += 1;
      const int i = b0;
      const double* e12 = &dout.p[i].e1;
      const int* err = &dout.p[i].error;
      if (prec == kF64)
        RLF_OK(launch_remove_f64(o, ob->data64.p, ob->sky64.p, dg.p + i, e12, err, opt.gaussian, st));
      else
        RLF_OK(launch_remove_mixed(o, ob->data32.p, ob->sky32.p, dg.p + i, e12, err, opt.gaussian, st));
    }
    RLF_OK(pt.mark(kPhaseRemove, st));
    if (graph) {
      cudaGraph_t gr = nullptr;
      RLF_CUDA(cudaStreamEndCapture(st, &gr));
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, gr, 0);
      cudaGraphDestroy(gr);
      if (ie != cudaSuccess) { fprintf(stderr, "rlf: cudaGraphInstantiate: %s\n", cudaGetErrorString(ie)); return (int)ie; }
      execs.push_back(ex);
      RLF_CUDA(cudaGraphLaunch(ex, st));
      ob->stats[RLF_STAT_GRAPHS] += 1;
    }
  }
  if (!extract_only) RLF_OK(dout.download(out.data(), n, st));
  unsigned long long changed = 0;
  if (dchanged.p) RLF_CUDA(copy_async(&changed, dchanged.p, sizeof(changed), cudaMemcpyDeviceToHost, st));
  long long hstats[RLF_NSTATS];
  RLF_CUDA(copy_async(hstats, dstats.p, sizeof(hstats), cudaMemcpyDeviceToHost, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  ob->stats[RLF_STAT_CHANGED] += (long long)changed;
  for (int k = 0; k < RLF_NSTATS; ++k) ob->stats[k] += hstats[k];
  if (ms3) {
    double seq_ms = 0;
    pt.sum(ms3, &seq_ms);
    ob->stats[RLF_STAT_EXTRACT_SEQ_US] += (long long)(seq_ms * 1000.0 + 0.5);
  }
  return 0;
}

// the two passes of RadioLensfit2.cpp:597-606 over a device-resident observation
static int process(rlf_observation* ob, int n_gal, const double* flux, const double* scale, const double* l,
                   const double* m, int numr, const double* ro, const rlf_options& opt, rlf_fit_result* res,
                   int* n_bad, cudaStream_t st) {
  const unsigned fmax = facet_size(kRMax, ob->len);
  std::vector<GalaxyParams> gals = make_gals(n_gal, flux, scale, nullptr, nullptr, l, m, ob->len, fmax);
  std::vector<int> order(n_gal);
  for (int i = 0; i < n_gal; ++i) order[i] = i;
  double ms3[3] = {0, 0, 0};
  for (auto& x : ob->stats) x = 0;
  cudaEvent_t e0, e1;
  RLF_CUDA(cudaEventCreate(&e0));
  RLF_CUDA(cudaEventCreate(&e1));
  RLF_CUDA(cudaEventRecord(e0, st));
  std::vector<FitOut> out;
  RLF_OK(run_pass(ob, gals, order, numr, ro, opt, out, st, ms3));
  std::vector<int> bad;
  for (int i = 0; i < n_gal; ++i) {
    memcpy(&res[i], &out[i], sizeof(rlf_fit_result));
    if (out[i].error) bad.push_back(i);
  }
  int nb = (int)bad.size();
  if (opt.refit && nb > 0) {
    std::vector<FitOut> out2;
    RLF_OK(run_pass(ob, gals, bad, numr, ro, opt, out2, st, ms3));
    nb = 0;
    for (size_t k = 0; k < bad.size(); ++k) {
      memcpy(&res[bad[k]], &out2[k], sizeof(rlf_fit_result));
      if (out2[k].error) {  // data_processing.c:97-103: written with e = 0
        res[bad[k]].e1 = 0.;
        res[bad[k]].e2 = 0.;
        nb++;
      }
    }
  }
  RLF_CUDA(cudaEventRecord(e1, st));
  RLF_CUDA(cudaEventSynchronize(e1));
  float tot = 0;
  cudaEventElapsedTime(&tot, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ob->ms[0] = tot; ob->ms[1] = ms3[0]; ob->ms[2] = ms3[1]; ob->ms[3] = ms3[2];
  if (n_bad) *n_bad = nb;
  return 0;
}

// Rows of a new mixed-precision observation into uv order: perm, inv, and uvw, variances and flags
// (in the caller's order on entry) gathered to their positions.
static int obs_permute_rows(rlf_observation* ob, cudaStream_t st) {
  const int n = ob->n_rows;
  DevBuf<int> bins;
  RLF_OK(bins.ensure((size_t)kOrderBins * kOrderBins));
  RLF_OK(ob->perm.ensure(n));
  RLF_OK(ob->inv.ensure(n));
  RLF_OK(launch_row_order(n, ob->uu.p, ob->vv.p, ob->wavenumbers[0] / (2 * kPi), ob->len, ob->perm.p, bins.p, st));
  RLF_OK(launch_invert_perm(n, ob->perm.p, ob->inv.p, st));
  for (DevBuf<double>* a : {&ob->uu, &ob->vv, &ob->ww}) {
    DevBuf<double> t;
    RLF_OK(t.ensure(n));
    RLF_OK(launch_gather_rows_f64(n, a->p, ob->perm.p, t.p, st));
    std::swap(a->p, t.p);
    std::swap(a->n, t.n);
  }
  {
    DevBuf<float> t;
    RLF_OK(t.ensure((size_t)ob->n_vis));
    RLF_OK(launch_scatter_rows<float>(0, ob->n_vis, n, ob->sigma2.p, ob->inv.p, t.p, st));
    std::swap(ob->sigma2.p, t.p);
    std::swap(ob->sigma2.n, t.n);
  }
  if (ob->flag.p) {
    DevBuf<uint8_t> t;
    RLF_OK(t.ensure((size_t)ob->n_vis));
    RLF_OK(launch_scatter_rows<uint8_t>(0, ob->n_vis, n, ob->flag.p, ob->inv.p, t.p, st));
    std::swap(ob->flag.p, t.p);
    std::swap(ob->flag.n, t.n);
  }
  RLF_CUDA(cudaStreamSynchronize(st));  // the swapped-out buffers are freed on return
  return 0;
}

static rlf_observation* obs_create(int n_rows, int n_ch, const double* uu, const double* vv, const double* ww,
                                   const double* wavenumbers, const double* spec, double len, const float* sigma2,
                                   const uint8_t* flag, int precision, cudaStream_t st) {
  if (n_rows <= 0 || n_ch <= 0 || n_ch > kMaxCh) { fprintf(stderr, "rlf: bad observation shape\n"); return nullptr; }
  rlf_observation* ob = new rlf_observation();
  ob->n_rows = n_rows;
  ob->n_ch = n_ch;
  ob->n_vis = (long long)n_rows * n_ch;
  ob->precision = precision;
  ob->len = len;
  ob->wavenumbers.assign(wavenumbers, wavenumbers + n_ch);
  ob->spec.assign(spec, spec + n_ch);
  ob->n_part = grid_partial_blocks(n_rows);
  for (int i = 0; i < n_rows; ++i)
    ob->max_delay_m = std::max(ob->max_delay_m, fabs(uu[i]) + fabs(vv[i]) + fabs(ww[i]));
  int r = ob->uu.upload(uu, n_rows, st);
  if (!r) r = ob->vv.upload(vv, n_rows, st);
  if (!r) r = ob->ww.upload(ww, n_rows, st);
  if (!r) r = ob->sigma2.upload(sigma2, (size_t)ob->n_vis, st);
  if (!r && flag) r = ob->flag.upload(flag, (size_t)ob->n_vis, st);
  if (!r && precision != RLF_F64) r = obs_permute_rows(ob, st);
  if (!r && precision == RLF_F64) {
    r = ob->data64.ensure(ob->n_vis);
    if (!r) r = ob->sky64.ensure(ob->n_vis);
    if (!r) r = (int)cudaMemsetAsync(ob->data64.p, 0, ob->n_vis * sizeof(double2), st);
    if (!r) r = (int)cudaMemsetAsync(ob->sky64.p, 0, ob->n_vis * sizeof(double2), st);
  } else if (!r) {
    r = ob->data32.ensure(ob->n_vis);
    if (!r) r = ob->sky32.ensure(ob->n_vis);
    if (!r) r = (int)cudaMemsetAsync(ob->data32.p, 0, ob->n_vis * sizeof(float2), st);
    if (!r) r = (int)cudaMemsetAsync(ob->sky32.p, 0, ob->n_vis * sizeof(float2), st);
  }
  if (!r) r = set_channels(n_ch, wavenumbers, spec, st);
  if (!r) r = (int)cudaStreamSynchronize(st);
  if (r) { delete ob; return nullptr; }
  return ob;
}

// Device address of page-locked host memory registered with CUDA (cudaHostAlloc, cudaHostRegister),
// or nullptr for other memory.  The conversion kernels read and write such buffers directly over the
// host link, which takes one pass instead of a staging copy plus a conversion.
static void* mapped_host(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// upload host complex128 [n] into the observation's data or sky array
static int obs_put_c128(rlf_observation* ob, const double* h, bool sky, cudaStream_t st) {
  const long long n = ob->n_vis;
  if (ob->precision == RLF_F64) {
    double2* d = sky ? ob->sky64.p : ob->data64.p;
    if (h) RLF_CUDA(copy_async(d, h, n * sizeof(double2), cudaMemcpyHostToDevice, st));
    else RLF_CUDA(cudaMemsetAsync(d, 0, n * sizeof(double2), st));
    return 0;
  }
  float2* d = sky ? ob->sky32.p : ob->data32.p;
  if (!h) { RLF_CUDA(cudaMemsetAsync(d, 0, n * sizeof(float2), st)); return 0; }
  // the caller's order read in sequence, each row scattered to its position (inv)
  if (const void* hd = mapped_host(h)) {
    __atomic_add_fetch(&g_h2d_bytes, (unsigned long long)n * sizeof(double2), __ATOMIC_RELAXED);
    RLF_OK(launch_c64_to_f32_scatter(0, n, ob->n_rows, static_cast<const double2*>(hd), ob->inv.p, d, st));
    RLF_CUDA(cudaStreamSynchronize(st));
    return 0;
  }
  // stage in chunks through a device FP64 buffer
  const long long chunk = 1LL << 24;
  DevBuf<double2> tmp;
  RLF_OK(tmp.ensure((size_t)std::min(chunk, n)));
  for (long long i = 0; i < n; i += chunk) {
    const long long c = std::min(chunk, n - i);
    RLF_CUDA(copy_async(tmp.p, h + 2 * i, c * sizeof(double2), cudaMemcpyHostToDevice, st));
    RLF_OK(launch_c64_to_f32_scatter(i, c, ob->n_rows, tmp.p, ob->inv.p, d, st));
  }
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

static int obs_get_c128(rlf_observation* ob, double* h, bool sky, cudaStream_t st) {
  const long long n = ob->n_vis;
  if (!h) return 0;
  if (ob->precision == RLF_F64) {
    RLF_CUDA(copy_async(h, sky ? ob->sky64.p : ob->data64.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st));
    RLF_CUDA(cudaStreamSynchronize(st));
    return 0;
  }
  const float2* d = sky ? ob->sky32.p : ob->data32.p;
  // each row gathered from its position (inv), the caller's order written in sequence
  if (void* hd = mapped_host(h)) {
    __atomic_add_fetch(&g_d2h_bytes, (unsigned long long)n * sizeof(double2), __ATOMIC_RELAXED);
    RLF_OK(launch_f32_to_c64_gather(0, n, ob->n_rows, d, ob->inv.p, static_cast<double2*>(hd), st));
    RLF_CUDA(cudaStreamSynchronize(st));
    return 0;
  }
  const long long chunk = 1LL << 24;
  DevBuf<double2> tmp;
  RLF_OK(tmp.ensure((size_t)std::min(chunk, n)));
  for (long long i = 0; i < n; i += chunk) {
    const long long c = std::min(chunk, n - i);
    RLF_OK(launch_f32_to_c64_gather(i, c, ob->n_rows, d, ob->inv.p, tmp.p, st));
    RLF_CUDA(copy_async(h + 2 * i, tmp.p, c * sizeof(double2), cudaMemcpyDeviceToHost, st));
    RLF_CUDA(cudaStreamSynchronize(st));
  }
  return 0;
}

// facet arrays of a likelihood_params (FACET) uploaded as a one-galaxy FacetBatch (F64)
struct OneFacet {
  DevBuf<double> gu, gv, dre, dim, sig2, rprior;
  DevBuf<int> off, cnt;
  FacetBatch fb;
  int load(const likelihood_params* par, cudaStream_t st) {
    const int n = (int)par->ncoords;
    std::vector<double> re(n > 0 ? n : 1), im(n > 0 ? n : 1), pr(kMaxNodes, 0.0);
    for (int i = 0; i < n; ++i) { re[i] = par->data[i].real; im[i] = par->data[i].imag; }
    for (int i = 0; i < par->numr && i < kMaxNodes; ++i) pr[i] = par->rprior[i];
    RLF_OK(gu.upload(par->uu, n, st));
    RLF_OK(gv.upload(par->vv, n, st));
    RLF_OK(dre.upload(re.data(), n, st));
    RLF_OK(dim.upload(im.data(), n, st));
    RLF_OK(sig2.upload(par->sigma2, n, st));
    RLF_OK(rprior.upload(pr.data(), kMaxNodes, st));
    int z = 0;
    RLF_OK(off.upload(&z, 1, st));
    RLF_OK(cnt.upload(&n, 1, st));
    FitConfigHost fc;
    memset(&fc, 0, sizeof(fc));
    if (par->numr < 2 || par->numr > kMaxNodes) { fprintf(stderr, "rlf: numr %d unsupported\n", par->numr); return 1; }
    fc.numr = par->numr;
    fc.gaussian = g_lib.opt.gaussian;
    fc.np_max = kNpMax;
    for (int i = 0; i < par->numr; ++i) fc.ro[i] = par->ro[i];
    RLF_OK(fit_set_config(fc, st));
    fb.n_gal = 1;
    fb.max_cells = n;
    fb.offset = off.p;
    fb.count = cnt.p;
    fb.gu = gu.p; fb.gv = gv.p; fb.dre = dre.p; fb.dim = dim.p; fb.sig2 = sig2.p;
    fb.rprior = rprior.p;
    fb.start = nullptr;
    fb.active = nullptr;
    fb.out = nullptr;
    fb.queue = nullptr;
    fb.trace = nullptr;
    fb.trace_cap = 0;
    fb.board = SampleBoard{};
    return 0;
  }
};

// last spline built by marginalise_posterior_r, for marf (marginalise_r.c:231-238)
static std::vector<double> g_marf_x, g_marf_y;

// Opt-in native backtrace on a fatal signal (RLF_DEBUG_SEGV=1), for diagnosing host crashes.
static void segv_trace(int sig) {
  void* buf[64];
  const int n = backtrace(buf, 64);
  static const char msg[] = "rlf: fatal signal, native backtrace:\n";
  if (write(2, msg, sizeof(msg) - 1) < 0) {}
  backtrace_symbols_fd(buf, n, 2);
  signal(sig, SIG_DFL);
  raise(sig);
}
__attribute__((constructor)) static void install_segv_trace() {
  if (getenv("RLF_DEBUG_SEGV")) {
    signal(SIGSEGV, segv_trace);
    signal(SIGBUS, segv_trace);
  }
}

}  // namespace rlf

using namespace rlf;

// =========================================================== batched / device API
// an input block on the device: page-locked host memory is read in place, other memory copied
template <class T>
static const T* device_in(const T* h, size_t n, DevBuf<T>& buf, cudaStream_t st) {
  if (const void* d = mapped_host(h)) {
    __atomic_add_fetch(&g_h2d_bytes, (unsigned long long)n * sizeof(T), __ATOMIC_RELAXED);
    return static_cast<const T*>(d);
  }
  if (buf.upload(h, n, st)) return nullptr;
  return buf.p;
}

extern "C" {

const char* rlf_version(void) { return "rlf-gb300 0.1 (sm_103a)"; }

long long rlf_launch_count(void) { return rlf::launch_count(); }

double rlf_fp32_peak_gflops(void) {
  cudaStream_t st;
  if (lib_stream(&st)) return 0.0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return rlf::fp32_probe_gflops(sms * 8, 20000, st);
}

int rlf_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int rlf_configure(const rlf_options* opt) {
  if (opt) g_lib.opt = *opt;
  if (g_lib.opt.batch < 1) g_lib.opt.batch = 1;
  return 0;
}

rlf_observation* rlf_obs_create(int n_rows, int n_ch, const double* uu, const double* vv, const double* ww,
                                const double* wavenumbers, const double* spec, double len, const float* sigma2,
                                const uint8_t* flag, int precision) {
  cudaStream_t st;
  if (lib_stream(&st)) return nullptr;
  return obs_create(n_rows, n_ch, uu, vv, ww, wavenumbers, spec, len, sigma2, flag, precision, st);
}

void rlf_obs_destroy(rlf_observation* obs) { delete obs; }

int rlf_obs_set_vis(rlf_observation* obs, const double* data_c128, const double* sky_c128) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  RLF_OK(obs_put_c128(obs, data_c128, false, st));
  RLF_OK(obs_put_c128(obs, sky_c128, true, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_set_data_c64(rlf_observation* obs, const float* data_c64) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const long long n = obs->n_vis;
  if (obs->precision == RLF_F64) {
    DevBuf<float2> tmp;
    RLF_OK(tmp.upload(reinterpret_cast<const float2*>(data_c64), (size_t)n, st));
    RLF_OK(launch_convert_f32_to_c64(n, tmp.p, obs->data64.p, st));
    RLF_CUDA(cudaStreamSynchronize(st));
  } else {
    // staged in chunks, each row scattered to its position
    const long long chunk = 1LL << 24;
    DevBuf<float2> tmp;
    RLF_OK(tmp.ensure((size_t)std::min(chunk, n)));
    for (long long i = 0; i < n; i += chunk) {
      const long long c = std::min(chunk, n - i);
      RLF_CUDA(copy_async(tmp.p, data_c64 + 2 * i, c * sizeof(float2), cudaMemcpyHostToDevice, st));
      RLF_OK(launch_scatter_rows<float2>(i, c, obs->n_rows, tmp.p, obs->inv.p, obs->data32.p, st));
    }
    RLF_CUDA(cudaStreamSynchronize(st));
  }
  return 0;
}

// DATA block of the Measurement Set straight into the observation's data (measurement_set.cpp:345-400)
int rlf_obs_set_data_ms(rlf_observation* obs, const float* data_block, unsigned int num_pols) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const long long n = obs->n_vis * (long long)num_pols;
  DevBuf<float2> in;
  const float2* src = static_cast<const float2*>(mapped_host(data_block));
  if (src) {
    __atomic_add_fetch(&g_h2d_bytes, (unsigned long long)n * sizeof(float2), __ATOMIC_RELAXED);
  } else {
    RLF_OK(in.upload(reinterpret_cast<const float2*>(data_block), (size_t)n, st));
    src = in.p;
  }
  if (obs->precision == RLF_F64) RLF_OK(launch_ms_vis_c128(src, obs->n_rows, obs->n_ch, (int)num_pols, obs->data64.p, st));
  else RLF_OK(launch_ms_vis_f32(src, obs->n_rows, obs->n_ch, (int)num_pols, obs->inv.p, obs->data32.p, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

// ---- Measurement Set readers and writer on column blocks the caller read from the table

double rlf_ms_read_coords(const double* uvw_block, unsigned int num_coords, double* uu, double* vv, double* ww) {
  cudaStream_t st;
  if (lib_stream(&st) || num_coords == 0) return 0.;
  DevBuf<double> in, u, v, w;
  DevBuf<unsigned long long> mx;
  const double* d = device_in(uvw_block, (size_t)3 * num_coords, in, st);
  if (!d || u.ensure(num_coords) || v.ensure(num_coords) || w.ensure(num_coords) || mx.ensure(1)) return 0.;
  cudaMemsetAsync(mx.p, 0, sizeof(unsigned long long), st);
  if (launch_ms_coords(d, num_coords, u.p, v.p, w.p, mx.p, st)) return 0.;
  unsigned long long bits = 0;
  u.download(uu, num_coords, st);
  v.download(vv, num_coords, st);
  w.download(ww, num_coords, st);
  copy_async(&bits, mx.p, sizeof(bits), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  double m;
  memcpy(&m, &bits, sizeof(m));
  return ceil(m);
}

unsigned long rlf_ms_read_flag(const uint8_t* flag_block, unsigned int num_coords, unsigned int num_channels,
                               unsigned int num_pols, uint8_t* flag) {
  cudaStream_t st;
  if (lib_stream(&st) || num_coords == 0 || num_channels == 0) return 0;
  const size_t nv = (size_t)num_coords * num_channels;
  DevBuf<uint8_t> in, out;
  DevBuf<unsigned long long> cnt;
  const uint8_t* d = device_in(flag_block, nv * num_pols, in, st);
  if (!d || out.ensure(nv) || cnt.ensure(1)) return 0;
  cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), st);
  if (launch_ms_flags(d, num_coords, (int)num_channels, (int)num_pols, out.p, cnt.p, st)) return 0;
  unsigned long long c = 0;
  out.download(flag, nv, st);
  copy_async(&c, cnt.p, sizeof(c), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return (unsigned long)c;
}

int rlf_ms_read_vis(const float* data_block, unsigned int num_coords, unsigned int num_channels, unsigned int num_pols,
                    double* vis_c128) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  if (num_coords == 0 || num_channels == 0) return 0;
  const size_t nv = (size_t)num_coords * num_channels;
  DevBuf<float2> in;
  DevBuf<double2> out;
  const float2* d = device_in(reinterpret_cast<const float2*>(data_block), nv * num_pols, in, st);
  if (!d) return 1;
  double2* o = static_cast<double2*>(mapped_host(vis_c128));
  if (o) __atomic_add_fetch(&g_d2h_bytes, (unsigned long long)nv * sizeof(double2), __ATOMIC_RELAXED);
  else { RLF_OK(out.ensure(nv)); o = out.p; }
  RLF_OK(launch_ms_vis_c128(d, num_coords, (int)num_channels, (int)num_pols, o, st));
  if (o == out.p) RLF_OK(out.download(reinterpret_cast<double2*>(vis_c128), nv, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_ms_read_sigma2(const float* sigma_block, unsigned int num_coords, unsigned int num_channels,
                       float sigma2_theory, float* sigma2_vis) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const size_t nv = (size_t)num_coords * num_channels;
  if (nv == 0) return 0;
  DevBuf<float> in, out;
  const float* d = sigma_block ? device_in(sigma_block, num_coords, in, st) : nullptr;
  if (sigma_block && !d) return 1;
  RLF_OK(out.ensure(nv));
  // without a SIGMA column every entry takes the theoretical variance (RadioLensfit2.cpp:258-263)
  RLF_OK(launch_ms_sigma2(d, d ? num_coords : 0, (long long)nv, sigma2_theory, out.p, st));
  RLF_OK(out.download(sigma2_vis, nv, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_ms_write_vis(const double* vis_c128, unsigned int num_coords, unsigned int num_channels, float* data_block) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const size_t nv = (size_t)num_coords * num_channels;
  if (nv == 0) return 0;
  DevBuf<double2> in;
  DevBuf<float2> out;
  const double2* d = device_in(reinterpret_cast<const double2*>(vis_c128), nv, in, st);
  if (!d) return 1;
  float2* o = static_cast<float2*>(mapped_host(data_block));
  if (o) __atomic_add_fetch(&g_d2h_bytes, (unsigned long long)nv * sizeof(float2), __ATOMIC_RELAXED);
  else { RLF_OK(out.ensure(nv)); o = out.p; }
  RLF_OK(launch_ms_write(d, num_coords, (int)num_channels, o, st));
  if (o == out.p) RLF_OK(out.download(reinterpret_cast<float2*>(data_block), nv, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_get_vis(rlf_observation* obs, double* data_c128, double* sky_c128) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(obs_get_c128(obs, data_c128, false, st));
  RLF_OK(obs_get_c128(obs, sky_c128, true, st));
  return 0;
}

}  // extern "C"

namespace rlf {
// data (use_e = 1, sheared models) or sky model (use_e = 0, round models) += the models of n_gal
// galaxies; FP32 observations with evenly spaced channels take the batched kernel, the others
// the per-visibility kernels
static int add_models(rlf_observation* obs, const GalaxyParams* dg, int n_gal, int use_e, int gaussian,
                      cudaStream_t st) {
  const Observation o = obs->view();
  const int chunk = 256;  // galaxies per launch keeps each launch short
  int bc = -1;
  if (obs->precision != RLF_F64) {
    bc = batch_set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), obs->max_delay_m, st);
    if (bc > 0) return bc;
    if (bc == 0 && !obs->rows.p) {
      RLF_OK(obs->rows.ensure(obs->n_rows));
      RLF_OK(launch_row_table(obs->n_rows, obs->uu.p, obs->vv.p, obs->ww.p, obs->rows.p, st));
    }
  }
  for (int g0 = 0; g0 < n_gal; g0 += chunk) {
    const int gn = std::min(chunk, n_gal - g0);
    if (obs->precision == RLF_F64) {
      RLF_OK(launch_sky_model_f64(o, use_e ? obs->data64.p : obs->sky64.p, dg + g0, gn, use_e, gaussian, st));
    } else if (bc == 0) {
      RLF_OK(launch_model_sum_batch(obs->n_rows, obs->rows.p, use_e ? obs->data32.p : obs->sky32.p, dg + g0, gn,
                                    use_e, gaussian, st));
    } else {
      RLF_OK(launch_sky_model_mixed(o, use_e ? obs->data32.p : obs->sky32.p, dg + g0, gn, use_e, gaussian, st));
    }
  }
  return 0;
}
}  // namespace rlf

extern "C" {

int rlf_obs_simulate(rlf_observation* obs, int n_gal, const double* flux, const double* scale, const double* e1,
                     const double* e2, const double* l, const double* m, double noise_sigma, uint64_t seed,
                     int gaussian) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  std::vector<GalaxyParams> g = make_gals(n_gal, flux, scale, e1, e2, l, m, obs->len, 0);
  DevBuf<GalaxyParams> dg;
  RLF_OK(dg.upload(g.data(), g.size(), st));
  RLF_OK(add_models(obs, dg.p, n_gal, 1, gaussian, st));
  if (noise_sigma > 0) {
    if (obs->precision == RLF_F64)
      k_add_noise<double2><<<4096, 256, 0, st>>>(obs->n_vis, obs->data64.p, noise_sigma, seed, nullptr, obs->n_rows);
    else
      k_add_noise<float2><<<4096, 256, 0, st>>>(obs->n_vis, obs->data32.p, noise_sigma, seed, obs->perm.p, obs->n_rows);
    RLF_CUDA(cudaGetLastError());
  }
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_sky_model(rlf_observation* obs, int n_gal, const double* flux, const double* scale, const double* l,
                      const double* m, int gaussian) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  std::vector<GalaxyParams> g = make_gals(n_gal, flux, scale, nullptr, nullptr, l, m, obs->len, 0);
  DevBuf<GalaxyParams> dg;
  RLF_OK(dg.upload(g.data(), g.size(), st));
  RLF_OK(add_models(obs, dg.p, n_gal, 0, gaussian, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_snapshot(rlf_observation* obs) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const size_t n = (size_t)obs->n_vis;
  if (obs->precision == RLF_F64) {
    RLF_OK(obs->data64_0.ensure(n));
    RLF_OK(obs->sky64_0.ensure(n));
    RLF_CUDA(copy_async(obs->data64_0.p, obs->data64.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    RLF_CUDA(copy_async(obs->sky64_0.p, obs->sky64.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  } else {
    RLF_OK(obs->data32_0.ensure(n));
    RLF_OK(obs->sky32_0.ensure(n));
    RLF_CUDA(copy_async(obs->data32_0.p, obs->data32.p, n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    RLF_CUDA(copy_async(obs->sky32_0.p, obs->sky32.p, n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  }
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_restore(rlf_observation* obs) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const size_t n = (size_t)obs->n_vis;
  if (obs->precision == RLF_F64) {
    if (!obs->data64_0.p) return 1;
    RLF_CUDA(copy_async(obs->data64.p, obs->data64_0.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    RLF_CUDA(copy_async(obs->sky64.p, obs->sky64_0.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  } else {
    if (!obs->data32_0.p) return 1;
    RLF_CUDA(copy_async(obs->data32.p, obs->data32_0.p, n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
    RLF_CUDA(copy_async(obs->sky32.p, obs->sky32_0.p, n * sizeof(float2), cudaMemcpyDeviceToDevice, st));
  }
  return 0;
}

int rlf_obs_process(rlf_observation* obs, int n_gal, const double* flux, const double* scale, const double* l,
                    const double* m, int numr, const double* ro, const rlf_options* opt, rlf_fit_result* out,
                    int* n_bad) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  rlf_options o = opt ? *opt : g_lib.opt;
  return process(obs, n_gal, flux, scale, l, m, numr, ro, o, out, n_bad, st);
}

int rlf_obs_extract(rlf_observation* obs, int n_gal, const double* flux, const double* scale, const double* l,
                    const double* m, int batch, double* facets, int stride, int* ncoords) {
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  const unsigned fmax = rlf::facet_size(kRMax, obs->len);
  std::vector<GalaxyParams> gals = make_gals(n_gal, flux, scale, nullptr, nullptr, l, m, obs->len, fmax);
  std::vector<int> order(n_gal);
  for (int i = 0; i < n_gal; ++i) order[i] = i;
  rlf_options o = g_lib.opt;
  o.batch = batch;
  std::vector<FitOut> out;
  std::vector<double> ro(kMaxNodes, 1.0);
  return run_pass(obs, gals, order, 24, ro.data(), o, out, st, nullptr, facets, ncoords, stride);
}

// -------------------------------------------------------------- channel shards
// The reference's MPI decomposition (data_processing-mpi.c:65-216): every rank holds the
// visibilities of its own channels, extracts every galaxy of a round into un-averaged facet sums
// over those channels, the sums of all ranks are added (data_processing-mpi.c:95-124), the owner of
// a galaxy fits the summed facet and every rank removes the fitted galaxies from its own channels
// (:169-210).  These three steps are the entry points below; the exchange between them is the
// caller's (radiolensfit2_gb300.shard: torch.distributed all-reduce and all-gather).

int rlf_obs_facet_partials(rlf_observation* obs, int n_gal, const double* flux, const double* scale,
                           const double* l, const double* m, double* out, int stride) {
  if (!obs || n_gal < 0 || (n_gal && !out)) return 1;
  if (n_gal == 0) return 0;
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  const unsigned fmax = rlf::facet_size(kRMax, obs->len);
  if ((unsigned)stride < fmax * fmax) { fprintf(stderr, "rlf: partials stride %d below %u\n", stride, fmax * fmax); return 1; }
  std::vector<GalaxyParams> gals = make_gals(n_gal, flux, scale, nullptr, nullptr, l, m, obs->len, fmax);
  std::vector<int> order(n_gal);
  for (int i = 0; i < n_gal; ++i) order[i] = i;
  // every galaxy extracted against the same data (no removal in between): FP32 observations take the
  // sequential batch extraction's first round for sub-batches of galaxies, FP64 ones (and galaxies
  // with facets beyond the batched kernels) one pass per galaxy
  rlf_options o = g_lib.opt;
  o.batch = kSeqMaxGal;
  std::vector<FitOut> res;
  std::vector<double> ro(kMaxNodes, 1.0);
  return run_pass(obs, gals, order, 24, ro.data(), o, res, st, nullptr, nullptr, nullptr, 0, out, stride);
}

int rlf_fit_partials(int n_gal, const double* partials, int stride, const double* flux, const double* scale,
                     double len, int numr, const double* ro, const rlf_options* opt, rlf_fit_result* out) {
  if (n_gal < 0 || (n_gal && (!partials || !out))) return 1;
  if (n_gal == 0) return 0;
  if (numr < 2 || numr > kMaxNodes) { fprintf(stderr, "rlf: %d scalelength nodes unsupported\n", numr); return 1; }
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  const rlf_options o = opt ? *opt : g_lib.opt;
  const Precision fprec = o.fit_precision == RLF_MIXED ? kMixed : kF64;
  const unsigned fmax = rlf::facet_size(kRMax, len);
  if ((unsigned)stride < fmax * fmax) { fprintf(stderr, "rlf: partials stride %d below %u\n", stride, fmax * fmax); return 1; }
  const std::vector<double> zero(n_gal, 0.0);  // positions play no part in the fit
  std::vector<GalaxyParams> gals = make_gals(n_gal, flux, scale, nullptr, nullptr, zero.data(), zero.data(), len, fmax);
  // sums as k_facet_finalize takes them: per galaxy [re (F^2) | im (F^2)] at 2 * stride; ss, sw planes
  std::vector<double> sums((size_t)n_gal * 2 * stride, 0.0), ss((size_t)n_gal * stride, 0.0), sw((size_t)n_gal * stride, 0.0);
  std::vector<int> facets(n_gal), offs(n_gal);
  std::vector<double> rprior((size_t)n_gal * kMaxNodes, 0.0);
  int max_cells = 0;
  for (int g = 0; g < n_gal; ++g) {
    const int F = gals[g].facet, nc = F * F;
    facets[g] = F;
    max_cells = std::max(max_cells, nc);
    const double* row = partials + (size_t)g * 4 * stride;
    std::copy(row, row + nc, sums.begin() + (size_t)g * 2 * stride);
    std::copy(row + stride, row + stride + nc, sums.begin() + (size_t)g * 2 * stride + nc);
    std::copy(row + 2 * stride, row + 2 * stride + nc, ss.begin() + (size_t)g * stride);
    std::copy(row + 3 * stride, row + 3 * stride + nc, sw.begin() + (size_t)g * stride);
    const double mu = scale_mean(flux[g]);
    for (int r = 1; r < numr; ++r) rprior[(size_t)g * kMaxNodes + r] = rfunc(mu, kRStd, ro[r]);
  }
  for (int g = 0; g < n_gal; ++g) offs[g] = g * max_cells;
  DevBuf<double> dsums, dss, dsw, dprior;
  DevBuf<const double*> pss, psw;
  DevBuf<int> dfac, doff, dnc, dqueue;
  RLF_OK(dsums.upload(sums.data(), sums.size(), st));
  RLF_OK(dss.upload(ss.data(), ss.size(), st));
  RLF_OK(dsw.upload(sw.data(), sw.size(), st));
  std::vector<const double*> pssh(n_gal), pswh(n_gal);
  for (int g = 0; g < n_gal; ++g) {
    pssh[g] = dss.p + (size_t)g * stride;
    pswh[g] = dsw.p + (size_t)g * stride;
  }
  RLF_OK(pss.upload(pssh.data(), n_gal, st));
  RLF_OK(psw.upload(pswh.data(), n_gal, st));
  RLF_OK(dfac.upload(facets.data(), n_gal, st));
  RLF_OK(doff.upload(offs.data(), n_gal, st));
  RLF_OK(dnc.ensure(n_gal));
  RLF_OK(dprior.upload(rprior.data(), rprior.size(), st));
  RLF_OK(dqueue.ensure(1));
  const size_t esz = fprec == kF64 ? sizeof(double) : sizeof(float);
  const size_t plane = (size_t)n_gal * max_cells * esz;
  DevBuf<unsigned char> cells;
  RLF_OK(cells.ensure(5 * plane));
  FacetOut fo;
  fo.offset = doff.p;
  fo.ncoords = dnc.p;
  fo.gu = cells.p; fo.gv = cells.p + plane; fo.dre = cells.p + 2 * plane; fo.dim = cells.p + 3 * plane;
  fo.sig2 = cells.p + 4 * plane;
  fo.as_float = fprec == kMixed;
  RLF_OK(launch_facet_finalize(n_gal, dfac.p, dsums.p, 1, 2LL * stride, pss.p, psw.p, len, fo, st));
  FitConfigHost fc;
  memset(&fc, 0, sizeof(fc));
  fc.numr = numr;
  fc.gaussian = o.gaussian;
  fc.np_max = kNpMax;
  for (int i = 0; i < numr; ++i) fc.ro[i] = ro[i];
  RLF_OK(fit_set_config(fc, st));
  DevBuf<FitOut> dout;
  RLF_OK(dout.ensure(n_gal));
  RLF_CUDA(cudaMemsetAsync(dout.p, 0, n_gal * sizeof(FitOut), st));
  DevBuf<SampleSlot> bslot;
  DevBuf<double> bL;
  DevBuf<int> berr, bflag, bnewton, bdone;
  RLF_OK(bslot.ensure(n_gal));
  RLF_OK(bL.ensure((size_t)n_gal * 2 * kBoardCap));
  RLF_OK(berr.ensure((size_t)n_gal * 2 * kBoardCap));
  RLF_OK(bflag.ensure((size_t)n_gal * 2 * kBoardCap));
  RLF_OK(bnewton.ensure(n_gal));
  RLF_OK(bdone.ensure(1));
  RLF_CUDA(cudaMemsetAsync(bslot.p, 0, (size_t)n_gal * sizeof(SampleSlot), st));
  RLF_CUDA(cudaMemsetAsync(bflag.p, 0, (size_t)n_gal * 2 * kBoardCap * sizeof(int), st));
  RLF_CUDA(cudaMemsetAsync(bnewton.p, 0, (size_t)n_gal * sizeof(int), st));
  RLF_CUDA(cudaMemsetAsync(bdone.p, 0, sizeof(int), st));
  RLF_CUDA(cudaMemsetAsync(dqueue.p, 0, sizeof(int), st));
  FacetBatch fb{};
  fb.n_gal = n_gal;
  fb.max_cells = max_cells;
  fb.offset = doff.p;
  fb.count = dnc.p;
  fb.gu = fo.gu; fb.gv = fo.gv; fb.dre = fo.dre; fb.dim = fo.dim; fb.sig2 = fo.sig2;
  fb.rprior = dprior.p;
  fb.start = nullptr;
  fb.active = nullptr;
  fb.out = dout.p;
  fb.queue = dqueue.p;
  fb.trace = nullptr;
  fb.trace_cap = 0;
  fb.board.slot = bslot.p;
  fb.board.L = bL.p;
  fb.board.err = berr.p;
  fb.board.flag = bflag.p;
  fb.board.newton = bnewton.p;
  fb.board.done_gal = bdone.p;
  fb.board.wait_ns = o.board_wait_us > 0 ? (unsigned long long)o.board_wait_us * 1000ull : 0ull;
  int sms = 0, dev = 0;
  RLF_CUDA(cudaGetDevice(&dev));
  RLF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int grid = o.fit_ctas_per_sm > 0 ? std::min(fit_max_grid(fprec), sms * o.fit_ctas_per_sm) : fit_max_grid(fprec);
  RLF_OK(fit_launch(fb, fprec, grid, st));
  std::vector<FitOut> h(n_gal);
  RLF_OK(dout.download(h.data(), n_gal, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  for (int g = 0; g < n_gal; ++g) memcpy(&out[g], &h[g], sizeof(rlf_fit_result));
  return 0;
}

int rlf_obs_remove(rlf_observation* obs, int n_gal, const double* flux, const double* scale, const double* l,
                   const double* m, const rlf_fit_result* fits) {
  if (!obs || n_gal < 0 || (n_gal && !fits)) return 1;
  if (n_gal == 0) return 0;
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  RLF_OK(set_channels(obs->n_ch, obs->wavenumbers.data(), obs->spec.data(), st));
  const unsigned fmax = rlf::facet_size(kRMax, obs->len);
  std::vector<GalaxyParams> gals = make_gals(n_gal, flux, scale, nullptr, nullptr, l, m, obs->len, fmax);
  std::vector<FitOut> f(n_gal);
  for (int g = 0; g < n_gal; ++g) memcpy(&f[g], &fits[g], sizeof(rlf_fit_result));
  DevBuf<GalaxyParams> dg;
  DevBuf<FitOut> df;
  RLF_OK(dg.upload(gals.data(), n_gal, st));
  RLF_OK(df.upload(f.data(), n_gal, st));
  const Observation o = obs->view();
  // in catalogue order, one galaxy at a time (data_processing.c:109-135), bad fits skipped
  for (int g = 0; g < n_gal; ++g) {
    const double* e12 = &df.p[g].e1;
    const int* err = &df.p[g].error;
    if (obs->precision == RLF_F64)
      RLF_OK(launch_remove_f64(o, obs->data64.p, obs->sky64.p, dg.p + g, e12, err, g_lib.opt.gaussian, st));
    else
      RLF_OK(launch_remove_mixed(o, obs->data32.p, obs->sky32.p, dg.p + g, e12, err, g_lib.opt.gaussian, st));
  }
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_obs_last_stats(rlf_observation* obs, long long* stats) {
  if (!obs || !stats) return 1;
  for (int k = 0; k < RLF_NSTATS; ++k) stats[k] = obs->stats[k];
  return 0;
}

int rlf_obs_last_timing(rlf_observation* obs, double* ms4) {
  for (int k = 0; k < 4; ++k) ms4[k] = obs->ms[k];
  return 0;
}

// =========================================================== reference-named ABI
// evaluate_uv_grid.c:50-55
unsigned int facet_size(double theta_med, double len) { return rlf::facet_size(theta_med, len); }

// galaxy_visibilities.c:40-53
double gaussian_shape(double k1, double k2, double scale_factor, double wave_factor) {
  return rlf::gaussian_shape(k1, k2, scale_factor, wave_factor);
}
double sersic_shape(double k1, double k2, double scale_factor, double wave_factor) {
  return rlf::sersic_shape(k1, k2, scale_factor, wave_factor);
}

// likelihood.c:376-421
double marginalise_over_position_shift(double x) { return rlf::position_marginal(x); }

// distributions.c:59-87
double rfunc(const double mu, const double sigma, double r) { return rlf::rfunc(mu, sigma, r); }
double scale_mean(double flux) { return rlf::scale_mean(flux); }

// evaluate_uv_grid.c:58-109 (single process)
unsigned int evaluate_uv_grid_size(int rank, int nprocs, double len, double* wavenumbers, unsigned int num_channels,
                                   unsigned int ncoords, double* u, double* v, unsigned int sizeg, bool* flag) {
  (void)rank;
  (void)nprocs;
  cudaStream_t st;
  if (lib_stream(&st)) return 0;
  if (set_channels((int)num_channels, wavenumbers, nullptr, st)) return 0;
  const size_t nv = (size_t)num_channels * ncoords;
  Observation o;
  o.n_rows = (int)ncoords; o.n_ch = (int)num_channels; o.lay.s_row = 1; o.lay.s_ch = ncoords;
  if (g_lib.d0.upload(u, ncoords, st) || g_lib.d1.upload(v, ncoords, st)) return 0;
  if (g_lib.b0.upload(reinterpret_cast<const uint8_t*>(flag), nv, st)) return 0;
  if (g_lib.u16.ensure(nv) || g_lib.ucount.ensure((size_t)sizeg * sizeg + 1)) return 0;
  o.uu = g_lib.d0.p; o.vv = g_lib.d1.p; o.ww = g_lib.d1.p; o.len = len;
  if (launch_cell_index(o, g_lib.b0.p, sizeg, g_lib.u16.p, st)) return 0;
  if (launch_count_cells(o, g_lib.u16.p, sizeg, g_lib.ucount.p, st)) return 0;
  unsigned n = 0;
  copy_async(&n, g_lib.ucount.p + (size_t)sizeg * sizeg, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return n;
}

// evaluate_uv_grid.c:113-133
unsigned int evaluate_facet_coords(double* grid_u, double* grid_v, double len, unsigned int sizeg, double* count_w) {
  cudaStream_t st;
  if (lib_stream(&st)) return 0;
  const size_t nc = (size_t)sizeg * sizeg;
  if (g_lib.d0.upload(count_w, nc, st) || g_lib.d1.ensure(nc) || g_lib.d2.ensure(nc) || g_lib.ucount.ensure(1)) return 0;
  if (launch_facet_coords(g_lib.d1.p, g_lib.d2.p, len, sizeg, g_lib.d0.p, g_lib.ucount.p, st)) return 0;
  unsigned n = 0;
  copy_async(&n, g_lib.ucount.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  copy_async(grid_u, g_lib.d1.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  copy_async(grid_v, g_lib.d2.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return n;
}

// evaluate_uv_grid.c:143-211 (non-MPI branch)
void gridding_visibilities(double* wavenumbers, unsigned int num_channels, unsigned int ncoords, double* u, double* v,
                           complexd* vis, float* sigma2, double len, unsigned int sizeg, complexd* new_vis,
                           double* new_sigma2, bool* flag, double* sum_w) {
  cudaStream_t st;
  if (lib_stream(&st)) return;
  if (set_channels((int)num_channels, wavenumbers, nullptr, st)) return;
  const size_t nv = (size_t)num_channels * ncoords, nc = (size_t)sizeg * sizeg;
  const int n_part = grid_partial_blocks((int)ncoords);
  Observation o;
  o.n_rows = (int)ncoords; o.n_ch = (int)num_channels; o.lay.s_row = 1; o.lay.s_ch = ncoords; o.len = len;
  if (g_lib.d0.upload(u, ncoords, st) || g_lib.d1.upload(v, ncoords, st)) return;
  if (g_lib.c0.upload(reinterpret_cast<const double2*>(vis), nv, st)) return;
  if (g_lib.f0.upload(sigma2, nv, st)) return;
  if (g_lib.b0.upload(reinterpret_cast<const uint8_t*>(flag), nv, st)) return;
  if (g_lib.d2.ensure((size_t)n_part * 4 * nc + 4 * nc) || g_lib.c1.ensure(nc) || g_lib.d3.ensure(nc) ||
      g_lib.d4.ensure(nc))
    return;
  o.uu = g_lib.d0.p; o.vv = g_lib.d1.p; o.ww = g_lib.d1.p;
  if (launch_grid_vis_f64(o, g_lib.c0.p, g_lib.f0.p, g_lib.b0.p, sizeg, g_lib.d2.p, n_part, st)) return;
  if (launch_grid_vis_finalize(g_lib.d2.p, n_part, sizeg, g_lib.c1.p, g_lib.d3.p, g_lib.d4.p, st)) return;
  std::vector<double> sw(nc);
  copy_async(sw.data(), g_lib.d4.p, nc * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  size_t n = 0;
  for (size_t p = 0; p < nc; ++p) n += sw[p] != 0.0;
  memcpy(sum_w, sw.data(), nc * sizeof(double));
  copy_async(new_vis, g_lib.c1.p, n * sizeof(double2), cudaMemcpyDeviceToHost, st);
  copy_async(new_sigma2, g_lib.d3.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
}

// evaluate_uv_grid.c:216-230
void average_facets(unsigned long int size, complexd* grid_vis, double* grid_sigma2, double* sum_w) {
  cudaStream_t st;
  if (lib_stream(&st)) return;
  if (g_lib.c0.upload(reinterpret_cast<const double2*>(grid_vis), size, st) ||
      g_lib.d0.upload(grid_sigma2, size, st) || g_lib.d1.upload(sum_w, size, st))
    return;
  if (launch_average_facets((long long)size, g_lib.c0.p, g_lib.d0.p, g_lib.d1.p, st)) return;
  copy_async(grid_vis, g_lib.c0.p, size * sizeof(double2), cudaMemcpyDeviceToHost, st);
  copy_async(grid_sigma2, g_lib.d0.p, size * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
}

// galaxy_visibilities.c:59-91
void model_galaxy_visibilities_at_zero(double e1, double e2, double scale, unsigned int num_coords, double* grid_u,
                                       double* grid_v, const double* sigma2, double* Modvis) {
  cudaStream_t st;
  if (lib_stream(&st)) return;
  if (g_lib.d0.upload(grid_u, num_coords, st) || g_lib.d1.upload(grid_v, num_coords, st) ||
      g_lib.d2.upload(sigma2, num_coords, st) || g_lib.d3.ensure(num_coords))
    return;
  if (launch_model_at_zero(e1, e2, scale, (int)num_coords, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, g_lib.d3.p,
                           g_lib.opt.gaussian, st))
    return;
  copy_async(Modvis, g_lib.d3.p, num_coords * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
}

// galaxy_visibilities.c:154-190
void data_galaxy_visibilities(double spectra, double wavenumber, double band_factor, double acc_time, double e1,
                              double e2, double scale, double flux, double l, double m, unsigned int num_coords,
                              double* uu_metres, double* vv_metres, double* ww_metres, complexd* vis) {
  (void)band_factor;
  (void)acc_time;  // smearing terms are commented out in the reference (galaxy_visibilities.c:179)
  cudaStream_t st;
  if (lib_stream(&st)) return;
  if (g_lib.d0.upload(uu_metres, num_coords, st) || g_lib.d1.upload(vv_metres, num_coords, st) ||
      g_lib.d2.upload(ww_metres, num_coords, st) || g_lib.c0.ensure(num_coords))
    return;
  if (launch_galaxy_vis_channel((int)num_coords, spectra, wavenumber, e1, e2, scale, flux, l, m, g_lib.d0.p,
                                g_lib.d1.p, g_lib.d2.p, g_lib.c0.p, g_lib.opt.gaussian, st))
    return;
  copy_async(vis, g_lib.c0.p, num_coords * sizeof(double2), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
}

// galaxy_visibilities.c:244-270
void data_visibilities_phase_shift(double wavenumber, double l, double m, unsigned int num_coords, double* uu_metres,
                                   double* vv_metres, double* ww_metres, complexd* vis) {
  cudaStream_t st;
  if (lib_stream(&st)) return;
  if (g_lib.d0.upload(uu_metres, num_coords, st) || g_lib.d1.upload(vv_metres, num_coords, st) ||
      g_lib.d2.upload(ww_metres, num_coords, st) ||
      g_lib.c0.upload(reinterpret_cast<const double2*>(vis), num_coords, st))
    return;
  if (launch_phase_shift_channel((int)num_coords, wavenumber, l, m, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, g_lib.c0.p,
                                 st))
    return;
  copy_async(vis, g_lib.c0.p, num_coords * sizeof(double2), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
}

// likelihood.c:156-187
double loglikelihood_r(double ee1, double ee2, double scale, unsigned long int n_uv_coords, const double* variance,
                       double* grid_u, double* grid_v, complexd* visData, double* visM) {
  cudaStream_t st;
  if (lib_stream(&st)) return kBad;
  const size_t n = n_uv_coords;
  std::vector<double> re(n ? n : 1), im(n ? n : 1);
  for (size_t i = 0; i < n; ++i) { re[i] = visData[i].real; im[i] = visData[i].imag; }
  if (g_lib.d0.upload(grid_u, n, st) || g_lib.d1.upload(grid_v, n, st) || g_lib.d2.upload(re.data(), n, st) ||
      g_lib.d3.upload(im.data(), n, st) || g_lib.d4.upload(variance, n, st) || g_lib.d5.ensure(n) ||
      g_lib.d6.ensure(2))
    return kBad;
  if (launch_loglikelihood_r(ee1, ee2, scale, (int)n, g_lib.d4.p, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, g_lib.d3.p,
                             g_lib.d5.p, g_lib.d6.p, g_lib.opt.gaussian, st))
    return kBad;
  double L[2];
  copy_async(L, g_lib.d6.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  copy_async(visM, g_lib.d5.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  return L[0];
}

// likelihood.c:194-358
int cross_correlation(unsigned long int n_uv_coords, double* grid_u, double* grid_v, complexd* visData,
                      double* visMod, double* ho, double* det_sigma) {
  cudaStream_t st;
  if (lib_stream(&st)) return 1;
  const size_t n = n_uv_coords;
  std::vector<double> re(n ? n : 1), im(n ? n : 1);
  for (size_t i = 0; i < n; ++i) { re[i] = visData[i].real; im[i] = visData[i].imag; }
  if (g_lib.d0.upload(grid_u, n, st) || g_lib.d1.upload(grid_v, n, st) || g_lib.d2.upload(re.data(), n, st) ||
      g_lib.d3.upload(im.data(), n, st) || g_lib.d4.upload(visMod, n, st) || g_lib.d6.ensure(4))
    return 1;
  if (launch_cross_correlation((int)n, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, g_lib.d3.p, g_lib.d4.p, g_lib.d6.p, st))
    return 1;
  double r[4];
  copy_async(r, g_lib.d6.p, 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *ho = r[0];
  *det_sigma = r[1];
  return (int)r[2];
}

// likelihood.c:106-149
double loglikelihood(void* params, double ee1, double ee2, int* error) {
  likelihood_params* par = (likelihood_params*)params;
  cudaStream_t st;
  *error = 1;
  if (lib_stream(&st)) return kBad;
  OneFacet f;
  if (f.load(par, st) || g_lib.d6.ensure(2)) return kBad;
  if (launch_loglikelihood(f.fb, ee1, ee2, g_lib.d6.p, nullptr, st)) return kBad;
  double r[2];
  copy_async(r, g_lib.d6.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *error = (int)r[1];
  return r[0];
}

// likelihood.c:87-100
double f_likelihood(const rlf_gsl_vector_layout* v, void* params) {
  int error = 0;
  const double e1 = v->data[0], e2 = v->data[v->stride];
  double L;
  if (e1 * e1 + e2 * e2 < 0.65) L = loglikelihood(params, e1, e2, &error);
  else L = -1.e+10;
  return -L;
}

// likelihood.c:428-554
void likelihood_sampling(double* mes_e1, double* mes_e2, double maxL, void* params, int np_max, double* var_e1,
                         double* var_e2, double* oneDimvar) {
  likelihood_params* par = (likelihood_params*)params;
  cudaStream_t st;
  if (lib_stream(&st)) return;
  OneFacet f;
  if (f.load(par, st) || g_lib.d6.ensure(5)) return;
  if (launch_likelihood_sampling(f.fb, *mes_e1, *mes_e2, maxL, np_max, g_lib.d6.p, st)) return;
  double r[5];
  copy_async(r, g_lib.d6.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *mes_e1 = r[0]; *mes_e2 = r[1]; *var_e1 = r[2]; *var_e2 = r[3]; *oneDimvar = r[4];
}

// marginalise_r.c:29-64
void rlf_set_posterior_values(int numR, double* L_r, double* rprior, double* Ro, double* xmarvals, double* ymarvals,
                              int* numvals) {
  cudaStream_t st;
  *numvals = 0;
  if (lib_stream(&st)) return;
  if (g_lib.d0.upload(L_r, numR, st) || g_lib.d1.upload(rprior, numR, st) || g_lib.d2.upload(Ro, numR, st) ||
      g_lib.d3.ensure(numR) || g_lib.d4.ensure(numR) || g_lib.i0.ensure(1))
    return;
  if (launch_set_posterior_values(numR, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, g_lib.d3.p, g_lib.d4.p, g_lib.i0.p, st))
    return;
  int n = 0;
  copy_async(&n, g_lib.i0.p, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  copy_async(xmarvals, g_lib.d3.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  copy_async(ymarvals, g_lib.d4.p, n * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *numvals = n;
}

// marginalise_r.c:81-223
double rlf_marginalise_posterior_r(int num_marvals, double* xmarvals, double* ymarvals) {
  cudaStream_t st;
  if (lib_stream(&st)) return kBad;
  if (num_marvals < 3 || num_marvals > kMaxNodes) return kBad;
  if (g_lib.d0.upload(xmarvals, num_marvals, st) || g_lib.d1.upload(ymarvals, num_marvals, st) || g_lib.d2.ensure(1))
    return kBad;
  if (launch_marginalise_posterior_r(num_marvals, g_lib.d0.p, g_lib.d1.p, g_lib.d2.p, st)) return kBad;
  double L = kBad;
  copy_async(&L, g_lib.d2.p, sizeof(double), cudaMemcpyDeviceToHost, st);
  copy_async(ymarvals, g_lib.d1.p, num_marvals * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  g_marf_x.assign(xmarvals, xmarvals + num_marvals);
  g_marf_y.assign(ymarvals, ymarvals + num_marvals);
  return L;
}

// marginalise_r.c:231-238: exp of the natural cubic spline through the last marginalised points
double rlf_marf(double x, void* params) {
  (void)params;
  const int n = (int)g_marf_x.size();
  if (n < 3 || x < g_marf_x[0] || x > g_marf_x[n - 1]) return 0.;
  std::vector<double> c(n, 0.0), diag(n), off(n), g(n), alpha(n), gamma(n), z(n);
  const int m = n - 2;
  for (int i = 0; i < m; i++) {
    const double h_i = g_marf_x[i + 1] - g_marf_x[i], h_ip1 = g_marf_x[i + 2] - g_marf_x[i + 1];
    off[i] = h_ip1;
    diag[i] = 2.0 * (h_ip1 + h_i);
    g[i] = 3.0 * ((g_marf_y[i + 2] - g_marf_y[i + 1]) / h_ip1 - (g_marf_y[i + 1] - g_marf_y[i]) / h_i);
  }
  if (m == 1) c[1] = g[0] / diag[0];
  else {
    alpha[0] = diag[0];
    gamma[0] = off[0] / alpha[0];
    for (int i = 1; i < m - 1; i++) { alpha[i] = diag[i] - off[i - 1] * gamma[i - 1]; gamma[i] = off[i] / alpha[i]; }
    alpha[m - 1] = diag[m - 1] - off[m - 2] * gamma[m - 2];
    z[0] = g[0];
    for (int i = 1; i < m; i++) z[i] = g[i] - gamma[i - 1] * z[i - 1];
    for (int i = 0; i < m; i++) z[i] /= alpha[i];
    c[m] = z[m - 1];
    for (int k = m - 1; k-- > 0;) c[k + 1] = z[k] - gamma[k] * c[k + 2];
  }
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) { int mid = (lo + hi) / 2; if (g_marf_x[mid] > x) hi = mid; else lo = mid; }
  const double dx = g_marf_x[lo + 1] - g_marf_x[lo], dy = g_marf_y[lo + 1] - g_marf_y[lo], delx = x - g_marf_x[lo];
  const double b = dy / dx - dx * (c[lo + 1] + 2.0 * c[lo]) / 3.0, d = (c[lo + 1] - c[lo]) / (3.0 * dx);
  return exp(g_marf_y[lo] + delx * (b + delx * (c[lo] + delx * d)));
}

// galaxy_fitting.c:41-117
int source_fitting(int rank, likelihood_params* par, double* mes_e1, double* mes_e2, double* var_e1, double* var_e2,
                   double* oneDimvar, double* maxL) {
  cudaStream_t st;
  if (lib_stream(&st)) return 1;
  OneFacet f;
  if (f.load(par, st) || g_lib.fo.ensure(1) || g_lib.i0.ensure(1)) return 1;
  cudaMemsetAsync(g_lib.i0.p, 0, sizeof(int), st);
  f.fb.out = g_lib.fo.p;
  f.fb.queue = g_lib.i0.p;
  if (fit_launch(f.fb, kF64, 1, st)) return 1;
  FitOut o;
  copy_async(&o, g_lib.fo.p, sizeof(FitOut), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  *mes_e1 = o.e1; *mes_e2 = o.e2; *var_e1 = o.var_e1; *var_e2 = o.var_e2; *oneDimvar = o.oneDimvar; *maxL = o.maxL;
  if (g_lib.opt.verbose) {
    if (o.maxL > -1.e+10) printf("rank %d: average: %f,%f variance: %e,%e 1Dvar: %e\n", rank, o.e1, o.e2, o.var_e1,
                                 o.var_e2, o.oneDimvar);
    else printf("rank %d: BAD - NO likelihood sampling!\n", rank);
  }
  return o.error;
}

// source_fitting with a record of every likelihood evaluation (e1, e2, L, error) for debugging
// the facet of a likelihood_params as FP32 cells (the layout the mixed policy reads)
static int upload_mixed_cells(const likelihood_params* par, DevBuf<float>& fcells, FacetBatch& fb, cudaStream_t st) {
  const int n = (int)par->ncoords;
  std::vector<float> h((size_t)5 * (n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    h[i] = (float)par->uu[i];
    h[n + i] = (float)par->vv[i];
    h[2 * n + i] = (float)par->data[i].real;
    h[3 * n + i] = (float)par->data[i].imag;
    h[4 * n + i] = (float)par->sigma2[i];
  }
  RLF_OK(fcells.upload(h.data(), h.size(), st));
  fb.gu = fcells.p; fb.gv = fcells.p + n; fb.dre = fcells.p + 2 * n; fb.dim = fcells.p + 3 * n;
  fb.sig2 = fcells.p + 4 * n;
  RLF_CUDA(cudaStreamSynchronize(st));  // h is released on return
  return 0;
}

int rlf_debug_fit_trace(void* pv, double* trace, int cap, double* out6, int precision) {
  likelihood_params* par = (likelihood_params*)pv;
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  OneFacet f;
  DevBuf<double> dt;
  RLF_OK(f.load(par, st));
  DevBuf<float> fcells;
  if (precision == RLF_MIXED) RLF_OK(upload_mixed_cells(par, fcells, f.fb, st));
  RLF_OK(g_lib.fo.ensure(1));
  RLF_OK(g_lib.i0.ensure(1));
  RLF_OK(dt.ensure((size_t)cap * 4));
  RLF_CUDA(cudaMemsetAsync(dt.p, 0, (size_t)cap * 4 * sizeof(double), st));
  RLF_CUDA(cudaMemsetAsync(g_lib.i0.p, 0, sizeof(int), st));
  f.fb.out = g_lib.fo.p;
  f.fb.queue = g_lib.i0.p;
  f.fb.trace = dt.p;
  f.fb.trace_cap = cap;
  RLF_OK(fit_launch(f.fb, precision == RLF_MIXED ? kMixed : kF64, 1, st));
  FitOut o;
  RLF_CUDA(copy_async(&o, g_lib.fo.p, sizeof(FitOut), cudaMemcpyDeviceToHost, st));
  RLF_CUDA(copy_async(trace, dt.p, (size_t)cap * 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  out6[0] = o.e1; out6[1] = o.e2; out6[2] = o.max_e1; out6[3] = o.max_e2; out6[4] = o.maxL; out6[5] = o.nevals;
  return 0;
}

int rlf_debug_df_math(int op, int n, const double* x, const double* y, double* out) {
  if (op < 0 || op > 6 || n < 0 || (n > 0 && (!x || !out || (op == 3 && !y)))) return 1;
  if (n == 0) return 0;
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  DevBuf<double> dx, dy, dout;
  RLF_OK(dx.upload(x, (size_t)n, st));
  if (op == 3) RLF_OK(dy.upload(y, (size_t)n, st));
  RLF_OK(dout.ensure((size_t)n));
  RLF_OK(launch_df_math(op, n, dx.p, op == 3 ? dy.p : nullptr, dout.p, st));
  RLF_OK(dout.download(out, (size_t)n, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int rlf_debug_loglike_nodes(void* pv, double e1, double e2, int precision, double* out2, double* node_L) {
  likelihood_params* par = (likelihood_params*)pv;
  cudaStream_t st;
  RLF_OK(lib_stream(&st));
  OneFacet f;
  RLF_OK(f.load(par, st));
  DevBuf<float> fcells;
  if (precision == RLF_MIXED) RLF_OK(upload_mixed_cells(par, fcells, f.fb, st));
  DevBuf<double> d;
  RLF_OK(d.ensure(2 + kMaxNodes));
  RLF_OK(launch_loglikelihood_prec(f.fb, e1, e2, d.p, d.p + 2, precision == RLF_MIXED ? kMixed : kF64, st));
  double h[2 + kMaxNodes];
  RLF_CUDA(copy_async(h, d.p, sizeof(h), cudaMemcpyDeviceToHost, st));
  RLF_CUDA(cudaStreamSynchronize(st));
  out2[0] = h[0]; out2[1] = h[1];
  for (int k = 0; k < par->numr && k < kMaxNodes; ++k) node_L[k] = h[2 + k];
  return 0;
}

// source_extraction.c:36-68 (FACET): visGal is used as scratch only
void source_extraction(int rank, unsigned int facet, likelihood_params* par, complexd* facet_vis, double* facet_sigma2,
                       double* sum_w, double l0, double m0, double flux, double mu, double e1, double e2,
                       complexd* visSkyMod, complexd* visData, complexd* visGal, float* sigma2_vis, bool* flag,
                       unsigned long int num_coords, double* uu_metres, double* vv_metres, double* ww_metres,
                       double len) {
  (void)rank;
  (void)visGal;
  cudaStream_t st;
  if (lib_stream(&st)) return;
  rlf_observation* ob = obs_create((int)num_coords, (int)par->nchannels, uu_metres, vv_metres, ww_metres,
                                   par->wavenumbers, par->spec, len, sigma2_vis, reinterpret_cast<const uint8_t*>(flag),
                                   RLF_F64, st);
  if (!ob) return;
  const long long nv = ob->n_vis;
  copy_async(ob->data64.p, visData, nv * sizeof(double2), cudaMemcpyHostToDevice, st);
  copy_async(ob->sky64.p, visSkyMod, nv * sizeof(double2), cudaMemcpyHostToDevice, st);
  FacetCache* fc = nullptr;
  if (obs_facet(ob, facet, &fc, st)) { delete ob; return; }
  GalaxyParams g;
  g.l = l0; g.m = m0; g.flux = flux; g.scale = mu; g.e1 = e1; g.e2 = e2; g.facet = (int)facet; g.pad = 0;
  DevBuf<GalaxyParams> dg;
  DevBuf<int> dfac, doff, dnc;
  DevBuf<const double*> dss, dsw;
  DevBuf<double> cells;
  const int F = (int)facet, nc = F * F;
  const double* ssp = fc->ss.p;
  const double* swp = fc->sw.p;
  int zero = 0;
  if (dg.upload(&g, 1, st) || dfac.upload(&F, 1, st) || doff.upload(&zero, 1, st) || dnc.ensure(1) ||
      dss.upload(&ssp, 1, st) || dsw.upload(&swp, 1, st) || cells.ensure((size_t)5 * nc)) {
    delete ob;
    return;
  }
  const Observation o = ob->view();
  if (launch_extract_f64(o, ob->data64.p, ob->sky64.p, fc->cell.p, dg.p, facet, g_lib.opt.gaussian, ob->partial.p,
                         ob->n_part, st)) { delete ob; return; }
  FacetOut fo;
  fo.offset = doff.p;
  fo.ncoords = dnc.p;
  fo.gu = cells.p; fo.gv = cells.p + nc; fo.dre = cells.p + 2 * nc; fo.dim = cells.p + 3 * nc; fo.sig2 = cells.p + 4 * nc;
  fo.as_float = 0;
  double* sums = ob->partial.p + (size_t)ob->n_part * 2 * nc;
  if (launch_reduce_partials(ob->partial.p, ob->n_part, 2 * nc, sums, st) ||
      launch_facet_finalize(1, dfac.p, sums, 1, 0, dss.p, dsw.p, len, fo, st)) { delete ob; return; }
  int n = 0;
  std::vector<double> h((size_t)5 * nc);
  copy_async(&n, dnc.p, sizeof(int), cudaMemcpyDeviceToHost, st);
  copy_async(h.data(), cells.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
  copy_async(sum_w, fc->sw.p, nc * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  for (int i = 0; i < n; ++i) {
    facet_vis[i].real = h[(size_t)2 * nc + i];
    facet_vis[i].imag = h[(size_t)3 * nc + i];
    facet_sigma2[i] = h[(size_t)4 * nc + i];
  }
  delete ob;
}

// data_simulation.c:131-165 (SCALELENGTH_ON)
void sky_model(double* wavenumbers, double* spec, double channel_bandwidth_hz, int time_acc, unsigned int num_channels,
               unsigned int n_gal, double* gflux, double* gscale, double* l, double* m, unsigned long int num_coords,
               double* uu_metres, double* vv_metres, double* ww_metres, complexd* visGal, complexd* visMod) {
  (void)channel_bandwidth_hz;
  (void)time_acc;
  (void)visGal;
  cudaStream_t st;
  if (lib_stream(&st)) return;
  std::vector<float> s2((size_t)num_channels * num_coords, 1.0f);
  rlf_observation* ob = obs_create((int)num_coords, (int)num_channels, uu_metres, vv_metres, ww_metres, wavenumbers,
                                   spec, 1.0, s2.data(), nullptr, RLF_F64, st);
  if (!ob) return;
  copy_async(ob->sky64.p, visMod, ob->n_vis * sizeof(double2), cudaMemcpyHostToDevice, st);
  std::vector<GalaxyParams> g = make_gals((int)n_gal, gflux, gscale, nullptr, nullptr, l, m, 1.0, 0);
  DevBuf<GalaxyParams> dg;
  if (dg.upload(g.data(), g.size(), st)) { delete ob; return; }
  const Observation o = ob->view();
  for (unsigned g0 = 0; g0 < n_gal; g0 += 256) {
    const int gn = (int)std::min<unsigned>(256, n_gal - g0);
    if (launch_sky_model_f64(o, ob->sky64.p, dg.p + g0, gn, 0, g_lib.opt.gaussian, st)) { delete ob; return; }
  }
  copy_async(visMod, ob->sky64.p, ob->n_vis * sizeof(double2), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  delete ob;
}

// With rlf_options.reuse_obs = 1, the observation of the last data_processing call is kept with its
// device copies (uvw, variances, flags, row table) and the facet tables built from them while later
// calls pass the same arrays: the reference driver passes the same uvw, sigma2_vis, flag and channel
// arrays to both passes (RadioLensfit2.cpp:597-606).  The key holds the arrays' addresses and sizes
// and a fingerprint of their sampled contents (all channel values, 4096 evenly spaced rows and
// visibilities), so a different observation placed at the same addresses is rebuilt; a change at an
// unsampled position is the caller's promise not to make.  The default (reuse_obs = 0) builds the
// observation on every call, as the reference reads its arrays on every call
// (data_processing.c:82-84).  Visibilities and sky model are uploaded on every call; rlf_release
// frees a kept observation.
struct ObsKey {
  int n_rows = 0, n_ch = 0, precision = -1, has_flag = 0;
  const void *uu = nullptr, *vv = nullptr, *ww = nullptr, *sigma2 = nullptr, *flag = nullptr;
  double len = 0;
  unsigned long long fp = 0;
  bool operator==(const ObsKey& o) const {
    return n_rows == o.n_rows && n_ch == o.n_ch && precision == o.precision && has_flag == o.has_flag && uu == o.uu &&
           vv == o.vv && ww == o.ww && sigma2 == o.sigma2 && flag == o.flag && len == o.len && fp == o.fp;
  }
};
static unsigned long long fnv1a(unsigned long long h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
  return h;
}
static ObsKey obs_key(int n_rows, int n_ch, const double* uu, const double* vv, const double* ww,
                      const double* wavenumbers, const double* spec, double len, const float* sigma2,
                      const uint8_t* flag, int precision) {
  ObsKey k;
  k.n_rows = n_rows; k.n_ch = n_ch; k.precision = precision; k.has_flag = flag != nullptr;
  k.uu = uu; k.vv = vv; k.ww = ww; k.sigma2 = sigma2; k.flag = flag; k.len = len;
  unsigned long long h = 1469598103934665603ull;
  h = fnv1a(h, wavenumbers, sizeof(double) * n_ch);
  h = fnv1a(h, spec, sizeof(double) * n_ch);
  const long long nv = (long long)n_rows * n_ch;
  for (int i = 0; i <= 4096; ++i) {
    const long long r = (long long)(n_rows - 1) * i / 4096, v = (nv - 1) * i / 4096;
    h = fnv1a(h, uu + r, sizeof(double));
    h = fnv1a(h, vv + r, sizeof(double));
    h = fnv1a(h, ww + r, sizeof(double));
    h = fnv1a(h, sigma2 + v, sizeof(float));
    if (flag) h = fnv1a(h, flag + v, 1);
  }
  k.fp = h;
  return k;
}
static rlf_observation* g_obs_cached = nullptr;
static ObsKey g_obs_key;

// data_processing.c:47-147: one pass over the catalogue (re_fitting = false) or the bad list
void data_processing(bool re_fitting, unsigned int* bad_list, int nsources, double len, unsigned int num_coords,
                     FILE* pFile, likelihood_params* par, double* l, double* m, double* gflux, double* gscale,
                     double* ge1, double* ge2, double* SNR_vis, double* sum_w, complexd* visGal, complexd* visSkyMod,
                     complexd* visData, float* sigma2_vis, bool* flag, double* uu_metres, double* vv_metres,
                     double* ww_metres, double* fitting_time, int* bad) {
  (void)sum_w;
  (void)visGal;
  cudaStream_t st;
  if (lib_stream(&st)) return;
  const rlf_options opt = g_lib.opt;
  const uint8_t* flag8 = reinterpret_cast<const uint8_t*>(flag);
  rlf_observation* ob = nullptr;
  const ObsKey key = obs_key((int)num_coords, (int)par->nchannels, uu_metres, vv_metres, ww_metres, par->wavenumbers,
                             par->spec, len, sigma2_vis, flag8, opt.precision);
  if (opt.reuse_obs && g_obs_cached && key == g_obs_key) {
    ob = g_obs_cached;
  } else {
    delete g_obs_cached;
    g_obs_cached = nullptr;
    ob = obs_create((int)num_coords, (int)par->nchannels, uu_metres, vv_metres, ww_metres, par->wavenumbers, par->spec,
                    len, sigma2_vis, flag8, opt.precision, st);
    if (!ob) return;
    if (opt.reuse_obs) { g_obs_cached = ob; g_obs_key = key; }
  }
  // the observation is freed on the way out unless it is the cached one
  struct Release {
    rlf_observation* o;
    ~Release() { if (o != g_obs_cached) delete o; }
  } release{ob};
  if (obs_put_c128(ob, reinterpret_cast<const double*>(visData), false, st) ||
      obs_put_c128(ob, reinterpret_cast<const double*>(visSkyMod), true, st)) return;
  // galaxies: the catalogue (in order) or the bad list
  std::vector<int> order(nsources > 0 ? nsources : 0);
  for (int g = 0; g < nsources; ++g) order[g] = re_fitting ? (int)bad_list[g] : g;
  int ncat = 0;
  for (int g : order) ncat = std::max(ncat, g + 1);
  const unsigned fmax = rlf::facet_size(kRMax, len);
  std::vector<GalaxyParams> gals = make_gals(ncat, gflux, gscale, nullptr, nullptr, l, m, len, fmax);
  std::vector<FitOut> out;
  double ms3[3] = {0, 0, 0};
  if (run_pass(ob, gals, order, par->numr, par->ro, opt, out, st, ms3)) return;
  int nbad = 0;
  for (int g = 0; g < nsources; ++g) {
    const int gal = order[g];
    FitOut r = out[g];
    if (opt.verbose) printf("n. %d flux = %f: measured e = %f , %f \n", gal, gflux[gal], r.e1, r.e2);
    if (r.error) {
      if (re_fitting) {
        r.e1 = 0.;
        r.e2 = 0.;
        if (pFile)
          fprintf(pFile, "%f | %f | %f | %f | %f | %f | %f | %f | %f | %f | %f \n", gflux[gal], ge1[gal], r.e1,
                  sqrt(r.var_e1), ge2[gal], r.e2, sqrt(r.var_e2), r.oneDimvar, SNR_vis[gal], l[gal] / (kPi / 648000.0),
                  m[gal] / (kPi / 648000.0));
      } else {
        bad_list[nbad] = (unsigned)gal;
      }
      nbad++;
    } else if (pFile) {
      fprintf(pFile, "%f | %f | %f | %f | %f | %f | %f | %f | %f | %f | %f \n", gflux[gal], ge1[gal], r.e1,
              sqrt(r.var_e1), ge2[gal], r.e2, sqrt(r.var_e2), r.oneDimvar, SNR_vis[gal], l[gal] / (kPi / 648000.0),
              m[gal] / (kPi / 648000.0));
    }
  }
  *bad = nbad;
  *fitting_time += ms3[1] / 1000.0;
  obs_get_c128(ob, reinterpret_cast<double*>(visData), false, st);
  obs_get_c128(ob, reinterpret_cast<double*>(visSkyMod), true, st);
}

void rlf_release(void) {
  delete g_obs_cached;
  g_obs_cached = nullptr;
  g_obs_key = ObsKey{};
}

void rlf_transfer_bytes(unsigned long long* h2d, unsigned long long* d2h) {
  if (h2d) *h2d = __atomic_load_n(&g_h2d_bytes, __ATOMIC_RELAXED);
  if (d2h) *d2h = __atomic_load_n(&g_d2h_bytes, __ATOMIC_RELAXED);
}

}  // extern "C"

// marginalise_r.h:24-27 declares these with C++ linkage
void set_posterior_values(int numR, double* L_r, double* rprior, double* Ro, double* xmarvals, double* ymarvals,
                          int* numvals) {
  rlf_set_posterior_values(numR, L_r, rprior, Ro, xmarvals, ymarvals, numvals);
}
double marginalise_posterior_r(int num_marvals, double* xmarvals, double* ymarvals) {
  return rlf_marginalise_posterior_r(num_marvals, xmarvals, ymarvals);
}
double marf(double x, void* params) { return rlf_marf(x, params); }

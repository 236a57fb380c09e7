// Facet likelihood, scalelength marginalisation and ellipticity fit on the GPU.
//
// One CTA fits one galaxy at a time, taking galaxies from a device work queue (persistent
// kernel).  Inside a CTA:
//   * warp w evaluates the likelihood at scalelength node w+1 (likelihood.c:117-131 runs these
//     nodes as an OpenMP loop): facet model (galaxy_visibilities.c:59-91), cross-correlation and
//     Newton search for the position shift (likelihood.c:194-358), analytic position
//     marginalisation (likelihood.c:376-421);
//   * warp 0 then marginalises over scalelength (marginalise_r.c:29-223): natural cubic spline of
//     the log-posterior and adaptive Gauss-Kronrod 41 (QAG) quadrature of its exponential, the 41
//     integrand points evaluated by the lanes in parallel;
//   * the Nelder-Mead simplex (galaxy_fitting.c:41-82, GSL nmsimplex2) and the likelihood
//     sampling (likelihood.c:428-554) run replicated in every thread, so every decision is taken
//     identically by all threads and each likelihood evaluation is a CTA-collective call.
//
// Two arithmetic policies:
//   F64   -- all double, the reference's arithmetic; the parity path and FP64 GPU oracle.
//   Mixed -- FP32 cell arithmetic (model, products, phase rotations: the work that scales with
//            the facet size) with compensated sums (Kahan per lane, double-float across lanes,
//            reduced into double).  The per-node scalars (Newton step, determinant, position
//            marginal), the marginalisation over scalelength and the simplex/sampling logic run in
//            FP64: a few hundred lane-uniform operations per evaluation, small beside the cell
//            loops, and they keep the log-likelihood within 1e-6 relative of the FP64 result.
#include "rlf_fit.cuh"
#include <stdio.h>

namespace rlf {

#ifndef RLF_FIT_WARPS
#define RLF_FIT_WARPS 8
#endif
// warps of a fit CTA (one galaxy); the scalelength nodes are spread over them, and small CTAs run
// several galaxies per SM, so that one galaxy's serial phases overlap another's cell passes
constexpr int kFitWarps = RLF_FIT_WARPS;
constexpr int kFitThreads = kFitWarps * 32;
constexpr int kFitMinBlocks = kFitWarps <= 6 ? 4 : (kFitWarps <= 8 ? 3 : (kFitWarps <= 12 ? 2 : 1));
constexpr int kQagCap = 128;       // intervals held by the device QAG (more: status bit 2, an error)
constexpr int kNewtonMax = 50;     // likelihood.c:290
constexpr int kSimplexMax = 50;    // galaxy_fitting.c:80
constexpr int kModelCache = 4;     // facet cells per lane whose model stays in registers
constexpr int kNodePart = 8;       // partials per cross-correlation sum left by a node's lanes
constexpr int kNodeCache = 64;     // facet cells per node whose model stays in shared memory
constexpr int kNodeStride = kNodeCache + 8;  // padded row of the per-node caches (bank spread)
constexpr int kNodesPerWarp = 32 / kNodePart;  // nodes whose cell passes share a warp
constexpr int kEiTab = 101;        // Ei(k) and e^k for k = 0..100 (the position marginal's range)
constexpr int kEiTerms = 48;       // terms of the per-lane Ei expansions (at most ~26 are used)
constexpr int kInvTab = 128;       // 1/k for k < kInvTab

__constant__ double c_ei_tab[kEiTab];      // Ei(k), computed on the host in extended precision
__constant__ double c_exp_tab[kEiTab];     // e^k
__constant__ float2 c_invk2[kInvTab];       // 1 / k as a float pair (hi, lo)
__constant__ float2 c_invfact2[kEiTerms];   // 1 / k! as a float pair

struct FitConst {
  int numr;
  int gaussian;
  int np_max;
  int pad;
  double ro[kMaxNodes];
};
__constant__ FitConst c_fit;

// 41-point Gauss-Kronrod rule (QUADPACK qk41): Kronrod abscissae, Kronrod weights and the
// weights of the embedded 20-point Gauss rule (abscissae xgk[1], xgk[3], ...).
__constant__ double c_xgk[21] = {
    0.998859031588277663838315576545863, 0.993128599185094924786122388471320,
    0.981507877450250259193342994720217, 0.963971927277913791267666131197277,
    0.940822633831754753519982722212443, 0.912234428251325905867752441203298,
    0.878276811252281976077442995113078, 0.839116971822218823394529061701521,
    0.795041428837551198350638833272788, 0.746331906460150792614305070355642,
    0.693237656334751384805490711845932, 0.636053680726515025452836696226286,
    0.575140446819710315342946036586425, 0.510867001950827098004364050955251,
    0.443593175238725103199992213492640, 0.373706088715419560672548177024927,
    0.301627868114913004320555356858592, 0.227785851141645078080496195368575,
    0.152605465240922675505220241022678, 0.076526521133497333754640409398838,
    0.000000000000000000000000000000000};
__constant__ double c_wgk[21] = {
    0.003073583718520531501218293246031, 0.008600269855642942198661787950102,
    0.014626169256971252983787960308868, 0.020388373461266523598010231432755,
    0.025882133604951158834505067096153, 0.031287306777032798958543119323801,
    0.036600169758200798030557240707211, 0.041668873327973686263788305936895,
    0.046434821867497674720231880926108, 0.050944573923728691932707670050345,
    0.055195105348285994744832372419777, 0.059111400880639572374967220648594,
    0.062653237554781168025870122174255, 0.065834597133618422111563556969398,
    0.068648672928521619345623411885368, 0.071054423553444068305790361723210,
    0.073030690332786667495189417658913, 0.074582875400499188986581418362488,
    0.075704497684556674659542775376617, 0.076377867672080736705502835038061,
    0.076600711917999656445049901530102};
__constant__ double c_wg[10] = {
    0.017614007139152118311861962351853, 0.040601429800386941331039952274932,
    0.062672048334109063569506535187042, 0.083276741576704748724758143222046,
    0.101930119817240435036750135480350, 0.118194531961518417312377377711382,
    0.131688638449176626898494499748163, 0.142096109318382051329298325067165,
    0.149172986472603746787828737001969, 0.152753387130725850698084331955098};

// ------------------------------------------------------------------ policies
struct PolicyF64 {
  using Cell = double;
  using S = double;
  static constexpr bool kMixed = false;
};
struct PolicyMixed {
  using Cell = float;
  using S = double;
  static constexpr bool kMixed = true;
};

template <class S> struct Consts;
template <> struct Consts<double> {
  static __device__ __forceinline__ double dbl_eps() { return 2.2204460492503131e-16; }
  static __device__ __forceinline__ double dbl_min() { return 2.2250738585072014e-308; }
};
template <> struct Consts<float> {
  static __device__ __forceinline__ float dbl_eps() { return 1.1920929e-07f; }
  static __device__ __forceinline__ float dbl_min() { return 1.17549435e-38f; }
};

__device__ __forceinline__ double s_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float s_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double s_log(double x) { return log(x); }
__device__ __forceinline__ float s_log(float x) { return logf(x); }
__device__ __forceinline__ double s_exp(double x) { return exp(x); }
__device__ __forceinline__ float s_exp(float x) { return expf(x); }
__device__ __forceinline__ double s_abs(double x) { return fabs(x); }
__device__ __forceinline__ float s_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double s_pow15(double x) { return x * sqrt(x); }
__device__ __forceinline__ float s_pow15(float x) { return x * sqrtf(x); }
__device__ __forceinline__ void s_sincos(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ void s_sincos(float a, float* s, float* c) { sincosf(a, s, c); }

// Uniform (lane-identical) warp sums.  Double: butterfly (a+b == b+a, so every lane ends with
// the same bits).  Float: per-lane Kahan partials combined in double-float, operands ordered by
// lane so both partners of a butterfly step compute identical bits.
__device__ __forceinline__ double uwarp_sum(double v) { return warp_sum(v); }
// butterfly of (hi, lo) double-float partials; afterwards every lane holds the same pair
__device__ __forceinline__ void df_butterfly(float& hi, float& lo) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    float ohi = __shfl_xor_sync(0xffffffffu, hi, m);
    float olo = __shfl_xor_sync(0xffffffffu, lo, m);
    const bool first = (lane & m) == 0;
    float ahi = first ? hi : ohi, alo = first ? lo : olo;
    float bhi = first ? ohi : hi, blo = first ? olo : lo;
    f2 s = two_sum(ahi, bhi);
    float e = s.lo + (alo + blo);
    f2 r = quick_two_sum(s.hi, e);
    hi = r.hi;
    lo = r.lo;
  }
}
// double-float warp sum returned as double, keeping the compensated low part
__device__ __forceinline__ double uwarp_sum_dfd(float hi, float lo) {
  df_butterfly(hi, lo);
  return (double)hi + (double)lo;
}

template <class S> struct Acc;
template <> struct Acc<double> {
  double s;
  __device__ __forceinline__ void zero() { s = 0.; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void sub(double x) { s -= x; }
  __device__ __forceinline__ double reduce() const { return uwarp_sum(s); }
};
template <> struct Acc<float> {
  float s, c;  // Kahan: running sum and compensation (true sum ~ s - c)
  __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ void sub(float x) { add(-x); }
  __device__ __forceinline__ double reduce() const { return uwarp_sum_dfd(s, -c); }
};

// ----------------------------------------------------------- position marginal
// likelihood.c:376-421 evaluated by a whole warp (every lane calls it with the same x).  Ei(x)
// comes from its power series  gamma + ln x + sum_k a_k / k,  a_k = x^k / k!,  or, for large x,
// from the asymptotic series  e^x / x sum_k k! / x^k  stopped before its smallest term.  The
// 32 lanes take 32 consecutive k per round and form a_k as a prefix product of x/k across the
// warp (Hillis-Steele scan), so a series of up to ~100 terms costs 4 rounds instead of 100
// dependent steps with divisions.
template <class S> __device__ __forceinline__ S wsum(S v);
template <> __device__ __forceinline__ double wsum<double>(double v) { return uwarp_sum(v); }

template <class S>
__device__ __forceinline__ S warp_prefix_prod(S f) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const S g = __shfl_up_sync(0xffffffffu, f, o);
    if (lane >= o) f *= g;
  }
  return f;
}

// sum_{k>=1} x^k / (k k!)
template <class S>
__device__ __forceinline__ S ei_series_sum_warp(S x, S eps) {
  const int lane = threadIdx.x & 31;
  S base = S(1), sum = S(0);
  for (int j = 0; j < 12; ++j) {
    const S k = S(32 * j + lane + 1);
    const S a = base * warp_prefix_prod<S>(x / k);
    const S t = a / k;
    sum += wsum<S>(t);
    base = __shfl_sync(0xffffffffu, a, 31);
    const S last = __shfl_sync(0xffffffffu, t, 31);
    if (S(32 * j + 32) > x && last < eps * sum) break;
  }
  return sum;
}

// sum_{k>=0} k!/x^k over the decreasing part of the asymptotic series
template <class S>
__device__ __forceinline__ S ei_asym_sum_warp(S x, S eps) {
  const int lane = threadIdx.x & 31;
  S base = S(1), sum = S(1);
  for (int j = 0; j < 8; ++j) {
    const S k = S(32 * j + lane + 1);
    const S b = base * warp_prefix_prod<S>(k / x);
    const bool keep = (k < x) && (b >= eps);
    sum += wsum<S>(keep ? b : S(0));
    base = __shfl_sync(0xffffffffu, b, 31);
    if (!(S(32 * j + 32) < x) || base < eps) break;
  }
  return sum;
}

__device__ __forceinline__ double ei_warp(double x) {
  if (x <= 40.0) return kEulerGamma + log(x) + ei_series_sum_warp<double>(x, 1e-18);
  return exp(x) / x * ei_asym_sum_warp<double>(x, 1e-18);
}

__device__ double pos_marg(double x) {
  const double Delta = 0.5 * 5.991;
  if (x <= Delta) return kBad;
  if (x > 100.) return x - log(Delta) - exp(-Delta);
  if ((x - Delta) < 0.0001) x = Delta + 0.0001;
  const double yc = ei_warp(x), ys = ei_warp(x - Delta);
  return log((yc - ys) / log(x / (x - Delta)));
}

// --------------------------------------------------------------- cell model
template <class S>
__device__ __forceinline__ S cell_shape(int gaussian, S a1, S a2, S a3, S u, S v, S sfw) {
  S k1 = a1 * u + a2 * v;
  S k2 = a2 * u + a3 * v;
  S q = sfw * (k1 * k1 + k2 * k2);
  if (gaussian) return s_exp(S(-0.5) * q);
  S den = S(1) + q;
  return S(1) / (den * s_sqrt(den));
}

// The same model for the fit's cell passes: (1 + q)^(-3/2) as rsqrt(1 + q)^3, one FP64 square-root
// approximation and two products instead of a square root and a division (a few ulp apart).
__device__ __forceinline__ double s_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float s_rsqrt(float x) { return rsqrtf(x); }
template <class S>
__device__ __forceinline__ S cell_shape_fit(int gaussian, S a1, S a2, S a3, S u, S v, S sfw) {
  S k1 = a1 * u + a2 * v;
  S k2 = a2 * u + a3 * v;
  S q = sfw * (k1 * k1 + k2 * k2);
  if (gaussian) return s_exp(S(-0.5) * q);
  const S r = s_rsqrt(S(1) + q);
  return r * r * r;
}

// Warp-level likelihood at one scalelength node, likelihood.c:156-187 with the model of
// galaxy_visibilities.c:59-91 and the cross-correlation of likelihood.c:194-358.
// Cell arithmetic runs in P::Cell (the per-cell model, products and phase rotations); the six
// cross-correlation sums are reduced into P::S, and the Newton step, determinant, position
// marginal and log terms are evaluated in P::S (double in both policies).
// model_in (optional) replaces the computed model (cross_correlation's own entry point);
// model_out (optional) receives the normalised model (loglikelihood_r writes visM).
template <class P>
__device__ typename P::S node_loglike(const typename P::Cell* gu, const typename P::Cell* gv,
                                      const typename P::Cell* dre, const typename P::Cell* dim,
                                      const typename P::Cell* sig2, int n, typename P::S e1,
                                      typename P::S e2, typename P::S r, int gaussian, int* iters,
                                      double* model_out,
                                      const double* model_in, typename P::S* ho_out,
                                      typename P::S* det_out) {
  using S = typename P::S;
  using T = typename P::Cell;
  const int lane = threadIdx.x & 31;
  const T a1 = T(S(1) + e1), a2 = T(e2), a3 = T(S(1) - e1);
  // galaxy_visibilities.c:63-65 then the 4 pi^2 wave factor of :69
  const S detA = S(1) - e1 * e1 - e2 * e2;
  const S sc = r * S(kPi / 648000.0);
  const T sfw = T(((sc * sc) / (detA * detA)) * S(4 * kPi * kPi));
  const T cc = T(2 * kPi);
  S s_norm = S(1);
  T inv_s = T(1);
  // the unnormalised model of the first kModelCache cells of this lane, kept in registers for
  // the cross-correlation passes (the model does not change during the Newton search)
  T mc[kModelCache];
  if (!model_in) {
    Acc<T> acc;
    acc.zero();
#pragma unroll
    for (int t = 0; t < kModelCache; ++t) {
      const int i = lane + 32 * t;
      mc[t] = T(0);
      if (i < n) {
        const T m = cell_shape<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw);
        mc[t] = m;
        acc.add(m * m / T(sig2[i]));
      }
    }
    for (int i = lane + 32 * kModelCache; i < n; i += 32) {
      T m = cell_shape<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw);
      acc.add(m * m / T(sig2[i]));
    }
    const S sum = acc.reduce();
    s_norm = s_sqrt(sum);
    inv_s = T(S(1) / s_norm);
  }
  const T t_norm = T(s_norm);
  auto normalise = [&](T m) -> T {
    if (P::kMixed) return m * inv_s;
    return m / t_norm;  // the reference divides (galaxy_visibilities.c:90)
  };
  if (!model_in) {
#pragma unroll
    for (int t = 0; t < kModelCache; ++t) mc[t] = normalise(mc[t]);
  }
  // normalised model of cell i beyond the cached ones
  auto model_tail = [&](int i) -> T {
    if (model_in) return T(model_in[i]);
    return normalise(cell_shape<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw));
  };
  Acc<T> val, dx, dy, d2x, d2y, dxy;
  val.zero(); dx.zero(); dy.zero(); d2x.zero(); d2y.zero(); dxy.zero();
  auto first_cell = [&](int i, T m) {
    if (model_out) model_out[i] = (double)m;
    T hre = T(dre[i]) * m;
    T him = -T(dim[i]) * m;
    T u = cc * T(gu[i]);
    T v = cc * T(gv[i]);
    val.add(hre);
    dx.sub(him * u);
    dy.sub(him * v);
    d2x.sub(hre * u * u);
    d2y.sub(hre * v * v);
    dxy.sub(hre * u * v);
  };
  // cells in the order i = lane, lane + 32, ... (cached ones first, then the rest)
#pragma unroll
  for (int t = 0; t < kModelCache; ++t) {
    const int i = lane + 32 * t;
    if (i < n) first_cell(i, model_in ? T(model_in[i]) : mc[t]);
  }
  for (int i = lane + 32 * kModelCache; i < n; i += 32) first_cell(i, model_tail(i));
  S Sval = val.reduce(), Sdx = dx.reduce(), Sdy = dy.reduce();
  S Sd2x = d2x.reduce(), Sd2y = d2y.reduce(), Sdxy = dxy.reduce();
  S det = Sd2x * Sd2y - Sdxy * Sdxy;
  S xo = S(0), yo = S(0), norm = S(1);
  const S tol = S(1.e-7);
  int iter = 0;
  while (det > S(0) && (norm > tol) && iter < kNewtonMax) {
    iter++;
    S incx = (Sdx * Sd2y - Sdy * Sdxy) / det;
    S incy = (Sdy * Sd2x - Sdx * Sdxy) / det;
    xo -= incx;
    yo -= incy;
    const T txo = T(xo), tyo = T(yo);
    val.zero(); dx.zero(); dy.zero(); d2x.zero(); d2y.zero(); dxy.zero();
    auto newton_cell = [&](int i, T m) {
      T hre = T(dre[i]) * m;
      T him = -T(dim[i]) * m;
      T u = cc * T(gu[i]);
      T v = cc * T(gv[i]);
      T a = txo * u + tyo * v;
      T sa, ca;
      s_sincos(a, &sa, &ca);
      T rp = (hre * ca - him * sa);
      T ip = (hre * sa + him * ca);
      val.add(rp);
      dx.sub(ip * u);
      dy.sub(ip * v);
      d2x.sub(rp * u * u);
      d2y.sub(rp * v * v);
      dxy.sub(rp * u * v);
    };
#pragma unroll
    for (int t = 0; t < kModelCache; ++t) {
      const int i = lane + 32 * t;
      if (i < n) newton_cell(i, model_in ? T(model_in[i]) : mc[t]);
    }
    for (int i = lane + 32 * kModelCache; i < n; i += 32) newton_cell(i, model_tail(i));
    Sval = val.reduce(); Sdx = dx.reduce(); Sdy = dy.reduce();
    Sd2x = d2x.reduce(); Sd2y = d2y.reduce(); Sdxy = dxy.reduce();
    det = Sd2x * Sd2y - Sdxy * Sdxy;
    norm = s_sqrt(incx * incx + incy * incy);
  }
  // lane-uniform by construction; broadcast from lane 0 as a guard
  Sval = __shfl_sync(0xffffffffu, Sval, 0);
  det = __shfl_sync(0xffffffffu, det, 0);
  *iters = iter;
  if (ho_out) *ho_out = Sval;
  if (det_out) *det_out = det;
  if (det <= S(0)) return S(kBad);
  S B = (Sval * Sval) * S(0.5);
  S L = pos_marg(B);
  if (isnan(L)) return S(kBad);
  return L - S(0.5) * s_log(det);
}

// ------------------------------------------------------------- shared state
// Per-node state of the phased node evaluation (eval_nodes), in dynamic shared memory sized by the
// number of scalelength nodes (row 0 unused, as Ro[0]): the partial sums each node's lanes leave, and
// caches of the first kNodeCache cells of every node.  Phase A leaves the unnormalised model in hre;
// phase B replaces it by the real part of data x normalised model and fills him (the model does not
// change during the Newton search, so the Newton passes read both back and evaluate no model).
// The FP64 policy keeps the Newton inputs as double-float pairs (f2), the mixed policy as double.
union CacheSlot {
  double d;
  f2 f;
};
struct NodeCache {
  double* part;       // [7][nr][kNodePart]: 0 model norm; 1..6 val, dx, dy, d2x, d2y, dxy
  CacheSlot* hre;     // [nr][kNodeStride]
  CacheSlot* him;     // [nr][kNodeStride]
  double *cu, *cv;    // [kNodeCache] 2 pi u and 2 pi v of the cells
  double* isg;        // [kNodeCache] 1 / variance of the cells
  f2 *cu2, *cv2;      // [kNodeCache] 2 pi u, 2 pi v as double-float pairs
  f2 *gu2, *gv2;      // [kNodeCache] u, v (FP64 policy, exponential profile: the double-float passes)
  f2 *dre2, *dim2;    // [kNodeCache] facet visibility / variance
  f2* isg2;           // [kNodeCache] 1 / variance
  int nr;
  __device__ __forceinline__ double* P(int k, int node) const { return part + ((size_t)k * nr + node) * kNodePart; }
  __device__ __forceinline__ CacheSlot& H(int node, int i) const { return hre[node * kNodeStride + i]; }
  __device__ __forceinline__ CacheSlot& M(int node, int i) const { return him[node * kNodeStride + i]; }
};
// bytes of a NodeCache for nr node rows (a multiple of 16)
__host__ __device__ __forceinline__ size_t node_cache_bytes(int nr) {
  return (size_t)7 * nr * kNodePart * sizeof(double) + (size_t)2 * nr * kNodeStride * sizeof(CacheSlot) +
         (size_t)kNodeCache * (3 * sizeof(double) + 7 * sizeof(f2));
}
__device__ __forceinline__ NodeCache node_cache_view(unsigned char* base, int nr) {
  NodeCache c;
  c.nr = nr;
  c.part = reinterpret_cast<double*>(base);
  c.hre = reinterpret_cast<CacheSlot*>(c.part + (size_t)7 * nr * kNodePart);
  c.him = c.hre + (size_t)nr * kNodeStride;
  c.cu = reinterpret_cast<double*>(c.him + (size_t)nr * kNodeStride);
  c.cv = c.cu + kNodeCache;
  c.isg = c.cv + kNodeCache;
  c.cu2 = reinterpret_cast<f2*>(c.isg + kNodeCache);
  c.cv2 = c.cu2 + kNodeCache;
  c.gu2 = c.cv2 + kNodeCache;
  c.gv2 = c.gu2 + kNodeCache;
  c.dre2 = c.gv2 + kNodeCache;
  c.dim2 = c.dre2 + kNodeCache;
  c.isg2 = c.dim2 + kNodeCache;
  return c;
}

// ---- double-float (unevaluated sum of two floats) arithmetic for sin/cos on the FP32 pipes
__device__ __forceinline__ f2 df_mul(f2 a, f2 b) {
  f2 p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ f2 df_add(f2 a, f2 b) {
  f2 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ f2 df_neg(f2 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ f2 df_sub(f2 a, f2 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ double df_to_double(f2 a) { return (double)a.hi + (double)a.lo; }
// P * y + c
__device__ __forceinline__ f2 df_horner(f2 P, f2 y, float c_hi, float c_lo) {
  return df_add(df_mul(P, y), f2{c_hi, c_lo});
}

// ---- double-float division, square root, exp and log for the fit's serial phases.  Dependent
// FP64 operations on this GPU take 64 cycles (fma) to ~550 (division), ~700 (square root), ~1150
// (exp) and ~2100 (log); an FP32 fma ~5 and a double-float multiply ~22.  Largest relative errors
// against FP64 (tests/test_gpu_dfmath.py): division 1e-14, square root 6e-15, exp 1e-13 over
// [-40, 40] (the squarings of its reduced argument amplify), log 5e-13 of max(|log|, 1) over
// e^[-80, 80], log of a double 4e-14.
__device__ __forceinline__ f2 df_sqr(f2 a) {
  f2 p = two_prod(a.hi, a.hi);
  p.lo = fmaf(2.f * a.hi, a.lo, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ f2 df_scale(f2 a, float s) { return f2{a.hi * s, a.lo * s}; }  // s a power of 2
// a / b: the quotient of the high parts from an approximate reciprocal, refined twice by the
// double-float remainder a - q b
__device__ __forceinline__ f2 df_div(f2 a, f2 b) {
  const float r = __fdividef(1.f, b.hi);
  const float q1 = a.hi * r;
  f2 rem = df_sub(a, df_mul(f2{q1, 0.f}, b));
  const float q2 = rem.hi * r;
  f2 q = quick_two_sum(q1, q2);
  rem = df_sub(a, df_mul(q, b));
  return df_add(q, f2{rem.hi * r, 0.f});
}
// sqrt(a): s = a rsqrt(a) refined twice by s + (a - s^2) / (2 s); 0 for 0, NaN below
__device__ __forceinline__ f2 df_sqrt(f2 a) {
  if (!(a.hi > 0.f)) return f2{a.hi == 0.f ? 0.f : __int_as_float(0x7fc00000), 0.f};
  const float y = rsqrtf(a.hi);
  f2 s{a.hi * y, 0.f};
  f2 e = df_sub(a, df_sqr(s));
  s = df_add(s, f2{e.hi * 0.5f * y, 0.f});
  e = df_sub(a, df_sqr(s));
  return df_add(s, f2{e.hi * 0.5f * y, 0.f});
}
// exp(a): a = k ln2 + r, |r| <= ln2 / 2, with ln2 split in three so that k * (first part) is exact
// and k * (second part) exact as a pair; exp(r) = exp(r / 8)^8 with exp(r / 8) from its Taylor
// series to degree 10 (remainder below 1e-23); 0 below the float range, inf above it
__constant__ float2 c_df_invfact[11] = {
    {1.0f, 0.f}, {1.0f, 0.f}, {0.5f, 0.f}, {0.1666666716337204f, -4.967053879312289e-09f},
    {0.0416666679084301f, -1.2417634698280722e-09f}, {0.008333333767950535f, -4.34617203337595e-10f},
    {0.0013888889225199819f, -3.3631094437103215e-11f}, {0.00019841270113829523f, -2.725596874933456e-12f},
    {2.4801587642286904e-05f, -3.40699609366682e-13f}, {2.7557318844628753e-06f, 3.793571224297229e-14f},
    {2.755731998149713e-07f, -7.575112209051195e-15f}};
__device__ __forceinline__ f2 df_exp(f2 a) {
  if (isnan(a.hi)) return a;
  if (a.hi < -87.f) return f2{0.f, 0.f};
  if (a.hi > 88.f) return f2{__int_as_float(0x7f800000), 0.f};
  const float k = rintf(a.hi * 1.4426950216293335f);
  f2 r = df_add(a, f2{-k * 0.693115234375f, 0.f});      // 2839 / 4096: 12 significant bits
  r = df_sub(r, two_prod(k, 3.194618329871446e-05f));
  r = df_add(r, f2{-k * 1.6465949697480609e-12f, 0.f});
  const f2 t = df_scale(r, 0.125f);
  f2 p{c_df_invfact[10].x, c_df_invfact[10].y};
#pragma unroll
  for (int n = 9; n >= 0; --n) p = df_add(df_mul(p, t), f2{c_df_invfact[n].x, c_df_invfact[n].y});
  p = df_sqr(df_sqr(df_sqr(p)));
  // 2^k in two factors, each inside the float exponent range
  const int ki = (int)k, k1 = ki / 2, k2 = ki - k1;
  const float s1 = __int_as_float((k1 + 127) << 23), s2 = __int_as_float((k2 + 127) << 23);
  return df_scale(df_scale(p, s1), s2);
}
// e ln2 as a pair (|e| < 2^11: the first product is exact)
__device__ __forceinline__ f2 df_ln2_times(float e) {
  f2 l = df_add(two_prod(e, 3.194618329871446e-05f), f2{e * 1.6465949697480609e-12f, 0.f});
  return df_add(f2{e * 0.693115234375f, 0.f}, l);
}
// log(a), a > 0 within the float range: a = m 2^e with m in [1, 2) (an exact scaling), then
// y0 = log(m.hi) from the SFU and log(m) = y0 + log(1 + d), d = m exp(-y0) - 1 (|d| ~1e-6):
// y0 + d - d^2 / 2, plus e ln2; -inf for 0, NaN below, inf for inf
__device__ __forceinline__ f2 df_log(f2 a) {
  if (!(a.hi > 0.f) || isinf(a.hi))
    return f2{a.hi == 0.f ? -__int_as_float(0x7f800000) : (a.hi > 0.f ? a.hi : __int_as_float(0x7fc00000)), 0.f};
  int e = ((__float_as_int(a.hi) >> 23) & 0xff) - 127;  // -127 for subnormal high parts
  if (e > 126) e = 126;
  const f2 m = df_scale(a, __int_as_float((127 - e) << 23));
  const float y0 = __logf(m.hi);
  const f2 d = df_sub(df_mul(m, df_exp(f2{-y0, 0.f})), f2{1.f, 0.f});
  return df_add(df_add(f2{y0, 0.f}, df_add(d, f2{-0.5f * d.hi * d.hi, 0.f})), df_ln2_times((float)e));
}
// log(x) of a positive normal double of any magnitude: x = m 2^e with m in [1, 2) split into a
// float pair from its bits (the low part's 29 bits rounded to 24), log m + e ln2
__device__ __forceinline__ f2 df_log_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  const unsigned long long frac = b & 0x000fffffffffffffull;
  const float hi = __uint_as_float(0x3f800000u | (unsigned)(frac >> 29));
  const float lo = (float)(unsigned)(frac & 0x1fffffffull) * 2.220446049250313e-16f;  // 2^-52
  return df_add(df_log(quick_two_sum(hi, lo)), df_ln2_times((float)e));
}


// ---- a double-float number type for the F64 fit's marginalisation over the scalelength (the
// natural spline, QUADPACK qag and its 41-point rule, exp and log): the FP64 code instantiated on
// the FP32 pipes, where each of its dependent operations takes ~15-40 cycles instead of 64-2100
struct DF {
  float hi, lo;
  DF() = default;
  __device__ __forceinline__ DF(f2 a) : hi(a.hi), lo(a.lo) {}
  __device__ __forceinline__ DF(double d) {
    hi = (float)d;
    lo = isfinite(hi) ? (float)(d - (double)hi) : 0.f;
  }
  __device__ __forceinline__ f2 p() const { return f2{hi, lo}; }
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ DF operator+(DF a, DF b) { return DF(df_add(a.p(), b.p())); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return DF(df_sub(a.p(), b.p())); }
__device__ __forceinline__ DF operator-(DF a) { return DF(f2{-a.hi, -a.lo}); }
__device__ __forceinline__ DF operator*(DF a, DF b) { return DF(df_mul(a.p(), b.p())); }
__device__ __forceinline__ DF operator/(DF a, DF b) { return DF(df_div(a.p(), b.p())); }
__device__ __forceinline__ DF& operator+=(DF& a, DF b) { return a = a + b; }
__device__ __forceinline__ DF& operator-=(DF& a, DF b) { return a = a - b; }
__device__ __forceinline__ DF& operator*=(DF& a, DF b) { return a = a * b; }
__device__ __forceinline__ bool operator<(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(DF a, DF b) { return b < a; }
__device__ __forceinline__ bool operator<=(DF a, DF b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(DF a, DF b) { return !(a < b); }
__device__ __forceinline__ bool operator==(DF a, DF b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(DF a, DF b) { return !(a == b); }
__device__ __forceinline__ DF s_abs(DF a) { return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? -a : a; }
__device__ __forceinline__ DF s_exp(DF a) { return DF(df_exp(a.p())); }
__device__ __forceinline__ DF s_log(DF a) { return DF(df_log(a.p())); }
__device__ __forceinline__ DF s_pow15(DF a) { return a * DF(df_sqrt(a.p())); }
__device__ __forceinline__ double s_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double s_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float s_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float s_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ DF s_max(DF a, DF b) { return a < b ? b : a; }
__device__ __forceinline__ DF s_min(DF a, DF b) { return b < a ? b : a; }
template <> struct Consts<DF> {
  static __device__ __forceinline__ DF dbl_eps() { return DF(2.2204460492503131e-16); }
  static __device__ __forceinline__ DF dbl_min() { return DF(f2{0.f, 0.f}); }  // below the float range
};
// warp shuffles of the marginalisation's number types
__device__ __forceinline__ double sshfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float sshfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ DF sshfl_xor(DF v, int m) {
  return DF(f2{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)});
}
__device__ __forceinline__ double sshfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float sshfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ DF sshfl(DF v, int src) {
  return DF(f2{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)});
}
template <> __device__ __forceinline__ DF wsum<DF>(DF v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v = v + sshfl_xor(v, m);
  return v;
}
// the 41-point rule's abscissae and weights (c_xgk, c_wgk, c_wg) as float pairs
__constant__ float2 c_xgk2[21] = {
    {0.9988590478897095f, -1.6301431315923764e-08f}, {0.9931285977363586f, 1.4487362420823047e-09f},
    {0.9815078973770142f, -1.9926764238675787e-08f}, {0.9639719128608704f, 1.4417043558978548e-08f},
    {0.9408226609230042f, -2.709125013211633e-08f}, {0.9122344255447388f, 2.7065871766041028e-09f},
    {0.8782768249511719f, -1.3698890022340038e-08f}, {0.8391169905662537f, -1.874403565693683e-08f},
    {0.7950414419174194f, -1.3079867855481098e-08f}, {0.7463319301605225f, -2.3700371443169388e-08f},
    {0.6932376623153687f, -5.9806173346999e-09f}, {0.6360536813735962f, -6.470811664271992e-10f},
    {0.5751404762268066f, -2.9407097201783472e-08f}, {0.5108669996261597f, 2.324667569553185e-09f},
    {0.44359317421913147f, 1.0195936317458631e-09f}, {0.3737061023712158f, -1.3655796493594607e-08f},
    {0.30162787437438965f, -6.259476492687099e-09f}, {0.2277858555316925f, -4.390047436686473e-09f},
    {0.15260545909404755f, 6.146875008994357e-09f}, {0.07652652263641357f, -1.502916235907037e-09f},
    {0.0f, 0.0f}};
__constant__ float2 c_wgk2[21] = {
    {0.003073583822697401f, -1.0417686852060015e-10f}, {0.008600269444286823f, 4.113561158369805e-10f},
    {0.014626169577240944f, -3.2026969964960017e-10f}, {0.020388374105095863f, -6.438293231880721e-10f},
    {0.025882134214043617f, -6.090924431489952e-10f}, {0.0312873050570488f, 1.719984044079581e-09f},
    {0.03660016879439354f, 9.638072562268007e-10f}, {0.04166887328028679f, 4.768689609857546e-11f},
    {0.04643482342362404f, -1.5561263388974567e-09f}, {0.05094457417726517f, -2.535364695965825e-10f},
    {0.05519510433077812f, 1.0175078557494999e-09f}, {0.059111401438713074f, -5.580734763199757e-10f},
    {0.06265323609113693f, 1.4636442058346688e-09f}, {0.06583459675312042f, 3.80497994223461e-10f},
    {0.06864867359399796f, -6.654763406999109e-10f}, {0.07105442136526108f, 2.188182968154706e-09f},
    {0.07303068786859512f, 2.4641915175038775e-09f}, {0.07458287477493286f, 6.255663209664419e-10f},
    {0.07570450007915497f, -2.3945982974282742e-09f}, {0.07637786865234375f, -9.802629818977948e-10f},
    {0.07660071551799774f, -3.5999980774192863e-09f}};
__constant__ float2 c_wg2[10] = {
    {0.017614006996154785f, 1.429973361943837e-10f}, {0.04060142859816551f, 1.2022214335161152e-09f},
    {0.06267204880714417f, -4.730351110815434e-10f}, {0.08327674120664597f, 3.7005878916751556e-10f},
    {0.10193011909723282f, 7.200076090896346e-10f}, {0.11819453537464142f, -3.4131231174683307e-09f},
    {0.13168863952159882f, -1.0724221510827192e-09f}, {0.14209610223770142f, 7.080680486382107e-09f},
    {0.14917299151420593f, -5.041602246791399e-09f}, {0.15275338292121887f, 4.2095069652248185e-09f}};
template <class S> __device__ __forceinline__ S kr(double d, float2 f) { return S(d); }
template <> __device__ __forceinline__ DF kr<DF>(double d, float2 f) { return DF(f2{f.x, f.y}); }

// state of the marginalisation over the scalelength (marginalise_posterior_warp)
template <class T>
struct MargShared {
  // natural spline rows and the factorisation of its matrix for the abscissae fac_x[0..fac_n)
  T soff[kMaxNodes], sdiag[kMaxNodes], sg[kMaxNodes], sz[kMaxNodes], salpha[kMaxNodes], sgamma[kMaxNodes];
  T fac_x[kMaxNodes];
  int fac_n;
  T xs[kMaxNodes], ys[kMaxNodes], cs[kMaxNodes];
  T sb[kMaxNodes], sd[kMaxNodes];         // linear and cubic spline coefficients of each interval
  T qa[kQagCap], qb[kQagCap], qr[kQagCap], qe[kQagCap];
  int status;
};
// the marginalisation's number type of a fit policy: double-float for the FP64 fit
template <class S> struct MargNumT { using T = S; };
template <> struct MargNumT<double> { using T = DF; };
template <class S> using MargNum = typename MargNumT<S>::T;

template <class S>
struct FitShared {
  // phased node evaluation (eval_nodes): per-node state
  double nx[kMaxNodes], ny[kMaxNodes];    // position shift of each node's Newton search
  double nnorm[kMaxNodes];                // 1 / the node's model normalisation
  int alist[kMaxNodes];                   // nodes with a Newton pass pending
  int nact;
  S Lr[kMaxNodes];
  S rprior[kMaxNodes];
  MargShared<MargNum<S>> mg;              // the marginalisation over the scalelength
  S bcast_L;
  int bcast_err;
  int g;
  int newton;
  // sampling board: a claimed grid point and its chunk (owner and helper CTAs)
  SampleSlot claim_prm;
  int claim_g, claim_seq, claim_idx, claim_state;
  int bcast_np;
  int status;
};

// ------------------------------------------------- scalelength marginalisation
template <class S>
__device__ __forceinline__ S spline_eval(const MargShared<S>& sh, int n, bool cubic, S x, bool* ok) {
  if (x < sh.xs[0] || x > sh.xs[n - 1]) { *ok = false; return S(0); }
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (sh.xs[mid] > x) hi = mid; else lo = mid;
  }
  const S x_lo = sh.xs[lo], x_hi = sh.xs[lo + 1];
  const S y_lo = sh.ys[lo], y_hi = sh.ys[lo + 1];
  const S dx = x_hi - x_lo, dy = y_hi - y_lo, delx = x - x_lo;
  *ok = true;
  // cubic: the coefficients of gsl_interp_cspline's evaluation, made once per spline (spline_coeffs)
  if (cubic) return y_lo + delx * (sh.sb[lo] + delx * (sh.cs[lo] + delx * sh.sd[lo]));
  return y_lo + delx / dx * dy;
}

// b_i and d_i of every interval of the natural cubic spline (xs, ys, cs), lane i: as the
// reference's interpolation evaluates them per point (gsl_interp_cspline), once per spline
template <class S>
__device__ __forceinline__ void spline_coeffs(MargShared<S>& sh, int n) {
  const int i = threadIdx.x & 31;
  if (i < n - 1) {
    const S dx = sh.xs[i + 1] - sh.xs[i], dy = sh.ys[i + 1] - sh.ys[i];
    const S c_i = sh.cs[i], c_ip1 = sh.cs[i + 1];
    sh.sb[i] = (dy / dx) - dx * (c_ip1 + S(2) * c_i) / S(3);
    sh.sd[i] = (c_ip1 - c_i) / (S(3) * dx);
  }
  __syncwarp();
}

// integrand of marginalise_r.c:231-238: exp(spline(x)), 0 outside the nodes
template <class S>
__device__ __forceinline__ S marf(const MargShared<S>& sh, int n, bool cubic, S x) {
  bool ok;
  S y = spline_eval(sh, n, cubic, x, &ok);
  return ok ? s_exp(y) : S(0);
}

template <class S>
__device__ __forceinline__ S rescale_error(S err, S result_abs, S result_asc) {
  err = s_abs(err);
  if (result_asc != S(0) && err != S(0)) {
    S scale = s_pow15(S(200) * err / result_asc);
    err = (scale < S(1)) ? result_asc * scale : result_asc;
  }
  if (result_abs > Consts<S>::dbl_min() / (S(50) * Consts<S>::dbl_eps())) {
    S min_err = S(50) * Consts<S>::dbl_eps() * result_abs;
    if (min_err > err) err = min_err;
  }
  return err;
}

// QUADPACK qk41 on one warp: lane j < 21 evaluates the integrand at centre -+ half*xgk[j].
template <class S>
__device__ __noinline__ void qk41_warp(const MargShared<S>& sh, int n, bool cubic, S a, S b, S* result, S* abserr,
                          S* resabs, S* resasc) {
  const int j = threadIdx.x & 31;
  const S center = S(0.5) * (a + b);
  const S half = S(0.5) * (b - a);
  const S abs_half = s_abs(half);
  S f1 = S(0), f2 = S(0);
  if (j < 21) {
    const S absc = half * kr<S>(c_xgk[j], c_xgk2[j]);
    f1 = marf(sh, n, cubic, center - absc);
    f2 = (j == 20) ? f1 : marf(sh, n, cubic, center + absc);
  }
  const S fc = sshfl(f1, 20);
  const S wk = (j < 20) ? kr<S>(c_wgk[j], c_wgk2[j]) : S(0);
  const S wg = (j < 20 && (j & 1)) ? kr<S>(c_wg[j >> 1], c_wg2[j >> 1]) : S(0);
  const S fsum = f1 + f2;
  S rk = wsum<S>(wk * fsum) + fc * kr<S>(c_wgk[20], c_wgk2[20]);
  S rg = wsum<S>(wg * fsum);
  S ra = wsum<S>(wk * (s_abs(f1) + s_abs(f2))) + s_abs(fc * kr<S>(c_wgk[20], c_wgk2[20]));
  const S mean = rk * S(0.5);
  S rasc = wsum<S>(wk * (s_abs(f1 - mean) + s_abs(f2 - mean))) + kr<S>(c_wgk[20], c_wgk2[20]) * s_abs(fc - mean);
  const S err = (rk - rg) * half;
  rk *= half;
  ra *= abs_half;
  rasc *= abs_half;
  *result = rk;
  *resabs = ra;
  *resasc = rasc;
  *abserr = rescale_error<S>(err, ra, rasc);
}

// QUADPACK qag (GSL gsl_integration_qag, key GSL_INTEG_GAUSS41, epsabs 0, epsrel 1e-3):
// global adaptive bisection of the interval with the largest error.  Control is replicated in
// the lanes of warp 0; interval lists live in shared memory (kQagCap entries).
// Returns 0 on success, nonzero as GSL's status would be.
template <class S>
__device__ __noinline__ int qag_warp(MargShared<S>& sh, int n, bool cubic, S a, S b, S* out) {
  const int lane = threadIdx.x & 31;
  const S epsabs = S(0), epsrel = S(1.e-3);
  S result0, abserr0, resabs0, resasc0;
  qk41_warp<S>(sh, n, cubic, a, b, &result0, &abserr0, &resabs0, &resasc0);
  S tolerance = s_max(epsabs, epsrel * s_abs(result0));
  const S round_off = S(50) * Consts<S>::dbl_eps() * resabs0;
  *out = result0;
  if (abserr0 <= round_off && abserr0 > tolerance) return 18;        // GSL_EROUND
  if ((abserr0 <= tolerance && abserr0 != resasc0) || abserr0 == S(0)) return 0;
  if (lane == 0) { sh.qa[0] = a; sh.qb[0] = b; sh.qr[0] = result0; sh.qe[0] = abserr0; }
  __syncwarp();
  S area = result0, errsum = abserr0;
  int nint = 1, iteration = 1, roundoff1 = 0, roundoff2 = 0, error_type = 0;
  const int limit = 1000;
  do {
    // interval with the largest error (lowest index on ties)
    S best = S(-1);
    int bi = 0x7fffffff;
    for (int k = lane; k < nint; k += 32) {
      S e = sh.qe[k];
      if (e > best) { best = e; bi = k; }
    }
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
      S ob = sshfl_xor(best, m);
      int oi = __shfl_xor_sync(0xffffffffu, bi, m);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int imax = bi;
    const S a_i = sh.qa[imax], b_i = sh.qb[imax], r_i = sh.qr[imax], e_i = sh.qe[imax];
    const S a1 = a_i, b1 = S(0.5) * (a_i + b_i), a2 = b1, b2 = b_i;
    S area1, area2, error1, error2, resabs1, resabs2, resasc1, resasc2;
    qk41_warp<S>(sh, n, cubic, a1, b1, &area1, &error1, &resabs1, &resasc1);
    qk41_warp<S>(sh, n, cubic, a2, b2, &area2, &error2, &resabs2, &resasc2);
    const S area12 = area1 + area2, error12 = error1 + error2;
    errsum += (error12 - e_i);
    area += area12 - r_i;
    if (resasc1 != error1 && resasc2 != error2) {
      const S delta = r_i - area12;
      if (s_abs(delta) <= S(1.0e-5) * s_abs(area12) && error12 >= S(0.99) * e_i) roundoff1++;
      if (iteration >= 10 && error12 > e_i) roundoff2++;
    }
    tolerance = s_max(epsabs, epsrel * s_abs(area));
    if (errsum > tolerance) {
      if (roundoff1 >= 6 || roundoff2 >= 20) error_type = 2;
      const S tmp = (S(1) + S(100) * Consts<S>::dbl_eps()) * (s_abs(a2) + S(1000) * Consts<S>::dbl_min());
      if (s_abs(a1) <= tmp && s_abs(b2) <= tmp) error_type = 3;
    }
    __syncwarp();
    if (lane == 0) {
      sh.qa[imax] = a1; sh.qb[imax] = b1; sh.qr[imax] = area1; sh.qe[imax] = error1;
      sh.qa[nint] = a2; sh.qb[nint] = b2; sh.qr[nint] = area2; sh.qe[nint] = error2;
    }
    __syncwarp();
    nint++;
    iteration++;
    if (nint >= kQagCap && errsum > tolerance && !error_type) {
      if (lane == 0) sh.status |= 2;
      error_type = 4;  // device interval capacity: reported like GSL_EMAXITER
    }
  } while (iteration < limit && !error_type && errsum > tolerance);
  S sum = S(0);
  for (int k = lane; k < nint; k += 32) sum += sh.qr[k];
  sum = wsum<S>(sum);
  *out = sum;
  if (errsum <= tolerance) return 0;
  if (error_type == 2) return 18;
  if (error_type == 3) return 21;
  return 11;
}

// marginalise_r.c:81-223 on warp 0; (xs, ys, numvals) already in shared memory.
template <class S>
__device__ __noinline__ S marginalise_posterior_warp(MargShared<S>& sh, int n) {
  const int lane = threadIdx.x & 31;
  const bool in = lane < n;
  const S y_l = in ? sh.ys[lane] : S(0);
  const S x_l = in ? sh.xs[lane] : S(0);
  // ymax: the first maximum above -10 (strict comparison from ymax = -10, marginalise_r.c:90-96)
  S ymax = (in && y_l > S(-10.0)) ? y_l : S(-10.0);
  int ypos = (in && y_l > S(-10.0)) ? lane : 0x7fffffff;
  // xmin, xmax: the node range (it contains the maximum's neighbours, marginalise_r.c:97-106)
  S xmin = in ? x_l : S(1e300), xmax = in ? x_l : S(-1e300);
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    const S oy = sshfl_xor(ymax, m);
    const int op = __shfl_xor_sync(0xffffffffu, ypos, m);
    if (oy > ymax || (oy == ymax && op < ypos)) { ymax = oy; ypos = op; }
    xmin = s_min(xmin, sshfl_xor(xmin, m));
    xmax = s_max(xmax, sshfl_xor(xmax, m));
  }
  if (in) { sh.ys[lane] = y_l - ymax; sh.cs[lane] = S(0); }
  // natural cubic spline: c_0 = c_{n-1} = 0, interior from the symmetric tridiagonal system
  // solved by LDL^T (as gsl_interp_cspline).  The lanes form the rows; the factorisation
  // (alpha, gamma) depends only on the abscissae and is kept while they do not change.
  const int m = n - 2;
  __syncwarp();
  if (lane < m) {
    const int i = lane;
    const S h_i = sh.xs[i + 1] - sh.xs[i], h_ip1 = sh.xs[i + 2] - sh.xs[i + 1];
    const S dy_i = sh.ys[i + 1] - sh.ys[i], dy_ip1 = sh.ys[i + 2] - sh.ys[i + 1];
    const S g_i = (h_i != S(0)) ? S(1) / h_i : S(0);
    const S g_ip1 = (h_ip1 != S(0)) ? S(1) / h_ip1 : S(0);
    sh.soff[i] = h_ip1;
    sh.sdiag[i] = S(2) * (h_ip1 + h_i);
    sh.sg[i] = S(3) * (dy_ip1 * g_ip1 - dy_i * g_i);
  }
  const bool same = __all_sync(0xffffffffu, !in || sh.fac_x[lane] == x_l) && sh.fac_n == n;
  __syncwarp();
  if (m == 1) {
    if (lane == 0) sh.cs[1] = sh.sg[0] / sh.sdiag[0];
  } else if (m > 1) {
    if (!same) {
      if (lane == 0) {
        sh.salpha[0] = sh.sdiag[0];
        sh.sgamma[0] = sh.soff[0] / sh.salpha[0];
        for (int i = 1; i < m - 1; i++) {
          sh.salpha[i] = sh.sdiag[i] - sh.soff[i - 1] * sh.sgamma[i - 1];
          sh.sgamma[i] = sh.soff[i] / sh.salpha[i];
        }
        sh.salpha[m - 1] = sh.sdiag[m - 1] - sh.soff[m - 2] * sh.sgamma[m - 2];
        sh.fac_n = n;
      }
      if (in) sh.fac_x[lane] = x_l;
    }
    __syncwarp();
    if (lane == 0) {
      S z = sh.sg[0];
      sh.sz[0] = z;
      for (int i = 1; i < m; i++) {
        z = sh.sg[i] - sh.sgamma[i - 1] * z;
        sh.sz[i] = z;
      }
    }
    __syncwarp();
    if (lane < m) sh.sz[lane] = sh.sz[lane] / sh.salpha[lane];
    __syncwarp();
    if (lane == 0) {
      S c = sh.sz[m - 1];
      sh.cs[m] = c;
      for (int k = m - 1; k-- > 0;) {
        c = sh.sz[k] - sh.sgamma[k] * c;
        sh.cs[k + 1] = c;
      }
    }
  }
  __syncwarp();
  spline_coeffs<S>(sh, n);
  if (xmax <= xmin) return S(kBad);  // the reference exits the process here
  S sump;
  int status = qag_warp<S>(sh, n, true, xmin, xmax, &sump);
  if (status) status = qag_warp<S>(sh, n, false, xmin, xmax, &sump);
  if (status) return S(kBad);
  return s_log(sump) + ymax;
}

// ------------------------------------------------------------ phased nodes
// Ei(x1) and Ei(x2), 0 < x <= 100, evaluated by one lane (each lane its own x).
//   x <= 2.5: the power series  gamma + ln x + sum_k x^k / (k k!)  (at most 26 terms);
//   x > 2.5: the Taylor expansion about the nearest integer x0 of
//       Ei(x) = Ei(x0) + e^x0 int_0^s e^t / (x0 + t) dt,   s = x - x0,  |s| <= 1/2,
//     with e^t / (x0 + t) = sum_n c_n t^n,  c_0 = 1/x0,  c_n = (1/n! - c_(n-1)) / x0  (from
//     (x0 + t) sum c_n t^n = e^t), so  Ei(x) = Ei(x0) + e^x0 sum_n c_n s^(n+1) / (n+1);  the terms
//     shrink at least as (1/6)^n.  Ei(x0) and e^x0 come from a table made on the host in extended
//     precision.
// The recurrences run in double-float on the FP32 pipes (dependent FP64 operations take 64 cycles
// and more here), the two in one loop so that their latencies overlap; each expansion stops at its
// first term below 2^-53 of its sum, under the pair's ~2^-47 precision (the series alone would
// need up to ~100 terms over (0, 100]).  The closing sums and the tables stay in double.
__device__ __forceinline__ f2 df_c(float2 v) { return f2{v.x, v.y}; }
__device__ __forceinline__ void ei_pair_df(double x1, double x2, double* e1, double* e2) {
  const bool ser1 = x1 <= 2.5, ser2 = x2 <= 2.5;
  const int k1 = ser1 ? 0 : (int)(x1 + 0.5), k2 = ser2 ? 0 : (int)(x2 + 0.5);
  const f2 s1 = df_from_double(ser1 ? x1 : x1 - k1), s2 = df_from_double(ser2 ? x2 : x2 - k2);
  const f2 i1 = df_c(c_invk2[k1]), i2 = df_c(c_invk2[k2]);
  // series: c = s^k / k!, term c / k;  Taylor: c = c_k, p = s^(k+1), term c p / (k+1)
  f2 c1 = ser1 ? f2{1.f, 0.f} : i1, c2 = ser2 ? f2{1.f, 0.f} : i2;
  f2 p1 = s1, p2 = s2;
  f2 a1 = ser1 ? f2{0.f, 0.f} : df_mul(i1, s1), a2 = ser2 ? f2{0.f, 0.f} : df_mul(i2, s2);
  bool run1 = true, run2 = true;
  for (int k = 1; k < kEiTerms - 1 && (run1 || run2); ++k) {
    const f2 ik = df_c(c_invk2[k]), ik1 = df_c(c_invk2[k + 1]), ifk = df_c(c_invfact2[k]);
    if (run1) {
      f2 t;
      if (ser1) { c1 = df_mul(df_mul(c1, s1), ik); t = df_mul(c1, ik); }
      else { c1 = df_mul(df_sub(ifk, c1), i1); p1 = df_mul(p1, s1); t = df_mul(df_mul(c1, p1), ik1); }
      a1 = df_add(a1, t);
      if (fabsf(t.hi) < 1.1102230246251565e-16f * fabsf(a1.hi)) run1 = false;
    }
    if (run2) {
      f2 t;
      if (ser2) { c2 = df_mul(df_mul(c2, s2), ik); t = df_mul(c2, ik); }
      else { c2 = df_mul(df_sub(ifk, c2), i2); p2 = df_mul(p2, s2); t = df_mul(df_mul(c2, p2), ik1); }
      a2 = df_add(a2, t);
      if (fabsf(t.hi) < 1.1102230246251565e-16f * fabsf(a2.hi)) run2 = false;
    }
  }
  const double d1 = df_to_double(a1), d2 = df_to_double(a2);
  *e1 = ser1 ? kEulerGamma + log(x1) + d1 : c_ei_tab[k1] + c_exp_tab[k1] * d1;
  *e2 = ser2 ? kEulerGamma + log(x2) + d2 : c_ei_tab[k2] + c_exp_tab[k2] * d2;
}

// likelihood.c:376-421 for one lane's own x = S^2 / 2, with - log(det) / 2 of likelihood.c:171
// added (det > 0): the logs and quotients in double-float.  log(Delta) and exp(-Delta) are the
// double values of the reference's expressions.
__device__ double pos_marg_lane(double x, double det) {
  const double Delta = 0.5 * 5.991;
  if (x <= Delta) return kBad;
  const f2 ld = df_log_double(det);
  if (x > 100.) return x - 1.0971111625418426 - 0.05001161502657909 - 0.5 * df_to_double(ld);
  if ((x - Delta) < 0.0001) x = Delta + 0.0001;
  double yc, ys;
  ei_pair_df(x, x - Delta, &yc, &ys);
  // log((yc - ys) / log(x / (x - Delta))) - log(det) / 2
  const f2 lr = df_log(df_div(df_from_double(x), df_from_double(x - Delta)));
  return df_to_double(df_sub(df_sub(df_log_double(yc - ys), df_log(lr)), df_scale(ld, 0.5f)));
}

// sin and cos of a double |a| <= pi/4 from their Taylor series (coefficients 1/n!, split into
// float pairs), the low-order terms in double-float and the terms below ~2e-9 of the result in
// float:  sin a = a * sum_k (-1)^k y^k / (2k+1)!,  cos a = sum_k (-1)^k y^k / (2k)!,  y = a^2.
// Relative error ~1e-14 (double-float carries 48 bits).  About 150 FP32 operations replace the
// ~40 FP64 ones of sincos(), which at this GPU's FP64 rate cost as much as ~3000 FP32 ones.
__device__ __forceinline__ void df_sincos_small(f2 x, f2* sa, f2* ca) {
  const f2 y = df_mul(x, x);
  const float yf = y.hi;
  // sin: tail k = 5..9 in float, k = 0..4 in double-float
  float t = -8.220635078476521e-18f;                                        // -1/19!
  t = fmaf(t, yf, 2.8114573589663704e-15f);                                 // 1/17!
  t = fmaf(t, yf, -7.647163609812713e-13f);                                 // -1/15!
  t = fmaf(t, yf, 1.6059044372074283e-10f);                                 // 1/13!
  t = fmaf(t, yf, -2.5052107943679403e-08f);                                // -1/11!
  f2 P{t, 0.f};
  P = df_horner(P, y, 2.7557318844628753e-06f, 3.793571224297229e-14f);   // 1/9!
  P = df_horner(P, y, -0.00019841270113829523f, 2.725596874933456e-12f);  // -1/7!
  P = df_horner(P, y, 0.008333333767950535f, -4.34617203337595e-10f);     // 1/5!
  P = df_horner(P, y, -0.1666666716337204f, 4.967053879312289e-09f);     // -1/3!
  P = df_horner(P, y, 1.f, 0.f);
  const f2 sv = df_mul(x, P);
  // cos: tail k = 6..10 in float, k = 0..5 in double-float
  float u = 4.110317590937049e-19f;                                        // 1/20!
  u = fmaf(u, yf, -1.5619206814541513e-16f);                                // -1/18!
  u = fmaf(u, yf, 4.7794772561329454e-14f);                                 // 1/16!
  u = fmaf(u, yf, -1.147074536050896e-11f);                                 // -1/14!
  u = fmaf(u, yf, 2.0876755879584152e-09f);                                 // 1/12!
  f2 Q{u, 0.f};
  Q = df_horner(Q, y, -2.755731998149713e-07f, 7.575112209051195e-15f);   // -1/10!
  Q = df_horner(Q, y, 2.4801587642286904e-05f, -3.40699609366682e-13f);   // 1/8!
  Q = df_horner(Q, y, -0.0013888889225199819f, 3.3631094437103215e-11f);  // -1/6!
  Q = df_horner(Q, y, 0.0416666679084301f, -1.2417634698280722e-09f);     // 1/4!
  Q = df_horner(Q, y, -0.5f, 0.f);                                         // -1/2!
  Q = df_horner(Q, y, 1.f, 0.f);
  *sa = sv;
  *ca = Q;
}
__device__ __forceinline__ void dsincos_small(double a, double* sa, double* ca) {
  f2 s, c;
  df_sincos_small(df_from_double(a), &s, &c);
  *sa = df_to_double(s);
  *ca = df_to_double(c);
}
// a double as a float pair from its bits with integer operations (a conversion through the FP64
// pipe costs ~80 cycles here): hi = the sign, exponent and top 23 fraction bits, lo = the low 29
// bits (rounded to 24) scaled to their place (a normal float for exponents from -74).  Zero and
// subnormal doubles give 0; other exponents below -74 or above 127 take the FP64 conversion.
__device__ __forceinline__ f2 df_from_double_bits(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -74 || e > 127) return (b & 0x7ff0000000000000ull) ? df_from_double(d) : f2{0.f, 0.f};
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  const float scale = __uint_as_float((unsigned)(e - 52 + 127) << 23);  // 2^(e - 52), e - 52 >= -126
  const float lo = (float)(unsigned)(b & 0x1fffffffull) * scale;
  return f2{hi, sign ? -lo : lo};
}

// (1 + q)^(-3/2), q >= 0, in double-float.  With y the FP32 estimate of (1 + q)^(-1/2) and
// e = 1 - (1 + q) y^2 (|e| ~1e-7), (1 + q)^(-1/2) = y (1 - e)^(-1/2) = y (1 + e/2 + 3e^2/8 + ...)
// by the binomial series; the terms kept leave O(e^3) ~1e-21, below the pair's precision.
__device__ __forceinline__ f2 df_profile_exp(f2 q) {
  const f2 den = df_add(f2{1.f, 0.f}, q);
  const float y = rsqrtf(den.hi);
  const f2 e = df_sub(f2{1.f, 0.f}, df_mul(den, two_prod(y, y)));
  const f2 c = df_add(f2{0.5f * e.hi, 0.5f * e.lo}, f2{0.375f * e.hi * e.hi, 0.f});
  const f2 r = df_add(f2{y, 0.f}, df_mul(f2{y, 0.f}, c));
  return df_mul(df_sqr(r), r);
}
// the exponential-profile model of one cell (galaxy_visibilities.c:48-53 with the sheared k of
// :63-69), double-float: k1 = a1 u + a2 v, k2 = a2 u + a3 v, (1 + sfw (k1^2 + k2^2))^(-3/2)
__device__ __forceinline__ f2 df_cell_model(f2 a1, f2 a2, f2 a3, f2 u, f2 v, f2 sfw) {
  const f2 k1 = df_add(df_mul(a1, u), df_mul(a2, v));
  const f2 k2 = df_add(df_mul(a2, u), df_mul(a3, v));
  return df_profile_exp(df_mul(sfw, df_add(df_sqr(k1), df_sqr(k2))));
}

__device__ __forceinline__ void pass_sincos(double a, double* sa, double* ca) {
  if (fabs(a) <= 0.78539816339744831) dsincos_small(a, sa, ca);
  else sincos(a, sa, ca);
}
__device__ __forceinline__ void pass_sincos(float a, float* sa, float* ca) { sincosf(a, sa, ca); }

// one lane's partial of a cross-correlation sum, as double
template <class A>
__device__ __forceinline__ double acc_value(const A& a);
template <>
__device__ __forceinline__ double acc_value(const Acc<double>& a) { return a.s; }
template <>
__device__ __forceinline__ double acc_value(const Acc<float>& a) { return (double)a.s - (double)a.c; }
__device__ __forceinline__ double node_sum(const double* p) {
  double s = p[0];
#pragma unroll
  for (int k = 1; k < kNodePart; ++k) s += p[k];
  return s;
}

// The likelihood at every scalelength node (likelihood.c:117-187 with the cross-correlation and
// Newton search of :194-358 and the position marginal of :376-421), into sh.Lr[1..numr-1].
//
// Cell passes: a node's cells run on a segment of kNodePart lanes (four nodes per warp; lane
// 8j + c takes cells c, c + 8, ... of the warp's j-th node) and every lane leaves its own partial
// of each sum in shared memory.  Most facets hold a few dozen cells, so a whole warp per node
// would leave most lanes idle, and an FP64 instruction costs this GPU's SM the same whatever
// number of its lanes are active.  Warp 0 then carries every node at once (lane = node): the
// sums, determinant and Newton step of each node and its position marginal.  The nodes step
// through their Newton iterations in lock-step rounds, each stopping by the reference's own test;
// a round's cell pass takes only the nodes still iterating, packed into consecutive segments.
template <class P>
__device__ void eval_nodes(FitShared<typename P::S>& sh, NodeCache& nc, const typename P::Cell* gu,
                           const typename P::Cell* gv, const typename P::Cell* dre,
                           const typename P::Cell* dim, const typename P::Cell* sig2, int n, double e1,
                           double e2) {
  using T = typename P::Cell;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int numR = c_fit.numr;
  const int gaussian = c_fit.gaussian;
  const T a1 = T(1.0 + e1), a2 = T(e2), a3 = T(1.0 - e1);
  const double detA = 1.0 - e1 * e1 - e2 * e2;
  const T cc = T(2 * kPi);
  const int seg = lane >> 3, c0 = lane & (kNodePart - 1);
  const int ncache = n < kNodeCache ? n : kNodeCache;
  // galaxy_visibilities.c:63-65 then the 4 pi^2 wave factor of :69
  auto sfw_of = [&](int node) -> T {
    const double sc = c_fit.ro[node] * (kPi / 648000.0);
    return T(((sc * sc) / (detA * detA)) * (4 * kPi * kPi));
  };
  // normalised model of an uncached cell (galaxy_visibilities.c:90 divides by the norm; the fit
  // multiplies by its reciprocal)
  auto model = [&](int i, T sfw, T inn) -> T {
    return cell_shape_fit<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw) * inn;
  };
  const int groups = (numR - 1 + kNodesPerWarp - 1) / kNodesPerWarp;
  // ---- A: model and its norm
  for (int i = threadIdx.x; i < ncache; i += blockDim.x) {
    nc.cu[i] = (double)(cc * T(gu[i]));
    nc.cv[i] = (double)(cc * T(gv[i]));
    nc.cu2[i] = df_from_double(nc.cu[i]);
    nc.cv2[i] = df_from_double(nc.cv[i]);
    nc.isg[i] = (double)(T(1) / T(sig2[i]));
    if (!P::kMixed && !gaussian) {
      nc.gu2[i] = df_from_double((double)gu[i]);
      nc.gv2[i] = df_from_double((double)gv[i]);
      nc.dre2[i] = df_from_double((double)dre[i]);
      nc.dim2[i] = df_from_double((double)dim[i]);
      nc.isg2[i] = df_from_double(nc.isg[i]);
    }
  }
  __syncthreads();
  // FP64 policy, exponential profile: the model and zero-shift passes and the model of the cells
  // beyond the cache in double-float (an FP64 (1 + q)^(-3/2) chain costs ~1200 cycles here)
  const bool dfm = !P::kMixed && !gaussian;
  const f2 a1d = df_from_double(1.0 + e1), a2d = df_from_double(e2), a3d = df_from_double(1.0 - e1);
  auto sfw_df = [&](int node) -> f2 {
    const double sc = c_fit.ro[node] * (kPi / 648000.0);
    return df_from_double(((sc * sc) / (detA * detA)) * (4 * kPi * kPi));
  };
  auto model_df = [&](int i, f2 sfw, f2 inn) -> f2 {
    return df_mul(df_cell_model(a1d, a2d, a3d, df_from_double_bits((double)gu[i]), df_from_double_bits((double)gv[i]),
                                sfw), inn);
  };
  for (int g = warp; g < groups; g += nw) {
    const int node = 1 + g * kNodesPerWarp + seg;
    if (dfm && node < numR) {
      const f2 sfw = sfw_df(node);
      f2 acc{0.f, 0.f};
      int i = c0;
      for (; i < ncache; i += kNodePart) {
        const f2 m = df_cell_model(a1d, a2d, a3d, nc.gu2[i], nc.gv2[i], sfw);
        nc.H(node, i).f = m;
        acc = df_add(acc, df_mul(df_sqr(m), nc.isg2[i]));
      }
      for (; i < n; i += kNodePart) {
        const f2 m = df_cell_model(a1d, a2d, a3d, df_from_double_bits((double)gu[i]), df_from_double_bits((double)gv[i]),
                                   sfw);
        acc = df_add(acc, df_div(df_sqr(m), df_from_double_bits((double)sig2[i])));
      }
      nc.P(0, node)[c0] = df_to_double(acc);
    } else if (node < numR) {
      const T sfw = sfw_of(node);
      Acc<T> acc;
      acc.zero();
      int i = c0;
      for (; i < ncache; i += kNodePart) {
        const T m = cell_shape_fit<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw);
        nc.H(node, i).d = (double)m;
        acc.add(m * m * T(nc.isg[i]));
      }
      for (; i < n; i += kNodePart) {
        const T m = cell_shape_fit<T>(gaussian, a1, a2, a3, T(gu[i]), T(gv[i]), sfw);
        acc.add(m * m / T(sig2[i]));
      }
      nc.P(0, node)[c0] = acc_value(acc);
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int node = lane;
    if (node >= 1 && node < numR) {
      const double s_norm = sqrt(node_sum(nc.P(0, node)));
      sh.nnorm[node] = 1.0 / s_norm;
    }
  }
  __syncthreads();
  // ---- B: cross-correlation at zero shift; caches data x model
  for (int g = warp; g < groups; g += nw) {
    const int node = 1 + g * kNodesPerWarp + seg;
    if (dfm && node < numR) {
      const f2 sfw = sfw_df(node), inn = df_from_double(sh.nnorm[node]);
      f2 val{0.f, 0.f}, dx{0.f, 0.f}, dy{0.f, 0.f}, d2x{0.f, 0.f}, d2y{0.f, 0.f}, dxy{0.f, 0.f};
      for (int i = c0; i < n; i += kNodePart) {
        const bool cached = i < kNodeCache;
        const f2 m = cached ? df_mul(nc.H(node, i).f, inn) : model_df(i, sfw, inn);
        const f2 hre = df_mul(cached ? nc.dre2[i] : df_from_double_bits((double)dre[i]), m);
        const f2 him = df_neg(df_mul(cached ? nc.dim2[i] : df_from_double_bits((double)dim[i]), m));
        if (cached) {
          nc.H(node, i).f = hre;
          nc.M(node, i).f = him;
        }
        const f2 u = cached ? nc.cu2[i] : df_from_double_bits((2 * kPi) * (double)gu[i]);
        const f2 v = cached ? nc.cv2[i] : df_from_double_bits((2 * kPi) * (double)gv[i]);
        val = df_add(val, hre);
        dx = df_sub(dx, df_mul(him, u));
        dy = df_sub(dy, df_mul(him, v));
        const f2 ru = df_mul(hre, u), rv = df_mul(hre, v);
        d2x = df_sub(d2x, df_mul(ru, u));
        d2y = df_sub(d2y, df_mul(rv, v));
        dxy = df_sub(dxy, df_mul(ru, v));
      }
      nc.P(1, node)[c0] = df_to_double(val); nc.P(2, node)[c0] = df_to_double(dx);
      nc.P(3, node)[c0] = df_to_double(dy); nc.P(4, node)[c0] = df_to_double(d2x);
      nc.P(5, node)[c0] = df_to_double(d2y); nc.P(6, node)[c0] = df_to_double(dxy);
    } else if (node < numR) {
      const T sfw = sfw_of(node), nn = T(sh.nnorm[node]);
      Acc<T> val, dx, dy, d2x, d2y, dxy;
      val.zero(); dx.zero(); dy.zero(); d2x.zero(); d2y.zero(); dxy.zero();
      for (int i = c0; i < n; i += kNodePart) {
        const T m = i < kNodeCache ? T(nc.H(node, i).d) * nn : model(i, sfw, nn);
        const T hre = T(dre[i]) * m, him = -T(dim[i]) * m;
        if (i < kNodeCache) {
          if constexpr (P::kMixed) {
            nc.H(node, i).d = (double)hre;
            nc.M(node, i).d = (double)him;
          } else {
            nc.H(node, i).f = df_from_double(hre);
            nc.M(node, i).f = df_from_double(him);
          }
        }
        const T u = cc * T(gu[i]), v = cc * T(gv[i]);
        val.add(hre);
        dx.sub(him * u);
        dy.sub(him * v);
        d2x.sub(hre * u * u);
        d2y.sub(hre * v * v);
        dxy.sub(hre * u * v);
      }
      nc.P(1, node)[c0] = acc_value(val); nc.P(2, node)[c0] = acc_value(dx);
      nc.P(3, node)[c0] = acc_value(dy); nc.P(4, node)[c0] = acc_value(d2x);
      nc.P(5, node)[c0] = acc_value(d2y); nc.P(6, node)[c0] = acc_value(dxy);
    }
  }
  __syncthreads();
  // ---- Newton rounds; warp 0 holds each node's state in its lane
  double Sval = 0, Sdx = 0, Sdy = 0, Sd2x = 0, Sd2y = 0, Sdxy = 0, det = 0;
  double xo = 0, yo = 0, norm = 1, normv = 0;
  int iter = 0;
  bool pending = true;  // this lane's node had a pass in the last round
  const bool mine = warp == 0 && lane >= 1 && lane < numR;
  const double tol = 1.e-7;
  while (true) {
    if (warp == 0) {
      bool act = false;
      if (mine && pending) {
        const int node = lane;
        Sval = node_sum(nc.P(1, node)); Sdx = node_sum(nc.P(2, node)); Sdy = node_sum(nc.P(3, node));
        Sd2x = node_sum(nc.P(4, node)); Sd2y = node_sum(nc.P(5, node)); Sdxy = node_sum(nc.P(6, node));
        det = Sd2x * Sd2y - Sdxy * Sdxy;
        if (iter > 0) norm = normv;
        if (det > 0 && norm > tol && iter < kNewtonMax) {
          iter++;
          const double incx = (Sdx * Sd2y - Sdy * Sdxy) / det;
          const double incy = (Sdy * Sd2x - Sdx * Sdxy) / det;
          xo -= incx;
          yo -= incy;
          normv = sqrt(incx * incx + incy * incy);
          sh.nx[node] = xo;
          sh.ny[node] = yo;
          act = true;
        }
      }
      pending = act;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (act) sh.alist[__popc(am & ((1u << lane) - 1u))] = lane;
      if (lane == 0) sh.nact = __popc(am);
    }
    __syncthreads();
    const int nact = sh.nact;
    if (!nact) break;
    const int agroups = (nact + kNodesPerWarp - 1) / kNodesPerWarp;
    for (int g = warp; g < agroups; g += nw) {
      const int k = g * kNodesPerWarp + seg;
      if (k >= nact) continue;
      const int node = sh.alist[k];
      const T sfw = sfw_of(node), nn = T(sh.nnorm[node]);
      if constexpr (!P::kMixed) {
        // FP64 policy: the Newton pass in double-float (FP32 pairs, ~48-bit significands): phase,
        // sin/cos, rotation and the six sums stay on the FP32 pipes
        const f2 xo2 = df_from_double(sh.nx[node]), yo2 = df_from_double(sh.ny[node]);
        f2 val{0.f, 0.f}, dx{0.f, 0.f}, dy{0.f, 0.f}, d2x{0.f, 0.f}, d2y{0.f, 0.f}, dxy{0.f, 0.f};
        auto cell = [&](f2 hre, f2 him, f2 u, f2 v) {
          const f2 a = df_add(df_mul(xo2, u), df_mul(yo2, v));
          f2 sa, ca;
          if (fabsf(a.hi) <= 0.785398f) {
            df_sincos_small(a, &sa, &ca);
          } else {
            double s8, c8;
            sincos(df_to_double(a), &s8, &c8);
            sa = df_from_double(s8);
            ca = df_from_double(c8);
          }
          const f2 rp = df_sub(df_mul(hre, ca), df_mul(him, sa));
          const f2 ip = df_add(df_mul(hre, sa), df_mul(him, ca));
          val = df_add(val, rp);
          dx = df_sub(dx, df_mul(ip, u));
          dy = df_sub(dy, df_mul(ip, v));
          const f2 ru = df_mul(rp, u), rv = df_mul(rp, v);
          d2x = df_sub(d2x, df_mul(ru, u));
          d2y = df_sub(d2y, df_mul(rv, v));
          dxy = df_sub(dxy, df_mul(ru, v));
        };
        int i = c0;
        for (; i < ncache; i += kNodePart) cell(nc.H(node, i).f, nc.M(node, i).f, nc.cu2[i], nc.cv2[i]);
        f2 sfwd{0.f, 0.f}, innd{0.f, 0.f};
        if (dfm && i < n) {
          sfwd = sfw_df(node);
          innd = df_from_double(sh.nnorm[node]);
        }
        for (; i < n; i += kNodePart) {
          if (dfm) {
            const f2 m = model_df(i, sfwd, innd);
            cell(df_mul(df_from_double_bits((double)dre[i]), m), df_neg(df_mul(df_from_double_bits((double)dim[i]), m)),
                 df_from_double_bits((2 * kPi) * (double)gu[i]), df_from_double_bits((2 * kPi) * (double)gv[i]));
          } else {
            const T m = model(i, sfw, nn);
            cell(df_from_double(T(dre[i]) * m), df_from_double(-T(dim[i]) * m), df_from_double(cc * T(gu[i])),
                 df_from_double(cc * T(gv[i])));
          }
        }
        nc.P(1, node)[c0] = df_to_double(val); nc.P(2, node)[c0] = df_to_double(dx);
        nc.P(3, node)[c0] = df_to_double(dy); nc.P(4, node)[c0] = df_to_double(d2x);
        nc.P(5, node)[c0] = df_to_double(d2y); nc.P(6, node)[c0] = df_to_double(dxy);
        continue;
      }
      const T txo = T(sh.nx[node]), tyo = T(sh.ny[node]);
      Acc<T> val, dx, dy, d2x, d2y, dxy;
      val.zero(); dx.zero(); dy.zero(); d2x.zero(); d2y.zero(); dxy.zero();
      auto cell = [&](T hre, T him, T u, T v) {
        const T a = txo * u + tyo * v;
        T sa, ca;
        pass_sincos(a, &sa, &ca);
        const T rp = (hre * ca - him * sa);
        const T ip = (hre * sa + him * ca);
        val.add(rp);
        dx.sub(ip * u);
        dy.sub(ip * v);
        d2x.sub(rp * u * u);
        d2y.sub(rp * v * v);
        dxy.sub(rp * u * v);
      };
      int i = c0;
      for (; i < ncache; i += kNodePart) cell(T(nc.H(node, i).d), T(nc.M(node, i).d), T(nc.cu[i]), T(nc.cv[i]));
      for (; i < n; i += kNodePart) {
        const T m = model(i, sfw, nn);
        cell(T(dre[i]) * m, -T(dim[i]) * m, cc * T(gu[i]), cc * T(gv[i]));
      }
      nc.P(1, node)[c0] = acc_value(val); nc.P(2, node)[c0] = acc_value(dx);
      nc.P(3, node)[c0] = acc_value(dy); nc.P(4, node)[c0] = acc_value(d2x);
      nc.P(5, node)[c0] = acc_value(d2y); nc.P(6, node)[c0] = acc_value(dxy);
    }
    __syncthreads();
  }
  // ---- position marginal and determinant term of every node
  if (mine) {
    double L = kBad;
    if (det > 0) {
      L = pos_marg_lane((Sval * Sval) * 0.5, det);
      if (isnan(L)) L = kBad;
    }
    sh.Lr[lane] = typename P::S(L);
  }
  if (warp == 0) {
    int it = mine ? iter : 0;
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) it += __shfl_xor_sync(0xffffffffu, it, m);
    if (lane == 0) sh.newton += it;
  }
  __syncthreads();
}

// CTA-collective loglikelihood(e1, e2) (likelihood.c:106-149).
template <class P>
__device__ typename P::S eval_loglike(FitShared<typename P::S>& sh, NodeCache& nc, const typename P::Cell* gu,
                                      const typename P::Cell* gv, const typename P::Cell* dre,
                                      const typename P::Cell* dim, const typename P::Cell* sig2,
                                      int n, typename P::S e1, typename P::S e2, int* error) {
  using S = typename P::S;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int numR = c_fit.numr;
  (void)nw;
  eval_nodes<P>(sh, nc, gu, gv, dre, dim, sig2, n, (double)e1, (double)e2);
  if (warp == 0) {
    // set_posterior_values (marginalise_r.c:29-64): the nodes with a likelihood, in node order
    const bool ok = lane >= 1 && lane < numR && sh.Lr[lane] > S(kBad);
    const unsigned okm = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const int pos = __popc(okm & ((1u << lane) - 1u));
      sh.mg.xs[pos] = MargNum<S>(c_fit.ro[lane]);
      sh.mg.ys[pos] = MargNum<S>(sh.Lr[lane] + sh.rprior[lane]);
    }
    const int num = __popc(okm);
    __syncwarp();
    S L_e;
    int err = 0;
    if (num > 4) {
      L_e = S(marginalise_posterior_warp<MargNum<S>>(sh.mg, num));
    } else {
      err = 1;
      L_e = S(kBad);
    }
    if (L_e == S(kBad)) err = 1;
    if (lane == 0) {
      sh.bcast_L = L_e;
      sh.bcast_err = err;
    }
  }
  __syncthreads();
  *error = sh.bcast_err;
  return sh.bcast_L;
}

// -------------------------------------------------------------- galaxy fit
template <class P>
struct FitCtx {
  FitShared<typename P::S>* sh;
  NodeCache* nc;
  const typename P::Cell *gu, *gv, *dre, *dim, *sig2;
  int n;
  int nevals;
  double* trace;   // optional evaluation record (thread 0 writes)
  int trace_cap;
  SampleBoard board;  // slot == nullptr: the sampling grid is evaluated by this CTA alone
  int g;              // the galaxy's index in the batch (board rows)
  int seq;            // chunks published so far
};

// ------------------------------------------------------------ sampling board
constexpr unsigned long long kBoardWaitNs = 2000000000ull;  // wait limit of owners and idle helpers

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ size_t board_row(int g, int seq) { return ((size_t)g * 2 + (seq & 1)) * kBoardCap; }

// a chunk's parameters as the owner published them (read after the claim, behind a fence)
__device__ __forceinline__ SampleSlot board_params(const SampleSlot* sl) {
  const volatile SampleSlot* v = sl;
  SampleSlot q;
  q.claim = 0;
  q.npts = v->npts; q.p0 = v->p0; q.lo1 = v->lo1; q.lo2 = v->lo2; q.n2 = v->n2;
  q.sampling = v->sampling; q.me1 = v->me1; q.me2 = v->me2; q.pad = 0;
  return q;
}

// Grid point idx of a published chunk (likelihood.c:507-514): evaluates the log-likelihood unless
// the point is the centre or outside |e| < 1 (err = -1), and publishes the result (thread 0 writes
// value, then the chunk sequence as the point's flag).  CTA-collective.
template <class P>
__device__ void board_point(FitShared<typename P::S>& sh, NodeCache& nc, const typename P::Cell* gu,
                            const typename P::Cell* gv, const typename P::Cell* dre, const typename P::Cell* dim,
                            const typename P::Cell* sig2, int n, const SampleBoard& bd, int g, int seq, int idx,
                            const SampleSlot& prm, int newton_before);

template <class P>
__device__ typename P::S eval_loglike(FitShared<typename P::S>& sh, NodeCache& nc, const typename P::Cell* gu,
                                      const typename P::Cell* gv, const typename P::Cell* dre,
                                      const typename P::Cell* dim, const typename P::Cell* sig2,
                                      int n, typename P::S e1, typename P::S e2, int* error);

template <class P>
__device__ void board_point(FitShared<typename P::S>& sh, NodeCache& nc, const typename P::Cell* gu,
                            const typename P::Cell* gv, const typename P::Cell* dre, const typename P::Cell* dim,
                            const typename P::Cell* sig2, int n, const SampleBoard& bd, int g, int seq, int idx,
                            const SampleSlot& prm, int newton_before) {
  using S = typename P::S;
  const int p = prm.p0 + idx;
  const int ie1 = prm.lo1 + 2 * (p / prm.n2), ie2 = prm.lo2 + 2 * (p % prm.n2);
  const S x_e1 = S(prm.me1) + ie1 * prm.sampling;
  const S x_e2 = S(prm.me2) + ie2 * prm.sampling;
  const S mod2 = x_e1 * x_e1 + x_e2 * x_e2;
  int err = -1;
  S L = S(0);
  if ((ie1 != 0 || ie2 != 0) && mod2 < S(1)) L = eval_loglike<P>(sh, nc, gu, gv, dre, dim, sig2, n, x_e1, x_e2, &err);
  if (threadIdx.x == 0) {
    const size_t o = board_row(g, seq) + idx;
    bd.L[o] = (double)L;
    bd.err[o] = err;
    if (newton_before >= 0) atomicAdd(&bd.newton[g], sh.newton - newton_before);
    __threadfence();
    atomicExch(&bd.flag[o], seq);
  }
}

// Owner side of one chunk: publish it, evaluate points until all are claimed, then wait (bounded)
// for the helpers' results.  CTA-collective; returns with the results visible to every thread.
template <class P>
__device__ void board_chunk(FitCtx<P>& c, int seq, const SampleSlot& prm) {
  FitShared<typename P::S>& sh = *c.sh;
  const SampleBoard& bd = c.board;
  SampleSlot* sl = bd.slot + c.g;
  if (threadIdx.x == 0) {
    volatile SampleSlot* v = sl;
    v->npts = prm.npts; v->p0 = prm.p0; v->lo1 = prm.lo1; v->lo2 = prm.lo2; v->n2 = prm.n2;
    v->sampling = prm.sampling; v->me1 = prm.me1; v->me2 = prm.me2;
    __threadfence();
    atomicExch(&sl->claim, (unsigned long long)seq << 32);
  }
  while (true) {
    if (threadIdx.x == 0) sh.claim_idx = (int)(atomicAdd(&sl->claim, 1ull) & 0xffffffffull);
    __syncthreads();
    const int idx = sh.claim_idx;
    if (idx >= prm.npts) break;
    board_point<P>(sh, *c.nc, c.gu, c.gv, c.dre, c.dim, c.sig2, c.n, bd, c.g, seq, idx, prm, -1);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const size_t row = board_row(c.g, seq);
    const unsigned long long t0 = global_ns();
    const unsigned long long limit = bd.wait_ns ? bd.wait_ns : kBoardWaitNs;
    for (int k = 0; k < prm.npts; ++k) {
      const volatile int* f = bd.flag + row + k;
      while (*f != seq) {
        if (global_ns() - t0 > limit) break;
        __nanosleep(200);
      }
      if (*f != seq) {  // a helper did not deliver within the limit: the point counts as an error
        bd.err[row + k] = 1;
        sh.status |= 8;
      }
    }
    __threadfence();
  }
  __syncthreads();
}

template <class P>
__device__ __noinline__ typename P::S loglike(FitCtx<P>& c, typename P::S e1, typename P::S e2,
                                              int* error) {
  c.nevals++;
  const typename P::S L = eval_loglike<P>(*c.sh, *c.nc, c.gu, c.gv, c.dre, c.dim, c.sig2, c.n, e1, e2, error);
  if (c.trace && threadIdx.x == 0 && c.nevals <= c.trace_cap) {
    double* t = c.trace + 4 * (size_t)(c.nevals - 1);
    t[0] = (double)e1; t[1] = (double)e2; t[2] = (double)L; t[3] = (double)*error;
  }
  return L;
}

// likelihood.c:87-100
template <class P>
__device__ __forceinline__ typename P::S f_likelihood(FitCtx<P>& c, typename P::S e1, typename P::S e2) {
  using S = typename P::S;
  int error = 0;
  S L;
  if (e1 * e1 + e2 * e2 < S(0.65)) L = loglike<P>(c, e1, e2, &error);
  else L = S(-1.e+10);
  return -L;
}

template <class S>
__device__ __forceinline__ bool s_finite(S x) { return isfinite(x); }

// GSL nmsimplex2 state for n = 2 (three vertices), replicated per thread.
template <class S>
struct Simplex {
  S x[3][2];
  S y[3];
  S c[2];
  S S2;
  S size;
};

template <class S>
__device__ __forceinline__ void nm_center(Simplex<S>& s) {
  for (int j = 0; j < 2; ++j) {
    S a = S(0);
    for (int i = 0; i < 3; ++i) a += s.x[i][j];
    s.c[j] = a * (S(1) / S(3));
  }
}
template <class S>
__device__ __forceinline__ S nm_size(Simplex<S>& s) {
  S ss = S(0);
  for (int i = 0; i < 3; ++i) {
    S t2 = S(0);
    for (int j = 0; j < 2; ++j) {
      S d = s.x[i][j] - s.c[j];
      t2 += d * d;
    }
    ss += t2;
  }
  s.S2 = ss / S(3);
  return s_sqrt(s.S2);
}
template <class S>
__device__ __forceinline__ void nm_update(Simplex<S>& s, int i, const S* xn, S val) {
  const S P = S(3);
  S dd = S(0), xmcd = S(0), dl[2];
  for (int j = 0; j < 2; ++j) {
    dl[j] = xn[j] - s.x[i][j];
    S xmc = s.x[i][j] - s.c[j];
    dd += dl[j] * dl[j];
    xmcd += xmc * dl[j];
  }
  const S d = s_sqrt(dd);
  s.S2 += (S(2) / P) * xmcd + ((P - S(1)) / P) * (d * d / P);
  for (int j = 0; j < 2; ++j) s.c[j] += (S(1) / P) * dl[j];
  for (int j = 0; j < 2; ++j) s.x[i][j] = xn[j];
  s.y[i] = val;
}

template <class P>
__device__ __forceinline__ typename P::S nm_corner(FitCtx<P>& c, Simplex<typename P::S>& s, typename P::S coeff,
                                                   int corner, typename P::S* xc) {
  using S = typename P::S;
  const S Pn = S(3);
  const S alpha = (S(1) - coeff) * Pn / (Pn - S(1));
  const S beta = (Pn * coeff - S(1)) / (Pn - S(1));
  for (int j = 0; j < 2; ++j) {
    xc[j] = alpha * s.c[j];
    xc[j] += beta * s.x[corner][j];
  }
  return f_likelihood<P>(c, xc[0], xc[1]);
}

// one nmsimplex2 iteration; returns 0 (GSL_SUCCESS) or 5 (GSL_EFAILED)
template <class P>
__device__ int nm_iterate(FitCtx<P>& c, Simplex<typename P::S>& s) {
  using S = typename P::S;
  S xc[2], xc2[2], val, val2;
  int hi = 0, s_hi = 1, lo = 0;
  S dhi = s.y[0], dlo = s.y[0], ds_hi = s.y[1];
  for (int i = 1; i < 3; ++i) {
    val = s.y[i];
    if (val < dlo) { dlo = val; lo = i; }
    else if (val > dhi) { ds_hi = dhi; s_hi = hi; dhi = val; hi = i; }
    else if (val > ds_hi) { ds_hi = val; s_hi = i; }
  }
  val = nm_corner<P>(c, s, S(-1), hi, xc);
  if (s_finite(val) && val < s.y[lo]) {
    val2 = nm_corner<P>(c, s, S(-2), hi, xc2);
    if (s_finite(val2) && val2 < s.y[lo]) nm_update(s, hi, xc2, val2);
    else nm_update(s, hi, xc, val);
  } else if (!s_finite(val) || val > s.y[s_hi]) {
    if (s_finite(val) && val <= s.y[hi]) nm_update(s, hi, xc, val);
    val2 = nm_corner<P>(c, s, S(0.5), hi, xc2);
    if (s_finite(val2) && val2 <= s.y[hi]) {
      nm_update(s, hi, xc2, val2);
    } else {
      bool bad = false;
      for (int i = 0; i < 3; ++i) {
        if (i == lo) continue;
        for (int j = 0; j < 2; ++j) s.x[i][j] = S(0.5) * (s.x[i][j] + s.x[lo][j]);
        S v = f_likelihood<P>(c, s.x[i][0], s.x[i][1]);
        s.y[i] = v;
        if (!s_finite(v)) bad = true;
      }
      nm_center(s);
      nm_size(s);
      if (bad) return 5;
    }
  } else {
    nm_update(s, hi, xc, val);  // plain reflection accepted
  }
  if (s.S2 > S(0)) s.size = s_sqrt(s.S2);
  else s.size = nm_size(s);
  return 0;
}

template <class S>
__device__ __forceinline__ int nm_lowest(const Simplex<S>& s) {
  int lo = 0;
  for (int i = 1; i < 3; ++i) if (s.y[i] < s.y[lo]) lo = i;
  return lo;
}

// likelihood.c:428-554; sampling/edim/start are float as in the reference, the other reals are S
// (double for F64, float for the mixed policy).
template <class P>
__device__ __noinline__ void likelihood_sampling(FitCtx<P>& c, typename P::S* mes_e1, typename P::S* mes_e2,
                                    typename P::S maxL, int np_max, typename P::S* var_e1,
                                    typename P::S* var_e2, typename P::S* oneDimvar) {
  using S = typename P::S;
  int error = 0;
  int ie1, ie2, np;
  S totL, L_e, average_1, average_2, cov, var1, var2, x_e1, x_e2;
  S xL1, xL2, mod2 = S(0);
  S L = S(1);
  const S threshold = S(0.05);
  const S max_e1 = *mes_e1, max_e2 = *mes_e2;
  average_1 = max_e1;
  average_2 = max_e2;
  var1 = max_e1 * max_e1;
  var2 = max_e2 * max_e2;
  cov = max_e1 * max_e2;
  totL = S(1);
  np = 1;
  float sampling = 0.05;
  if (max_e1 < S(0)) sampling = -0.05;
  int k1 = 0;
  x_e1 = max_e1;
  while (L > threshold && mod2 < S(1) && !error) {
    x_e1 += sampling;
    mod2 = x_e1 * x_e1 + max_e2 * max_e2;
    if (mod2 < S(1)) {
      L_e = loglike<P>(c, x_e1, max_e2, &error);
      if (!error) { L = s_exp(L_e - maxL); k1++; }
    }
  }
  if (L < threshold && k1 > 1) k1--;
  L = S(1);
  int k2 = 0;
  sampling = 0.05;
  if (max_e2 < S(0)) sampling = -0.05;
  x_e2 = max_e2;
  while (L > threshold && mod2 < S(1) && !error) {
    x_e2 += sampling;
    mod2 = x_e2 * x_e2 + max_e1 * max_e1;
    if (mod2 < S(1)) {
      L_e = loglike<P>(c, max_e1, x_e2, &error);
      if (!error) { L = s_exp(L_e - maxL); k2++; }
    }
  }
  if (L < threshold && k2 > 1) k2--;
  if (c.trace && threadIdx.x == 0 && c.trace_cap > 0) {  // debugging record: line-search extents
    double* t = c.trace + 4 * (size_t)(c.trace_cap - 1);
    t[0] = k1; t[1] = k2; t[2] = (double)L; t[3] = (double)np_max;
  }
  sampling = 0.05;
  float edim1 = k1 * sampling;
  float edim2 = k2 * sampling;
  float start1 = edim1;
  float start2 = edim2;
  while (np < np_max && sampling > kERes) {
    // loop bounds of likelihood.c:504-506, in float as there: first index -start/sampling
    // converted to int, last index while (float)ie <= start/sampling
    const float q1 = start1 / sampling, q2 = start2 / sampling;
    const int lo1 = (int)(-start1 / sampling), lo2 = (int)(-start2 / sampling);
    if (c.board.slot) {
      // the same points in the same order, evaluated through the sampling board
      int n1 = 0, n2 = 0;
      for (ie1 = lo1; (float)ie1 <= q1; ie1 += 2) n1++;
      for (ie2 = lo2; (float)ie2 <= q2; ie2 += 2) n2++;
      const int total = n1 * n2;
      for (int p0 = 0; p0 < total; p0 += kBoardCap) {
        SampleSlot prm;
        prm.claim = 0; prm.pad = 0;
        prm.npts = min(kBoardCap, total - p0);
        prm.p0 = p0; prm.lo1 = lo1; prm.lo2 = lo2; prm.n2 = n2;
        prm.sampling = sampling; prm.me1 = (double)max_e1; prm.me2 = (double)max_e2;
        c.seq++;
        board_chunk<P>(c, c.seq, prm);
        const size_t row = board_row(c.g, c.seq);
        // the accumulation runs on thread 0 alone: only it writes the galaxy's result, and the
        // replicated FP64 arithmetic (an exp per point) would cost every warp of the CTA
        if (threadIdx.x == 0)
        for (int k = 0; k < prm.npts; ++k) {
          const int e = c.board.err[row + k];
          if (e < 0) continue;
          const int p = p0 + k;
          ie1 = lo1 + 2 * (p / n2);
          ie2 = lo2 + 2 * (p % n2);
          x_e1 = max_e1 + ie1 * sampling;
          x_e2 = max_e2 + ie2 * sampling;
          c.nevals++;
          error = e;
          if (!error) {
            L_e = S(c.board.L[row + k]);
            L = s_exp(L_e - maxL);
            if (L >= threshold && !isinf(L)) {
              np++;
              xL1 = x_e1 * L;
              xL2 = x_e2 * L;
              average_1 += xL1;
              average_2 += xL2;
              var1 += x_e1 * xL1;
              var2 += x_e2 * xL2;
              cov += x_e1 * xL2;
              totL += L;
            }
          }
        }
      }
      // the level's point count decides the next level for every thread
      if (threadIdx.x == 0) c.sh->bcast_np = np;
      __syncthreads();
      np = c.sh->bcast_np;
      __syncthreads();
    } else {
      for (ie1 = lo1; (float)ie1 <= q1; ie1 += 2) {
        for (ie2 = lo2; (float)ie2 <= q2; ie2 += 2) {
          if (ie1 != 0 || ie2 != 0) {
            x_e1 = max_e1 + ie1 * sampling;
            x_e2 = max_e2 + ie2 * sampling;
            mod2 = x_e1 * x_e1 + x_e2 * x_e2;
            if (mod2 < S(1)) {
              L_e = loglike<P>(c, x_e1, x_e2, &error);
              if (!error) {
                L = s_exp(L_e - maxL);
                if (L >= threshold && !isinf(L)) {
                  np++;
                  xL1 = x_e1 * L;
                  xL2 = x_e2 * L;
                  average_1 += xL1;
                  average_2 += xL2;
                  var1 += x_e1 * xL1;
                  var2 += x_e2 * xL2;
                  cov += x_e1 * xL2;
                  totL += L;
                }
              }
            }
          }
        }
      }
    }
    sampling *= 0.5;
    start1 = edim1 - sampling;
    start2 = edim2 - sampling;
  }
  average_1 /= totL;
  average_2 /= totL;
  var1 /= totL; var1 -= average_1 * average_1;
  var2 /= totL; var2 -= average_2 * average_2;
  cov /= totL; cov -= average_1 * average_2;
  *mes_e1 = average_1;
  *mes_e2 = average_2;
  *var_e1 = var1;
  *var_e2 = var2;
  *oneDimvar = s_sqrt((var1) * (var2) - cov * cov);
}

// galaxy_fitting.c:41-117 with a configurable start point and step (reference: (0,0), 0.1)
template <class P>
__device__ __noinline__ FitOut fit_galaxy(FitCtx<P>& c, double start_e1, double start_e2, double step, int np_max) {
  using S = typename P::S;
  FitOut o;
  Simplex<S> s;
  int bad_start = 0;
  // gsl_multimin_fminimizer_set: x0 and x0 + step along each axis
  s.x[0][0] = S(start_e1); s.x[0][1] = S(start_e2);
  s.y[0] = f_likelihood<P>(c, s.x[0][0], s.x[0][1]);
  for (int i = 0; i < 2; ++i) {
    s.x[i + 1][0] = S(start_e1); s.x[i + 1][1] = S(start_e2);
    s.x[i + 1][i] = (i == 0 ? S(start_e1) : S(start_e2)) + S(step);
    s.y[i + 1] = f_likelihood<P>(c, s.x[i + 1][0], s.x[i + 1][1]);
  }
  for (int i = 0; i < 3; ++i) if (!s_finite(s.y[i])) bad_start = 1;
  nm_center(s);
  s.size = nm_size(s);
  int iter = 0, status = 0;
  S fval = s.y[0];
  int lo = 0;
  if (!bad_start) {
    do {
      iter++;
      status = nm_iterate<P>(c, s);
      lo = nm_lowest(s);
      fval = s.y[lo];
      if (status) break;
      status = (s.size < S(kTol)) ? 0 : -2;  // gsl_multimin_test_size
    } while (status == -2 && iter < kSimplexMax && fval < S(0));
  }
  S e1 = s.x[lo][0], e2 = s.x[lo][1];
  S maxL = -fval;
  if (e1 * e1 + e2 * e2 > S(0.65)) maxL = S(-1e+10);
  int error = 0;
  S v1 = S(0), v2 = S(0), od = S(0);
  if (bad_start) maxL = S(-1e+10);
  if (maxL > S(-1.e+10)) {
    likelihood_sampling<P>(c, &e1, &e2, maxL, np_max, &v1, &v2, &od);
    if (v1 < S(kVar) || v2 < S(kVar) || od < S(kVar)) error = 1;
  } else {
    error = 1;
  }
  o.max_e1 = (double)s.x[lo][0];
  o.max_e2 = (double)s.x[lo][1];
  o.e1 = e1; o.e2 = e2; o.var_e1 = v1; o.var_e2 = v2; o.oneDimvar = od; o.maxL = maxL;
  o.error = error; o.iters = iter; o.nevals = c.nevals;
  o.status = bad_start ? 4 : 0;
  return o;
}

// ------------------------------------------------------------------ kernels
template <class P>
__device__ __forceinline__ size_t cells_smem_bytes(int max_cells) {
  return (size_t)5 * max_cells * sizeof(typename P::Cell);
}

// galaxy g's facet cells (read in place from global memory: a few KB, read-only during the fit,
// they stay in L1) and its scalelength prior into sh.rprior; returns the number of cells
template <class P>
__device__ int bind_galaxy(const FacetBatch& b, int g, const typename P::Cell** cells, FitShared<typename P::S>& sh) {
  using Cell = typename P::Cell;
  using S = typename P::S;
  const int off = b.offset[g];
  cells[0] = reinterpret_cast<const Cell*>(b.gu) + off;
  cells[1] = reinterpret_cast<const Cell*>(b.gv) + off;
  cells[2] = reinterpret_cast<const Cell*>(b.dre) + off;
  cells[3] = reinterpret_cast<const Cell*>(b.dim) + off;
  cells[4] = reinterpret_cast<const Cell*>(b.sig2) + off;
  for (int i = threadIdx.x; i < kMaxNodes; i += blockDim.x) sh.rprior[i] = S(b.rprior[(size_t)g * kMaxNodes + i]);
  return b.count[g];
}

// Helper side of the sampling board, run by a CTA once the galaxy queue is empty: warp 0 scans
// the slots of the launch for a chunk with unclaimed points and claims one; the CTA evaluates it
// with the galaxy's cells and prior.  Returns when every galaxy of the launch is finished, or after
// kBoardWaitNs without finding work.
template <class P>
__device__ void board_help(const FacetBatch& b, FitShared<typename P::S>& sh, NodeCache& nc) {
  const SampleBoard& bd = b.board;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int staged = -1, n = 0;
  const typename P::Cell* cp[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  unsigned long long idle0 = global_ns();
  while (true) {
    if (warp == 0) {
      int state = 0;
      while (state == 0) {
        if (*(volatile int*)bd.done_gal >= b.n_gal) { state = -1; break; }
        for (int base = 0; base < b.n_gal && state == 0; base += 32) {
          const int gg = (int)((blockIdx.x + (unsigned)base + lane) % (unsigned)b.n_gal);
          bool cand = false;
          if (base + lane < b.n_gal) {
            const unsigned long long w = *(volatile unsigned long long*)&bd.slot[gg].claim;
            const int npts = *(volatile int*)&bd.slot[gg].npts;
            cand = (w >> 32) != 0 && (int)(w & 0xffffffffull) < npts;
          }
          unsigned m = __ballot_sync(0xffffffffu, cand);
          while (m && state == 0) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            int got = 0;
            if (lane == src) {
              const unsigned long long w = atomicAdd(&bd.slot[gg].claim, 1ull);
              __threadfence();
              const SampleSlot prm = board_params(&bd.slot[gg]);
              const int idx = (int)(w & 0xffffffffull);
              if (idx < prm.npts) {
                sh.claim_prm = prm;
                sh.claim_g = gg;
                sh.claim_seq = (int)(w >> 32);
                sh.claim_idx = idx;
                got = 1;
              }
            }
            if (__shfl_sync(0xffffffffu, got, src)) state = 1;
          }
        }
        if (state == 0) {
          if (global_ns() - idle0 > kBoardWaitNs) state = -1;
          else __nanosleep(1000);
        }
      }
      if (lane == 0) sh.claim_state = state;
    }
    __syncthreads();
    if (sh.claim_state < 0) return;
    const int gg = sh.claim_g;
    if (gg != staged) {
      n = bind_galaxy<P>(b, gg, cp, sh);
      staged = gg;
    }
    const SampleSlot prm = sh.claim_prm;
    const int seq = sh.claim_seq, idx = sh.claim_idx;
    const int before = sh.newton;
    __syncthreads();
    board_point<P>(sh, nc, cp[0], cp[1], cp[2], cp[3], cp[4], n, bd, gg, seq, idx, prm, before);
    idle0 = global_ns();
    __syncthreads();
  }
}

template <class P>
__global__ void __launch_bounds__(kFitThreads, kFitMinBlocks) k_fit(FacetBatch b) {
  using Cell = typename P::Cell;
  __shared__ FitShared<typename P::S> sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  NodeCache nc = node_cache_view(dyn, c_fit.numr);
  const int tid = threadIdx.x;
  if (tid == 0) { sh.newton = 0; sh.status = 0; sh.mg.status = 0; sh.mg.fac_n = -1; }
  while (true) {
    if (tid == 0) sh.g = atomicAdd(b.queue, 1);
    __syncthreads();
    const int g = sh.g;
    if (g >= b.n_gal) break;
    if (b.active && !b.active[g]) {
      if (tid == 0 && b.board.slot) atomicAdd(b.board.done_gal, 1);
      __syncthreads();
      continue;
    }
    const Cell* cp[5];
    const int n = bind_galaxy<P>(b, g, cp, sh);
    if (tid == 0) { sh.newton = 0; sh.status = 0; sh.mg.status = 0; }
    __syncthreads();
    double se1 = 0., se2 = 0., step = 0.1;
    if (b.start) { se1 = b.start[3 * g]; se2 = b.start[3 * g + 1]; step = b.start[3 * g + 2]; }
    FitCtx<P> c{&sh, &nc, cp[0], cp[1], cp[2], cp[3], cp[4], n, 0,
                b.trace ? b.trace + (size_t)g * b.trace_cap * 4 : nullptr, b.trace_cap, b.board, g, 0};
    FitOut o = fit_galaxy<P>(c, se1, se2, step, c_fit.np_max);
    __syncthreads();
    if (tid == 0) {
      o.newton_iters = sh.newton + (b.board.slot ? *(volatile int*)&b.board.newton[g] : 0);
      o.status |= sh.status | sh.mg.status;
      o.ncoords = n;
      b.out[g] = o;
      if (b.board.slot) {
        __threadfence();
        atomicAdd(b.board.done_gal, 1);
      }
    }
    __syncthreads();
  }
  if (b.board.slot) board_help<P>(b, sh, nc);
}

// one loglikelihood evaluation of galaxy 0 of the batch (C entry point loglikelihood)
template <class P>
__global__ void __launch_bounds__(kFitThreads, 1) k_loglike_once(FacetBatch b, double e1, double e2,
                                                                  double* out2, double* node_L) {
  using Cell = typename P::Cell;
  using S = typename P::S;
  __shared__ FitShared<S> sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  NodeCache nc = node_cache_view(dyn, c_fit.numr);
  const int n = b.count[0];
  const int tid = threadIdx.x;
  for (int i = tid; i < kMaxNodes; i += blockDim.x) sh.rprior[i] = S(b.rprior[i]);
  if (tid == 0) { sh.newton = 0; sh.status = 0; sh.mg.status = 0; sh.mg.fac_n = -1; }
  __syncthreads();
  int err = 0;
  S L = eval_loglike<P>(sh, nc, reinterpret_cast<const Cell*>(b.gu), reinterpret_cast<const Cell*>(b.gv),
                        reinterpret_cast<const Cell*>(b.dre), reinterpret_cast<const Cell*>(b.dim),
                        reinterpret_cast<const Cell*>(b.sig2), n, S(e1), S(e2), &err);
  if (tid == 0) { out2[0] = (double)L; out2[1] = (double)err; }
  if (node_L && tid < kMaxNodes) node_L[tid] = (tid >= 1 && tid < c_fit.numr) ? (double)sh.Lr[tid] : 0.0;
}

template <class P>
__global__ void __launch_bounds__(kFitThreads, 1) k_sampling_once(FacetBatch b, double e1, double e2,
                                                                   double maxL, int np_max, double* out5) {
  using Cell = typename P::Cell;
  using S = typename P::S;
  __shared__ FitShared<S> sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  NodeCache nc = node_cache_view(dyn, c_fit.numr);
  const int n = b.count[0];
  const int tid = threadIdx.x;
  for (int i = tid; i < kMaxNodes; i += blockDim.x) sh.rprior[i] = S(b.rprior[i]);
  if (tid == 0) { sh.newton = 0; sh.status = 0; sh.mg.status = 0; sh.mg.fac_n = -1; }
  __syncthreads();
  FitCtx<P> c{&sh, &nc, reinterpret_cast<const Cell*>(b.gu), reinterpret_cast<const Cell*>(b.gv),
              reinterpret_cast<const Cell*>(b.dre), reinterpret_cast<const Cell*>(b.dim),
              reinterpret_cast<const Cell*>(b.sig2), n, 0, b.trace, b.trace_cap};
  S m1 = S(e1), m2 = S(e2), v1, v2, od;
  likelihood_sampling<P>(c, &m1, &m2, S(maxL), np_max, &v1, &v2, &od);
  if (tid == 0) { out5[0] = m1; out5[1] = m2; out5[2] = v1; out5[3] = v2; out5[4] = od; }
}

// loglikelihood_r (likelihood.c:156-187): one warp, writes the normalised model to visM
__global__ void k_loglike_r(double e1, double e2, double scale, int n, const double* variance,
                            const double* gu, const double* gv, const double* dre, const double* dim,
                            double* visM, double* out_L, int gaussian) {
  int it;
  double L = node_loglike<PolicyF64>(gu, gv, dre, dim, variance, n, e1, e2, scale, gaussian, &it, visM,
                                     nullptr, nullptr, nullptr);
  if (threadIdx.x == 0) { out_L[0] = L; out_L[1] = it; }
}

// cross_correlation (likelihood.c:194-358) with a caller-supplied model: out = (ho, det, error)
__global__ void k_xcorr(int n, const double* gu, const double* gv, const double* dre, const double* dim,
                        const double* visMod, double* out3) {
  int it;
  double ho = 0, det = 0;
  node_loglike<PolicyF64>(gu, gv, dre, dim, nullptr, n, 0., 0., 1., 0, &it, nullptr, visMod, &ho, &det);
  if (threadIdx.x == 0) { out3[0] = ho; out3[1] = det; out3[2] = (det <= 0) ? 1.0 : 0.0; out3[3] = it; }
}

__global__ void k_marginalise_once(int n, const double* x, double* y, double* out1) {
  __shared__ MargShared<double> sh;
  const int lane = threadIdx.x;
  if (lane == 0) { sh.status = 0; sh.fac_n = -1; for (int i = 0; i < n; ++i) { sh.xs[i] = x[i]; sh.ys[i] = y[i]; } }
  __syncwarp();
  double L = marginalise_posterior_warp<double>(sh, n);
  __syncwarp();
  if (lane == 0) { out1[0] = L; for (int i = 0; i < n; ++i) y[i] = sh.ys[i]; }
}

__global__ void k_set_posterior(int numR, const double* Lr, const double* rprior, const double* ro,
                                double* x, double* y, int* numvals) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int num = 0, nRo = 1;
  while (nRo < numR && (Lr[nRo] <= kBad)) nRo++;
  if (nRo < numR) {
    for (nRo = 1; nRo < numR; nRo++) {
      double lv = Lr[nRo];
      if (lv > kBad) { x[num] = ro[nRo]; y[num] = lv + rprior[nRo]; num++; }
    }
  }
  *numvals = num;
}

__global__ void k_position_marginal(int n, const double* x, double* y) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = position_marginal(x[i]);
}

// ----------------------------------------------------------------- launchers
static int check(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "rlf: %s: %s\n", what, cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}

static int g_fit_numr = kMaxNodes;  // host copy of c_fit.numr (sizes the node caches)

int fit_set_config(const FitConfigHost& cfg, cudaStream_t st) {
  FitConst h;
  memset(&h, 0, sizeof(h));
  h.numr = cfg.numr;
  g_fit_numr = cfg.numr;
  h.gaussian = cfg.gaussian;
  h.np_max = cfg.np_max;
  for (int i = 0; i < kMaxNodes; ++i) {
    h.ro[i] = (i < cfg.numr) ? cfg.ro[i] : 0.0;
  }
  static double invk[kInvTab], invfact[kEiTerms], eitab[kEiTab], exptab[kEiTab];
  for (int k = 0; k < kInvTab; ++k) invk[k] = k ? 1.0 / k : 0.0;
  long double f = 1.0L;
  for (int k = 0; k < kEiTerms; ++k) {
    if (k) f *= k;
    invfact[k] = (double)(1.0L / f);
  }
  // Ei(k) = gamma + ln k + sum_j k^j / (j j!) and e^k in extended precision (all terms positive)
  eitab[0] = 0.0;
  exptab[0] = 1.0;
  for (int k = 1; k < kEiTab; ++k) {
    const long double x = k;
    long double term = 1.0L, sum = 0.0L;
    for (int j = 1; j < 2000; ++j) {
      term *= x / j;
      const long double t = term / j;
      sum += t;
      if (t < 1e-30L * sum) break;
    }
    eitab[k] = (double)(0.577215664901532860606512090082402431L + logl(x) + sum);
    exptab[k] = (double)expl(x);
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_fit, &h, sizeof(h), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_ei_tab, eitab, sizeof(eitab), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_exp_tab, exptab, sizeof(exptab), 0, cudaMemcpyHostToDevice, st);
  static float2 invk2[kInvTab], invfact2[kEiTerms];
  for (int k = 0; k < kInvTab; ++k) {
    invk2[k].x = (float)invk[k];
    invk2[k].y = (float)(invk[k] - (double)invk2[k].x);
  }
  for (int k = 0; k < kEiTerms; ++k) {
    invfact2[k].x = (float)invfact[k];
    invfact2[k].y = (float)(invfact[k] - (double)invfact2[k].x);
  }
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_invk2, invk2, sizeof(invk2), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_invfact2, invfact2, sizeof(invfact2), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // h is released on return
  if (e != cudaSuccess) { fprintf(stderr, "rlf: fit config: %s\n", cudaGetErrorString(e)); return (int)e; }
  return 0;
}

template <class P>
static int fit_launch_t(const FacetBatch& b, int grid, cudaStream_t st) {
  const size_t dyn = node_cache_bytes(g_fit_numr);
  constexpr size_t kDynMax = 190 * 1024;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_fit<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDynMax);
    attr_set = true;
  }
  if (dyn > kDynMax) { fprintf(stderr, "rlf: too many scalelength nodes for the fit kernel\n"); return 1; }
  // persistent CTAs: as many as fit on the GPU with this batch's facet staging
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fit<P>, kFitThreads, dyn);
  if (per < 1) per = 1;
  if (grid > sms * per) grid = sms * per;
  k_fit<P><<<grid, kFitThreads, dyn, st>>>(b);
  return check("k_fit");
}

int fit_launch(const FacetBatch& b, Precision p, int grid, cudaStream_t st) {
  if (b.n_gal <= 0) return 0;
  if (!b.board.slot && grid > b.n_gal) grid = b.n_gal;
  if (grid < 1) grid = 1;
  return p == kF64 ? fit_launch_t<PolicyF64>(b, grid, st) : fit_launch_t<PolicyMixed>(b, grid, st);
}

int fit_max_grid(Precision p) {
  (void)p;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms * kFitMinBlocks;  // fit_launch lowers it to the occupancy of the launch's staging
}

int launch_loglikelihood_r(double e1, double e2, double scale, int n, const double* variance,
                           const double* gu, const double* gv, const double* dre, const double* dim,
                           double* visM, double* out_L, int gaussian, cudaStream_t st) {
  k_loglike_r<<<1, 32, 0, st>>>(e1, e2, scale, n, variance, gu, gv, dre, dim, visM, out_L, gaussian);
  return check("k_loglike_r");
}
int launch_cross_correlation(int n, const double* gu, const double* gv, const double* dre,
                             const double* dim, const double* visMod, double* out3, cudaStream_t st) {
  k_xcorr<<<1, 32, 0, st>>>(n, gu, gv, dre, dim, visMod, out3);
  return check("k_xcorr");
}
// the single-evaluation kernels take the per-node caches in dynamic shared memory, above the
// default 48 KB together with their static state
template <class K>
static void allow_node_cache(K kernel) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)node_cache_bytes(g_fit_numr));
}
int launch_loglikelihood(const FacetBatch& b, double e1, double e2, double* out2, double* node_L,
                         cudaStream_t st) {
  allow_node_cache(k_loglike_once<PolicyF64>);
  k_loglike_once<PolicyF64><<<1, kFitThreads, node_cache_bytes(g_fit_numr), st>>>(b, e1, e2, out2, node_L);
  return check("k_loglike_once");
}
int launch_loglikelihood_prec(const FacetBatch& b, double e1, double e2, double* out2, double* node_L,
                              Precision prec, cudaStream_t st) {
  if (prec == kMixed) {
    allow_node_cache(k_loglike_once<PolicyMixed>);
    k_loglike_once<PolicyMixed><<<1, kFitThreads, node_cache_bytes(g_fit_numr), st>>>(b, e1, e2, out2, node_L);
    return check("k_loglike_once<mixed>");
  }
  return launch_loglikelihood(b, e1, e2, out2, node_L, st);
}
int launch_likelihood_sampling(const FacetBatch& b, double e1, double e2, double maxL, int np_max,
                               double* out5, cudaStream_t st) {
  allow_node_cache(k_sampling_once<PolicyF64>);
  k_sampling_once<PolicyF64><<<1, kFitThreads, node_cache_bytes(g_fit_numr), st>>>(b, e1, e2, maxL, np_max, out5);
  return check("k_sampling_once");
}
int launch_marginalise_posterior_r(int n, const double* x, double* y, double* out1, cudaStream_t st) {
  k_marginalise_once<<<1, 32, 0, st>>>(n, x, y, out1);
  return check("k_marginalise_once");
}
__global__ void k_df_math(int op, int n, const double* __restrict__ x, const double* __restrict__ y,
                          double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const f2 a = df_from_double(x[i]);
    f2 r{0.f, 0.f};
    switch (op) {
      case 0: r = df_exp(a); break;
      case 1: r = df_log(a); break;
      case 2: r = df_log_double(x[i]); break;
      case 3: r = df_div(a, df_from_double(y[i])); break;
      case 4: r = df_sqrt(a); break;
      case 5: r = df_profile_exp(a); break;
      default: r = df_from_double_bits(x[i]); break;
    }
    out[i] = df_to_double(r);
  }
}
int launch_df_math(int op, int n, const double* x, const double* y, double* out, cudaStream_t st) {
  if (op < 0 || op > 6) return 1;
  if (n <= 0) return 0;
  k_df_math<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, st>>>(op, n, x, y, out);
  return check("k_df_math");
}
int launch_set_posterior_values(int numR, const double* Lr, const double* rprior, const double* ro,
                                double* x, double* y, int* numvals, cudaStream_t st) {
  k_set_posterior<<<1, 32, 0, st>>>(numR, Lr, rprior, ro, x, y, numvals);
  return check("k_set_posterior");
}
int launch_position_marginal(int n, const double* x, double* y, cudaStream_t st) {
  if (n <= 0) return 0;
  k_position_marginal<<<(n + 127) / 128, 128, 0, st>>>(n, x, y);
  return check("k_position_marginal");
}

}  // namespace rlf

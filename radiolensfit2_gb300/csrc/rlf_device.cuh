// Device-side building blocks shared by every kernel of the shape-measurement path.
//
// Numeric constants are those of the reference (default_params.h, datatype.h); scalar functions
// are __host__ __device__ so the C ABI's scalar entry points and the kernels share one
// definition.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define RLF_HD __host__ __device__ __forceinline__

namespace rlf {

// kernels launched by this library since load (incremented by every launch-site check)
void count_launch();
long long launch_count();

constexpr double kPi = 3.14159265358979323846;
constexpr double kC0 = 299792458.0;
constexpr int kPsfNat = 38;
constexpr double kRMin = 0.3;
constexpr double kRMax = 3.5;
constexpr int kNumR = 29;
constexpr double kAdd = -0.93;
constexpr double kEsp = 0.33;
constexpr double kRStd = 0.3136;
constexpr double kTol = 1.0e-3;
constexpr int kNpMax = 30;
constexpr double kERes = 3.0e-3;
constexpr double kVar = 1e-4;
constexpr double kBad = -1.e+10;        // likelihood sentinel (likelihood.c:96,141,177)
constexpr int kMaxNodes = 32;           // capacity for scalelength nodes (the reference uses 24)
constexpr unsigned kMaxFacet = 255;     // facet cell index fits in 16 bits
constexpr uint16_t kNoCell = 0xFFFF;    // flagged or out-of-grid visibility

// ---------------------------------------------------------------- profiles
// galaxy_visibilities.c:40-53
RLF_HD double gaussian_shape(double k1, double k2, double scale_factor, double wave_factor) {
  return exp(-0.5 * scale_factor * wave_factor * (k1 * k1 + k2 * k2));
}
RLF_HD double sersic_shape(double k1, double k2, double scale_factor, double wave_factor) {
  double den = 1. + scale_factor * wave_factor * (k1 * k1 + k2 * k2);
  return 1. / (den * sqrt(den));
}
RLF_HD double shape(int gaussian, double k1, double k2, double sf, double wf) {
  return gaussian ? gaussian_shape(k1, k2, sf, wf) : sersic_shape(k1, k2, sf, wf);
}
// scale (arcsec) -> (scale[rad])^2 / detA^2, as galaxy_visibilities.c:63-65
RLF_HD double scale_factor(double e1, double e2, double scale_arcsec) {
  double detA = 1. - e1 * e1 - e2 * e2;
  double s = scale_arcsec * (kPi / 648000.0);
  return (s * s) / (detA * detA);
}

// evaluate_uv_grid.c:50-55; the unparenthesised ARCS2RAD macro makes this
// ((len*38*theta)*PI)/648000 evaluated left to right.
RLF_HD unsigned facet_size(double theta_med, double len) {
  return (unsigned)(2.0 * ceil(len * kPsfNat * theta_med * kPi / 648000.0));
}

// distributions.c:59-87
RLF_HD double scale_mean(double flux) { return kAdd + kEsp * log(flux); }
RLF_HD double rfunc(double mu, double sigma, double r) {
  double x = (log(r) - mu) / sigma;
  return -(x * x) * 0.5 - log(r * sigma);
}

// ------------------------------------------------------------ Ei(x), x > 0
// Exponential integral from its power series  Ei(x) = gamma + ln x + sum_k x^k/(k k!)  for
// x <= 40 and the asymptotic series  e^x/x sum_k k!/x^k  (stopped at its smallest term) above.
constexpr double kEulerGamma = 0.57721566490153286060651209008240243;
RLF_HD double ei_pos(double x) {
  if (x <= 40.0) {
    double term = 1.0, sum = 0.0;
    for (int k = 1; k < 400; ++k) {
      term *= x / k;
      double t = term / k;
      sum += t;
      if (t < 1e-18 * sum) break;
    }
    return kEulerGamma + log(x) + sum;
  }
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 200; ++k) {
    double next = term * k / x;
    if (next >= term || next < 1e-18 * sum) break;
    term = next;
    sum += term;
  }
  return exp(x) / x * sum;
}

// likelihood.c:376-421: log of the likelihood analytically marginalised over a uniform prior on
// the position shift inside the 95% confidence radius.
RLF_HD double position_marginal(double x) {
  const double Delta = 0.5 * 5.991;
  if (x <= Delta) return kBad;
  if (x > 100.) return x - log(Delta) - exp(-Delta);
  if ((x - Delta) < 0.0001) x = Delta + 0.0001;
  double yc = ei_pos(x), ys = ei_pos(x - Delta);
  return log((yc - ys) / log(x / (x - Delta)));
}

// ---------------------------------------------------------------- warps
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  return v;
}

// ------------------------------------------------------ double-float arithmetic
// Unevaluated sums hi+lo of two floats (Dekker / Knuth error-free transformations) carry the
// FP64 phase argument through FP32 code without FP64 instructions in the inner loops.
struct f2 { float hi, lo; };
__device__ __forceinline__ f2 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ f2 quick_two_sum(float a, float b) {  // |a| >= |b|
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ f2 two_prod(float a, float b) {
  float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ f2 df_from_double(double d) {
  float h = (float)d;
  return {h, (float)(d - (double)h)};
}

}  // namespace rlf

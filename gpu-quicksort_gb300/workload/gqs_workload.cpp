// Seeded synthetic workloads for the sort benchmarks and tests.
//
// Every key is a pure function of (seed, index): a counter-based splitmix64
// stream, so generation is embarrassingly parallel and identical on x86-64
// and AArch64. Transcendental functions (log, exp, sin, cos) are computed by
// the series below from +, -, *, / only, and this file is compiled with
// -ffp-contract=off, so no platform libm or FMA contraction can change a bit.
//
// Distributions follow the sort configurations: uniform u32 over [0, 2^32);
// sorted; reverse sorted; 16 distinct values; Zipf(s=1.1) over 2^20 ranks;
// Gaussian u32 (mean 2^31, sd 2^28); f32 N(0, 1e3); f64 U[-1e9, 1e9]; the
// reference's known-answer input (a shuffled 1..n permutation,
// GPU-Quicksort_OpenCL_1.2/QuicksortMain.cpp:415-416); segment tables with
// log-uniform lengths. No generator emits NaN, Inf or -0.0.

#include <cstdint>
#include <cstddef>
#include <cstring>
#include <vector>
#include <algorithm>

#include "gqs_workload.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Draw number `k` of key `i` under `seed`.
inline uint64_t draw(uint64_t seed, uint64_t i, uint64_t k) {
  return splitmix64(splitmix64(seed * 0xD1B54A32D192ED03ull + k) ^ (i * 0x9E3779B97F4A7C15ull));
}

inline double unit_open0(uint64_t x) {  // (0, 1]
  return (double)((x >> 11) + 1) * (1.0 / 9007199254740992.0);
}
inline double unit_closed0(uint64_t x) {  // [0, 1)
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

const double kLn2Hi = 6.93147180369123816490e-01;
const double kLn2Lo = 1.90821492927058770002e-10;
const double kPi = 3.14159265358979311600e+00;

// ln(x) for x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(z), z = (m - 1) / (m + 1), |z| <= 0.1716.
double det_log(double x) {
  int e = 0;
  // frexp is exact on every IEEE platform.
  double m = __builtin_frexp(x, &e);  // m in [0.5, 1)
  if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
  double z = (m - 1.0) / (m + 1.0);
  double z2 = z * z;
  double term = z, sum = 0.0;
  for (int k = 1; k <= 41; k += 2) { sum += term / (double)k; term *= z2; }
  return 2.0 * sum + (double)e * kLn2Lo + (double)e * kLn2Hi;
}

// exp(x): x = k ln2 + r, |r| <= ln2/2, Taylor series in r.
double det_exp(double x) {
  double kf = x / (kLn2Hi + kLn2Lo);
  long k = (long)(kf < 0 ? kf - 0.5 : kf + 0.5);
  double r = (x - (double)k * kLn2Hi) - (double)k * kLn2Lo;
  double term = 1.0, sum = 1.0;
  for (int n = 1; n <= 24; ++n) { term *= r / (double)n; sum += term; }
  return __builtin_ldexp(sum, (int)k);
}

// sin and cos of a in [0, pi/2] by Taylor series.
double det_sin_q(double a) {
  double a2 = a * a, term = a, sum = a;
  for (int n = 1; n <= 14; ++n) { term *= -a2 / (double)((2 * n) * (2 * n + 1)); sum += term; }
  return sum;
}
double det_cos_q(double a) {
  double a2 = a * a, term = 1.0, sum = 1.0;
  for (int n = 1; n <= 14; ++n) { term *= -a2 / (double)((2 * n - 1) * (2 * n)); sum += term; }
  return sum;
}
// cos(2 pi u) for u in [0, 1).
double det_cos_2pi(double u) {
  double t = 4.0 * u;
  int q = (int)t;
  double a = (t - (double)q) * (kPi / 2.0);
  switch (q & 3) {
    case 0: return det_cos_q(a);
    case 1: return -det_sin_q(a);
    case 2: return -det_cos_q(a);
    default: return det_sin_q(a);
  }
}

// Standard normal deviate for key i (Box-Muller, cosine branch).
inline double gauss(uint64_t seed, uint64_t i) {
  double u1 = unit_open0(draw(seed, i, 1));
  double u2 = unit_closed0(draw(seed, i, 2));
  double r = __builtin_sqrt(-2.0 * det_log(u1));
  return r * det_cos_2pi(u2);
}

inline float no_neg_zero(float f) {
  uint32_t b;
  std::memcpy(&b, &f, 4);
  if (b == 0x80000000u) return 0.0f;
  return f;
}
inline double no_neg_zero(double f) {
  uint64_t b;
  std::memcpy(&b, &f, 8);
  if (b == 0x8000000000000000ull) return 0.0;
  return f;
}

// Zipf(s) over `ranks` ranks: cumulative table, built once per (s, ranks).
struct ZipfTable {
  std::vector<double> cdf;
  explicit ZipfTable(uint32_t ranks, double s) : cdf(ranks) {
    double acc = 0.0;
    for (uint32_t r = 0; r < ranks; ++r) {
      acc += det_exp(-s * det_log((double)(r + 1)));
      cdf[r] = acc;
    }
    for (uint32_t r = 0; r < ranks; ++r) cdf[r] /= acc;
  }
  uint32_t rank(double u) const {  // first r with cdf[r] > u
    size_t lo = 0, hi = cdf.size() - 1;
    while (lo < hi) {
      size_t mid = (lo + hi) / 2;
      if (cdf[mid] > u) hi = mid; else lo = mid + 1;
    }
    return (uint32_t)lo;
  }
};

// Fisher-Yates shuffle of 1..n, the known-answer input.
template <class T>
void kat_fill(uint64_t seed, size_t n, T* out) {
  for (size_t i = 0; i < n; ++i) out[i] = (T)(i + 1);
  for (size_t i = n; i > 1; --i) {
    uint64_t x = draw(seed, i, 7);
    size_t j = (size_t)(((unsigned __int128)x * i) >> 64);
    std::swap(out[i - 1], out[j]);
  }
}

}  // namespace

extern "C" {

int gqs_workload_u32(int dist, uint64_t seed, size_t n, uint32_t* out) {
  if (!out && n) return -1;
  switch (dist) {
    case GQS_DIST_UNIFORM:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = (uint32_t)(draw(seed, i, 0) >> 32);
      return 0;
    case GQS_DIST_SORTED:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = (uint32_t)(((unsigned __int128)i << 32) / n);
      return 0;
    case GQS_DIST_REVERSE:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = (uint32_t)(((unsigned __int128)(n - 1 - i) << 32) / n);
      return 0;
    case GQS_DIST_DISTINCT16: {
      uint32_t vals[16];
      for (int v = 0; v < 16; ++v) vals[v] = (uint32_t)(draw(seed, v, 3) >> 32);
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = vals[(uint32_t)(draw(seed, i, 0) >> 60)];
      return 0;
    }
    case GQS_DIST_ZIPF: {
      ZipfTable zt(1u << 20, 1.1);
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) {
        uint32_t r = zt.rank(unit_closed0(draw(seed, i, 0)));
        out[i] = (uint32_t)((uint64_t)(r + 1) * 2654435761ull);
      }
      return 0;
    }
    case GQS_DIST_GAUSSIAN:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) {
        double g = 2147483648.0 + 268435456.0 * gauss(seed, i);
        double r = __builtin_floor(g + 0.5);
        if (r < 0.0) r = 0.0;
        if (r > 4294967295.0) r = 4294967295.0;
        out[i] = (uint32_t)r;
      }
      return 0;
    case GQS_DIST_KAT:
      kat_fill<uint32_t>(seed, n, out);
      return 0;
    case GQS_DIST_ALLEQUAL: {
      uint32_t v = (uint32_t)(draw(seed, 0, 4) >> 32);
      for (size_t i = 0; i < n; ++i) out[i] = v;
      return 0;
    }
    default:
      return -2;
  }
}

int gqs_workload_f32(int dist, uint64_t seed, size_t n, float* out) {
  if (!out && n) return -1;
  switch (dist) {
    case GQS_DIST_GAUSSIAN:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = no_neg_zero((float)(1000.0 * gauss(seed, i)));
      return 0;
    case GQS_DIST_UNIFORM:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = no_neg_zero((float)(-1e9 + 2e9 * unit_closed0(draw(seed, i, 0))));
      return 0;
    case GQS_DIST_SORTED:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = no_neg_zero((float)(-1e9 + 2e9 * ((double)i / (double)n)));
      return 0;
    case GQS_DIST_REVERSE:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = no_neg_zero((float)(-1e9 + 2e9 * ((double)(n - 1 - i) / (double)n)));
      return 0;
    case GQS_DIST_DISTINCT16: {
      float vals[16];
      for (int v = 0; v < 16; ++v) vals[v] = no_neg_zero((float)(1000.0 * gauss(seed ^ 0x5151u, v)));
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = vals[(uint32_t)(draw(seed, i, 0) >> 60)];
      return 0;
    }
    case GQS_DIST_KAT:
      kat_fill<float>(seed, n, out);
      return 0;
    case GQS_DIST_ALLEQUAL: {
      float v = no_neg_zero((float)(1000.0 * gauss(seed, 0)));
      for (size_t i = 0; i < n; ++i) out[i] = v;
      return 0;
    }
    default:
      return -2;
  }
}

int gqs_workload_f64(int dist, uint64_t seed, size_t n, double* out) {
  if (!out && n) return -1;
  switch (dist) {
    case GQS_DIST_UNIFORM:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = no_neg_zero(-1e9 + 2e9 * unit_closed0(draw(seed, i, 0)));
      return 0;
    case GQS_DIST_GAUSSIAN:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = no_neg_zero(1000.0 * gauss(seed, i));
      return 0;
    case GQS_DIST_SORTED:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = no_neg_zero(-1e9 + 2e9 * ((double)i / (double)n));
      return 0;
    case GQS_DIST_REVERSE:
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i)
        out[i] = no_neg_zero(-1e9 + 2e9 * ((double)(n - 1 - i) / (double)n));
      return 0;
    case GQS_DIST_DISTINCT16: {
      double vals[16];
      for (int v = 0; v < 16; ++v) vals[v] = no_neg_zero(-1e9 + 2e9 * unit_closed0(draw(seed, v, 3)));
#pragma omp parallel for schedule(static)
      for (long long i = 0; i < (long long)n; ++i) out[i] = vals[(uint32_t)(draw(seed, i, 0) >> 60)];
      return 0;
    }
    case GQS_DIST_KAT:
      kat_fill<double>(seed, n, out);
      return 0;
    case GQS_DIST_ALLEQUAL: {
      double v = no_neg_zero(-1e9 + 2e9 * unit_closed0(draw(seed, 0, 4)));
      for (size_t i = 0; i < n; ++i) out[i] = v;
      return 0;
    }
    default:
      return -2;
  }
}

// Segment table with lengths floor(exp(U(ln minlen, ln maxlen))), written as
// nseg + 1 offsets (offsets[0] = 0). Returns the total key count.
uint64_t gqs_workload_segments(uint64_t seed, size_t nseg, uint64_t minlen, uint64_t maxlen,
                               uint64_t* offsets) {
  double lo = det_log((double)minlen), hi = det_log((double)maxlen);
  uint64_t acc = 0;
  offsets[0] = 0;
  for (size_t s = 0; s < nseg; ++s) {
    double u = unit_closed0(draw(seed, s, 5));
    uint64_t len = (uint64_t)__builtin_floor(det_exp(lo + (hi - lo) * u));
    if (len < minlen) len = minlen;
    if (len > maxlen) len = maxlen;
    acc += len;
    offsets[s + 1] = acc;
  }
  return acc;
}

// Deterministic log/exp exposed for the generator's own tests.
double gqs_workload_det_log(double x) { return det_log(x); }
double gqs_workload_det_exp(double x) { return det_exp(x); }
double gqs_workload_det_cos2pi(double u) { return det_cos_2pi(u); }

}  // extern "C"

// Device-side building blocks shared by every kernel of the GB300 library:
// order-preserving keys, boundary mapping, the median midpoint and percentile
// interpolation contracts, compensated sums and canonical-NaN stores.
//
// Every float64 operation whose result must match the reference bit for bit
// uses a round-to-nearest intrinsic (__dadd_rn, __dmul_rn, ...), which nvcc
// never contracts into an FMA.
#pragma once

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "plan.h"

namespace ndf {

enum Mode : int32_t { kReflect = 0, kConstant = 1, kNearest = 2, kMirror = 3, kWrap = 4 };

enum Kind : int32_t {
  kMedian = 0,
  kMedianNetwork = 1,
  kMedianHistogram = 2,
  kMean = 3,
  kMeanRolling = 4,
  kMin = 5,
  kMax = 6,
  kVar = 7,
  kStd = 8,
  kRank = 9,
  kRankHistogram = 10,
  kPercentile = 11,
  // Robust reductions (src/robust.rs:137-185).
  kMad = 12,
  kMode = 13,
  kBiweightLocation = 14,
  kBiweightScale = 15,
  kSigmaMean = 16,
  kSigmaMedian = 17,
  kSigmaMode = 18,
};

// Error flags a kernel can raise in the plan's device status word.
enum DeviceError : uint32_t {
  kDevOk = 0,
  kDevSupportOverflow = 1u << 0,  // a histogram support exceeded its rank codes
  kDevScratchOverflow = 1u << 1,  // a kernel ran out of its scratch capacity
};

// ---------------------------------------------------------------------------
// Order-preserving unsigned keys. Unsigned key order equals IEEE total order
// (-0 before +0) for every non-NaN value. The reference encodes the same order
// as signed integers (src/median_network.rs:21-31); an unsigned key keeps
// the sentinel (all ones) above +inf, so a dropped sample sorts last.

template <typename T>
struct KeyOf;

template <>
struct KeyOf<float> {
  using K = uint32_t;
  static constexpr uint32_t kSentinel = 0xFFFFFFFFu;
  __device__ __forceinline__ static uint32_t key(float v) {
    uint32_t b = __float_as_uint(v);
    return b ^ ((uint32_t)((int32_t)b >> 31) | 0x80000000u);
  }
  __device__ __forceinline__ static float value(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k ^ 0x80000000u) : ~k;
    return __uint_as_float(b);
  }
};

template <>
struct KeyOf<double> {
  using K = unsigned long long;
  static constexpr unsigned long long kSentinel = ~0ull;
  __device__ __forceinline__ static unsigned long long key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return b ^ ((unsigned long long)((long long)b >> 63) | 0x8000000000000000ull);
  }
  __device__ __forceinline__ static double value(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k ^ 0x8000000000000000ull) : ~k;
    return __longlong_as_double((long long)b);
  }
};

// A sample is dropped (keyed as the sentinel) when it is NaN, or infinite
// while infinities are ignored (src/reduction.rs:85-101,
// src/median_network.rs:40-63). Under the propagate policy a dropped NaN
// makes the window NaN; the caller detects it from the retained count.
template <typename T>
__device__ __forceinline__ typename KeyOf<T>::K sample_key(T v, bool drop_inf) {
  bool drop = isnan(v) || (drop_inf && isinf(v));
  return drop ? KeyOf<T>::kSentinel : KeyOf<T>::key(v);
}

// ---------------------------------------------------------------------------
// Canonical NaN stores: 0x7fc00000 / 0x7ff8000000000000 (docs/semantics.md).

__device__ __forceinline__ float canonical(float v) {
  return isnan(v) ? __uint_as_float(0x7fc00000u) : v;
}
__device__ __forceinline__ double canonical(double v) {
  return isnan(v) ? __longlong_as_double(0x7ff8000000000000ll) : v;
}
__device__ __forceinline__ float nan_of(float) { return __uint_as_float(0x7fc00000u); }
__device__ __forceinline__ double nan_of(double) {
  return __longlong_as_double(0x7ff8000000000000ll);
}

// float64 -> T with one round-to-nearest cast (T::from_f64 in the reference).
template <typename T>
__device__ __forceinline__ T from_f64(double v);
template <>
__device__ __forceinline__ float from_f64<float>(double v) {
  return __double2float_rn(v);
}
template <>
__device__ __forceinline__ double from_f64<double>(double v) {
  return v;
}

// ---------------------------------------------------------------------------
// Boundary mapping, src/boundary.rs:29-71. Returns false for a position
// outside a constant boundary. `length` is nonzero.

__host__ __device__ __forceinline__ long long rem_euclid(long long a, long long b) {
  long long r = a % b;
  return r < 0 ? r + b : r;
}

__host__ __device__ __forceinline__ bool map_index(long long index, long long length, int mode,
                                                   long long* out) {
  if (index >= 0 && index < length) {
    *out = index;
    return true;
  }
  switch (mode) {
    case kConstant:
      return false;
    case kNearest:
      *out = index < 0 ? 0 : length - 1;
      return true;
    case kWrap:
      *out = rem_euclid(index, length);
      return true;
    case kReflect: {
      if (length == 1) {
        *out = 0;
        return true;
      }
      long long period = 2 * length;
      long long r = rem_euclid(index, period);
      *out = r < length ? r : period - 1 - r;
      return true;
    }
    default: {  // kMirror
      if (length == 1) {
        *out = 0;
        return true;
      }
      long long period = 2 * (length - 1);
      long long r = rem_euclid(index, period);
      *out = r < length ? r : period - r;
      return true;
    }
  }
}

// ---------------------------------------------------------------------------
// Midpoint of the two middle retained values (lower <= upper in total
// order), the reducers 0.4.0 contract pinned by docs/semantics.md:74-88,
// tests/_reference.py:36-47 and src/reduction.rs:214-249.

__device__ __forceinline__ double midpoint(double lower, double upper) {
  if (signbit(lower) == signbit(upper) && lower == upper) return lower;
  if (lower == 0.0 && upper == 0.0) return 0.0;
  if (isinf(lower) || isinf(upper)) {
    if (isinf(lower) && isinf(upper)) return nan_of(0.0);
    return isinf(lower) ? lower : upper;
  }
  // x / 2 and x * 0.5 are the same correctly rounded value; the multiply
  // avoids a float64 division on the FP64 pipe.
  if (signbit(lower) == signbit(upper))
    return __dadd_rn(lower, __dmul_rn(__dsub_rn(upper, lower), 0.5));
  return __dmul_rn(__dadd_rn(lower, upper), 0.5);
}

// The same midpoint for two float32 values, cast once to float32. When
// both values are zero or normal with biased exponents in [30, 253] and
// their exponents differ by at most 28, the float64 computation above is
// exact ((a + b) / 2 needs at most 53 significant bits), so the result is
// the float32 rounding of (a + b) / 2. In that range RN32(a + b) * 0.5 is
// that rounding too: halving a normal float is exact and commutes with
// rounding. Everything else takes the float64 path.
__device__ __forceinline__ float midpoint_f32(float lower, float upper) {
  const unsigned int bl = __float_as_uint(lower), bu = __float_as_uint(upper);
  const int el = (int)((bl >> 23) & 0xFF), eu = (int)((bu >> 23) & 0xFF);
  const bool zl = (bl << 1) == 0u, zu = (bu << 1) == 0u;
  const bool nl = el >= 30 && el <= 253, nu = eu >= 30 && eu <= 253;
  const int diff = el > eu ? el - eu : eu - el;
  if ((zl || nl) && (zu || nu) && (zl || zu || diff <= 28)) {
    if (bl == bu) return lower;
    return __fmul_rn(__fadd_rn(lower, upper), 0.5f);
  }
  return __double2float_rn(midpoint((double)lower, (double)upper));
}

// Float64 classification and magnitude on the integer pipes (GB300's FP64
// pipe is narrow; these are exact bit tests, the same answers as isfinite /
// isnan / fabs and a magnitude comparison).
__device__ __forceinline__ unsigned long long mag_bits64(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ bool finite64(double x) { return mag_bits64(x) < 0x7FF0000000000000ull; }
__device__ __forceinline__ bool nan64(double x) { return mag_bits64(x) > 0x7FF0000000000000ull; }
__device__ __forceinline__ bool inf64_test(double x) { return mag_bits64(x) == 0x7FF0000000000000ull; }
__device__ __forceinline__ double abs64(double x) { return __longlong_as_double((long long)mag_bits64(x)); }

// Division of many dividends by one divisor s, correctly rounded (the same
// result as d / s): with r = RN(1/s), q = RN(d r) is corrected once by its
// exact residual (Markstein's method), and the corrected quotient is kept
// only when its own residual proves it is the nearest float: |d - q s| <
// ulp(q) |s| / 2, which holds exactly when q = RN(d / s) and no tie occurs
// (the residual is exact for q within one ulp; a wrong q has a residual of
// at least that bound, and rounding cannot bring it below a representable
// bound). Anything else (ties, powers of two, subnormal, zero or non-finite
// operands or results) takes the division.
struct Divisor {
  double s, r;
  bool fast;  // s normal and finite
};

__device__ __forceinline__ Divisor make_divisor(double s) {
  const unsigned long long m = (unsigned long long)__double_as_longlong(s) & 0x7FFFFFFFFFFFFFFFull;
  Divisor d;
  d.s = s;
  d.fast = m >= 0x0010000000000000ull && m < 0x7FF0000000000000ull;
  d.r = d.fast ? __drcp_rn(s) : 0.0;
  return d;
}

__device__ __forceinline__ double div_by(double x, const Divisor& d) {
  if (d.fast) {
    const double q0 = __dmul_rn(x, d.r);
    const double q = __fma_rn(__fma_rn(-q0, d.s, x), d.r, q0);
    const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
    const int qe = (int)((qb >> 52) & 0x7FF);
    const int se = (int)(((unsigned long long)__double_as_longlong(d.s) >> 52) & 0x7FF);
    // q normal, not a power of two, and the bound |s| 2^(E(q) - 53) normal.
    const int he = se + qe - 1023 - 53;
    if (qe >= 1 && qe < 0x7FF && (qb & 0x000FFFFFFFFFFFFFull) != 0 && he >= 1 && he <= 2046) {
      const double e = __fma_rn(-q, d.s, x);
      const unsigned long long hb =
          ((unsigned long long)__double_as_longlong(d.s) & 0x000FFFFFFFFFFFFFull) | ((unsigned long long)he << 52);
      if (((unsigned long long)__double_as_longlong(e) & 0x7FFFFFFFFFFFFFFFull) < hb) return q;
    }
  }
  return __ddiv_rn(x, d.s);
}

// Neumaier float64 sum, src/mean.rs:7-26. The |value| >= |x| test compares
// magnitude bits (the same order for every non-NaN pair; with a NaN operand
// the sum is NaN on either branch).
struct Sum64 {
  double value = 0.0, correction = 0.0;
  __device__ __forceinline__ void add(double x) {
    double next = __dadd_rn(value, x);
    if (mag_bits64(value) >= mag_bits64(x))
      correction = __dadd_rn(correction, __dadd_rn(__dsub_rn(value, next), x));
    else
      correction = __dadd_rn(correction, __dadd_rn(__dsub_rn(x, next), value));
    value = next;
  }
  __device__ __forceinline__ double total() const { return __dadd_rn(value, correction); }
};

// ---------------------------------------------------------------------------
// Exact sums equal to the sequential Neumaier sums (Sum64) of the same terms.
//
// The reference adds terms x_1..x_n in order with Neumaier's compensation
// (Sum64, src/mean.rs:7-26): s_i = RN(s_{i-1} + x_i), the error
// e_i of each addition computed exactly (Fast2Sum with the larger magnitude
// first), c_n = the rounded running sum of the e_i, result RN(s_n + c_n).
// With S the exact sum, s_n + sum(e_i) = S, so the result is RN(S + delta),
// delta = c_n - sum(e_i) the rounding of the correction sum. For n < 2^k
// terms below 2^H (n < 2^31, no overflow):
//  * sum|e_i| <= u n (1+u)^n sum|x_i| < 2^(2k + H - 52), u = 2^-53. When
//    every term is a multiple of 2^Q, so are every s_i, e_i and running sum
//    of the e_i; with Q >= 2k + H - 105 those running sums stay below
//    2^(Q + 53), are exact, delta = 0, and the result is RN(S) exactly
//    (ties included). This is the usual case for image data;
//  * otherwise |delta| <= gamma_{n-1} sum|e_i| < 2 n^3 u^2 2^H. ExactSum
//    rounds both ends of [S - E, S + E], E = 2^(3k + 55) units of the fixed
//    point (more than |delta| plus the n units of truncation); RN is
//    monotone, so when the ends agree every point between them rounds to the
//    same double, which is the sequential result.
// ExactSum adds the terms exactly, in any order (so threads can split
// them), in 192-bit fixed point with lowest bit 2^(H - 158) (bits below it
// truncated). When neither case decides (S within E of a rounding boundary,
// huge magnitudes, a result outside the normal range) the caller runs the
// sequential sum.

struct W3 {
  unsigned long long w0, w1, w2;  // 192-bit two's complement, w0 lowest
};

__device__ __forceinline__ void add3(W3& s, unsigned long long a0, unsigned long long a1, unsigned long long a2) {
  asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u64 %2, %2, %5;"
      : "+l"(s.w0), "+l"(s.w1), "+l"(s.w2)
      : "l"(a0), "l"(a1), "l"(a2));
}

__device__ __forceinline__ void sub3(W3& s, unsigned long long a0, unsigned long long a1, unsigned long long a2) {
  asm("sub.cc.u64 %0, %0, %3;\n\tsubc.cc.u64 %1, %1, %4;\n\tsubc.u64 %2, %2, %5;"
      : "+l"(s.w0), "+l"(s.w1), "+l"(s.w2)
      : "l"(a0), "l"(a1), "l"(a2));
}

// s += x / 2^L, |x| truncated to whole units; false when x is not finite or
// |x| >= 2^(L + 158). `low` takes the exponent of x's lowest set bit.
__device__ __forceinline__ bool add_fixed(W3& s, double x, int L, int& low) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
  if (mag >= 0x7FF0000000000000ull) return false;
  const int e = (int)(mag >> 52);
  const unsigned long long m = (mag & 0x000FFFFFFFFFFFFFull) | (e ? 0x0010000000000000ull : 0ull);
  if (m == 0) return true;
  const int sh = (e ? e - 1075 : -1074) - L;  // x = m 2^(sh + L)
  if (sh > 105) return false;
  low = min(low, sh + L + __ffsll((long long)m) - 1);
  unsigned long long a0 = 0, a1 = 0, a2 = 0;
  if (sh < 0) {
    a0 = sh > -64 ? m >> -sh : 0ull;
  } else {
    const int bs = sh & 63;
    const unsigned long long lo = m << bs, hi = bs ? m >> (64 - bs) : 0ull;
    if (sh < 64) {
      a0 = lo;
      a1 = hi;
    } else {
      a1 = lo;
      a2 = hi;
    }
  }
  if (b >> 63)
    sub3(s, a0, a1, a2);
  else
    add3(s, a0, a1, a2);
  return true;
}

// RN(s 2^L) for a 192-bit two's complement s with |s| < 2^190; false when s
// is zero or the result is not a normal double.
__device__ __forceinline__ bool fixed_rn(W3 s, int L, double* out) {
  const bool neg = (long long)s.w2 < 0;
  if (neg) {
    s.w0 = ~s.w0;
    s.w1 = ~s.w1;
    s.w2 = ~s.w2;
    add3(s, 1ull, 0ull, 0ull);
  }
  int top;
  if (s.w2)
    top = 191 - __clzll((long long)s.w2);
  else if (s.w1)
    top = 127 - __clzll((long long)s.w1);
  else if (s.w0)
    top = 63 - __clzll((long long)s.w0);
  else
    return false;
  // Shift the leading one to bit 191: 53 significand bits, then round and
  // sticky bits.
  int z = 191 - top;
  while (z >= 64) {
    s.w2 = s.w1;
    s.w1 = s.w0;
    s.w0 = 0;
    z -= 64;
  }
  if (z) {
    s.w2 = (s.w2 << z) | (s.w1 >> (64 - z));
    s.w1 = (s.w1 << z) | (s.w0 >> (64 - z));
    s.w0 <<= z;
  }
  unsigned long long sig = s.w2 >> 11;
  const bool half = (s.w2 >> 10) & 1ull;
  const bool sticky = (s.w2 & 0x3FFull) != 0 || s.w1 != 0 || s.w0 != 0;
  int exponent = L + top;  // s 2^L in [2^exponent, 2^(exponent + 1))
  if (half && (sticky || (sig & 1ull))) ++sig;
  if (sig >> 53) {
    sig >>= 1;
    ++exponent;
  }
  const int biased = exponent + 1023;
  if (biased < 1 || biased > 2046) return false;
  *out = __longlong_as_double((long long)(((unsigned long long)neg << 63) | ((unsigned long long)biased << 52) |
                                          (sig & 0x000FFFFFFFFFFFFFull)));
  return true;
}

// Smallest H with |x| < 2^H (x finite).
__device__ __forceinline__ int bound_exponent(double x) {
  const int e = (int)(mag_bits64(x) >> 52);
  return e ? e - 1022 : -1022;
}

struct ExactSum {
  W3 s;
  int H, low;
  bool ok;
  __device__ __forceinline__ explicit ExactSum(int bound) : s{0ull, 0ull, 0ull}, H(bound), low(INT_MAX), ok(true) {}
  __device__ __forceinline__ void add(double x) { ok = add_fixed(s, x, H - 158, low) && ok; }
  // The sequential Neumaier sum of the n added terms, when it is proven.
  __device__ __forceinline__ bool result(long long n, double* out) const {
    if (!ok || n < 1 || n >= (1ll << 31)) return false;
    const int k = 64 - __clzll(n);  // n < 2^k
    if (k + H > 1000) return false;
    const int L = H - 158;
    if (low >= 2 * k + H - 105) {
      // Exact correction sum: the result is RN(S).
      if ((s.w0 | s.w1 | s.w2) == 0ull) {
        *out = 0.0;
        return true;
      }
      return fixed_rn(s, L, out);
    }
    const int pos = 3 * k + 55;
    const unsigned long long e0 = pos < 64 ? 1ull << pos : 0ull;
    const unsigned long long e1 = pos >= 64 && pos < 128 ? 1ull << (pos - 64) : 0ull;
    const unsigned long long e2 = pos >= 128 ? 1ull << (pos - 128) : 0ull;
    W3 lo = s, hi = s;
    sub3(lo, e0, e1, e2);
    add3(hi, e0, e1, e2);
    double a, b;
    if (!fixed_rn(lo, L, &a) || !fixed_rn(hi, L, &b) || __double_as_longlong(a) != __double_as_longlong(b))
      return false;
    *out = a;
    return true;
  }
};

__device__ __forceinline__ double clamp64(double x, double lo, double hi) {
  if (x < lo) return lo;
  if (x > hi) return hi;
  return x;
}

// split / scale_binary / scaled_dot, src/convolution.rs:203-270.
struct Split {
  double mantissa;
  int exponent;
};

__device__ __forceinline__ Split split64(double value) {
  unsigned long long b = (unsigned long long)__double_as_longlong(value);
  int exponent = (int)((b >> 52) & 0x7ff);
  unsigned long long fraction = b & ((1ull << 52) - 1);
  if (exponent == 0) {
    int leading = 63 - __clzll((long long)fraction);
    double mantissa = __ddiv_rn((double)fraction, (double)(1ull << leading));
    return {copysign(mantissa, value), leading - 1074};
  }
  return {__longlong_as_double((long long)((b & ((1ull << 63) | ((1ull << 52) - 1))) |
                                           (1023ull << 52))),
          exponent - 1023};
}

__device__ __forceinline__ double scale_binary(double value, int exponent) {
  if (value == 0.0) return value;
  Split s = split64(value);
  int target = s.exponent + exponent;
  if (target > 1023) return copysign(__longlong_as_double(0x7ff0000000000000ll), value);
  if (target < -1075) return copysign(0.0, value);
  if (target >= -1022)
    return __dmul_rn(s.mantissa, __longlong_as_double((long long)(target + 1023) << 52));
  double remaining = __longlong_as_double((long long)(target + 1022 + 1023) << 52);
  return __dmul_rn(__dmul_rn(s.mantissa, 2.2250738585072014e-308), remaining);
}

// finite_weighted(&[(v0, w0), (v1, w1)], false), src/convolution.rs:287-361.
static __device__ __noinline__ double finite_weighted2(double v0, double w0, double v1, double w1) {
  const double values[2] = {v0, v1};
  const double weights[2] = {w0, w1};
  Sum64 sum;
  bool fallback = false;
  for (int i = 0; i < 2; ++i) {
    double product = __dmul_rn(values[i], weights[i]);
    if (!isfinite(product) || (values[i] != 0.0 && fabs(product) < 2.2250738585072014e-308)) {
      fallback = true;
      break;
    }
    sum.add(product);
  }
  if (!fallback) {
    double total = sum.total();
    if (isfinite(total)) return total;
  }
  // scaled_dot over two pairs: count bits of (2 - 1) = 1.
  bool any = false;
  int maximum = 0;
  for (int i = 0; i < 2; ++i) {
    if (values[i] == 0.0) continue;
    int e = split64(values[i]).exponent + split64(weights[i]).exponent;
    maximum = any ? max(maximum, e) : e;
    any = true;
  }
  if (!any) return scale_binary(0.0, 0);
  int exponent = maximum + 1 + 2;
  Sum64 scaled;
  for (int i = 0; i < 2; ++i) {
    if (values[i] == 0.0) continue;
    Split a = split64(values[i]);
    Split b = split64(weights[i]);
    scaled.add(scale_binary(__dmul_rn(a.mantissa, b.mantissa), a.exponent + b.exponent - exponent));
  }
  return scale_binary(scaled.total(), exponent);
}

// interpolate, src/robust.rs:305-341.
__device__ __forceinline__ double interpolate(double lower, double upper, double fraction) {
  if (fraction == 0.0 || __double_as_longlong(lower) == __double_as_longlong(upper)) return lower;
  if (fraction == 1.0) return upper;
  if (isinf(lower) || isinf(upper)) {
    if (lower < 0 && isinf(lower) && upper > 0 && isinf(upper)) return nan_of(0.0);
    return isinf(lower) ? lower : upper;
  }
  if (signbit(lower) != signbit(upper)) {
    if (!isfinite(__dsub_rn(upper, lower))) {
      double half_lower = __dmul_rn(lower, 0.5);
      double half_upper = __dmul_rn(upper, 0.5);
      double r = __dmul_rn(
          __dadd_rn(half_lower, __dmul_rn(__dsub_rn(half_upper, half_lower), fraction)), 2.0);
      return clamp64(r, lower, upper);
    }
    return finite_weighted2(lower, __dsub_rn(1.0, fraction), upper, fraction);
  }
  double difference = __dsub_rn(upper, lower);
  double result = fraction <= 0.5
                      ? __dadd_rn(lower, __dmul_rn(difference, fraction))
                      : __dsub_rn(upper, __dmul_rn(difference, __dsub_rn(1.0, fraction)));
  return clamp64(result, lower, upper);
}

// Percentile rank split, src/robust.rs:343-352: returns the lower and upper
// zero-based ranks and the fraction for `n` retained samples (q < 100).
struct PercentileRank {
  long long lower, upper;
  double fraction;
};

// `q_fraction` is q / 100.0, computed once on the host (the same float64).
__device__ __forceinline__ PercentileRank percentile_rank(double q_fraction, long long n) {
  double rank = __dmul_rn(q_fraction, (double)(n - 1));
  long long lower = (long long)floor(rank);
  long long upper = lower + 1 < n - 1 ? lower + 1 : n - 1;
  return {lower, upper, __dsub_rn(rank, (double)lower)};
}

// The split for n >= 1 retained samples: from the plan's table when it has
// one (an L1-resident load instead of six FP64-pipe operations, which run at
// a small fraction of the FP32 rate on this GPU), else computed.
struct PctSplit {
  int lower, upper, flags;
  double fraction, w;
};

__device__ __forceinline__ PctSplit pct_split(const Reduce& r, long long n) {
  PctSplit s;
  if (r.pct) {
    const PctEntry* e = r.pct + n;
    s.fraction = __ldg(&e->fraction);
    s.w = __ldg(&e->w);
    s.lower = __ldg(&e->lower);
    s.flags = __ldg(&e->flags);
  } else {
    PercentileRank pr = percentile_rank(r.q_fraction, n);
    s.lower = (int)pr.lower;
    s.fraction = pr.fraction;
    const bool low = pr.fraction <= 0.5;
    s.w = low ? pr.fraction : __dsub_rn(1.0, pr.fraction);
    s.flags = (pr.fraction == 0.0 ? kPctFracZero : 0) | (low ? kPctLowSide : 0) |
              (pr.fraction == 1.0 ? kPctFracOne : 0);
  }
  s.upper = s.lower + 1 < n - 1 ? s.lower + 1 : (int)(n - 1);
  return s;
}

// float -> float64 bits for a normal or zero float (exact; integer ops only).
__device__ __forceinline__ double f32_to_f64_exact(unsigned int b) {
  const unsigned int sign = b & 0x80000000u;
  const unsigned int e = (b >> 23) & 0xFFu;
  const unsigned int hi = e == 0 ? sign : sign | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
  const unsigned int lo = e == 0 ? 0u : (b & 7u) << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// Round a float64 to float (to nearest, ties to even) with integer ops when
// the result is a normal float; other results take the hardware conversion.
__device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  const int e32 = (int)((hi >> 20) & 0x7FFu) - 896;
  if (e32 < 1 || e32 > 254) return __double2float_rn(x);
  const unsigned int mant = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  const unsigned int rem = lo & 0x1FFFFFFFu;
  const unsigned int bits = (hi & 0x80000000u) | ((unsigned int)e32 << 23) | mant;
  const bool up = rem > 0x10000000u || (rem == 0x10000000u && (mant & 1u));
  return __uint_as_float(bits + (up ? 1u : 0u));  // a carry rounds into the exponent
}

// T(interpolate(lower, upper, fraction)) for order statistics lower <= upper.
template <typename T>
__device__ __forceinline__ T pct_value(const PctSplit& s, T lower, T upper);

template <>
__device__ __forceinline__ double pct_value<double>(const PctSplit& s, double lower, double upper) {
  return interpolate(lower, upper, s.fraction);
}

// float inputs: the common case (both normal or zero, same sign, distinct,
// 0 < fraction < 1) needs three FP64 operations; rounding the float64 result
// once to float and clamping in float equals clamping in float64 first,
// because lower and upper are floats and rounding is monotonic.
template <>
__device__ __forceinline__ float pct_value<float>(const PctSplit& s, float lower, float upper) {
  const unsigned int lb = __float_as_uint(lower), ub = __float_as_uint(upper);
  const unsigned int el = (lb >> 23) & 0xFFu, eu = (ub >> 23) & 0xFFu;
  const bool ok_l = (el - 1u) < 254u || (lb << 1) == 0u;
  const bool ok_u = (eu - 1u) < 254u || (ub << 1) == 0u;
  const bool fast = ok_l && ok_u && lb != ub && ((lb ^ ub) >> 31) == 0u &&
                    (s.flags & (kPctFracZero | kPctFracOne)) == 0;
  if (!fast) return __double2float_rn(interpolate((double)lower, (double)upper, s.fraction));
  const double dl = f32_to_f64_exact(lb), du = f32_to_f64_exact(ub);
  const double p = __dmul_rn(__dsub_rn(du, dl), s.w);
  const double r = (s.flags & kPctLowSide) ? __dadd_rn(dl, p) : __dsub_rn(du, p);
  const float x = f64_to_f32_rn(r);
  if (x < lower) return lower;
  if (x > upper) return upper;
  return x;
}

}  // namespace ndf

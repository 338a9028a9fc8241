// Robust window statistics: the MAD, iterative sigma clipping, the mode
// estimators and the biweight location / scale (device code; robust.cu and
// robust_f64.cu instantiate it for float32 and float64 inputs so the two
// compile in parallel).
//
// Replaces RobustReduction::finish for those kinds (src/robust.rs:244-299,
// 376-689) and the estimators of src/location.rs:36-240, applied per window
// by robust_into (src/robust.rs:725-785). Every step keeps the reference's
// float64 arithmetic, operation for operation (each operation correctly
// rounded, no contraction), so the results equal the reference's bit for
// bit; the one order the reference leaves unpublished (the sample order
// after its in-place median, which the biweight sums follow) is ascending
// order here, as in the oracle.
//
// GB300 design: one thread per output pixel (grid-stride). A thread gathers
// its window through the per-axis boundary maps (flat offsets for interior
// windows), keeps the retained samples twice, in tap order (the order of
// the reference's sums) and sorted by total order (insertion sort on
// order-preserving keys), and runs the estimator on those two arrays. The
// arrays live in thread-local memory for windows up to 256 samples and in a
// per-thread slice of a global scratch buffer beyond. The work is float64
// and branchy, so it runs on the FP64 pipe at a fraction of the FP32 rate;
// the windows the robust filters serve are small.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "moments.cuh"
#include "plan.h"

namespace ndf {
namespace {

constexpr int kRThreads = 128;
// Phi^-1(0.75), src/robust.rs:11.
constexpr double kNormalUpperQuartile = 0.6744897501960817;

struct Scaled {
  double value;
  int exponent;
};

__device__ __forceinline__ unsigned long long total_key(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// IEEE a == b and a < b on bit patterns (the integer pipe; GB300's float64
// pipe is narrow): NaN compares false, -0 equals +0.
__device__ __forceinline__ bool eq64(double a, double b) {
  if (nan64(a) || nan64(b)) return false;
  return (mag_bits64(a) | mag_bits64(b)) == 0ull || __double_as_longlong(a) == __double_as_longlong(b);
}

__device__ __forceinline__ bool lt64(double a, double b) {
  if (nan64(a) || nan64(b) || (mag_bits64(a) | mag_bits64(b)) == 0ull) return false;
  return total_key(a) < total_key(b);
}

// RN(2 v): one more in the exponent field for normal v below the overflow
// threshold (exact), the float64 multiply otherwise.
__device__ __forceinline__ double twice(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned int e = (unsigned int)((b >> 52) & 0x7FF);
  if (e >= 1 && e < 2046) return __longlong_as_double((long long)(b + (1ull << 52)));
  return __dmul_rn(v, 2.0);
}

// A float or float64 sample as float64: normal and zero floats by integer
// operations (exact), the rest by the hardware conversion.
__device__ __forceinline__ double widen(float x) {
  const unsigned int b = __float_as_uint(x);
  const unsigned int e = (b >> 23) & 0xFFu;
  if ((e != 0u && e != 255u) || (b << 1) == 0u) return f32_to_f64_exact(b);
  return (double)x;
}
__device__ __forceinline__ double widen(double x) { return x; }

__device__ __forceinline__ int total_cmp(double a, double b) {
  const unsigned long long ka = total_key(a), kb = total_key(b);
  return ka < kb ? -1 : (ka > kb ? 1 : 0);
}

__device__ void sort_total(double* a, int n) {
  for (int i = 1; i < n; ++i) {
    const double v = a[i];
    const unsigned long long k = total_key(v);
    int j = i - 1;
    while (j >= 0 && total_key(a[j]) > k) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = v;
  }
}

// The same order for up to 32 samples without thread-local traffic in the
// inner loop: total-order keys in registers through the Batcher network
// (slots past n hold the largest key and sort last), written back in order.
__device__ __forceinline__ void sort_total32(const double* v, double* s, int n) {
  unsigned long long k[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) k[i] = i < n ? total_key(v[i]) : ~0ull;
  net::batcher_sort<32>(k);
#pragma unroll
  for (int i = 0; i < 32; ++i)
    if (i < n) s[i] = __longlong_as_double((long long)((k[i] >> 63) ? (k[i] & 0x7FFFFFFFFFFFFFFFull) : ~k[i]));
}

// Up to MAXV samples (a multiple of 32): runs of 32 sorted as above, as
// keys, then merged pairwise level by level, the keys ping-ponging between
// `w` and `s` (both MAXV long), and written back in order as samples.
__device__ __forceinline__ double key_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

__device__ __forceinline__ void merge_keys(const unsigned long long* a, int na, const unsigned long long* b, int nb,
                                           unsigned long long* out) {
  int i = 0, j = 0;
  for (int o = 0; o < na + nb; ++o) out[o] = (j >= nb || (i < na && a[i] <= b[j])) ? a[i++] : b[j++];
}

template <int MAXV>
__device__ __forceinline__ void sort_total_runs(const double* v, double* s, double* w, int n) {
  unsigned long long* src = reinterpret_cast<unsigned long long*>(w);
  unsigned long long* dst = reinterpret_cast<unsigned long long*>(s);
#pragma unroll 1
  for (int base = 0; base < n; base += 32) {
    const int count = n - base < 32 ? n - base : 32;
    unsigned long long k[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) k[i] = i < count ? total_key(v[base + i]) : ~0ull;
    net::batcher_sort<32>(k);
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (i < count) src[base + i] = k[i];
  }
#pragma unroll 1
  for (int width = 32; width < n; width *= 2) {
    for (int lo = 0; lo < n; lo += 2 * width) {
      const int mid = lo + width < n ? lo + width : n, hi = lo + 2 * width < n ? lo + 2 * width : n;
      merge_keys(src + lo, mid - lo, src + mid, hi - mid, dst + lo);
    }
    unsigned long long* t = src;
    src = dst;
    dst = t;
  }
  // The sorted keys are in `src`, which is `w` or `s`; write the samples to s.
  for (int i = 0; i < n; ++i) s[i] = key_value(src[i]);
}

// 2^n by binary powering with a final reciprocal for negative n: exact
// unless 2^|n| overflows, when the reciprocal is zero.
__device__ double powi2(int n) {
  unsigned int m = n < 0 ? (unsigned int)(-(long long)n) : (unsigned int)n;
  double r = 1.0, a = 2.0;
  while (m) {
    if (m & 1) r = __dmul_rn(r, a);
    a = __dmul_rn(a, a);
    m >>= 1;
  }
  return n < 0 ? __ddiv_rn(1.0, r) : r;
}

// binary_parts, src/robust.rs:498-511 (positive finite values).
__device__ __forceinline__ Scaled binary_parts(double value) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(value);
  const int exponent = (int)((b >> 52) & 0x7ff);
  const unsigned long long fraction = b & ((1ull << 52) - 1);
  if (exponent == 0) {
    const int leading = 63 - __clzll((long long)fraction);
    return {__ddiv_rn((double)fraction, (double)(1ull << leading)), leading - 1074};
  }
  return {__longlong_as_double((long long)(fraction | (1023ull << 52))), exponent - 1023};
}

__device__ __forceinline__ double inf64() { return __longlong_as_double(0x7ff0000000000000ll); }

// absolute_deviation, src/robust.rs:438-466.
__device__ Scaled absolute_deviation(double value, Scaled center) {
  const double doubled = twice(value);
  if (center.exponent == -1 && finite64(doubled)) {
    const double difference = __dsub_rn(doubled, center.value);
    if (finite64(difference)) return {abs64(difference), -1};
  }
  const double midpoint = center.exponent == -1 ? __dmul_rn(center.value, 0.5) : center.value;
  const double difference = __dsub_rn(value, midpoint);
  if (finite64(difference) || inf64_test(value)) return {abs64(difference), 0};
  return {abs64(__dsub_rn(__dmul_rn(value, 0.5), __dmul_rn(midpoint, 0.5))), 1};
}

// compare_scaled, src/robust.rs:468-481.
__device__ int compare_scaled(Scaled left, Scaled right) {
  if (mag_bits64(left.value) == 0ull || mag_bits64(right.value) == 0ull || inf64_test(left.value) ||
      inf64_test(right.value))
    return total_cmp(left.value, right.value);
  const Scaled l = binary_parts(left.value), r = binary_parts(right.value);
  const int a = l.exponent + left.exponent, b = r.exponent + right.exponent;
  if (a != b) return a < b ? -1 : 1;
  return total_cmp(l.value, r.value);
}

// scaled_midpoint, src/robust.rs:483-496.
__device__ Scaled scaled_midpoint(Scaled left, Scaled right) {
  if (inf64_test(right.value) || right.value == 0.0) return right;
  const Scaled r = binary_parts(right.value);
  const int exponent = r.exponent + right.exponent;
  double lv = 0.0;
  if (left.value != 0.0) {
    const Scaled l = binary_parts(left.value);
    lv = __dmul_rn(l.value, powi2(l.exponent + left.exponent - exponent));
  }
  return {__dadd_rn(lv, r.value), exponent - 1};
}

// mad_parts, src/robust.rs:376-436, over samples sorted in total order.
__device__ Scaled mad_parts(const double* s, int n) {
  const double lower = s[(n - 1) / 2], upper = s[n / 2];
  Scaled center;
  if (!finite64(lower) || !finite64(upper))
    center = {interpolate(lower, upper, 0.5), 0};
  else if (finite64(__dadd_rn(lower, upper)))
    center = {__dadd_rn(lower, upper), -1};
  else
    center = {__dadd_rn(__dmul_rn(lower, 0.5), __dmul_rn(upper, 0.5)), 0};
  if (!finite64(center.value)) return {nan_of(0.0), 0};
  // The merge keeps the two candidate deviations (left and right of the
  // consumed middle run) and recomputes only the side it consumed.
  int left = n / 2, right = left;
  Scaled previous{0.0, 0}, selected = previous;
  Scaled dl = left > 0 ? absolute_deviation(s[left - 1], center) : selected;
  Scaled dr = right < n ? absolute_deviation(s[right], center) : selected;
  for (int step = 0; step <= n / 2; ++step) {
    previous = selected;
    const bool take_left = left > 0 && (right == n || compare_scaled(dl, dr) <= 0);
    if (take_left) {
      --left;
      selected = dl;
      if (left > 0) dl = absolute_deviation(s[left - 1], center);
    } else {
      selected = dr;
      ++right;
      if (right < n) dr = absolute_deviation(s[right], center);
    }
  }
  return n % 2 == 1 ? selected : scaled_midpoint(previous, selected);
}

// multiply_scaled, src/robust.rs:513-534.
__device__ double multiply_scaled(Scaled value, double multiplier) {
  if (!finite64(value.value)) return __dmul_rn(value.value, multiplier);
  if (value.value == 0.0 || multiplier == 0.0) return 0.0;
  const Scaled l = binary_parts(value.value), r = binary_parts(multiplier);
  const Scaled m = binary_parts(__dmul_rn(l.value, r.value));
  const int exponent = l.exponent + r.exponent + m.exponent + value.exponent;
  if (exponent > 1023) return inf64();
  if (exponent < -1075) return 0.0;
  if (exponent >= -1022) return __dmul_rn(m.value, __longlong_as_double((long long)(exponent + 1023) << 52));
  const double scale = __longlong_as_double((long long)(exponent + 2045) << 52);
  return __dmul_rn(__dmul_rn(m.value, 2.2250738585072014e-308), scale);
}

// within_limit, src/robust.rs:536-559, with the spread and the multiplier
// split once per clipping pass (make_limit) and only the distance per sample
// (inside): the same comparisons, in the same arithmetic.
struct Limit {
  bool zero;  // spread or sigma zero: only samples equal to the center pass
  Scaled limit;
  int exponent;
};

__device__ Limit make_limit(Scaled spread, double sigma) {
  Limit l;
  l.zero = spread.value == 0.0 || sigma == 0.0;
  if (l.zero) return l;
  const Scaled sc = binary_parts(spread.value), mu = binary_parts(sigma);
  l.limit = binary_parts(__dmul_rn(sc.value, mu.value));
  l.exponent = sc.exponent + mu.exponent + l.limit.exponent + spread.exponent;
  return l;
}

__device__ __forceinline__ bool inside(double value, double center, const Limit& l) {
  if (eq64(value, center)) return true;
  if (l.zero) return false;
  const double difference = __dsub_rn(value, center);
  Scaled d;
  if (finite64(difference)) {
    d = binary_parts(abs64(difference));
  } else {
    d = binary_parts(abs64(__dsub_rn(__dmul_rn(value, 0.5), __dmul_rn(center, 0.5))));
    d.exponent += 1;
  }
  return d.exponent < l.exponent || (d.exponent == l.exponent && d.value <= l.limit.value);
}

// percentile, src/robust.rs:343-352, over sorted samples.
__device__ double percentile_sorted(const double* s, int n, double q) {
  if (q == 100.0) return s[n - 1];
  const double rank = __dmul_rn(__ddiv_rn(q, 100.0), (double)(n - 1));
  const int lower = (int)floor(rank);
  const int upper = min(lower + 1, n - 1);
  return interpolate(s[lower], s[upper], __dsub_rn(rank, (double)lower));
}

// median_valid_in_place of the reducers crate over sorted samples: the
// middle value, or the midpoint of the two middle values.
__device__ __forceinline__ double median_sorted(const double* s, int n) {
  return n % 2 == 1 ? s[n / 2] : midpoint(s[n / 2 - 1], s[n / 2]);
}

// finite_mean, src/robust.rs:572-592, in tap order.
__device__ double finite_mean(const double* v, int n) {
  Sum64 sum;
  for (int i = 0; i < n; ++i) sum.add(v[i]);
  const double total = sum.total();
  if (finite64(total)) return __ddiv_rn(total, (double)n);
  const unsigned long long m = (unsigned long long)(n - 1);
  const int exponent = (m == 0 ? 0 : 64 - __clzll((long long)m)) + 1;
  const double scale = powi2(exponent);
  Sum64 scaled;
  double lower = inf64(), upper = -inf64();
  for (int i = 0; i < n; ++i) {
    scaled.add(__ddiv_rn(v[i], scale));
    lower = fmin(lower, v[i]);
    upper = fmax(upper, v[i]);
  }
  return clamp64(__ddiv_rn(scaled.total(), __ddiv_rn((double)n, scale)), lower, upper);
}

// finite_mean of finite samples `v` whose sorted copy is `s`: the Neumaier
// total proven from the exact sum (ExactSum), else the sequential code.
__device__ double finite_mean_exact(const double* v, const double* s, int n) {
  if (n > 0) {
    ExactSum e(bound_exponent(fmax(abs64(s[0]), abs64(s[n - 1]))));
    for (int i = 0; i < n; ++i) e.add(v[i]);
    double total;
    if (e.result(n, &total) && finite64(total)) return __ddiv_rn(total, (double)n);
  }
  return finite_mean(v, n);
}

// Sum of the scaled deviations w[0..n) (each at most 1 in magnitude: the
// scale is their largest magnitude) and of the squared residuals about
// their mean (each at most 4), in tap order.
__device__ __forceinline__ double scaled_total(const double* w, int n) {
  ExactSum e(1);
  for (int i = 0; i < n; ++i) e.add(w[i]);
  double total;
  if (e.result(n, &total)) return total;
  Sum64 sum;
  for (int i = 0; i < n; ++i) sum.add(w[i]);
  return sum.total();
}

__device__ __forceinline__ double residual_squares(const double* w, int n, double center) {
  ExactSum e(3);
  for (int i = 0; i < n; ++i) {
    const double residual = __dsub_rn(w[i], center);
    e.add(__dmul_rn(residual, residual));
  }
  double total;
  if (e.result(n, &total)) return total;
  Sum64 squares;
  for (int i = 0; i < n; ++i) {
    const double residual = __dsub_rn(w[i], center);
    squares.add(__dmul_rn(residual, residual));
  }
  return squares.total();
}

// The deltas v[i] - v[0] into w (all halved first when one overflows, as
// std_parts and dispersion_valid do) and their largest magnitude.
__device__ __forceinline__ double deltas(const double* v, int n, double* w, bool* halve) {
  const double reference = v[0];
  bool over = false;
  unsigned long long peak = 0ull;
  for (int i = 0; i < n; ++i) {
    w[i] = __dsub_rn(v[i], reference);
    over = over || !finite64(w[i]);
    peak = max(peak, mag_bits64(w[i]));
  }
  if (over) {
    peak = 0ull;
    for (int i = 0; i < n; ++i) {
      w[i] = __dsub_rn(__dmul_rn(v[i], 0.5), __dmul_rn(reference, 0.5));
      peak = max(peak, mag_bits64(w[i]));
    }
  }
  *halve = over;
  return __longlong_as_double((long long)peak);
}

// std_parts, src/robust.rs:594-630, in tap order. `w` keeps each sample's
// delta / scale between the two sums (the same quotient both times).
__device__ Scaled std_parts(const double* v, int n, double* w) {
  bool halve;
  const double scale = deltas(v, n, w, &halve);
  if (scale == 0.0) return {0.0, 0};
  const Divisor by = make_divisor(scale);
  for (int i = 0; i < n; ++i) w[i] = div_by(w[i], by);
  const double center = __ddiv_rn(scaled_total(w, n), (double)n);
  const double squares = residual_squares(w, n, center);
  const Scaled parts = binary_parts(scale);
  return {__dmul_rn(parts.value, __dsqrt_rn(__ddiv_rn(squares, (double)n))), parts.exponent + (halve ? 1 : 0)};
}

// mode_from_moments, src/location.rs:56-84.
__device__ double mode_from_moments(double mean, double median, double std_dev, int estimator, double pearson) {
  const double difference = __dsub_rn(median, mean);
  const double pearson_mode = __dadd_rn(median, __dmul_rn(__dsub_rn(pearson, 1.0), difference));
  if (estimator == kModeMmm) return pearson_mode;
  if (estimator == kModeIraf) return mean < median ? mean : pearson_mode;
  if (std_dev == 0.0) return mean;
  if (__ddiv_rn(abs64(difference), std_dev) >= 0.3) return median;
  return pearson_mode;
}

// dispersion_valid(values, 0, true), src/dispersion.rs:5-61, for finite
// samples in tap order; `w` keeps each delta / scale between the two sums.
__device__ double population_std(const double* v, int n, double* w) {
  bool halve;
  const double scale = deltas(v, n, w, &halve);
  if (scale == 0.0) return 0.0;
  const Divisor by = make_divisor(scale);
  for (int i = 0; i < n; ++i) w[i] = div_by(w[i], by);
  const double center = __ddiv_rn(scaled_total(w, n), (double)n);
  const double result = __dmul_rn(scale, __dsqrt_rn(__ddiv_rn(residual_squares(w, n, center), (double)n)));
  return halve ? __dmul_rn(result, 2.0) : result;
}

// mode_estimate, src/location.rs:36-54: mean and std in tap order (`v`),
// the median from the sorted samples (`s`).
__device__ double mode_estimate(const double* v, const double* s, int n, int estimator, double pearson,
                                double* w) {
  if (n == 0) return nan_of(0.0);
  const double mean = finite_mean_exact(v, s, n);
  const double std_dev = estimator == kModeSex ? population_std(v, n, w) : nan_of(0.0);
  return mode_from_moments(mean, median_sorted(s, n), std_dev, estimator, pearson);
}

// standardize + biweight_location / biweight_scale, src/location.rs:104-240,
// over samples sorted in total order; `dev` receives the standardized
// deviations in that order.
__device__ double biweight(const double* s, int n, double* dev, const RobustArgs& ra, bool location) {
  const double median = median_sorted(s, n);
  double factor = 1.0;
  bool overflow = false;
  for (int i = 0; i < n; ++i) {
    dev[i] = __dsub_rn(s[i], median);
    overflow = overflow || !finite64(dev[i]);
  }
  if (overflow) {
    factor = 2.0;
    for (int i = 0; i < n; ++i) dev[i] = __dsub_rn(__dmul_rn(s[i], 0.5), __dmul_rn(median, 0.5));
  }
  // Median of |dev|: the deviations ascend, so their magnitudes ascend
  // outwards from the smallest; merge both sides up to the middle ranks.
  int right = 0;
  while (right < n && lt64(dev[right], 0.0)) ++right;
  int left = right;
  double a = 0.0, b = 0.0;
  for (int k = 0; k <= n / 2; ++k) {
    double next;
    if (left > 0 && (right == n || mag_bits64(dev[left - 1]) <= mag_bits64(dev[right]))) {
      next = abs64(dev[--left]);
    } else {
      next = abs64(dev[right++]);
    }
    if (k == (n - 1) / 2) a = next;
    if (k == n / 2) b = next;
  }
  double mad = n % 2 == 1 ? b : midpoint(a, b);
  if (mad == 0.0) return location ? median : 0.0;
  const double c = ra.parameter;
  double extra = 1.0;
  while (!finite64(__dmul_rn(c, mad))) {
    mad = __dmul_rn(mad, 0.5);
    extra = __dmul_rn(extra, 2.0);
  }
  const double width = __dmul_rn(c, mad);
  factor = __dmul_rn(factor, extra);
  const Divisor by_extra = make_divisor(extra), by_width = make_divisor(width);
  const bool unit_extra = extra == 1.0;  // x / 1 is x exactly
  // The weighted terms lie below 1 in magnitude (|u| < 1, weights in
  // [0, 1]); the scale's denominator terms in (-4, 1].
  if (location) {
    ExactSum weighted_e(1), weights_e(1);
    int kept = 0;
    for (int i = 0; i < n; ++i) {
      const double u = div_by(unit_extra ? dev[i] : div_by(dev[i], by_extra), by_width);
      if (!(mag_bits64(u) < 0x3FF0000000000000ull)) continue;
      const double t = __dsub_rn(1.0, __dmul_rn(u, u));
      const double weight = __dmul_rn(t, t);
      weighted_e.add(__dmul_rn(u, weight));
      weights_e.add(weight);
      ++kept;
    }
    double weighted_total, weights_total;
    if (!weighted_e.result(kept, &weighted_total) || !weights_e.result(kept, &weights_total)) {
      Sum64 weighted, weights;
      for (int i = 0; i < n; ++i) {
        const double u = div_by(unit_extra ? dev[i] : div_by(dev[i], by_extra), by_width);
        if (!(mag_bits64(u) < 0x3FF0000000000000ull)) continue;
        const double t = __dsub_rn(1.0, __dmul_rn(u, u));
        const double weight = __dmul_rn(t, t);
        weighted.add(__dmul_rn(u, weight));
        weights.add(weight);
      }
      weighted_total = weighted.total();
      weights_total = weights.total();
    }
    const double correction = __dmul_rn(width, __ddiv_rn(weighted_total, weights_total));
    const double unscaled = __dmul_rn(correction, factor);
    if (finite64(unscaled)) return __dadd_rn(median, unscaled);
    return __dmul_rn(__dadd_rn(__ddiv_rn(median, factor), correction), factor);
  }
  ExactSum numerator_e(1), denominator_e(3);
  int kept = 0;
  for (int i = 0; i < n; ++i) {
    const double u = div_by(unit_extra ? dev[i] : div_by(dev[i], by_extra), by_width);
    if (!(mag_bits64(u) < 0x3FF0000000000000ull)) continue;
    const double u2 = __dmul_rn(u, u);
    const double w = __dsub_rn(1.0, u2);
    const double taper = __dmul_rn(w, w);
    numerator_e.add(__dmul_rn(__dmul_rn(u2, taper), taper));
    denominator_e.add(__dmul_rn(w, __dsub_rn(1.0, __dmul_rn(5.0, u2))));
    ++kept;
  }
  double numerator_total, denominator_total;
  if (!numerator_e.result(kept, &numerator_total) || !denominator_e.result(kept, &denominator_total)) {
    Sum64 numerator, denominator;
    for (int i = 0; i < n; ++i) {
      const double u = div_by(unit_extra ? dev[i] : div_by(dev[i], by_extra), by_width);
      if (!(mag_bits64(u) < 0x3FF0000000000000ull)) continue;
      const double u2 = __dmul_rn(u, u);
      const double w = __dsub_rn(1.0, u2);
      const double taper = __dmul_rn(w, w);
      numerator.add(__dmul_rn(__dmul_rn(u2, taper), taper));
      denominator.add(__dmul_rn(w, __dsub_rn(1.0, __dmul_rn(5.0, u2))));
    }
    numerator_total = numerator.total();
    denominator_total = denominator.total();
  }
  const double count = (double)(ra.modify_sample_size ? kept : n);
  const double ratio = __ddiv_rn(__dsqrt_rn(__dmul_rn(count, numerator_total)), abs64(denominator_total));
  return __dmul_rn(__dmul_rn(width, ratio), factor);
}

// clipped, src/robust.rs:632-689: `v` holds the finite samples in tap
// order and `s` the same samples sorted; both shrink together (`w` is
// scratch).
__device__ double clipped(double* v, double* s, double* w, int n, const RobustArgs& ra, int kind) {
  long long iteration = 0;
  while (n >= ra.clip_min_count && (ra.maxiters < 0 || iteration < ra.maxiters)) {
    const double center = ra.center == 0 ? finite_mean_exact(v, s, n) : percentile_sorted(s, n, 50.0);
    Scaled spread;
    if (ra.spread == 1) {
      const Scaled deviation = mad_parts(s, n);
      if (deviation.value > 0.0 && finite64(deviation.value)) {
        const Scaled parts = binary_parts(deviation.value);
        spread = {__ddiv_rn(parts.value, kNormalUpperQuartile), parts.exponent + deviation.exponent};
      } else {
        spread = deviation;
      }
    } else {
      spread = std_parts(v, n, w);
    }
    const Limit below = make_limit(spread, ra.lower), above = make_limit(spread, ra.upper);
    // The test depends on the value alone and the distance to the center
    // grows away from it on both sides (rounding is monotone), so the kept
    // sorted samples are one run [lo, hi): binary searches find it (the
    // first sample at or above the center, then the run's two ends), and the
    // tap-order samples are kept by their total-order key against the run's
    // ends (equal values share their fate, so no value straddles an end).
    auto in = [&](int i) { return inside(s[i], center, lt64(s[i], center) ? below : above); };
    int a = 0, b = n;
    while (a < b) {
      const int m = (a + b) / 2;
      if (lt64(s[m], center)) a = m + 1; else b = m;
    }
    const int c = a;
    int lo = 0;
    b = c;
    while (lo < b) {
      const int m = (lo + b) / 2;
      if (in(m)) b = m; else lo = m + 1;
    }
    int hi = c;
    b = n;
    while (hi < b) {
      const int m = (hi + b) / 2;
      if (in(m)) hi = m + 1; else b = m;
    }
    if (lo == c && hi == c) lo = hi = 0;
    int kept = 0;
    if (hi > lo) {
      const unsigned long long first = total_key(s[lo]), last = total_key(s[hi - 1]);
      for (int i = 0; i < n; ++i) {
        const unsigned long long k = total_key(v[i]);
        if (k >= first && k <= last) v[kept++] = v[i];
      }
    }
    s += lo;
    ++iteration;
    const bool stable = kept == n;
    n = kept;
    if (stable) break;
  }
  if (n < ra.clip_min_count) return nan_of(0.0);
  if (kind == kRobustSigmaMean) return finite_mean_exact(v, s, n);
  if (kind == kRobustSigmaMedian) return percentile_sorted(s, n, 50.0);
  return mode_estimate(v, s, n, ra.estimator, ra.pearson, w);
}

// One window: gather, the sample policy, the estimator.
template <int MAXV, bool MERGE, typename Fetch>
__device__ double robust_window(Fetch&& fetch, int V, const Reduce& r, const RobustArgs& ra, double* v,
                                double* s, double* w) {
  const bool clip = ra.kind >= kRobustSigmaMean;
  int n = 0;
  bool nan = false, inf = false;
  for (int i = 0; i < V; ++i) {
    const double x = fetch(i);
    if (clip) {
      if (finite64(x)) v[n++] = x;
      continue;
    }
    if (nan64(x)) {
      nan = nan || !r.omit;
      continue;
    }
    if (r.drop_inf && inf64_test(x)) continue;
    inf = inf || inf64_test(x);
    v[n++] = x;
  }
  if (!clip) {
    if (nan || (r.omit && n < r.min_count) || n == 0) return nan_of(0.0);
  }
  if constexpr (MAXV == 32) {
    sort_total32(v, s, n);
  } else if constexpr (MERGE) {
    sort_total_runs<MAXV>(v, s, w, n);
  } else {
    for (int i = 0; i < n; ++i) s[i] = v[i];
    sort_total(s, n);
  }
  switch (ra.kind) {
    case kRobustMad:
      return multiply_scaled(mad_parts(s, n), ra.parameter);
    case kRobustMode:
      return inf ? nan_of(0.0) : mode_estimate(v, s, n, ra.estimator, ra.pearson, w);
    case kRobustBiweightLocation:
    case kRobustBiweightScale:
      return inf ? nan_of(0.0) : biweight(s, n, v, ra, ra.kind == kRobustBiweightLocation);
    default:
      return clipped(v, s, w, n, ra, ra.kind);
  }
}

// MAXV > 0: thread-local arrays; MAXV == 0: per-thread slices of `scratch`.
template <typename T, int MAXV, bool MERGE>
__global__ void __launch_bounds__(kRThreads)
    robust_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ GenericArgs a,
                  const long long* __restrict__ taps, const __grid_constant__ RobustArgs ra,
                  double* __restrict__ scratch) {
  const int rank = a.rank;
  const int V = a.r.count;
  const long long* flat = taps + (long long)V * rank;
  const T cval = (T)a.r.cval;
  double local_v[MAXV > 0 ? MAXV : 1], local_s[MAXV > 0 ? MAXV : 1], local_w[MAXV > 0 ? MAXV : 1];
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double* v = MAXV > 0 ? local_v : scratch + tid * 3ll * V;
  double* s = MAXV > 0 ? local_s : v + V;
  double* w = MAXV > 0 ? local_w : s + V;
  for (long long o = tid; o < a.n_out; o += (long long)gridDim.x * blockDim.x) {
    long long coord[kMaxGenericRank];
    long long rem = o;
    bool interior = true;
    for (int d = 0; d < rank; ++d) {
      coord[d] = rem / a.stride[d];
      rem -= coord[d] * a.stride[d];
      interior = interior && coord[d] + a.low[d] >= 0 && coord[d] + a.high[d] < a.shape[d];
    }
    auto fetch = [&](int i) -> double {
      if (interior) return widen(__ldg(in + o + flat[i]));
      const long long* tap = taps + (long long)i * rank;
      long long src = 0;
      for (int d = 0; d < rank; ++d) {
        long long m;
        if (!map_index(coord[d] + tap[d], a.shape[d], a.mode[d], &m)) return widen(cval);
        src += m * a.stride[d];
      }
      return widen(__ldg(in + src));
    };
    const double result = robust_window<MAXV, MERGE>(fetch, V, a.r, ra, v, s, w);
    T value;
    if constexpr (sizeof(T) == 4)
      value = nan64(result) ? nan_of(0.0f) : __double2float_rn(result);
    else
      value = nan64(result) ? nan_of(0.0) : result;
    out[o] = value;
  }
}

template <typename T, int MAXV, bool MERGE = false>
cudaError_t launch_robust_v(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const long long blocks = MAXV > 0 ? std::max(1ll, std::min((p.n_out + kRThreads - 1) / kRThreads,
                                                             (long long)std::max(1, p.sm_count) * 16))
                                    : p.robust_threads / kRThreads;
  robust_kernel<T, MAXV, MERGE><<<(unsigned)blocks, kRThreads, 0, s>>>(in, out, p.generic, p.d_gen_taps, p.robust,
                                                                        reinterpret_cast<double*>(p.d_scratch));
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_robust_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const int V = p.r.count;
  if (V <= 32) return launch_robust_v<T, 32>(p, in, out, s);
  // Windows of 33-256 samples: runs sorted in registers and merged, except
  // for the clipping kinds, whose iterations run faster in the kernel
  // without it (fewer registers).
  const bool clip = p.robust.kind >= kRobustSigmaMean;
  if (V <= 64) return clip ? launch_robust_v<T, 64, false>(p, in, out, s) : launch_robust_v<T, 64, true>(p, in, out, s);
  if (V <= 128)
    return clip ? launch_robust_v<T, 128, false>(p, in, out, s) : launch_robust_v<T, 128, true>(p, in, out, s);
  if (V <= 256)
    return clip ? launch_robust_v<T, 256, false>(p, in, out, s) : launch_robust_v<T, 256, true>(p, in, out, s);
  return launch_robust_v<T, 0>(p, in, out, s);
}

}  // namespace
}  // namespace ndf

// CPU restatement of ndfiltrs' windowed-statistics hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA library is
// checked against, and the timed CPU baseline of bench.py. Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it. The product
// (ndfiltrs_gb300 and its C-ABI library) never links, loads or calls it.
//
// Every function restates the reference algorithm (ysBach/ndfiltrs v0.2.0,
// Rust crate) and cites the file:line it follows. The order statistics are
// bit-exact restatements; mean/var/std follow the reference's float64
// compensated arithmetic operation for operation (no FMA contraction: build
// with -ffp-contract=off).
//
// Parity pin: the reference's own known-answer tests (boundary literals, tap
// order, reducers midpoint contract, mean/dispersion/percentile literals,
// zero-one principle) are restated in tests/test_oracle_pins.py, and golden
// vectors produced by the reference's literal Python oracles
// (tests/_reference.py, tests/_statistics_reference.py,
// tests/_mean_reference.py) plus SciPy/NumPy are committed under
// tests/golden/ together with the script that made them.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <type_traits>
#include <tuple>
#include <utility>
#include <vector>

namespace {

// Error codes mirror src/error.rs:6-18 (same numbering as the C-ABI).
constexpr int kOk = 0;
constexpr int kEmptyAxis = 1;
constexpr int kInvalid = 2;
constexpr int kLength = 3;
constexpr int kMemory = 4;
constexpr int kOverflow = 5;

thread_local std::string g_message;

int fail(int code, const char* message) {
  g_message = message;
  return code;
}

enum Mode { kReflect = 0, kConstant = 1, kNearest = 2, kMirror = 3, kWrap = 4 };

enum Kind {
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
};

// InvalidPolicy, src/reduction.rs:6-18.
struct Policy {
  bool omit = false;
  bool ignore_inf = false;
  uint64_t min_count = 1;
};

constexpr double kNaN64 = std::numeric_limits<double>::quiet_NaN();

inline uint64_t bits64(double v) {
  uint64_t b;
  std::memcpy(&b, &v, 8);
  return b;
}
inline double from_bits64(uint64_t b) {
  double v;
  std::memcpy(&v, &b, 8);
  return v;
}

// Total-order key of a float64 (the f64 arm of NetworkFloat::sort_key,
// src/median_network.rs:21-31, expressed as an unsigned key). Float32 values
// are handled as their exact float64 conversions, which keeps their order.
inline uint64_t total_key(double v) {
  uint64_t b = bits64(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

inline bool retained(double v, const Policy& p) {
  if (std::isnan(v)) return false;
  if (p.omit && p.ignore_inf && !std::isfinite(v)) return false;
  return true;
}

int64_t rem_euclid(int64_t a, int64_t b) {
  int64_t r = a % b;
  return r < 0 ? r + b : r;
}

// map_index, src/boundary.rs:29-71. Returns 1 with *out set, 0 for a
// constant-mode position outside the array, -kEmptyAxis on an empty axis.
int map_index(int64_t index, int64_t length, int mode, int64_t* out) {
  if (length == 0) return -kEmptyAxis;
  if (index >= 0 && index < length) {
    *out = index;
    return 1;
  }
  switch (mode) {
    case kConstant:
      return 0;
    case kNearest:
      *out = index < 0 ? 0 : length - 1;
      return 1;
    case kWrap:
      *out = rem_euclid(index, length);
      return 1;
    case kReflect: {
      if (length == 1) {
        *out = 0;
        return 1;
      }
      int64_t period = 2 * length;
      int64_t reduced = rem_euclid(index, period);
      *out = reduced < length ? reduced : period - 1 - reduced;
      return 1;
    }
    case kMirror: {
      if (length == 1) {
        *out = 0;
        return 1;
      }
      int64_t period = 2 * (length - 1);
      int64_t reduced = rem_euclid(index, period);
      *out = reduced < length ? reduced : period - reduced;
      return 1;
    }
    default:
      return -kInvalid;
  }
}

// Window, src/window.rs:11-137: taps in C order over the footprint, offset
// k - (size/2 + origin) per axis, flat offsets, per-axis low/high.
struct Window {
  int rank = 0;
  std::vector<int64_t> shape, strides, low, high;
  std::vector<int> modes;
  std::vector<int64_t> taps;  // count * rank, tap-major
  std::vector<int64_t> flat;  // count
  size_t count = 0;
  size_t out_len = 0;
};

int window_new(int rank, const uint64_t* shape, const uint64_t* size, const uint8_t* footprint,
               const int64_t* origin, const int32_t* modes, Window* w, bool build_taps = true) {
  if (rank <= 0) return fail(kInvalid, "filtering requires at least one dimension");
  for (int a = 0; a < rank; ++a)
    if (size[a] == 0) return fail(kInvalid, "window sizes must be positive");
  for (int a = 0; a < rank; ++a)
    if (modes[a] < 0 || modes[a] > 4) return fail(kInvalid, "unsupported boundary mode");
  uint64_t volume = 1;
  for (int a = 0; a < rank; ++a) {
    if (size[a] > 0 && volume > UINT64_MAX / size[a])
      return fail(kOverflow, "shape or index arithmetic overflowed");
    volume *= size[a];
  }
  std::vector<int64_t> anchors(rank);
  for (int a = 0; a < rank; ++a) {
    int64_t length = (int64_t)size[a];
    if (origin[a] < -(length / 2) || origin[a] > (length - 1) / 2)
      return fail(kInvalid, "origin must satisfy -(size // 2) <= origin <= (size - 1) // 2");
    anchors[a] = length / 2 + origin[a];
  }
  w->rank = rank;
  w->shape.assign(shape, shape + rank);
  w->modes.assign(modes, modes + rank);
  w->strides.assign(rank, 1);
  uint64_t out_len = 1;
  for (int a = 0; a < rank; ++a) {
    if (shape[a] > 0 && out_len > UINT64_MAX / shape[a])
      return fail(kOverflow, "shape or index arithmetic overflowed");
    out_len *= shape[a];
  }
  w->out_len = out_len;
  for (int a = rank - 2; a >= 0; --a) w->strides[a] = w->strides[a + 1] * (int64_t)shape[a + 1];
  size_t count = 0;
  if (footprint) {
    for (uint64_t e = 0; e < volume; ++e) count += footprint[e] != 0;
  } else {
    count = volume;
  }
  if (count == 0) return fail(kInvalid, "footprint must select at least one element");
  w->count = count;
  if (!build_taps) return kOk;
  w->taps.clear();
  w->flat.clear();
  w->taps.reserve(count * rank);
  w->flat.reserve(count);
  w->low.assign(rank, INT64_MAX);
  w->high.assign(rank, INT64_MIN);
  std::vector<uint64_t> index(rank, 0);
  for (uint64_t e = 0; e < volume; ++e) {
    if (!footprint || footprint[e]) {
      int64_t flat = 0;
      for (int a = 0; a < rank; ++a) {
        int64_t offset = (int64_t)index[a] - anchors[a];
        flat += offset * w->strides[a];
        w->low[a] = std::min(w->low[a], offset);
        w->high[a] = std::max(w->high[a], offset);
        w->taps.push_back(offset);
      }
      w->flat.push_back(flat);
    }
    for (int a = rank - 1; a >= 0; --a) {
      if (++index[a] < size[a]) break;
      index[a] = 0;
    }
  }
  return kOk;
}

// Window::prepare, src/window.rs:254-269.
inline bool prepare(const Window& w, size_t center, int64_t* index) {
  size_t remainder = center;
  bool interior = true;
  for (int a = 0; a < w.rank; ++a) {
    index[a] = (int64_t)(remainder / (size_t)w.strides[a]);
    remainder %= (size_t)w.strides[a];
    interior = interior && index[a] + w.low[a] >= 0 && index[a] + w.high[a] < w.shape[a];
  }
  return interior;
}

// Window::visit / gather / visit_mapped, src/window.rs:211-294. Samples are
// delivered in tap order as float64 (exact for float32 input).
template <class T, class F>
inline void visit(const Window& w, const T* input, size_t center, double cval, int64_t* index,
                  F&& consume) {
  if (prepare(w, center, index)) {
    const T* base = input + center;
    for (size_t t = 0; t < w.count; ++t) consume((double)base[w.flat[t]]);
    return;
  }
  for (size_t t = 0; t < w.count; ++t) {
    const int64_t* tap = &w.taps[t * w.rank];
    int64_t source = 0;
    bool outside = false;
    for (int a = 0; a < w.rank; ++a) {
      int64_t mapped = 0;
      int r = map_index(index[a] + tap[a], w.shape[a], w.modes[a], &mapped);
      if (r == 0) {
        outside = true;
        break;
      }
      source += mapped * w.strides[a];
    }
    consume(outside ? cval : (double)input[source]);
  }
}

// ---------------------------------------------------------------------------
// Arithmetic contracts.

// Midpoint contract of reducers 0.4.0 median_valid_in_place for two middle
// values (lower <= upper in total order), pinned by docs/semantics.md:74-88,
// tests/_reference.py:36-47 and src/reduction.rs:214-249.
double midpoint(double lower, double upper) {
  if (std::signbit(lower) == std::signbit(upper) && lower == upper) return lower;
  if (lower == 0.0 && upper == 0.0) return 0.0;
  if (std::isinf(lower) || std::isinf(upper)) {
    if (std::isinf(lower) && std::isinf(upper)) return kNaN64;
    return std::isinf(lower) ? lower : upper;
  }
  if (std::signbit(lower) == std::signbit(upper)) return lower + (upper - lower) / 2.0;
  return (lower + upper) / 2.0;
}

// Sum (Neumaier), src/mean.rs:7-26.
struct Sum {
  double value = 0.0, correction = 0.0;
  void add(double x) {
    double next = value + x;
    if (std::fabs(value) >= std::fabs(x))
      correction += (value - next) + x;
    else
      correction += (x - next) + value;
    value = next;
  }
  double total() const { return value + correction; }
};

// Mean, src/mean.rs:28-84.
struct Mean {
  Sum sum;
  uint64_t count = 0;
  bool nan = false, positive_inf = false, negative_inf = false;
  void add(double value, const Policy& policy) {
    if (std::isnan(value)) {
      nan = nan || !policy.omit;
      return;
    }
    if (policy.omit && policy.ignore_inf && !std::isfinite(value)) return;
    count += 1;
    if (std::isinf(value)) {
      positive_inf = positive_inf || value > 0;
      negative_inf = negative_inf || value < 0;
    } else {
      sum.add(value);
    }
  }
  // Returns false only when finite summation overflowed (src/mean.rs:66-84).
  bool finish(const Policy& policy, double* out) const {
    if (nan || count == 0 || (policy.omit && count < policy.min_count)) {
      *out = kNaN64;
      return true;
    }
    if (positive_inf || negative_inf) {
      if (positive_inf && negative_inf)
        *out = kNaN64;
      else
        *out = positive_inf ? INFINITY : -INFINITY;
      return true;
    }
    double total = sum.total();
    if (!std::isfinite(total)) return false;
    *out = total / (double)count;
    return true;
  }
};

inline double clamp_f64(double x, double lo, double hi) {
  if (x < lo) return lo;
  if (x > hi) return hi;
  return x;
}

// mean_valid, src/mean.rs:87-113 (retained, non-NaN values).
double mean_valid(const double* values, size_t n) {
  Mean mean;
  Policy propagate;
  for (size_t i = 0; i < n; ++i) mean.add(values[i], propagate);
  double result;
  if (mean.finish(propagate, &result)) return result;
  double count = (double)n;
  uint64_t m = (uint64_t)(n - 1);
  int lz = m == 0 ? 64 : __builtin_clzll(m);
  int exponent = 64 - lz + 1;
  double scale = std::ldexp(1.0, exponent);
  Sum scaled;
  double lower = INFINITY, upper = -INFINITY;
  for (size_t i = 0; i < n; ++i) {
    double v = values[i];
    lower = std::fmin(lower, v);
    upper = std::fmax(upper, v);
    scaled.add(v / scale);
  }
  return clamp_f64((scaled.value + scaled.correction) / (count / scale), lower, upper);
}

// dispersion_valid, src/dispersion.rs:5-61.
double dispersion_valid(const double* values, size_t n, uint64_t ddof, bool want_std) {
  if (n <= ddof) return kNaN64;
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(values[i])) return kNaN64;
  double reference = values[0];
  bool halve = false;
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(values[i] - reference)) {
      halve = true;
      break;
    }
  auto delta = [&](double v) { return halve ? v / 2.0 - reference / 2.0 : v - reference; };
  double scale = 0.0;
  for (size_t i = 0; i < n; ++i) scale = std::fmax(scale, std::fabs(delta(values[i])));
  if (scale == 0.0) return 0.0;
  Sum sum;
  for (size_t i = 0; i < n; ++i) sum.add(delta(values[i]) / scale);
  double center = sum.total() / (double)n;
  Sum squares;
  for (size_t i = 0; i < n; ++i) {
    double residual = delta(values[i]) / scale - center;
    squares.add(residual * residual);
  }
  double normalized = squares.total() / (double)(n - ddof);
  if (want_std) {
    double result = scale * std::sqrt(normalized);
    return halve ? result * 2.0 : result;
  }
  double result = scale * (scale * normalized);
  return halve ? result * 4.0 : result;
}

// split / scale_binary / scaled_dot / WeightedSum / finite_weighted,
// src/convolution.rs:203-361 (only the two-term, normalize=false use from
// the percentile interpolation is on this path).
std::pair<double, int> split(double value) {
  uint64_t b = bits64(value);
  int exponent = (int)((b >> 52) & 0x7ff);
  uint64_t fraction = b & ((1ull << 52) - 1);
  if (exponent == 0) {
    int leading = 63 - __builtin_clzll(fraction);
    double mantissa = (double)fraction / (double)(1ull << leading);
    return {std::copysign(mantissa, value), leading - 1074};
  }
  return {from_bits64((b & ((1ull << 63) | ((1ull << 52) - 1))) | (1023ull << 52)),
          exponent - 1023};
}

double scale_binary(double value, int exponent) {
  if (value == 0.0) return value;
  auto [mantissa, value_exponent] = split(value);
  int target = value_exponent + exponent;
  if (target > 1023) return std::copysign(INFINITY, value);
  if (target < -1075) return std::copysign(0.0, value);
  if (target >= -1022) return mantissa * from_bits64((uint64_t)(target + 1023) << 52);
  double remaining = from_bits64((uint64_t)(target + 1022 + 1023) << 52);
  return (mantissa * 2.2250738585072014e-308) * remaining;
}

int count_bits(size_t len) {
  uint64_t m = (uint64_t)(len - 1);
  return m == 0 ? 0 : 64 - __builtin_clzll(m);
}

std::pair<double, int> scaled_dot(const double (*pairs)[2], size_t n) {
  bool any = false;
  int maximum = INT32_MIN;
  for (size_t i = 0; i < n; ++i) {
    if (pairs[i][0] == 0.0) continue;
    int e = split(pairs[i][0]).second + split(pairs[i][1]).second;
    maximum = any ? std::max(maximum, e) : e;
    any = true;
  }
  if (!any) return {0.0, 0};
  int exponent = maximum + count_bits(n) + 2;
  Sum sum;
  for (size_t i = 0; i < n; ++i) {
    if (pairs[i][0] == 0.0) continue;
    auto [vm, ve] = split(pairs[i][0]);
    auto [wm, we] = split(pairs[i][1]);
    sum.add(scale_binary(vm * wm, ve + we - exponent));
  }
  return {sum.total(), exponent};
}

double finite_weighted2(double v0, double w0, double v1, double w1) {
  const double pairs[2][2] = {{v0, w0}, {v1, w1}};
  // WeightedSum::add / finish with normalize = false.
  Sum sum;
  bool fallback = false;
  for (int i = 0; i < 2 && !fallback; ++i) {
    double value = pairs[i][0], weight = pairs[i][1];
    double product = value * weight;
    if (!std::isfinite(product) ||
        (value != 0.0 && std::fabs(product) < 2.2250738585072014e-308)) {
      fallback = true;
      break;
    }
    sum.add(product);
  }
  if (!fallback) {
    double total = sum.total();
    if (std::isfinite(total)) return total;
  }
  auto [total, exponent] = scaled_dot(pairs, 2);
  return scale_binary(total, exponent);
}

// interpolate, src/robust.rs:305-341.
double interpolate(double lower, double upper, double fraction) {
  if (fraction == 0.0 || bits64(lower) == bits64(upper)) return lower;
  if (fraction == 1.0) return upper;
  if (std::isinf(lower) || std::isinf(upper)) {
    if (lower == -INFINITY && upper == INFINITY) return kNaN64;
    return std::isinf(lower) ? lower : upper;
  }
  if (std::signbit(lower) != std::signbit(upper)) {
    if (!std::isfinite(upper - lower)) {
      double half_lower = lower / 2.0;
      double half_upper = upper / 2.0;
      return clamp_f64((half_lower + (half_upper - half_lower) * fraction) * 2.0, lower, upper);
    }
    return finite_weighted2(lower, 1.0 - fraction, upper, fraction);
  }
  double difference = upper - lower;
  double result = fraction <= 0.5 ? lower + difference * fraction
                                  : upper - difference * (1.0 - fraction);
  return clamp_f64(result, lower, upper);
}

inline bool key_less(double a, double b) { return total_key(a) < total_key(b); }

// k-th smallest in total order (select_nth_unstable_by total_cmp).
double select_nth(std::vector<double>& v, size_t k) {
  std::nth_element(v.begin(), v.begin() + k, v.end(), key_less);
  return v[k];
}

// percentile, src/robust.rs:343-352.
double percentile(std::vector<double>& values, double q) {
  std::sort(values.begin(), values.end(), key_less);
  size_t n = values.size();
  if (q == 100.0) return values[n - 1];
  double rank = (q / 100.0) * (double)(n - 1);
  size_t lower = (size_t)std::floor(rank);
  size_t upper = std::min(lower + 1, n - 1);
  return interpolate(values[lower], values[upper], rank - (double)lower);
}

// Median of retained values: exact middle for odd counts, midpoint of the
// two middle values (total order) for even counts.
double median_valid(std::vector<double>& values) {
  size_t n = values.size();
  if (n % 2 == 1) return select_nth(values, n / 2);
  double upper = select_nth(values, n / 2);
  double lower = *std::max_element(values.begin(), values.begin() + n / 2, key_less);
  return midpoint(lower, upper);
}

struct Reduction {
  int kind = kMedian;
  Policy policy;
  uint64_t parameter = 0;  // rank or ddof
  double q = 50.0;         // percentile
};

// Reduction::finish, src/reduction.rs:78-130 (and RobustReduction::finish,
// src/robust.rs:244-299, for the percentile kind). Returns float64; the
// caller casts once to the output dtype.
double finish(const Reduction& r, std::vector<double>& values) {
  if (!r.policy.omit) {
    for (double v : values)
      if (std::isnan(v)) return kNaN64;
  } else {
    size_t write = 0;
    for (size_t read = 0; read < values.size(); ++read)
      if (retained(values[read], r.policy)) values[write++] = values[read];
    values.resize(write);
    if (write < r.policy.min_count) return kNaN64;
  }
  switch (r.kind) {
    case kMedian:
    case kMedianNetwork:
    case kMedianHistogram:
      return values.empty() ? kNaN64 : median_valid(values);
    case kMean:
    case kMeanRolling:
      return mean_valid(values.data(), values.size());
    case kMin:
      return values.empty() ? kNaN64 : *std::min_element(values.begin(), values.end(), key_less);
    case kMax:
      return values.empty() ? kNaN64 : *std::max_element(values.begin(), values.end(), key_less);
    case kVar:
      return dispersion_valid(values.data(), values.size(), r.parameter, false);
    case kStd:
      return dispersion_valid(values.data(), values.size(), r.parameter, true);
    case kRank:
    case kRankHistogram:
      if (r.parameter >= values.size()) return kNaN64;
      return select_nth(values, (size_t)r.parameter);
    case kPercentile:
      if (values.empty()) return kNaN64;
      return percentile(values, r.q);
  }
  return kNaN64;
}

template <class T>
inline T cast_out(double v) {
  if (std::isnan(v)) return std::numeric_limits<T>::quiet_NaN();
  return (T)v;
}

// filter_offsets, src/filter_nd.rs:125-172 (the mean streams through Mean;
// everything else gathers the window and calls finish).
template <class T>
void filter_offsets(const Window& w, const T* input, double cval, const Reduction& r,
                    size_t start, size_t end, T* output) {
  std::vector<int64_t> index(w.rank);
  std::vector<double> scratch;
  scratch.reserve(w.count);
  for (size_t center = start; center < end; ++center) {
    if (r.kind == kMean) {
      Mean mean;
      visit(w, input, center, cval, index.data(), [&](double v) { mean.add(v, r.policy); });
      double result;
      if (mean.finish(r.policy, &result)) {
        output[center - start] = cast_out<T>(result);
        continue;
      }
    }
    scratch.clear();
    visit(w, input, center, cval, index.data(), [&](double v) { scratch.push_back(v); });
    output[center - start] = cast_out<T>(finish(r, scratch));
  }
}

// ---------------------------------------------------------------------------
// Exact rectangular mean (kind mean_rolling, method="boxcar"):
// src/boxcar.rs:142-399 with src/exact_sum.rs:215-349. Per window, the finite
// samples are summed exactly as a two's-complement fixed-point integer in
// units of 2^-1074 (35 words cover every finite binary64 value times any
// count below 2^64), and the mean is the exact quotient by the finite count,
// rounded once to nearest (ties to even) directly to the output type.
// Counts decide NaN / +-inf first, as Counts::value (src/boxcar.rs:59-77).

using u128 = unsigned __int128;

struct ExactAcc {
  static constexpr int kWords = 35;
  uint64_t w[kWords] = {};

  void add(double v) {
    uint64_t bits;
    std::memcpy(&bits, &v, 8);
    const int e = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & ((1ull << 52) - 1);
    const uint64_t m = e ? (frac | (1ull << 52)) : frac;
    if (m == 0) return;
    const int shift = e ? e - 1 : 0;  // v = m * 2^(shift - 1074)
    const u128 payload = (u128)m << (shift % 64);
    int i = shift / 64;
    const uint64_t lo = (uint64_t)payload, hi = (uint64_t)(payload >> 64);
    if ((bits >> 63) == 0) {
      u128 carry = 0;
      for (uint64_t part : {lo, hi}) {
        const u128 t = (u128)w[i] + part + carry;
        w[i++] = (uint64_t)t;
        carry = t >> 64;
      }
      while (carry && i < kWords) {
        const u128 t = (u128)w[i] + carry;
        w[i++] = (uint64_t)t;
        carry = t >> 64;
      }
    } else {
      uint64_t borrow = 0;
      for (uint64_t part : {lo, hi}) {
        const uint64_t a = w[i];
        const uint64_t d = a - part - borrow;
        borrow = (a < part || (a - part) < borrow) ? 1 : 0;
        w[i++] = d;
      }
      while (borrow && i < kWords) {
        const uint64_t a = w[i];
        w[i++] = a - 1;
        borrow = a == 0 ? 1 : 0;
      }
    }
  }
};

inline int bitlen128(u128 x) {
  const uint64_t hi = (uint64_t)(x >> 64), lo = (uint64_t)x;
  if (hi) return 128 - __builtin_clzll(hi);
  return lo ? 64 - __builtin_clzll(lo) : 0;
}

// RN_T(S * 2^(64 low - 1074) / n) for the exact sum S, held as `nw` words of
// two's complement, and a positive count n.
template <class T>
T exact_mean(const uint64_t* words, int nw, int low, uint64_t n) {
  constexpr int p = std::numeric_limits<T>::digits;             // 24 or 53
  constexpr int unit = sizeof(T) == 4 ? 1074 - 149 : 0;           // T's subnormal unit
  uint64_t m[ExactAcc::kWords];
  const bool negative = (words[nw - 1] >> 63) != 0;
  uint64_t carry = 1;
  for (int i = 0; i < nw; ++i) {
    m[i] = negative ? ~words[i] + carry : words[i];
    if (negative) carry = (carry && m[i] == 0) ? 1 : 0;
  }
  int top = nw - 1;
  while (top >= 0 && m[top] == 0) --top;
  using U = std::conditional_t<sizeof(T) == 4, uint32_t, uint64_t>;
  const U sign = negative ? (U)1 << (sizeof(T) * 8 - 1) : 0;
  T out;
  if (top < 0) {
    const U zero = 0;  // exact cancellation gives +0
    std::memcpy(&out, &zero, sizeof(T));
    return out;
  }
  // Bit positions below are absolute (units of 2^-1074).
  const long B = (long)(top + low) * 64 + (64 - __builtin_clzll(m[top]));
  const int t = 64 - __builtin_clzll(n);
  const long s = std::max<long>(B - t - p - 1, unit);
  auto word = [&](long i) -> uint64_t { return i >= low && i < low + nw ? m[i - low] : 0; };
  const long wi = s / 64;
  const int off = (int)(s % 64);
  u128 high = (u128)(word(wi) >> off);
  if (off) {
    high |= (u128)word(wi + 1) << (64 - off);
    high |= (u128)word(wi + 2) << (128 - off);
  } else {
    high |= (u128)word(wi + 1) << 64;
  }
  bool sticky = off && (word(wi) & ((1ull << off) - 1)) != 0;
  for (long i = low; i < wi && !sticky; ++i) sticky = word(i) != 0;
  const u128 q = high / n, r = high % n;
  const int k = std::max(bitlen128(q) - p, 0);
  u128 mant;
  bool up;
  if (k > 0) {
    mant = q >> k;
    const bool guard = ((q >> (k - 1)) & 1) != 0;
    const bool rest = (q & (((u128)1 << (k - 1)) - 1)) != 0 || r != 0 || sticky;
    up = guard && (rest || (mant & 1));
  } else {
    // Only at the subnormal grid (s == unit), where no sample has bits below.
    mant = q;
    const u128 twice = 2 * r;
    up = twice > n || (twice == n && (sticky || (mant & 1)));
  }
  const U bits = (U)(((u128)(s - unit + k) << (p - 1)) + mant + (up ? 1 : 0)) | sign;
  std::memcpy(&out, &bits, sizeof(T));
  return out;
}

template <class T>
T exact_mean(const ExactAcc& acc, uint64_t n) {
  return exact_mean<T>(acc.w, ExactAcc::kWords, 0, n);
}

struct BoxcarCounts {
  uint64_t finite = 0, nan = 0, positive = 0, negative = 0;
};

// One window of the exact boxcar mean (Counts::sample / Counts::value).
template <class T>
T boxcar_window(const Window& w, const T* input, size_t center, double cval, const Policy& pol,
                int64_t* index) {
  ExactAcc acc;
  BoxcarCounts c;
  visit(w, input, center, cval, index, [&](double v) {
    if (std::isnan(v)) {
      if (!pol.omit) ++c.nan;
    } else if (std::isfinite(v)) {
      ++c.finite;
      acc.add(v);
    } else if (!(pol.omit && pol.ignore_inf)) {
      if (v > 0) ++c.positive; else ++c.negative;
    }
  });
  const uint64_t kept = c.finite + c.positive + c.negative;
  if (c.nan || kept == 0 || (pol.omit && kept < pol.min_count) || (c.positive && c.negative))
    return std::numeric_limits<T>::quiet_NaN();
  if (c.positive) return std::numeric_limits<T>::infinity();
  if (c.negative) return -std::numeric_limits<T>::infinity();
  return exact_mean<T>(acc, c.finite);
}

// ---------------------------------------------------------------------------
// Sorting network, src/median_network.rs:9-209.

template <class T>
struct KeyOf;
template <>
struct KeyOf<float> {
  using K = int32_t;
  static K key(float v) {
    int32_t b;
    std::memcpy(&b, &v, 4);
    return b ^ (int32_t)((uint32_t)(b >> 31) >> 1);
  }
  static float value(K k) {
    int32_t b = k ^ (int32_t)((uint32_t)(k >> 31) >> 1);
    float v;
    std::memcpy(&v, &b, 4);
    return v;
  }
};
template <>
struct KeyOf<double> {
  using K = int64_t;
  static K key(double v) {
    int64_t b;
    std::memcpy(&b, &v, 8);
    return b ^ (int64_t)((uint64_t)(b >> 63) >> 1);
  }
  static double value(K k) {
    int64_t b = k ^ (int64_t)((uint64_t)(k >> 63) >> 1);
    double v;
    std::memcpy(&v, &b, 8);
    return v;
  }
};

struct Comparator {
  uint32_t lower, upper;
  bool keep_lower, keep_upper;
};

void net_merge(size_t start, size_t length, size_t stride, size_t count,
               std::vector<Comparator>& out) {
  if (start >= count) return;
  size_t step = stride * 2;
  if (step < length) {
    net_merge(start, length, step, count, out);
    net_merge(start + stride, length, step, count, out);
    for (size_t lower = start + stride; lower + stride < start + length; lower += step)
      if (lower + stride < count) out.push_back({(uint32_t)lower, (uint32_t)(lower + stride), true, true});
  } else if (start + stride < count) {
    out.push_back({(uint32_t)start, (uint32_t)(start + stride), true, true});
  }
}

void net_sort(size_t start, size_t length, size_t count, std::vector<Comparator>& out) {
  if (length > 1 && start < count) {
    size_t half = length / 2;
    net_sort(start, half, count, out);
    net_sort(start + half, half, count, out);
    net_merge(start, length, 1, count, out);
  }
}

// Network::new, src/median_network.rs:116-155.
std::vector<Comparator> network_new(size_t count, const Policy& policy) {
  size_t wires = 1;
  while (wires < count) wires <<= 1;
  std::vector<Comparator> comparisons;
  net_sort(0, wires, count, comparisons);
  std::vector<bool> live(count, false);
  if (!policy.omit) {
    live[count / 2] = true;
    live[(count - 1) / 2] = true;
  } else {
    std::fill(live.begin(), live.end(), true);
  }
  std::vector<Comparator> kept;
  for (auto it = comparisons.rbegin(); it != comparisons.rend(); ++it) {
    Comparator c = *it;
    if (!live[c.lower] && !live[c.upper]) continue;
    c.keep_lower = live[c.lower];
    c.keep_upper = live[c.upper];
    live[c.lower] = true;
    live[c.upper] = true;
    kept.push_back(c);
  }
  std::reverse(kept.begin(), kept.end());
  return kept;
}

// Window::row_run, src/window.rs:164-191.
bool row_run(const Window& w, size_t center, size_t limit, int64_t* index, size_t* width) {
  bool interior = prepare(w, center, index);
  int last = w.rank - 1;
  size_t row_left = (size_t)(w.shape[last] - index[last]);
  if (!interior) {
    bool other_inside = true;
    for (int a = 0; a < last; ++a)
      other_inside = other_inside && index[a] + w.low[a] >= 0 && index[a] + w.high[a] < w.shape[a];
    int64_t left_edge = index[last] + w.low[last];
    size_t wd = (other_inside && left_edge < 0) ? std::min(row_left, (size_t)(-left_edge)) : row_left;
    *width = std::min(limit, wd);
    return false;
  }
  size_t end = (size_t)(w.shape[last] - std::max<int64_t>(w.high[last], 0));
  *width = std::min(limit, end - (size_t)index[last]);
  return true;
}

// filter_range with the network, src/filter_nd.rs:62-123, encode_plane
// src/median_network.rs:40-63 and Network::apply :157-209.
template <class T>
void filter_range_network(const Window& w, const T* input, double cval, const Reduction& r,
                          const std::vector<Comparator>& net, size_t start, size_t end,
                          T* output) {
  using KO = KeyOf<T>;
  using K = typename KO::K;
  const K nan_key = KO::key(std::numeric_limits<T>::quiet_NaN());
  std::vector<int64_t> index(w.rank);
  std::vector<K> keys;
  std::vector<uint32_t> valid;
  size_t offset = start;
  const size_t count = w.count;
  while (offset < end) {
    size_t width;
    bool interior = row_run(w, offset, end - offset, index.data(), &width);
    if (!interior) {
      filter_offsets(w, input, cval, r, offset, offset + width, output + (offset - start));
      offset += width;
      continue;
    }
    keys.assign(count * width, nan_key);
    valid.assign(width, 0);
    for (size_t tap = 0; tap < count; ++tap) {
      const T* plane = input + offset + w.flat[tap];
      K* kp = keys.data() + tap * width;
      for (size_t c = 0; c < width; ++c) {
        T v = plane[c];
        bool drop = std::isnan(v) || (r.policy.omit && r.policy.ignore_inf && !std::isfinite(v));
        kp[c] = drop ? nan_key : KO::key(v);
        valid[c] += drop ? 0u : 1u;
      }
    }
    for (const Comparator& cmp : net) {
      K* lo = keys.data() + (size_t)cmp.lower * width;
      K* hi = keys.data() + (size_t)cmp.upper * width;
      if (cmp.keep_lower && cmp.keep_upper) {
        for (size_t c = 0; c < width; ++c) {
          K a = lo[c], b = hi[c];
          lo[c] = a < b ? a : b;
          hi[c] = a < b ? b : a;
        }
      } else if (cmp.keep_lower) {
        for (size_t c = 0; c < width; ++c) lo[c] = lo[c] < hi[c] ? lo[c] : hi[c];
      } else {
        for (size_t c = 0; c < width; ++c) hi[c] = lo[c] < hi[c] ? hi[c] : lo[c];
      }
    }
    T* out = output + (offset - start);
    for (size_t c = 0; c < width; ++c) {
      size_t v = valid[c];
      bool missing = !r.policy.omit ? v != count : v < r.policy.min_count;
      if (missing || v == 0) {
        out[c] = std::numeric_limits<T>::quiet_NaN();
      } else if (v % 2 == 1) {
        out[c] = KO::value(keys[(v / 2) * width + c]);
      } else {
        double lower = (double)KO::value(keys[(v / 2 - 1) * width + c]);
        double upper = (double)KO::value(keys[(v / 2) * width + c]);
        out[c] = cast_out<T>(midpoint(lower, upper));
      }
    }
    offset += width;
  }
}

// ---------------------------------------------------------------------------
// Block histogram, src/histogram.rs:37-631.

constexpr uint32_t kOmitted = UINT32_MAX;
constexpr uint32_t kPropagatedNaN = UINT32_MAX - 1;
constexpr int kGroupShift = 12;
constexpr uint64_t kMinBlock = 32;
constexpr int64_t kOutside = INT64_MIN;

std::vector<uint64_t> block_lengths(const std::vector<int64_t>& shape, const uint64_t* size) {
  std::vector<uint64_t> out(shape.size());
  for (size_t a = 0; a < shape.size(); ++a) {
    uint64_t length = (uint64_t)shape[a];
    uint64_t blocks = std::max<uint64_t>(length / std::max<uint64_t>(size[a], kMinBlock), 1);
    out[a] = std::max<uint64_t>((length + blocks - 1) / blocks, 1);
  }
  return out;
}

int validate_support(const std::vector<int64_t>& shape, const uint64_t* size) {
  auto block = block_lengths(shape, size);
  uint64_t support = 1;
  for (size_t a = 0; a < shape.size(); ++a) {
    uint64_t length = block[a] + size[a] - 1;
    if (length != 0 && support > UINT64_MAX / length)
      return fail(kOverflow, "shape or index arithmetic overflowed");
    support *= length;
  }
  if (support > kPropagatedNaN) return fail(kOverflow, "shape or index arithmetic overflowed");
  return kOk;
}

inline uint32_t select_in_word(uint64_t word, uint32_t k) {
  uint32_t position = 0;
  for (int width : {32, 16, 8, 4, 2, 1}) {
    uint32_t low = (uint32_t)__builtin_popcountll(word & ((1ull << width) - 1));
    if (k >= low) {
      k -= low;
      word >>= width;
      position += width;
    }
  }
  return position;
}

struct Histogram {
  std::vector<uint64_t> words;
  std::vector<uint32_t> groups;
  size_t count = 0, nan = 0;
  void add(uint32_t code) {
    if (code < kPropagatedNaN) {
      words[code >> 6] |= 1ull << (code & 63);
      groups[code >> kGroupShift] += 1;
      count += 1;
    } else if (code == kPropagatedNaN) {
      nan += 1;
    }
  }
  void remove(uint32_t code) {
    if (code < kPropagatedNaN) {
      words[code >> 6] &= ~(1ull << (code & 63));
      groups[code >> kGroupShift] -= 1;
      count -= 1;
    } else if (code == kPropagatedNaN) {
      nan -= 1;
    }
  }
  size_t select(size_t k) const {
    size_t group = 0;
    while (k >= groups[group]) {
      k -= groups[group];
      group += 1;
    }
    size_t index = group << (kGroupShift - 6);
    while (true) {
      size_t c = (size_t)__builtin_popcountll(words[index]);
      if (k < c) break;
      k -= c;
      index += 1;
    }
    return (index << 6) + select_in_word(words[index], (uint32_t)k);
  }
};

// for_each_in_box, src/histogram.rs:199-240.
template <class F>
void for_each_in_box(const std::vector<size_t>& low, const std::vector<size_t>& lengths,
                     const std::vector<size_t>& strides, F&& visit_fn) {
  int rank = (int)low.size();
  int inner = rank - 1;
  for (int a = rank - 1; a >= 0; --a)
    if (lengths[a] > 1) {
      inner = a;
      break;
    }
  std::vector<size_t> counter(rank, 0);
  size_t base = 0;
  for (int a = 0; a < rank; ++a) base += low[a] * strides[a];
  while (true) {
    size_t idx = base;
    for (size_t i = 0; i < lengths[inner]; ++i) {
      visit_fn(idx);
      idx += strides[inner];
    }
    int axis = rank;
    while (true) {
      if (axis == 0) return;
      axis -= 1;
      if (axis == inner) continue;
      counter[axis] += 1;
      base += strides[axis];
      if (counter[axis] < lengths[axis]) break;
      base -= strides[axis] * lengths[axis];
      counter[axis] = 0;
    }
  }
}

template <class T>
struct HistGeometry {
  const T* input;
  std::vector<int64_t> shape;
  std::vector<uint64_t> size;
  std::vector<int> modes;
  std::vector<int64_t> anchors, strides;
  std::vector<uint64_t> block;
  std::vector<int> order;
  double cval;
  Policy policy;
  bool median;
  uint64_t rank_k;
};

// Geometry::block, src/histogram.rs:302-486. Writes outputs in place.
template <class T>
void hist_block(const HistGeometry<T>& g, const std::vector<size_t>& start,
                const std::vector<size_t>& extent, T* output) {
  using KO = KeyOf<T>;
  using K = typename KO::K;
  int rank = (int)g.shape.size();
  std::vector<size_t> lengths(rank), sstr(rank, 1);
  for (int a = 0; a < rank; ++a) lengths[a] = extent[a] + g.size[a] - 1;
  for (int a = rank - 2; a >= 0; --a) sstr[a] = sstr[a + 1] * lengths[a + 1];
  size_t total = sstr[0] * lengths[0];
  std::vector<std::vector<int64_t>> maps(rank);
  for (int a = 0; a < rank; ++a) {
    int64_t first = (int64_t)start[a] - g.anchors[a];
    maps[a].resize(lengths[a]);
    for (size_t s = 0; s < lengths[a]; ++s) {
      int64_t m;
      int rr = map_index(first + (int64_t)s, g.shape[a], g.modes[a], &m);
      maps[a][s] = rr == 1 ? m * g.strides[a] : kOutside;
    }
  }
  std::vector<uint32_t> codes(total, kOmitted);
  std::vector<std::pair<K, uint32_t>> pairs;
  pairs.reserve(total);
  int last = rank - 1;
  std::vector<size_t> counter(rank, 0);
  size_t sidx = 0;
  while (true) {
    int64_t base = 0;
    bool outside = false;
    for (int a = 0; a < last; ++a) {
      int64_t off = maps[a][counter[a]];
      outside = outside || off == kOutside;
      base += off == kOutside ? 0 : off;
    }
    for (size_t s = 0; s < lengths[last]; ++s) {
      int64_t off = maps[last][s];
      T value = (outside || off == kOutside) ? (T)g.cval : g.input[base + off];
      bool keep = !std::isnan(value) &&
                  !(g.policy.omit && g.policy.ignore_inf && !std::isfinite(value));
      if (keep)
        pairs.push_back({KO::key(value), (uint32_t)sidx});
      else if (!g.policy.omit)
        codes[sidx] = kPropagatedNaN;
      sidx += 1;
    }
    int axis = last;
    bool done = false;
    while (true) {
      if (axis == 0) {
        done = true;
        break;
      }
      axis -= 1;
      if (++counter[axis] < lengths[axis]) break;
      counter[axis] = 0;
    }
    if (done) break;
  }
  std::sort(pairs.begin(), pairs.end());
  std::vector<T> values(pairs.size());
  for (size_t i = 0; i < pairs.size(); ++i) {
    codes[pairs[i].second] = (uint32_t)i;
    values[i] = KO::value(pairs[i].first);
  }
  size_t ranks = pairs.size();
  Histogram h;
  h.words.assign((ranks + 63) / 64, 0);
  h.groups.assign((ranks + (1u << kGroupShift) - 1) >> kGroupShift, 0);

  std::vector<size_t> position(rank, 0), low(rank, 0), box(g.size.begin(), g.size.end());
  std::vector<bool> direction(rank, true);
  for_each_in_box(position, box, sstr, [&](size_t i) { h.add(codes[i]); });
  while (true) {
    size_t offset = 0;
    for (int a = 0; a < rank; ++a) offset += (start[a] + position[a]) * (size_t)g.strides[a];
    // Histogram::finish, src/histogram.rs:145-190.
    T result;
    if ((!g.policy.omit && h.nan > 0) || (g.policy.omit && h.count < g.policy.min_count)) {
      result = std::numeric_limits<T>::quiet_NaN();
    } else if (g.median) {
      if (h.count % 2 == 1) {
        result = values[h.select(h.count / 2)];
      } else {
        double lo = (double)values[h.select(h.count / 2 - 1)];
        double hi = (double)values[h.select(h.count / 2)];
        result = cast_out<T>(midpoint(lo, hi));
      }
    } else {
      result = g.rank_k < h.count ? values[h.select((size_t)g.rank_k)]
                                  : std::numeric_limits<T>::quiet_NaN();
    }
    output[offset] = result;
    int moved = -1;
    for (int oi = rank - 1; oi >= 0; --oi) {
      int axis = g.order[oi];
      bool can_move = direction[axis] ? position[axis] + 1 < extent[axis] : position[axis] > 0;
      if (can_move) {
        moved = axis;
        break;
      }
      direction[axis] = !direction[axis];
    }
    if (moved < 0) break;
    int axis = moved;
    size_t removed, added;
    if (direction[axis]) {
      removed = position[axis];
      added = position[axis] + g.size[axis];
    } else {
      removed = position[axis] + g.size[axis] - 1;
      added = position[axis] - 1;
    }
    low = position;
    box[axis] = 1;
    low[axis] = removed;
    for_each_in_box(low, box, sstr, [&](size_t i) { h.remove(codes[i]); });
    low[axis] = added;
    for_each_in_box(low, box, sstr, [&](size_t i) { h.add(codes[i]); });
    box[axis] = g.size[axis];
    if (direction[axis])
      position[axis] += 1;
    else
      position[axis] -= 1;
  }
}

template <class Fn>
void run_parallel(size_t items, int threads, Fn&& fn) {
  if (threads <= 1 || items <= 1) {
    fn(0, items);
    return;
  }
  size_t chunk = (items + (size_t)threads - 1) / (size_t)threads;
  std::vector<std::thread> pool;
  for (size_t s = 0; s < items; s += chunk) {
    size_t e = std::min(items, s + chunk);
    pool.emplace_back([&fn, s, e] { fn(s, e); });
  }
  for (auto& t : pool) t.join();
}

// order_statistic_into, src/histogram.rs:494-566 (blocks in parallel).
template <class T>
int histogram_filter(const Window& w, const uint64_t* size, const int64_t* origin,
                     const T* input, double cval, const Policy& policy, bool median,
                     uint64_t rank_k, int threads, T* output) {
  HistGeometry<T> g;
  g.input = input;
  g.shape = w.shape;
  g.size.assign(size, size + w.rank);
  g.modes = w.modes;
  g.strides = w.strides;
  g.cval = cval;
  g.policy = policy;
  g.median = median;
  g.rank_k = rank_k;
  int rank = w.rank;
  int rc = validate_support(g.shape, size);
  if (rc) return rc;
  for (int a = 0; a < rank; ++a) g.anchors.push_back((int64_t)size[a] / 2 + origin[a]);
  int fastest = 0;
  for (int a = 0; a < rank; ++a)
    if (size[a] >= size[fastest]) fastest = a;
  for (int a = 0; a < rank; ++a)
    if (a != fastest) g.order.push_back(a);
  g.order.push_back(fastest);
  g.block = block_lengths(g.shape, size);
  std::vector<size_t> blocks(rank);
  size_t nblocks = 1;
  for (int a = 0; a < rank; ++a) {
    blocks[a] = (size_t)((g.shape[a] + g.block[a] - 1) / g.block[a]);
    nblocks *= blocks[a];
  }
  std::atomic<size_t> next{0};
  auto worker = [&](size_t, size_t) {
    std::vector<size_t> start(rank), extent(rank);
    while (true) {
      size_t b = next.fetch_add(1);
      if (b >= nblocks) break;
      size_t rem = b;
      for (int a = rank - 1; a >= 0; --a) {
        start[a] = (rem % blocks[a]) * g.block[a];
        rem /= blocks[a];
        extent[a] = std::min<size_t>(g.block[a], (size_t)g.shape[a] - start[a]);
      }
      hist_block(g, start, extent, output);
    }
  };
  if (threads <= 1) {
    worker(0, 0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back([&] { worker(0, 0); });
    for (auto& t : pool) t.join();
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Exact window moments for the precision study (not a reference algorithm:
// the FP64 "exact-sum" oracle). Double-double accumulation of pivot-shifted
// sums with error-free transformations gives about 104 significant bits.

struct DD {
  double hi = 0.0, lo = 0.0;
};
inline DD two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
inline DD two_prod(double a, double b) {
  double p = a * b;
  double e = std::fma(a, b, -p);
  return {p, e};
}
inline DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  DD t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return two_sum(s.hi, s.lo);
}
inline DD dd_mul(DD a, DD b) {
  DD p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return two_sum(p.hi, p.lo);
}
inline DD dd_div_d(DD a, double b) {
  double q1 = a.hi / b;
  DD p = two_prod(q1, b);
  DD r = dd_add(a, DD{-p.hi, -p.lo});
  double q2 = r.hi / b;
  DD p2 = two_prod(q2, b);
  DD r2 = dd_add(r, DD{-p2.hi, -p2.lo});
  double q3 = r2.hi / b;
  DD q = two_sum(q1, q2);
  return dd_add(q, DD{q3, 0.0});
}

// Mean, variance and standard deviation of retained finite values with
// about 100-bit accuracy, rounded to float64 once.
double exact_moment(const std::vector<double>& values, int which, uint64_t ddof) {
  size_t n = values.size();
  if (which == kMean) {
    bool pinf = false, ninf = false;
    for (double v : values) {
      pinf = pinf || v == INFINITY;
      ninf = ninf || v == -INFINITY;
    }
    if (n == 0) return kNaN64;
    if (pinf && ninf) return kNaN64;
    if (pinf) return INFINITY;
    if (ninf) return -INFINITY;
  } else {
    if (n <= ddof) return kNaN64;
    for (double v : values)
      if (!std::isfinite(v)) return kNaN64;
  }
  if (n == 0) return kNaN64;
  double pivot = values[0];
  DD s1, s2;
  for (double v : values) {
    DD d = two_sum(v, -pivot);
    s1 = dd_add(s1, d);
    s2 = dd_add(s2, dd_mul(d, d));
  }
  if (which == kMean) {
    DD m = dd_add(dd_div_d(s1, (double)n), DD{pivot, 0.0});
    return m.hi + m.lo;
  }
  // SS = S2 - S1^2 / n
  DD s1sq = dd_mul(s1, s1);
  DD corr = dd_div_d(s1sq, (double)n);
  DD ss = dd_add(s2, DD{-corr.hi, -corr.lo});
  DD var = dd_div_d(ss, (double)(n - ddof));
  if (which == kVar) return var.hi + var.lo;
  if (var.hi <= 0.0) return 0.0;
  double root = std::sqrt(var.hi);
  // One Newton step in double-double: r + (var - r^2) / (2r).
  DD r2 = two_prod(root, root);
  DD diff = dd_add(var, DD{-r2.hi, -r2.lo});
  return root + (diff.hi + diff.lo) / (2.0 * root);
}

// ---------------------------------------------------------------------------
// Separable passes for rectangular windows. WindowFilter::new
// (src/plan.rs:267-289) routes minimum / maximum without a footprint to
// extrema_into and every rolling mean to mean_into; both sweep one axis at a
// time over lines of the array, padded through map_index.

// A pass's boundary rule is the same for every line: source coordinate of
// each padded position, or -1 for a constant-mode position outside.
int map_line(int64_t length, int64_t first, int64_t count, int mode, std::vector<int64_t>* out) {
  out->resize((size_t)count);
  for (int64_t p = 0; p < count; ++p) {
    int64_t m = 0;
    int r = map_index(first + p, length, mode, &m);
    if (r < 0) return fail(kInvalid, "zero-length axes cannot be padded");
    (*out)[(size_t)p] = r == 1 ? m : -1;
  }
  return kOk;
}

// Summary, src/extrema.rs:11-62: the extremum so far and whether a
// propagated NaN was seen; the empty summary holds NaN with nan == false.
template <class T>
struct Extremum {
  T value;
  bool nan;
};

template <class T>
inline Extremum<T> extremum_sample(T v, const Policy& p) {
  if (!p.omit) return {v, std::isnan(v)};
  if (retained(v, p)) return {v, false};
  return {std::numeric_limits<T>::quiet_NaN(), false};
}

template <class T>
inline Extremum<T> extremum_combine(Extremum<T> a, Extremum<T> b, bool maximum) {
  if (a.nan || b.nan) return {std::numeric_limits<T>::quiet_NaN(), true};
  if (std::isnan(a.value)) return b;
  if (std::isnan(b.value)) return a;
  const uint64_t ka = total_key(a.value), kb = total_key(b.value);
  return (maximum ? ka < kb : ka > kb) ? b : a;
}

// extrema_into, src/extrema.rs:124-437 (van Herk / Gil-Werman): along each
// axis, prefix and suffix combinations within blocks of the window length
// give every window as suffix[p] + prefix[p + w - 1]; retained counts follow
// the same blocks when min_count > 1.
template <class T>
int extrema_separable(const Window& w, const uint64_t* size, const int64_t* origin,
                      const T* input, double cval_d, const Policy& pol, bool maximum,
                      int threads, T* output) {
  const size_t n = w.out_len;
  const T cval = (T)cval_d;
  std::vector<Extremum<T>> prev(n), next(n);
  const bool counting = pol.omit && pol.min_count > 1;
  std::vector<uint64_t> prev_n, next_n;
  run_parallel(n, threads, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) prev[i] = extremum_sample(input[i], pol);
  });
  if (counting) {
    prev_n.resize(n);
    next_n.resize(n);
    for (size_t i = 0; i < n; ++i) prev_n[i] = retained(input[i], pol) ? 1 : 0;
  }
  uint64_t prior_volume = 1;
  for (int axis = 0; axis < w.rank; ++axis) {
    const int64_t length = w.shape[axis], stride = w.strides[axis], block = length * stride;
    const int64_t win = (int64_t)size[axis], anchor = win / 2 + origin[axis];
    const int64_t padded = length + win - 1;
    std::vector<int64_t> source;
    int rc = map_line(length, -anchor, padded, w.modes[axis], &source);
    if (rc) return rc;
    const Extremum<T> outside = extremum_sample(cval, pol);
    const uint64_t outside_n = retained(cval, pol) ? prior_volume : 0;
    run_parallel(n / (size_t)length, threads, [&](size_t s, size_t e) {
      std::vector<Extremum<T>> pad(padded), pre(padded), suf(padded);
      std::vector<uint64_t> pn, cpre, csuf;
      if (counting) {
        pn.resize(padded);
        cpre.resize(padded);
        csuf.resize(padded);
      }
      for (size_t line = s; line < e; ++line) {
        const int64_t base = ((int64_t)line / stride) * block + (int64_t)line % stride;
        for (int64_t p = 0; p < padded; ++p) {
          const int64_t src = source[(size_t)p];
          pad[p] = src >= 0 ? prev[(size_t)(base + src * stride)] : outside;
          if (counting) pn[p] = src >= 0 ? prev_n[(size_t)(base + src * stride)] : outside_n;
        }
        for (int64_t p = 0; p < padded; ++p) {
          const bool start = p % win == 0;
          pre[p] = start ? pad[p] : extremum_combine(pre[p - 1], pad[p], maximum);
          if (counting) cpre[p] = start ? pn[p] : cpre[p - 1] + pn[p];
        }
        for (int64_t p = padded - 1; p >= 0; --p) {
          const bool stop = p == padded - 1 || p % win == win - 1;
          suf[p] = stop ? pad[p] : extremum_combine(pad[p], suf[p + 1], maximum);
          if (counting) csuf[p] = stop ? pn[p] : csuf[p + 1] + pn[p];
        }
        for (int64_t c = 0; c < length; ++c) {
          const int64_t end = c + win - 1;
          const size_t dst = (size_t)(base + c * stride);
          next[dst] = extremum_combine(suf[c], pre[end], maximum);
          if (counting)
            next_n[dst] = c / win == end / win ? cpre[end] - cpre[c] + pn[c] : csuf[c] + cpre[end];
        }
      }
    });
    std::swap(prev, next);
    std::swap(prev_n, next_n);
    prior_volume *= (uint64_t)win;
  }
  run_parallel(n, threads, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) {
      const bool missing = prev[i].nan || (counting && prev_n[i] < pol.min_count);
      output[i] = missing ? std::numeric_limits<T>::quiet_NaN() : prev[i].value;
    }
  });
  return kOk;
}

// Counts::sample, src/boxcar.rs:17-33.
inline BoxcarCounts boxcar_sample(double v, const Policy& p) {
  BoxcarCounts c;
  if (std::isnan(v)) {
    c.nan = p.omit ? 0 : 1;
  } else if (std::isfinite(v)) {
    c.finite = 1;
  } else if (!(p.omit && p.ignore_inf)) {
    c.positive = v > 0 ? 1 : 0;
    c.negative = v < 0 ? 1 : 0;
  }
  return c;
}

// Significand bits of a finite nonzero binary64 as (lowest, highest) bit
// positions in units of 2^-1074.
inline void bit_range(double v, int* lowest, int* highest) {
  const uint64_t bits = bits64(v);
  const int e = (int)((bits >> 52) & 0x7ff);
  const uint64_t m = (bits & ((1ull << 52) - 1)) | (e ? 1ull << 52 : 0);
  const int shift = e ? e - 1 : 0;
  *lowest = shift + __builtin_ctzll(m);
  *highest = shift + 63 - __builtin_clzll(m);
}

// v as a `words`-word two's-complement integer in units of 2^(64 low - 1074);
// the span guarantees that no set bit falls below the unit or above the top.
inline void encode_span(double v, int low, int words, uint64_t* out) {
  std::fill(out, out + words, 0);
  const uint64_t bits = bits64(v);
  const int e = (int)((bits >> 52) & 0x7ff);
  uint64_t m = (bits & ((1ull << 52) - 1)) | (e ? 1ull << 52 : 0);
  if (m == 0) return;
  int pos = (e ? e - 1 : 0) - 64 * low;
  if (pos < 0) {
    m >>= -pos;
    pos = 0;
  }
  const u128 payload = (u128)m << (pos % 64);
  const int i = pos / 64;
  out[i] = (uint64_t)payload;
  if (i + 1 < words) out[i + 1] = (uint64_t)(payload >> 64);
  if (bits >> 63) {
    uint64_t carry = 1;
    for (int k = 0; k < words; ++k) {
      out[k] = ~out[k] + carry;
      carry = (carry && out[k] == 0) ? 1 : 0;
    }
  }
}

inline void span_add(uint64_t* acc, const uint64_t* v, int words, bool subtract) {
  uint64_t carry = subtract ? 1 : 0;
  for (int k = 0; k < words; ++k) {
    const uint64_t x = subtract ? ~v[k] : v[k];
    const u128 t = (u128)acc[k] + x + carry;
    acc[k] = (uint64_t)t;
    carry = (uint64_t)(t >> 64);
  }
}

// mean_into, src/boxcar.rs:140-342, with word_span (src/boxcar.rs:104-138):
// one span of words for every intermediate sum, exact sliding sums along
// each axis (each pass stores its axis innermost, so the last pass restores
// C order), one correctly rounded division at the end.
template <class T>
int boxcar_separable(const Window& w, const uint64_t* size, const int64_t* origin,
                     const T* input, double cval_d, const Policy& pol, int threads, T* output) {
  const size_t n = w.out_len;
  const int rank = w.rank;
  const double cval = (double)(T)cval_d;
  uint64_t volume = 1;
  for (int a = 0; a < rank; ++a) volume *= size[a];
  bool constant = false;
  for (int a = 0; a < rank; ++a) constant = constant || w.modes[a] == kConstant;
  int lowest = INT32_MAX, highest = 0;
  for (size_t i = 0; i <= n; ++i) {
    const double v = i < n ? (double)input[i] : cval;
    if (i == n && !constant) break;
    if (!std::isfinite(v) || v == 0.0) continue;
    int lo, hi;
    bit_range(v, &lo, &hi);
    lowest = std::min(lowest, lo);
    highest = std::max(highest, hi);
  }
  int low = 0, words = 1;
  if (lowest != INT32_MAX) {
    const int count_bits = volume > 1 ? 64 - __builtin_clzll(volume - 1) : 0;
    low = lowest / 64;
    words = (highest + 1 + count_bits + 1 + 63) / 64 - low;
  }
  std::vector<uint64_t> prev(n * words), next(n * words);
  std::vector<BoxcarCounts> prev_c(n), next_c(n);
  run_parallel(n, threads, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) {
      const double v = (double)input[i];
      prev_c[i] = boxcar_sample(v, pol);
      if (std::isfinite(v)) encode_span(v, low, words, &prev[i * words]);
    }
  });
  std::vector<uint64_t> padding(words, 0);
  BoxcarCounts padding_c = boxcar_sample(cval, pol);
  if (std::isfinite(cval) && constant) encode_span(cval, low, words, padding.data());
  std::vector<int64_t> strides(w.strides.begin(), w.strides.end());
  for (int axis = 0; axis < rank; ++axis) {
    const int64_t length = w.shape[axis], stride = strides[axis];
    const int64_t win = (int64_t)size[axis], anchor = win / 2 + origin[axis];
    std::vector<int64_t> first, leaving, entering;
    int rc = map_line(length, -anchor, win, w.modes[axis], &first);
    if (!rc) rc = map_line(length, -anchor, length - 1, w.modes[axis], &leaving);
    if (!rc) rc = map_line(length, win - anchor, length - 1, w.modes[axis], &entering);
    if (rc) return rc;
    run_parallel(n / (size_t)length, threads, [&](size_t s, size_t e) {
      std::vector<uint64_t> sum(words);
      for (size_t line = s; line < e; ++line) {
        int64_t base = 0, rest = (int64_t)line;
        for (int other = rank - 1; other >= 0; --other) {
          if (other == axis) continue;
          base += (rest % w.shape[other]) * strides[other];
          rest /= w.shape[other];
        }
        auto words_at = [&](int64_t src) -> const uint64_t* {
          return src >= 0 ? &prev[(size_t)(base + src * stride) * words] : padding.data();
        };
        auto counts_at = [&](int64_t src) -> const BoxcarCounts& {
          return src >= 0 ? prev_c[(size_t)(base + src * stride)] : padding_c;
        };
        auto add_counts = [](BoxcarCounts& a, const BoxcarCounts& b, bool subtract) {
          if (subtract) {
            a.finite -= b.finite; a.nan -= b.nan; a.positive -= b.positive; a.negative -= b.negative;
          } else {
            a.finite += b.finite; a.nan += b.nan; a.positive += b.positive; a.negative += b.negative;
          }
        };
        std::fill(sum.begin(), sum.end(), 0);
        BoxcarCounts count;
        for (int64_t t = 0; t < win; ++t) {
          span_add(sum.data(), words_at(first[(size_t)t]), words, false);
          add_counts(count, counts_at(first[(size_t)t]), false);
        }
        uint64_t* dst = &next[(size_t)line * (size_t)length * words];
        BoxcarCounts* dst_c = &next_c[(size_t)line * (size_t)length];
        for (int64_t c = 0; c < length; ++c) {
          std::copy(sum.begin(), sum.end(), dst + (size_t)c * words);
          dst_c[c] = count;
          if (c + 1 < length) {
            span_add(sum.data(), words_at(leaving[(size_t)c]), words, true);
            add_counts(count, counts_at(leaving[(size_t)c]), true);
            span_add(sum.data(), words_at(entering[(size_t)c]), words, false);
            add_counts(count, counts_at(entering[(size_t)c]), false);
          }
        }
      }
    });
    std::swap(prev, next);
    std::swap(prev_c, next_c);
    strides[axis] = 1;
    int64_t step = length;
    for (int other = rank - 1; other >= 0; --other) {
      if (other == axis) continue;
      strides[other] = step;
      step *= w.shape[other];
    }
    u128 carry = 0;
    for (int k = 0; k < words; ++k) {
      const u128 t = (u128)padding[k] * (uint64_t)win + carry;
      padding[k] = (uint64_t)t;
      carry = t >> 64;
    }
    padding_c.finite *= win;
    padding_c.nan *= win;
    padding_c.positive *= win;
    padding_c.negative *= win;
  }
  run_parallel(n, threads, [&](size_t s, size_t e) {
    for (size_t i = s; i < e; ++i) {
      const BoxcarCounts& c = prev_c[i];
      const uint64_t kept = c.finite + c.positive + c.negative;
      T v;
      if (c.nan || kept == 0 || (pol.omit && kept < pol.min_count) || (c.positive && c.negative)) {
        v = std::numeric_limits<T>::quiet_NaN();
      } else if (c.positive) {
        v = std::numeric_limits<T>::infinity();
      } else if (c.negative) {
        v = -std::numeric_limits<T>::infinity();
      } else {
        v = exact_mean<T>(&prev[i * words], words, low, c.finite);
      }
      output[i] = v;
    }
  });
  return kOk;
}

// ---------------------------------------------------------------------------
// Robust reductions: RobustReduction::finish (src/robust.rs:244-299) for the
// MAD, sigma clipping, the mode and the biweight location / scale, with the
// helpers of src/robust.rs:376-697 and src/location.rs:36-240.

enum RobustKind {
  kRobustPercentile = 0,
  kRobustMad = 1,
  kRobustMode = 2,
  kRobustBiweightLocation = 3,
  kRobustBiweightScale = 4,
  kRobustSigmaMean = 5,
  kRobustSigmaMedian = 6,
  kRobustSigmaMode = 7,
};
enum ModeRule { kModeSex = 0, kModeMmm = 1, kModeIraf = 2 };

struct RobustSpec {
  int kind = kRobustPercentile;
  Policy policy;           // percentile / MAD / mode / biweight
  double parameter = 0.0;  // q, MAD scale or biweight c
  double lower = 3.0, upper = 3.0;
  int64_t maxiters = 5;    // < 0: until stable
  int center = 1;          // 0 mean, 1 median
  int spread = 0;          // 0 std, 1 MAD
  int estimator = kModeSex;
  bool modify_sample_size = false;
  double pearson = 2.5;
  uint64_t clip_min_count = 1;
};

// Phi^-1(0.75), src/robust.rs:11.
constexpr double kNormalUpperQuartile = 0.6744897501960817;

inline int total_cmp(double a, double b) {
  const uint64_t ka = total_key(a), kb = total_key(b);
  return ka < kb ? -1 : (ka > kb ? 1 : 0);
}

// 2^n by binary powering with a final reciprocal for negative n (the
// powi of the reference's toolchain): exact unless 2^|n| overflows, when
// the reciprocal is zero.
double powi2(int n) {
  unsigned int m = n < 0 ? (unsigned int)(-(long long)n) : (unsigned int)n;
  double r = 1.0, a = 2.0;
  while (m) {
    if (m & 1) r *= a;
    a *= a;
    m >>= 1;
  }
  return n < 0 ? 1.0 / r : r;
}

struct Scaled {
  double value;
  int exponent;
};

// binary_parts, src/robust.rs:498-511 (positive finite values).
std::pair<double, int> binary_parts(double value) {
  const uint64_t b = bits64(value);
  const int exponent = (int)((b >> 52) & 0x7ff);
  const uint64_t fraction = b & ((1ull << 52) - 1);
  if (exponent == 0) {
    const int leading = 63 - __builtin_clzll(fraction);
    return {(double)fraction / (double)(1ull << leading), leading - 1074};
  }
  return {from_bits64(fraction | (1023ull << 52)), exponent - 1023};
}

// absolute_deviation, src/robust.rs:438-466.
Scaled absolute_deviation(double value, Scaled center) {
  if (center.exponent == -1 && std::isfinite(value * 2.0)) {
    const double difference = value * 2.0 - center.value;
    if (std::isfinite(difference)) return {std::fabs(difference), -1};
  }
  const double midpoint = center.exponent == -1 ? center.value / 2.0 : center.value;
  const double difference = value - midpoint;
  if (std::isfinite(difference) || std::isinf(value)) return {std::fabs(difference), 0};
  return {std::fabs(value / 2.0 - midpoint / 2.0), 1};
}

// compare_scaled, src/robust.rs:468-481.
int compare_scaled(Scaled left, Scaled right) {
  if (left.value == 0.0 || right.value == 0.0 || std::isinf(left.value) || std::isinf(right.value))
    return total_cmp(left.value, right.value);
  const auto [lv, le] = binary_parts(left.value);
  const auto [rv, re] = binary_parts(right.value);
  const int a = le + left.exponent, b = re + right.exponent;
  if (a != b) return a < b ? -1 : 1;
  return total_cmp(lv, rv);
}

// scaled_midpoint, src/robust.rs:483-496.
Scaled scaled_midpoint(Scaled left, Scaled right) {
  if (std::isinf(right.value) || right.value == 0.0) return right;
  const auto [rv, re] = binary_parts(right.value);
  const int exponent = re + right.exponent;
  double lv = 0.0;
  if (left.value != 0.0) {
    const auto [v, le] = binary_parts(left.value);
    lv = v * powi2(le + left.exponent - exponent);
  }
  return {lv + rv, exponent - 1};
}

// mad_parts, src/robust.rs:376-436: the median absolute deviation as a
// scaled magnitude, merging the deviations on both sides of the median.
Scaled mad_parts(const std::vector<double>& values) {
  std::vector<double> s(values);
  std::sort(s.begin(), s.end(), key_less);
  const size_t n = s.size();
  const double lower = s[(n - 1) / 2], upper = s[n / 2];
  Scaled center;
  if (!std::isfinite(lower) || !std::isfinite(upper))
    center = {interpolate(lower, upper, 0.5), 0};
  else if (std::isfinite(lower + upper))
    center = {lower + upper, -1};
  else
    center = {lower / 2.0 + upper / 2.0, 0};
  if (!std::isfinite(center.value)) return {kNaN64, 0};
  size_t left = n / 2, right = left;
  Scaled previous{0.0, 0}, selected = previous;
  for (size_t step = 0; step <= n / 2; ++step) {
    previous = selected;
    const bool take_left =
        left > 0 && (right == n || compare_scaled(absolute_deviation(s[left - 1], center),
                                                  absolute_deviation(s[right], center)) <= 0);
    if (take_left) {
      --left;
      selected = absolute_deviation(s[left], center);
    } else {
      selected = absolute_deviation(s[right], center);
      ++right;
    }
  }
  return n % 2 == 1 ? selected : scaled_midpoint(previous, selected);
}

// multiply_scaled, src/robust.rs:513-534.
double multiply_scaled(Scaled value, double multiplier) {
  if (!std::isfinite(value.value)) return value.value * multiplier;
  if (value.value == 0.0 || multiplier == 0.0) return 0.0;
  const auto [left, le] = binary_parts(value.value);
  const auto [right, re] = binary_parts(multiplier);
  const auto [mantissa, adjustment] = binary_parts(left * right);
  const int exponent = le + re + adjustment + value.exponent;
  if (exponent > 1023) return INFINITY;
  if (exponent < -1075) return 0.0;
  if (exponent >= -1022) return mantissa * from_bits64((uint64_t)(exponent + 1023) << 52);
  const double scale = from_bits64((uint64_t)(exponent + 2045) << 52);
  return (mantissa * 2.2250738585072014e-308) * scale;
}

// within_limit, src/robust.rs:536-559.
bool within_limit(double value, double center, Scaled spread, double sigma) {
  if (value == center) return true;
  if (spread.value == 0.0 || sigma == 0.0) return false;
  const double difference = value - center;
  double distance;
  int distance_exp;
  if (std::isfinite(difference)) {
    std::tie(distance, distance_exp) = binary_parts(std::fabs(difference));
  } else {
    std::tie(distance, distance_exp) = binary_parts(std::fabs(value / 2.0 - center / 2.0));
    distance_exp += 1;
  }
  const auto [scale, scale_exp] = binary_parts(spread.value);
  const auto [multiplier, multiplier_exp] = binary_parts(sigma);
  const auto [limit, adjustment] = binary_parts(scale * multiplier);
  const int limit_exp = scale_exp + multiplier_exp + adjustment + spread.exponent;
  return distance_exp < limit_exp || (distance_exp == limit_exp && distance <= limit);
}

// finite_mean, src/robust.rs:572-592.
double finite_mean(const std::vector<double>& values) {
  Sum sum;
  for (double v : values) sum.add(v);
  const double total = sum.total();
  if (std::isfinite(total)) return total / (double)values.size();
  const uint64_t m = (uint64_t)(values.size() - 1);
  const int exponent = (m == 0 ? 0 : 64 - __builtin_clzll(m)) + 1;
  const double scale = powi2(exponent);
  Sum scaled;
  double lower = INFINITY, upper = -INFINITY;
  for (double v : values) {
    scaled.add(v / scale);
    lower = std::fmin(lower, v);
    upper = std::fmax(upper, v);
  }
  return clamp_f64(scaled.total() / ((double)values.size() / scale), lower, upper);
}

// location, src/robust.rs:561-570 (the median is the 50th percentile).
double clip_location(const std::vector<double>& values, int center) {
  if (center == 0) return finite_mean(values);
  std::vector<double> copy(values);
  return percentile(copy, 50.0);
}

// std_parts, src/robust.rs:594-630.
Scaled std_parts(const std::vector<double>& values) {
  const double reference = values[0];
  bool halve = false;
  for (double v : values) halve = halve || !std::isfinite(v - reference);
  auto delta = [&](double v) { return halve ? v / 2.0 - reference / 2.0 : v - reference; };
  double scale = 0.0;
  for (double v : values) scale = std::fmax(scale, std::fabs(delta(v)));
  if (scale == 0.0) return {0.0, 0};
  Sum sum;
  for (double v : values) sum.add(delta(v) / scale);
  const double center = sum.total() / (double)values.size();
  Sum squares;
  for (double v : values) {
    const double residual = delta(v) / scale - center;
    squares.add(residual * residual);
  }
  const auto [mantissa, exponent] = binary_parts(scale);
  return {mantissa * std::sqrt(squares.total() / (double)values.size()), exponent + (halve ? 1 : 0)};
}

// mode_from_moments / mode_estimate, src/location.rs:36-84.
double mode_from_moments(double mean, double median, double std_dev, int estimator, double pearson) {
  const double difference = median - mean;
  const double pearson_mode = median + (pearson - 1.0) * difference;
  if (estimator == kModeMmm) return pearson_mode;
  if (estimator == kModeIraf) return mean < median ? mean : pearson_mode;
  if (std_dev == 0.0) return mean;
  if (std::fabs(difference) / std_dev >= 0.3) return median;
  return pearson_mode;
}

double mode_estimate(std::vector<double>& values, int estimator, double pearson) {
  if (values.empty()) return kNaN64;
  const double mean = mean_valid(values.data(), values.size());
  const double std_dev =
      estimator == kModeSex ? dispersion_valid(values.data(), values.size(), 0, true) : kNaN64;
  const double median = median_valid(values);
  return mode_from_moments(mean, median, std_dev, estimator, pearson);
}

// standardize, src/location.rs:104-150. The reference's in-place median
// leaves the samples in an order its selection routine does not publish;
// the deviations here follow ascending total order, and the biweight sums
// below run in that order.
struct Standardized {
  int state = 0;  // 0 empty, 1 zero MAD, 2 spread
  double median = 0.0, width = 0.0, factor = 1.0;
  std::vector<double> u;
};

Standardized standardize(std::vector<double>& values, double c) {
  Standardized out;
  const size_t n = values.size();
  if (n == 0) return out;
  std::sort(values.begin(), values.end(), key_less);
  out.median = median_valid(values);
  std::sort(values.begin(), values.end(), key_less);
  std::vector<double> dev(n);
  double factor = 1.0;
  bool overflow = false;
  for (size_t i = 0; i < n; ++i) {
    dev[i] = values[i] - out.median;
    overflow = overflow || !std::isfinite(dev[i]);
  }
  if (overflow) {
    factor = 2.0;
    for (size_t i = 0; i < n; ++i) dev[i] = values[i] / 2.0 - out.median / 2.0;
  }
  std::vector<double> absolute(n);
  for (size_t i = 0; i < n; ++i) absolute[i] = std::fabs(dev[i]);
  double mad = median_valid(absolute);
  if (mad == 0.0) {
    out.state = 1;
    return out;
  }
  double extra = 1.0;
  while (!std::isfinite(c * mad)) {
    mad /= 2.0;
    extra *= 2.0;
  }
  const double width = c * mad;
  for (size_t i = 0; i < n; ++i) dev[i] = dev[i] / extra / width;
  out.state = 2;
  out.width = width;
  out.factor = factor * extra;
  out.u = std::move(dev);
  return out;
}

// biweight_location, src/location.rs:152-183.
double biweight_location(std::vector<double>& values, double c) {
  Standardized st = standardize(values, c);
  if (st.state == 0) return kNaN64;
  if (st.state == 1) return st.median;
  Sum weighted, weights;
  for (double u : st.u) {
    if (!(std::fabs(u) < 1.0)) continue;
    const double weight = (1.0 - u * u) * (1.0 - u * u);
    weighted.add(u * weight);
    weights.add(weight);
  }
  const double correction = st.width * (weighted.total() / weights.total());
  const double unscaled = correction * st.factor;
  if (std::isfinite(unscaled)) return st.median + unscaled;
  return (st.median / st.factor + correction) * st.factor;
}

// biweight_scale, src/location.rs:185-240.
double biweight_scale(std::vector<double>& values, double c, bool modify_sample_size) {
  const size_t total = values.size();
  Standardized st = standardize(values, c);
  if (st.state == 0) return kNaN64;
  if (st.state == 1) return 0.0;
  Sum numerator, denominator;
  size_t kept = 0;
  for (double u : st.u) {
    if (!(std::fabs(u) < 1.0)) continue;
    const double u2 = u * u;
    const double taper = (1.0 - u2) * (1.0 - u2);
    numerator.add(u2 * taper * taper);
    denominator.add((1.0 - u2) * (1.0 - 5.0 * u2));
    ++kept;
  }
  const double count = (double)(modify_sample_size ? kept : total);
  const double ratio = std::sqrt(count * numerator.total()) / std::fabs(denominator.total());
  return st.width * ratio * st.factor;
}

// clipped, src/robust.rs:632-689: values are the finite samples in tap order.
double clipped(std::vector<double>& values, const RobustSpec& spec) {
  int64_t iteration = 0;
  while (values.size() >= spec.clip_min_count && (spec.maxiters < 0 || iteration < spec.maxiters)) {
    const double center = clip_location(values, spec.center);
    Scaled spread;
    if (spec.spread == 1) {
      const Scaled deviation = mad_parts(values);
      if (deviation.value > 0.0 && std::isfinite(deviation.value)) {
        const auto [mantissa, exponent] = binary_parts(deviation.value);
        spread = {mantissa / kNormalUpperQuartile, exponent + deviation.exponent};
      } else {
        spread = deviation;
      }
    } else {
      spread = std_parts(values);
    }
    const size_t previous = values.size();
    size_t write = 0;
    for (size_t read = 0; read < values.size(); ++read) {
      const double v = values[read];
      if (within_limit(v, center, spread, v < center ? spec.lower : spec.upper)) values[write++] = v;
    }
    values.resize(write);
    ++iteration;
    if (values.size() == previous) break;
  }
  if (values.size() < spec.clip_min_count) return kNaN64;
  if (spec.kind == kRobustSigmaMean) return clip_location(values, 0);
  if (spec.kind == kRobustSigmaMedian) return clip_location(values, 1);
  return mode_estimate(values, spec.estimator, spec.pearson);
}

// RobustReduction::finish, src/robust.rs:244-299.
double robust_finish(const RobustSpec& spec, std::vector<double>& values) {
  if (spec.kind >= kRobustSigmaMean) {
    size_t write = 0;
    for (size_t read = 0; read < values.size(); ++read)
      if (std::isfinite(values[read])) values[write++] = values[read];
    values.resize(write);
    return clipped(values, spec);
  }
  if (!spec.policy.omit) {
    for (double v : values)
      if (std::isnan(v)) return kNaN64;
  } else {
    size_t write = 0;
    for (size_t read = 0; read < values.size(); ++read)
      if (retained(values[read], spec.policy)) values[write++] = values[read];
    values.resize(write);
    if (values.size() < spec.policy.min_count) return kNaN64;
  }
  if (values.empty()) return kNaN64;
  switch (spec.kind) {
    case kRobustPercentile:
      return percentile(values, spec.parameter);
    case kRobustMad:
      return multiply_scaled(mad_parts(values), spec.parameter);
    default:
      break;
  }
  for (double v : values)
    if (std::isinf(v)) return kNaN64;
  if (spec.kind == kRobustMode) return mode_estimate(values, spec.estimator, spec.pearson);
  if (spec.kind == kRobustBiweightLocation) return biweight_location(values, spec.parameter);
  return biweight_scale(values, spec.parameter, spec.modify_sample_size);
}

// ---------------------------------------------------------------------------
// Mesh background: MeshBackground::new / estimate / interpolate_into
// (src/background.rs:417-923), the per-mesh statistics (:924-1152), the
// natural spline (:1154-1212) and the SExtractor-compatible interpolation
// (src/background/sep_interpolation.rs).

struct MeshSpec {
  int estimator = 0;  // 0 SExtractor, 1 sigma clip
  double pearson = 2.5;
  double lower = 3.0, upper = 3.0;
  int64_t maxiters = 10;  // < 0: until stable
  int center = 1, spread = 0;
  int statistic = 2;  // 0 mean, 1 median, 2 mode
  int mode_estimator = kModeSex;
  int rms = 0;        // 0 std, 1 MAD std
  double min_valid_fraction = 0.5;
  int valid_count = 0;  // 0 finite, 1 retained
  int valid_base = 0;   // 0 mesh, 1 box
  int fill = 0;         // 0 nearest, 1 inverse distance
  uint64_t idw_neighbors = 10;
  double idw_power = 1.0;
  int filter_edge = 0;     // 0 shrink, 1 truncate
  int threshold_kind = 0;  // 0 all, 1 deviation, 2 above
  double threshold = 0.0;
  int interpolation = 0;   // 0 spline, 1 SExtractor
};

// median_sorted / median_of, src/background.rs:940-963.
double mesh_median_sorted(const double* v, size_t n) {
  if (n % 2 == 1) return v[n / 2];
  const double a = v[n / 2 - 1], b = v[n / 2];
  const double mid = (a + b) / 2.0;
  return std::isfinite(mid) ? mid : a / 2.0 + b / 2.0;
}

double mesh_median_of(std::vector<double> v) {
  if (v.empty()) return kNaN64;
  for (double x : v)
    if (std::isnan(x)) return kNaN64;
  std::sort(v.begin(), v.end(), key_less);
  return mesh_median_sorted(v.data(), v.size());
}

// mean_of, src/background.rs:965-978.
double mesh_mean_of(const double* v, size_t n) {
  Sum sum;
  for (size_t i = 0; i < n; ++i) sum.add(v[i]);
  const double total = sum.total();
  if (std::isfinite(total)) return total / (double)n;
  return mean_valid(v, n);
}

// std_about, src/background.rs:1000-1015.
double mesh_std_about(const double* v, size_t n, double mean) {
  if (n == 0) return kNaN64;
  const double scale = std::fmax(std::fabs(v[0] - mean), std::fabs(v[n - 1] - mean));
  if (scale == 0.0) return 0.0;
  if (!std::isfinite(scale)) return kNaN64;
  Sum squares;
  for (size_t i = 0; i < n; ++i) {
    const double deviation = (v[i] - mean) / scale;
    squares.add(deviation * deviation);
  }
  return scale * std::sqrt(squares.total() / (double)n);
}

// mad_std, src/background.rs:1017-1022.
double mesh_mad_std(const double* v, size_t n, double median) {
  std::vector<double> scratch(n);
  for (size_t i = 0; i < n; ++i) scratch[i] = std::fabs(v[i] - median);
  return mesh_median_of(std::move(scratch)) / kNormalUpperQuartile;
}

// within, src/background.rs:1024-1032.
std::pair<size_t, size_t> mesh_within(const std::vector<double>& v, std::pair<size_t, size_t> range,
                                      double low, double high) {
  const auto b = v.begin() + (ptrdiff_t)range.first, e = v.begin() + (ptrdiff_t)range.second;
  const size_t lo = range.first + (size_t)(std::partition_point(b, e, [&](double x) { return x < low; }) - b);
  const size_t hi = range.first + (size_t)(std::partition_point(b, e, [&](double x) { return x <= high; }) - b);
  return {lo, std::max(hi, lo)};
}

// clip_sorted, src/background.rs:1034-1069.
std::pair<size_t, size_t> mesh_clip_sorted(const std::vector<double>& v, std::pair<size_t, size_t> range,
                                           double lower, double upper, int64_t maxiters, int center,
                                           int spread, size_t min_count) {
  int64_t iteration = 0;
  while (range.second - range.first >= std::max<size_t>(min_count, 1) &&
         (maxiters < 0 || iteration < maxiters)) {
    const double* kept = v.data() + range.first;
    const size_t n = range.second - range.first;
    const double middle = center == 0 ? mesh_mean_of(kept, n) : mesh_median_sorted(kept, n);
    const double width = spread == 0 ? mesh_std_about(kept, n, mesh_mean_of(kept, n))
                                     : mesh_mad_std(kept, n, mesh_median_sorted(kept, n));
    const auto next = mesh_within(v, range, middle - lower * width, middle + upper * width);
    ++iteration;
    if (next == range) break;
    range = next;
  }
  return range;
}

struct MeshStat {
  double background = kNaN64, rms = kNaN64;
  uint64_t finite = 0, retained = 0;
  bool valid = false;
};

// sextractor_stats / clipped_stats / finish_stats, src/background.rs:652-705,
// 1071-1152, over the mesh's finite samples sorted in total order.
MeshStat mesh_finish(std::vector<double>& v, uint64_t volume, uint64_t box_volume, const MeshSpec& spec) {
  MeshStat st;
  st.finite = v.size();
  if (v.empty()) return st;
  std::sort(v.begin(), v.end(), key_less);
  const size_t n = v.size();
  double background = kNaN64, rms = kNaN64;
  size_t retained = 0;
  if (spec.estimator == 0) {
    const double mean = mesh_mean_of(v.data(), n);
    const double sd = mesh_std_about(v.data(), n, mean);
    const auto first = mesh_within(v, {0, n}, mean - 2.0 * sd, mean + 2.0 * sd);
    if (first.first != first.second) {
      const double* sub = v.data() + first.first;
      const size_t m = first.second - first.first;
      const double mean2 = mesh_mean_of(sub, m);
      const double sd2 = mesh_std_about(sub, m, mean2);
      const auto span = mesh_within(v, {0, n}, mean2 - 5.0 * sd2, mean2 + 5.0 * sd2);
      const auto kept = mesh_clip_sorted(v, span, 3.0, 3.0, 100, 1, 0, 1);
      if (kept.first != kept.second) {
        const double* k = v.data() + kept.first;
        const size_t c = kept.second - kept.first;
        const double mean3 = mesh_mean_of(k, c);
        const double sd3 = mesh_std_about(k, c, mean3);
        background = mode_from_moments(mean3, mesh_median_sorted(k, c), sd3, kModeSex, spec.pearson);
        rms = sd3;
        retained = c;
      }
    }
  } else {
    const auto kept = mesh_clip_sorted(v, {0, n}, spec.lower, spec.upper, spec.maxiters, spec.center,
                                       spec.spread, 1);
    const size_t c = kept.second - kept.first;
    retained = c;
    if (c > 0) {
      const double* k = v.data() + kept.first;
      const double mean = mesh_mean_of(k, c);
      const double median = mesh_median_sorted(k, c);
      if (spec.statistic == 0)
        background = mean;
      else if (spec.statistic == 1)
        background = median;
      else
        background = mode_from_moments(mean, median, mesh_std_about(k, c, mean), spec.mode_estimator,
                                       spec.pearson);
      rms = spec.rms == 0 ? mesh_std_about(k, c, mean) : mesh_mad_std(k, c, median);
    }
  }
  st.retained = retained;
  const uint64_t count = spec.valid_count == 0 ? st.finite : retained;
  const uint64_t base = spec.valid_base == 0 ? volume : box_volume;
  if (count > 0 && (double)count >= spec.min_valid_fraction * (double)base && std::isfinite(background) &&
      std::isfinite(rms)) {
    st.background = background;
    st.rms = rms;
    st.valid = true;
  }
  return st;
}

void mesh_index(size_t flat, const std::vector<size_t>& mesh_shape, size_t* index) {
  for (size_t a = mesh_shape.size(); a-- > 0;) {
    index[a] = flat % mesh_shape[a];
    flat /= mesh_shape[a];
  }
}

// fill_invalid / replacement, src/background.rs:715-798.
void mesh_fill(std::vector<double>& bg, std::vector<double>& rms, const std::vector<bool>& valid,
               const std::vector<size_t>& mesh_shape, const MeshSpec& spec) {
  const size_t len = bg.size(), ndim = mesh_shape.size();
  std::vector<size_t> good;
  for (size_t i = 0; i < len; ++i)
    if (valid[i]) good.push_back(i);
  if (good.size() == len || good.empty()) return;
  std::vector<size_t> gi(good.size() * ndim), idx(ndim);
  for (size_t s = 0; s < good.size(); ++s) mesh_index(good[s], mesh_shape, &gi[s * ndim]);
  std::vector<std::tuple<size_t, double, double>> out;
  std::vector<std::pair<uint64_t, size_t>> d;
  for (size_t flat = 0; flat < len; ++flat) {
    if (valid[flat]) continue;
    mesh_index(flat, mesh_shape, idx.data());
    d.clear();
    for (size_t s = 0; s < good.size(); ++s) {
      uint64_t d2 = 0;
      for (size_t a = 0; a < ndim; ++a) {
        const uint64_t diff = idx[a] > gi[s * ndim + a] ? idx[a] - gi[s * ndim + a] : gi[s * ndim + a] - idx[a];
        d2 += diff * diff;
      }
      d.push_back({d2, good[s]});
    }
    double value, spread;
    if (spec.fill == 0) {
      uint64_t nearest = UINT64_MAX;
      for (auto& e : d) nearest = std::min(nearest, e.first);
      Sum v, r;
      size_t count = 0;
      for (auto& e : d)
        if (e.first == nearest) {
          v.add(bg[e.second]);
          r.add(rms[e.second]);
          ++count;
        }
      value = v.total() / (double)count;
      spread = r.total() / (double)count;
    } else {
      std::sort(d.begin(), d.end());
      const uint64_t last = d[std::min<size_t>(spec.idw_neighbors, d.size()) - 1].first;
      Sum weighted, weighted_rms, total;
      for (auto& e : d) {
        if (e.first > last) break;
        const double weight = 1.0 / std::pow(std::sqrt((double)e.first), spec.idw_power);
        weighted.add(weight * bg[e.second]);
        weighted_rms.add(weight * rms[e.second]);
        total.add(weight);
      }
      value = weighted.total() / total.total();
      spread = weighted_rms.total() / total.total();
    }
    out.emplace_back(flat, value, spread);
  }
  for (auto& [flat, value, spread] : out) {
    bg[flat] = value;
    rms[flat] = spread;
  }
}

// filter, src/background.rs:800-856.
void mesh_filter(std::vector<double>& bg, std::vector<double>& rms, const std::vector<size_t>& mesh_shape,
                 const std::vector<size_t>& filter_size, const MeshSpec& spec) {
  bool off = bg.empty();
  bool all_one = true;
  for (size_t f : filter_size) all_one = all_one && f == 1;
  if (off || all_one) return;
  const size_t ndim = mesh_shape.size(), len = bg.size();
  std::vector<double> ob(bg), orms(rms), wb, wr;
  std::vector<size_t> idx(ndim), low(ndim), high(ndim);
  for (size_t flat = 0; flat < len; ++flat) {
    mesh_index(flat, mesh_shape, idx.data());
    for (size_t a = 0; a < ndim; ++a) {
      const size_t k = idx[a], n = mesh_shape[a], half = filter_size[a] / 2;
      if (spec.filter_edge == 0) {
        const size_t h = std::min(std::min(half, k), n - 1 - k);
        low[a] = k - h;
        high[a] = k + h;
      } else {
        low[a] = k >= half ? k - half : 0;
        high[a] = std::min(k + half, n - 1);
      }
    }
    wb.clear();
    wr.clear();
    size_t volume = 1;
    for (size_t a = 0; a < ndim; ++a) volume *= high[a] - low[a] + 1;
    for (size_t pos = 0; pos < volume; ++pos) {
      size_t rest = pos, offset = 0, stride = 1;
      for (size_t a = ndim; a-- > 0;) {
        const size_t width = high[a] - low[a] + 1;
        offset += (low[a] + rest % width) * stride;
        rest /= width;
        stride *= mesh_shape[a];
      }
      wb.push_back(bg[offset]);
      wr.push_back(rms[offset]);
    }
    const double median = mesh_median_of(wb);
    bool replace = true;
    if (spec.threshold_kind == 1) replace = std::fabs(median - bg[flat]) >= spec.threshold;
    if (spec.threshold_kind == 2) replace = bg[flat] > spec.threshold;
    if (replace) {
      ob[flat] = median;
      orms[flat] = mesh_median_of(wr);
    }
  }
  bg.swap(ob);
  rms.swap(orms);
}

// Tap, src/background.rs:349-397.
struct SplineTap {
  size_t seg;
  double a, b, c, d;
};

SplineTap spline_tap(double u, size_t nodes) {
  if (nodes < 2) return {0, 1.0, 0.0, 0.0, 0.0};
  const double fl = std::floor(u);
  size_t seg = fl > 0.0 ? (size_t)fl : 0;
  seg = std::min(seg, nodes - 2);
  const double t = u - (double)seg;
  const double a = 1.0 - t;
  return {seg, a, t, (a * a * a - a) / 6.0, (t * t * t - t) / 6.0};
}

// natural_pivots / natural_second_derivatives / columns_second_derivatives,
// src/background.rs:1154-1212.
std::vector<double> natural_pivots(size_t nodes) {
  std::vector<double> p(nodes, 0.0);
  double previous = 0.0;
  for (size_t i = 1; i + 1 < nodes; ++i) {
    p[i] = 1.0 / (4.0 - previous);
    previous = p[i];
  }
  return p;
}

void columns_second(const double* block, size_t nodes, size_t inner, const std::vector<double>& pivots,
                    double* second) {
  std::fill(second, second + nodes * inner, 0.0);
  if (nodes < 3) return;
  for (size_t i = 1; i + 1 < nodes; ++i)
    for (size_t j = 0; j < inner; ++j) {
      const double rhs = 6.0 * (block[(i - 1) * inner + j] - 2.0 * block[i * inner + j] + block[(i + 1) * inner + j]);
      second[i * inner + j] = (rhs - second[(i - 1) * inner + j]) * pivots[i];
    }
  for (size_t i = nodes - 2; i-- > 1;)
    for (size_t j = 0; j < inner; ++j) second[i * inner + j] -= pivots[i] * second[(i + 1) * inner + j];
}

// spline_into, src/background.rs:858-921.
template <class T>
void mesh_spline(const std::vector<double>& mesh, const std::vector<size_t>& shape,
                 const std::vector<size_t>& mesh_shape, const std::vector<size_t>& box, T* out) {
  const size_t ndim = shape.size();
  std::vector<double> current(mesh);
  for (size_t axis = 0; axis < ndim; ++axis) {
    size_t outer = 1, inner = 1;
    for (size_t a = 0; a < axis; ++a) outer *= shape[a];
    for (size_t a = axis + 1; a < ndim; ++a) inner *= mesh_shape[a];
    const size_t nodes = mesh_shape[axis], length = shape[axis];
    std::vector<SplineTap> taps(length);
    for (size_t p = 0; p < length; ++p) taps[p] = spline_tap(((double)p + 0.5) / (double)box[axis] - 0.5, nodes);
    const std::vector<double> pivots = natural_pivots(nodes);
    const size_t block = nodes * inner;
    std::vector<double> second(current.size());
    for (size_t o = 0; o < outer; ++o)
      columns_second(&current[o * block], nodes, inner, pivots, &second[o * block]);
    if (axis + 1 == ndim) {
      for (size_t line = 0; line < outer; ++line) {
        const double* y = &current[line * nodes];
        const double* m = &second[line * nodes];
        for (size_t p = 0; p < length; ++p) {
          const SplineTap& t = taps[p];
          double v;
          if (nodes < 2)
            v = y[0];
          else
            v = t.a * y[t.seg] + t.b * y[t.seg + 1] + t.c * m[t.seg] + t.d * m[t.seg + 1];
          out[line * length + p] = (T)v;
        }
      }
      return;
    }
    std::vector<double> next(outer * length * inner);
    for (size_t row = 0; row < outer * length; ++row) {
      const size_t o = row / length, p = row % length;
      const SplineTap& t = taps[p];
      const size_t base = o * block;
      double* dst = &next[row * inner];
      if (nodes < 2) {
        std::copy(&current[base], &current[base] + inner, dst);
        continue;
      }
      const size_t lo = base + t.seg * inner, hi = lo + inner;
      for (size_t j = 0; j < inner; ++j)
        dst[j] = t.a * current[lo + j] + t.b * current[hi + j] + t.c * second[lo + j] + t.d * second[hi + j];
    }
    current.swap(next);
  }
}

// sep_interpolation.rs: SExtractor-compatible 2-D interpolation.
inline double legacy_phase(double v) { return (double)(float)v; }

std::vector<double> sep_pivots(size_t nodes) {
  std::vector<double> p(nodes, 0.0);
  for (size_t i = 1; i + 1 < nodes; ++i) p[i] = 1.0 / (2.0 - 0.25 * p[i - 1]);
  return p;
}

void sep_coefficients(const double* values, const std::vector<double>& pivots, size_t lanes, double* coeff) {
  const size_t n = pivots.size();
  for (size_t i = 1; i + 1 < n; ++i)
    for (size_t j = 0; j < lanes; ++j) {
      const double left = values[(i - 1) * lanes + j], middle = values[i * lanes + j],
                   right = values[(i + 1) * lanes + j];
      const double difference = (right - middle) - (middle - left);
      coeff[i * lanes + j] = std::fma(3.0, difference, -0.5 * coeff[(i - 1) * lanes + j]) * pivots[i];
    }
  for (size_t i = n - 1; i-- > 1;) {
    const double multiplier = -0.5 * pivots[i];
    for (size_t j = 0; j < lanes; ++j)
      coeff[i * lanes + j] = std::fma(multiplier, coeff[(i + 1) * lanes + j], coeff[i * lanes + j]) / 6.0;
  }
}

struct SepWeight {
  double fraction, left_curve, right_curve;
};

template <class T>
void mesh_sep(const std::vector<double>& mesh, size_t ny, size_t nx, size_t height, size_t width, T* out) {
  const size_t rows = (ny + height - 1) / height, columns = (nx + width - 1) / width;
  if (mesh.size() == 1) {
    for (size_t i = 0; i < ny * nx; ++i) out[i] = (T)mesh[0];
    return;
  }
  double peak = 0.0;
  for (double v : mesh) peak = std::fmax(peak, std::fabs(v));
  const double scale = std::fmax(from_bits64(bits64(peak) & 0x7ff0000000000000ull), 2.2250738585072014e-308);
  const double inverse_scale = 1.0 / scale;
  std::vector<double> values(mesh.size());
  for (size_t i = 0; i < mesh.size(); ++i) values[i] = mesh[i] * inverse_scale;
  // Horizontal::new
  std::vector<size_t> lengths;
  std::vector<SepWeight> first, later;
  const bool have_x = columns > 1;
  if (have_x) {
    const double step = legacy_phase(1.0 / legacy_phase((double)width));
    auto weights = [&](double b, size_t length) {
      std::vector<SepWeight> w;
      for (size_t i = 0; i < length; ++i) {
        const double a = 1.0 - b;
        w.push_back({b, a * std::fma(a, a, -1.0), b * std::fma(b, b, -1.0)});
        b = legacy_phase(b + step);
      }
      return w;
    };
    const size_t intervals = width == 1 ? 1 : columns - 1;
    size_t start = 0;
    for (size_t i = 1; i <= intervals; ++i) {
      const size_t end = i == intervals ? nx : i * width + width / 2;
      lengths.push_back(end - start);
      start = end;
    }
    first = weights(legacy_phase(0.5 * step - 0.5), lengths[0]);
    size_t longest = 0;
    for (size_t i = 1; i < lengths.size(); ++i) longest = std::max(longest, lengths[i]);
    later = weights(width % 2 == 0 ? 0.5 * step : 0.0, longest);
  }
  auto row_out = [&](const double* vals, const double* coeff, auto&& store) {
    size_t pos = 0;
    for (size_t i = 0; i < lengths.size(); ++i) {
      const std::vector<SepWeight>& w = i == 0 ? first : later;
      const double left = vals[i], right = vals[i + 1], cl = coeff[i], cr = coeff[i + 1];
      const double slope = right - left;
      for (size_t k = 0; k < lengths[i]; ++k, ++pos) {
        const double linear = std::fma(w[k].fraction, slope, left);
        store(pos, std::fma(w[k].right_curve, cr, std::fma(w[k].left_curve, cl, linear)));
      }
    }
  };
  if (rows == 1 && have_x) {
    std::vector<double> zeros(columns, 0.0), profile(nx);
    row_out(values.data(), zeros.data(), [&](size_t p, double v) { profile[p] = v * scale; });
    for (size_t y = 0; y < ny; ++y)
      for (size_t x = 0; x < nx; ++x) out[y * nx + x] = (T)profile[x];
    return;
  }
  std::vector<double> y_coeff(mesh.size(), 0.0);
  sep_coefficients(values.data(), sep_pivots(rows), columns, y_coeff.data());
  const std::vector<double> x_pivots = have_x ? sep_pivots(columns) : std::vector<double>();
  const double phase_height = legacy_phase((double)height);
  std::vector<double> line(columns), x_coeff(columns);
  for (size_t y = 0; y < ny; ++y) {
    const double box_coordinate = legacy_phase(legacy_phase((double)y) / phase_height);
    const double z = legacy_phase(box_coordinate - 0.5);
    const size_t i = std::min(z > 0.0 ? (size_t)z : (size_t)0, rows - 2);
    const double b = z - (double)i, a = 1.0 - b;
    const double ca = std::fma(a * a, a, -a), cb = std::fma(b * b, b, -b);
    const double* top = &values[i * columns];
    const double* bottom = &values[(i + 1) * columns];
    const double* ct = &y_coeff[i * columns];
    const double* cbot = &y_coeff[(i + 1) * columns];
    for (size_t j = 0; j < columns; ++j) {
      const double linear = std::fma(b, bottom[j] - top[j], top[j]);
      line[j] = std::fma(cb, cbot[j], std::fma(ca, ct[j], linear));
    }
    if (have_x) {
      std::fill(x_coeff.begin(), x_coeff.end(), 0.0);
      sep_coefficients(line.data(), x_pivots, 1, x_coeff.data());
      row_out(line.data(), x_coeff.data(), [&](size_t p, double v) { out[y * nx + p] = (T)(v * scale); });
    } else {
      for (size_t x = 0; x < nx; ++x) out[y * nx + x] = (T)(line[0] * scale);
    }
  }
}

template <class T>
void mesh_interpolate(const std::vector<double>& mesh, const std::vector<size_t>& shape,
                      const std::vector<size_t>& mesh_shape, const std::vector<size_t>& box, const MeshSpec& spec,
                      T* out) {
  size_t len = 1;
  for (size_t v : shape) len *= v;
  if (len == 0) return;
  bool constant = true;
  for (double v : mesh) constant = constant && v == mesh[0];
  if (constant) {
    for (size_t i = 0; i < len; ++i) out[i] = (T)mesh[0];
    return;
  }
  if (spec.interpolation == 0)
    mesh_spline(mesh, shape, mesh_shape, box, out);
  else
    mesh_sep(mesh, shape[0], shape[1], box[0], box[1], out);
}

}  // namespace

// ---------------------------------------------------------------------------
// C-ABI of the oracle (ctypes from tests/ and bench.py only).

extern "C" {

const char* ndfo_last_error() { return g_message.c_str(); }

int ndfo_map_index(int64_t index, uint64_t length, int32_t mode, int64_t* out) {
  int r = map_index(index, (int64_t)length, mode, out);
  return r;
}

double ndfo_midpoint(double lower, double upper) { return midpoint(lower, upper); }
double ndfo_interpolate(double lower, double upper, double fraction) {
  return interpolate(lower, upper, fraction);
}
double ndfo_mean_valid(const double* values, uint64_t n) { return mean_valid(values, n); }
double ndfo_dispersion_valid(const double* values, uint64_t n, uint64_t ddof, int32_t want_std) {
  return dispersion_valid(values, n, ddof, want_std != 0);
}
double ndfo_percentile(const double* values, uint64_t n, double q) {
  std::vector<double> v(values, values + n);
  return percentile(v, q);
}

// Window taps (count * rank offsets, tap-major) for geometry tests.
int ndfo_window_taps(int32_t rank, const uint64_t* shape, const uint64_t* size,
                     const uint8_t* footprint, const int64_t* origin, const int32_t* modes,
                     int64_t* taps_out, uint64_t capacity, uint64_t* count_out) {
  Window w;
  int rc = window_new(rank, shape, size, footprint, origin, modes, &w);
  if (rc) return rc;
  *count_out = w.count;
  if (capacity < w.count * (uint64_t)rank) return kLength;
  std::memcpy(taps_out, w.taps.data(), w.taps.size() * sizeof(int64_t));
  return kOk;
}

// Network comparator count (for the zero-one and pruning tests).
uint64_t ndfo_network_size(uint64_t count, int32_t omit) {
  Policy p;
  p.omit = omit != 0;
  return network_new(count, p).size();
}

// window_filter / robust_filter(kind="percentile") over one C-contiguous
// array; `dtype` 0 = float32, 1 = float64. `kind` uses the C-ABI numbering.
// `direct` != 0 visits every window (the traversal that the separable
// passes must equal bit for bit, as src/extrema.rs:459-894 and
// src/boxcar.rs:344-421 check); 0 follows WindowFilter::new's choice.
int ndfo_filter_ex(int32_t dtype, int32_t rank, const uint64_t* shape, const void* input,
                   void* output, const uint64_t* size, const uint8_t* footprint,
                   const int64_t* origin, const int32_t* modes, double cval, int32_t kind,
                   int32_t omit_nan, int32_t ignore_inf, uint64_t min_count, uint64_t parameter,
                   double q, int32_t threads, int32_t direct) {
  Window w;
  // Histogram and separable plans validate the rectangle without
  // materializing taps (src/plan.rs:267-312 calls validate_rectangular, not
  // Window::new).
  bool hist_plan = kind == kMedianHistogram || kind == kRankHistogram;
  bool separable = !direct && ((!footprint && (kind == kMin || kind == kMax)) || kind == kMeanRolling);
  int rc = window_new(rank, shape, size, footprint, origin, modes, &w, !hist_plan && !separable);
  if (rc) return rc;
  Reduction r;
  r.kind = kind;
  r.policy.omit = omit_nan != 0;
  r.policy.ignore_inf = ignore_inf != 0;
  r.policy.min_count = min_count;
  r.parameter = parameter;
  r.q = q;
  if (r.policy.omit && (min_count == 0 || min_count > w.count))
    return fail(kInvalid, kind == kPercentile
                              ? "min_count must be between one and the number of window elements"
                              : "min_count must be between 1 and the number of window elements");
  if (kind == kPercentile && (!std::isfinite(q) || q < 0.0 || q > 100.0))
    return fail(kInvalid, "percentile must be finite and between zero and 100");
  if (kind == kMeanRolling && footprint)
    return fail(kInvalid, "rolling means require rectangular size, not footprint");
  bool hist = kind == kMedianHistogram || kind == kRankHistogram;
  if (hist) {
    if (footprint)
      return fail(kInvalid, "histogram reductions require rectangular size, not footprint");
    rc = validate_support(w.shape, size);
    if (rc) return rc;
  }
  size_t n = w.out_len;
  if (n == 0) return kOk;
  if (threads < 1) threads = 1;
  bool f32 = dtype == 0;
  if (f32) cval = (double)(float)cval;
  if (hist) {
    bool median = kind == kMedianHistogram;
    if (f32)
      return histogram_filter(w, size, origin, (const float*)input, cval, r.policy, median,
                              parameter, threads, (float*)output);
    return histogram_filter(w, size, origin, (const double*)input, cval, r.policy, median,
                            parameter, threads, (double*)output);
  }
  if (separable) {
    const bool maximum = kind == kMax;
    if (kind == kMeanRolling)
      return f32 ? boxcar_separable(w, size, origin, (const float*)input, cval, r.policy, threads,
                                    (float*)output)
                 : boxcar_separable(w, size, origin, (const double*)input, cval, r.policy,
                                    threads, (double*)output);
    return f32 ? extrema_separable(w, size, origin, (const float*)input, cval, r.policy, maximum,
                                   threads, (float*)output)
               : extrema_separable(w, size, origin, (const double*)input, cval, r.policy,
                                   maximum, threads, (double*)output);
  }
  if (kind == kMeanRolling) {
    auto run = [&](auto tag) {
      using T = decltype(tag);
      run_parallel(n, threads, [&](size_t s, size_t e) {
        std::vector<int64_t> index(w.rank);
        for (size_t center = s; center < e; ++center)
          ((T*)output)[center] = boxcar_window<T>(w, (const T*)input, center, cval, r.policy, index.data());
      });
    };
    if (f32)
      run(float());
    else
      run(double());
    return kOk;
  }
  if (kind == kMedianNetwork) {
    auto net = network_new(w.count, r.policy);
    if (f32) {
      run_parallel(n, threads, [&](size_t s, size_t e) {
        filter_range_network(w, (const float*)input, cval, r, net, s, e, (float*)output + s);
      });
    } else {
      run_parallel(n, threads, [&](size_t s, size_t e) {
        filter_range_network(w, (const double*)input, cval, r, net, s, e, (double*)output + s);
      });
    }
    return kOk;
  }
  if (f32) {
    run_parallel(n, threads, [&](size_t s, size_t e) {
      filter_offsets(w, (const float*)input, cval, r, s, e, (float*)output + s);
    });
  } else {
    run_parallel(n, threads, [&](size_t s, size_t e) {
      filter_offsets(w, (const double*)input, cval, r, s, e, (double*)output + s);
    });
  }
  return kOk;
}

int ndfo_filter(int32_t dtype, int32_t rank, const uint64_t* shape, const void* input,
                void* output, const uint64_t* size, const uint8_t* footprint,
                const int64_t* origin, const int32_t* modes, double cval, int32_t kind,
                int32_t omit_nan, int32_t ignore_inf, uint64_t min_count, uint64_t parameter,
                double q, int32_t threads) {
  return ndfo_filter_ex(dtype, rank, shape, input, output, size, footprint, origin, modes, cval,
                        kind, omit_nan, ignore_inf, min_count, parameter, q, threads, 0);
}

// One robust reduction of `n` float64 samples (the pinned literal tests).
// `kind` is a RobustKind; `maxiters` < 0 clips until stable.
double ndfo_robust_values(int32_t kind, const double* values, uint64_t n, int32_t omit_nan,
                          int32_t ignore_inf, uint64_t min_count, double parameter, double lower,
                          double upper, int64_t maxiters, int32_t center, int32_t spread,
                          int32_t estimator, int32_t modify_sample_size, double pearson) {
  RobustSpec spec;
  spec.kind = kind;
  spec.policy.omit = omit_nan != 0;
  spec.policy.ignore_inf = ignore_inf != 0;
  spec.policy.min_count = min_count;
  spec.parameter = parameter;
  spec.lower = lower;
  spec.upper = upper;
  spec.maxiters = maxiters;
  spec.center = center;
  spec.spread = spread;
  spec.estimator = estimator;
  spec.modify_sample_size = modify_sample_size != 0;
  spec.pearson = pearson;
  spec.clip_min_count = min_count;
  std::vector<double> v(values, values + n);
  return robust_finish(spec, v);
}

// robust_into, src/robust.rs:725-785: every window gathered in tap order as
// float64, reduced, and cast once (NaN as the canonical NaN).
int ndfo_robust_filter(int32_t dtype, int32_t rank, const uint64_t* shape, const void* input,
                       void* output, const uint64_t* size, const uint8_t* footprint,
                       const int64_t* origin, const int32_t* modes, double cval, int32_t kind,
                       int32_t omit_nan, int32_t ignore_inf, uint64_t min_count, double parameter,
                       double lower, double upper, int64_t maxiters, int32_t center, int32_t spread,
                       int32_t estimator, int32_t modify_sample_size, double pearson,
                       int32_t threads) {
  Window w;
  int rc = window_new(rank, shape, size, footprint, origin, modes, &w);
  if (rc) return rc;
  if (min_count == 0 || min_count > w.count)
    return fail(kInvalid, "min_count must be between one and the number of window elements");
  const size_t n = w.out_len;
  if (n == 0) return kOk;
  if (threads < 1) threads = 1;
  const bool f32 = dtype == 0;
  if (f32) cval = (double)(float)cval;
  auto run = [&](auto tag) {
    using T = decltype(tag);
    run_parallel(n, threads, [&](size_t s, size_t e) {
      std::vector<int64_t> index(w.rank);
      std::vector<double> values;
      for (size_t c = s; c < e; ++c) {
        values.clear();
        visit(w, (const T*)input, c, cval, index.data(), [&](double v) { values.push_back(v); });
        const double r = ndfo_robust_values(kind, values.data(), values.size(), omit_nan, ignore_inf,
                                            min_count, parameter, lower, upper, maxiters, center,
                                            spread, estimator, modify_sample_size, pearson);
        ((T*)output)[c] = cast_out<T>(r);
      }
    });
  };
  if (f32)
    run(float());
  else
    run(double());
  return kOk;
}

// MeshBackground::new + estimate + interpolate_into (background and RMS),
// src/background.rs:445-560. Returns the reference's error classes; outputs
// are the two full-resolution maps (dtype of the input), the mesh grids
// (float64, int64 counts, uint8 validity) and the two global medians.
int ndfo_mesh_background(int32_t dtype, int32_t ndim, const uint64_t* shape, const void* input,
                         const uint8_t* mask, const uint64_t* box_size, const uint64_t* filter_size,
                         int32_t estimator, double pearson, double lower, double upper, int64_t maxiters,
                         int32_t center, int32_t spread, int32_t statistic, int32_t mode_estimator,
                         int32_t rms_kind, double min_valid_fraction, int32_t valid_count, int32_t valid_base,
                         int32_t fill, uint64_t idw_neighbors, double idw_power, int32_t filter_edge,
                         int32_t threshold_kind, double threshold, int32_t interpolation, void* out_background,
                         void* out_rms, double* mesh_background, double* mesh_rms, uint8_t* mesh_valid,
                         int64_t* finite_count, int64_t* retained_count, double* globals, int32_t threads) {
  if (ndim <= 0) return fail(kInvalid, "shape must have at least one axis");
  for (int a = 0; a < ndim; ++a)
    if (box_size[a] == 0) return fail(kInvalid, "box sizes must be positive");
  for (int a = 0; a < ndim; ++a)
    if (filter_size[a] % 2 == 0) return fail(kInvalid, "filter sizes must be odd and positive");
  MeshSpec spec;
  spec.estimator = estimator;
  spec.pearson = pearson;
  spec.lower = lower;
  spec.upper = upper;
  spec.maxiters = maxiters;
  spec.center = center;
  spec.spread = spread;
  spec.statistic = statistic;
  spec.mode_estimator = mode_estimator;
  spec.rms = rms_kind;
  spec.min_valid_fraction = min_valid_fraction;
  spec.valid_count = valid_count;
  spec.valid_base = valid_base;
  spec.fill = fill;
  spec.idw_neighbors = idw_neighbors;
  spec.idw_power = idw_power;
  spec.filter_edge = filter_edge;
  spec.threshold_kind = threshold_kind;
  spec.threshold = threshold;
  spec.interpolation = interpolation;
  // MeshConfig::validate, src/background.rs:230-289.
  if (!(std::isfinite(pearson) && pearson >= 1.0))
    return fail(kInvalid, "pearson must be finite and at least one");
  if (estimator == 1 && (!std::isfinite(lower) || !std::isfinite(upper) || lower < 0.0 || upper < 0.0))
    return fail(kInvalid, "clipping limits must be finite and nonnegative");
  if (!(min_valid_fraction >= 0.0 && min_valid_fraction <= 1.0))
    return fail(kInvalid, "minimum valid fraction must be between zero and one");
  if (fill == 1 && (idw_neighbors == 0 || !std::isfinite(idw_power) || idw_power < 0.0))
    return fail(kInvalid,
                "inverse-distance fill needs at least one neighbor and a finite nonnegative power");
  if (threshold_kind != 0 && !std::isfinite(threshold)) return fail(kInvalid, "filter threshold must be finite");
  if (interpolation == 1 && ndim != 2) return fail(kInvalid, "SExtractor interpolation needs a 2-D shape");
  std::vector<size_t> sh(shape, shape + ndim), box(box_size, box_size + ndim), filt(filter_size, filter_size + ndim),
      mesh_shape(ndim);
  size_t len = 1, mesh_len = 1;
  uint64_t box_volume = 1;
  for (int a = 0; a < ndim; ++a) {
    mesh_shape[a] = (sh[a] + box[a] - 1) / box[a];
    len *= sh[a];
    mesh_len *= mesh_shape[a];
    if (box[a] != 0 && box_volume > UINT64_MAX / box[a]) return fail(kOverflow, "box volume overflowed");
    box_volume *= box[a];
  }
  std::vector<MeshStat> stats(mesh_len);
  // Meshes in parallel, as the reference's estimate (src/background.rs:533-541).
  run_parallel(mesh_len, threads, [&](size_t first_mesh, size_t end_mesh) {
  std::vector<size_t> idx(ndim);
  for (size_t mesh = first_mesh; mesh < end_mesh; ++mesh) {
    mesh_index(mesh, mesh_shape, idx.data());
    std::vector<size_t> start(ndim), stop(ndim);
    uint64_t volume = 1;
    for (int a = 0; a < ndim; ++a) {
      start[a] = idx[a] * box[a];
      stop[a] = std::min(start[a] + box[a], sh[a]);
      volume *= stop[a] - start[a];
    }
    std::vector<double> values;
    std::vector<size_t> pos(start);
    if (volume > 0) {
      while (true) {
        size_t offset = 0;
        for (int a = 0; a < ndim; ++a) offset = offset * sh[a] + pos[a];
        const double v = dtype == 0 ? (double)((const float*)input)[offset] : ((const double*)input)[offset];
        if (std::isfinite(v) && !(mask && mask[offset])) values.push_back(v);
        int a = ndim - 1;
        for (; a >= 0; --a) {
          if (++pos[a] < stop[a]) break;
          pos[a] = start[a];
        }
        if (a < 0) break;
      }
    }
    stats[mesh] = mesh_finish(values, volume, box_volume, spec);
  }
  });
  std::vector<double> bg(mesh_len), rms(mesh_len);
  std::vector<bool> valid(mesh_len);
  for (size_t i = 0; i < mesh_len; ++i) {
    bg[i] = stats[i].background;
    rms[i] = stats[i].rms;
    valid[i] = stats[i].valid;
  }
  mesh_fill(bg, rms, valid, mesh_shape, spec);
  mesh_filter(bg, rms, mesh_shape, filt, spec);
  for (size_t i = 0; i < mesh_len; ++i) {
    mesh_background[i] = bg[i];
    mesh_rms[i] = rms[i];
    mesh_valid[i] = valid[i] ? 1 : 0;
    finite_count[i] = (int64_t)stats[i].finite;
    retained_count[i] = (int64_t)stats[i].retained;
  }
  globals[0] = mesh_median_of(bg);
  globals[1] = mesh_median_of(rms);
  if (dtype == 0) {
    mesh_interpolate(bg, sh, mesh_shape, box, spec, (float*)out_background);
    mesh_interpolate(rms, sh, mesh_shape, box, spec, (float*)out_rms);
  } else {
    mesh_interpolate(bg, sh, mesh_shape, box, spec, (double*)out_background);
    mesh_interpolate(rms, sh, mesh_shape, box, spec, (double*)out_rms);
  }
  return kOk;
}

// Exact (double-double) mean/var/std of every window, rounded to float64,
// for the precision study. `kind` is kMean, kVar or kStd. Output is float64.
int ndfo_exact_moments(int32_t dtype, int32_t rank, const uint64_t* shape, const void* input,
                       double* output, const uint64_t* size, const uint8_t* footprint,
                       const int64_t* origin, const int32_t* modes, double cval, int32_t kind,
                       int32_t omit_nan, int32_t ignore_inf, uint64_t min_count, uint64_t ddof,
                       int32_t threads) {
  Window w;
  int rc = window_new(rank, shape, size, footprint, origin, modes, &w);
  if (rc) return rc;
  Policy p;
  p.omit = omit_nan != 0;
  p.ignore_inf = ignore_inf != 0;
  p.min_count = min_count;
  if (dtype == 0) cval = (double)(float)cval;
  size_t n = w.out_len;
  auto body = [&](auto tag, size_t s, size_t e) {
    using T = decltype(tag);
    const T* in = (const T*)input;
    std::vector<int64_t> index(w.rank);
    std::vector<double> values;
    for (size_t c = s; c < e; ++c) {
      values.clear();
      bool nan = false;
      visit(w, in, c, cval, index.data(), [&](double v) {
        if (std::isnan(v)) {
          nan = nan || !p.omit;
          return;
        }
        if (p.omit && p.ignore_inf && !std::isfinite(v)) return;
        values.push_back(v);
      });
      if (nan || (p.omit && values.size() < p.min_count)) {
        output[c] = kNaN64;
        continue;
      }
      output[c] = exact_moment(values, kind, ddof);
    }
  };
  if (dtype == 0)
    run_parallel(n, threads, [&](size_t s, size_t e) { body(float{}, s, e); });
  else
    run_parallel(n, threads, [&](size_t s, size_t e) { body(double{}, s, e); });
  return kOk;
}

}  // extern "C"

// Window moments (mean / var / std) device code shared by the single-image
// and batched kernels. See moments.cu for the two arithmetic paths.
#pragma once

#include "common.cuh"
#include "network.cuh"
#include "plan.h"
#include "staging.cuh"

namespace ndf {
namespace mom {


// ---------------------------------------------------------------------------
// Reference float64 path. `fetch(i)` returns tap i as float64.

template <typename Fetch>
__device__ double mean_exact(Fetch&& fetch, const Reduce& r) {
  const int V = r.count;
  Sum64 sum;
  long long count = 0;
  bool nan = false, pinf = false, ninf = false;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (isnan(v)) {
      nan = nan || !r.omit;
      continue;
    }
    if (r.drop_inf && isinf(v)) continue;
    count += 1;
    if (isinf(v)) {
      pinf = pinf || v > 0;
      ninf = ninf || v < 0;
    } else {
      sum.add(v);
    }
  }
  if (nan || count == 0 || (r.omit && count < r.min_count)) return nan_of(0.0);
  if (pinf || ninf) {
    if (pinf && ninf) return nan_of(0.0);
    return pinf ? __longlong_as_double(0x7ff0000000000000ll)
                : __longlong_as_double((long long)0xfff0000000000000ull);
  }
  double total = sum.total();
  if (isfinite(total)) return __ddiv_rn(total, (double)count);
  // Finite overflow: mean_valid's power-of-two rescaling (src/mean.rs:87-113).
  unsigned long long m = (unsigned long long)(count - 1);
  int exponent = (m == 0 ? 0 : 64 - __clzll((long long)m)) + 1;
  double scale = ldexp(1.0, exponent);
  Sum64 scaled;
  double lower = __longlong_as_double(0x7ff0000000000000ll);
  double upper = -lower;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (isnan(v) || (r.drop_inf && isinf(v))) continue;
    lower = fmin(lower, v);
    upper = fmax(upper, v);
    scaled.add(__ddiv_rn(v, scale));
  }
  double result = __ddiv_rn(__dadd_rn(scaled.value, scaled.correction), __ddiv_rn((double)count, scale));
  return clamp64(result, lower, upper);
}

template <typename Fetch>
__device__ double dispersion_exact(Fetch&& fetch, const Reduce& r, bool want_std) {
  const int V = r.count;
  long long n = 0;
  bool nan = false, nonfinite = false, halve = false;
  double ref = 0.0;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (isnan(v)) {
      nan = nan || !r.omit;
      continue;
    }
    if (r.drop_inf && isinf(v)) continue;
    if (n == 0) ref = v;
    n += 1;
    nonfinite = nonfinite || !isfinite(v);
    halve = halve || !isfinite(__dsub_rn(v, ref));
  }
  if (nan || (r.omit && n < r.min_count)) return nan_of(0.0);
  if (n <= r.param || nonfinite) return nan_of(0.0);
  auto delta = [&](double v) {
    return halve ? __dsub_rn(__ddiv_rn(v, 2.0), __ddiv_rn(ref, 2.0)) : __dsub_rn(v, ref);
  };
  auto kept = [&](double v) { return !isnan(v) && !(r.drop_inf && isinf(v)); };
  double scale = 0.0;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (kept(v)) scale = fmax(scale, fabs(delta(v)));
  }
  if (scale == 0.0) return 0.0;
  Sum64 sum;
  const Divisor by = make_divisor(scale);
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (kept(v)) sum.add(div_by(delta(v), by));
  }
  double center = __ddiv_rn(sum.total(), (double)n);
  Sum64 squares;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (!kept(v)) continue;
    double residual = __dsub_rn(div_by(delta(v), by), center);
    squares.add(__dmul_rn(residual, residual));
  }
  double normalized = __ddiv_rn(squares.total(), (double)(n - r.param));
  if (want_std) {
    double result = __dmul_rn(scale, __dsqrt_rn(normalized));
    return halve ? __dmul_rn(result, 2.0) : result;
  }
  double result = __dmul_rn(scale, __dmul_rn(scale, normalized));
  return halve ? __dmul_rn(result, 4.0) : result;
}

template <typename Fetch>
__device__ __forceinline__ double moments_exact(Fetch&& fetch, const Reduce& r) {
  if (r.kind == kMean) return mean_exact(fetch, r);
  return dispersion_exact(fetch, r, r.kind == kStd);
}

// ---------------------------------------------------------------------------
// FP32 compensated path.

// Neumaier sum in FP32.
struct Sum32 {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    float t = __fadd_rn(s, x);
    float e = fabsf(s) >= fabsf(x) ? __fadd_rn(__fsub_rn(s, t), x) : __fadd_rn(__fsub_rn(x, t), s);
    c = __fadd_rn(c, e);
    s = t;
  }
};

// Float-float sum (hi + lo, renormalized after every addition).
struct SumFF {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float xh, float xl) {
    float s = __fadd_rn(hi, xh);
    float bp = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(xh, bp));
    e = __fadd_rn(e, __fadd_rn(lo, xl));
    hi = __fadd_rn(s, e);
    lo = __fsub_rn(e, __fsub_rn(hi, s));
  }
};

// Exact a - b as hi + lo (two-sum).
__device__ __forceinline__ void two_diff(float a, float b, float& hi, float& lo) {
  hi = __fsub_rn(a, b);
  float bp = __fsub_rn(hi, a);
  lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bp)), __fsub_rn(-b, bp));
}

// Deviations whose squares stay inside FP32's normal range without loss.
constexpr float kSafeLow = 1.0e-12f;
constexpr float kSafeHigh = 1.0e15f;

// Final combine in FP64. Returns false to request the FP64 path.
__device__ __forceinline__ bool combine(const Reduce& r, long long n, double p, double s1,
                                        double s2, double* out) {
  if (r.kind == kMean) {
    double m = p + s1 / (double)n;
    if (!isfinite(m)) return false;
    *out = m;
    return true;
  }
  double ss = s2 - s1 * (s1 / (double)n);
  if (!isfinite(ss)) return false;
  if (ss < 0.0) ss = 0.0;
  double var = ss / (double)(n - r.param);
  *out = r.kind == kStd ? sqrt(var) : var;
  return isfinite(*out);
}

// Classify a window the way the reference does before any arithmetic.
// Returns 1 = result decided (*out set), 0 = finite arithmetic needed.
__device__ __forceinline__ int decide_special(const Reduce& r, long long n, bool nan, bool pinf,
                                              bool ninf, double* out) {
  if (nan || n == 0 || (r.omit && n < r.min_count)) {
    *out = nan_of(0.0);
    return 1;
  }
  if (r.kind == kMean) {
    if (pinf || ninf) {
      *out = (pinf && ninf) ? nan_of(0.0)
                            : (pinf ? __longlong_as_double(0x7ff0000000000000ll)
                                    : __longlong_as_double((long long)0xfff0000000000000ull));
      return 1;
    }
    return 0;
  }
  if (n <= r.param || pinf || ninf) {
    *out = nan_of(0.0);
    return 1;
  }
  return 0;
}

// Kahan sum in FP32: s - c is the running total.
struct Kahan32 {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// float32 input: samples staged as float. `visit(f)` calls f(v) for every
// tap of the window; `first(i)` returns tap i (for the pivot search).
//
// Every retained sample is shifted by the pivot p (the window's first finite
// retained sample) exactly, as a two-sum (dh + dl = v - p); the sums of dh
// and of dh^2 run as Kahan sums, and the rounding parts (dl, and the
// two-product error of dh^2 plus 2 dh dl) are summed plainly: their total
// is below an ulp of the result's scale.
template <typename Visit, typename First>
__device__ __forceinline__ bool moments_fp32c_f32(Visit&& visit, First&& first, const Reduce& r,
                                                  double* out) {
  const int V = r.count;
  const float kInf = __uint_as_float(0x7f800000u);
  float p = 0.0f;
  for (int i = 0; i < V; ++i) {
    const float v = first(i);
    if (fabsf(v) < kInf) {
      p = v;
      break;
    }
  }
  int n = 0;
  bool nan = false, pinf = false, ninf = false;
  float maxdev = 0.0f, c1 = 0.0f, c2 = 0.0f;
  Kahan32 s1, s2;
  const bool omit = r.omit, drop_inf = r.drop_inf;
  visit([&](float v) {
    if (!(fabsf(v) < kInf)) {
      if (isnan(v)) {
        nan = nan || !omit;
      } else if (!drop_inf) {
        n += 1;
        pinf = pinf || v > 0.0f;
        ninf = ninf || v < 0.0f;
      }
      return;
    }
    n += 1;
    float dh, dl;
    two_diff(v, p, dh, dl);
    maxdev = fmaxf(maxdev, fabsf(dh));
    s1.add(dh);
    c1 = __fadd_rn(c1, dl);
    const float sq = __fmul_rn(dh, dh);
    float sqe = fmaf(dh, dh, -sq);
    sqe = fmaf(__fmul_rn(2.0f, dh), dl, sqe);
    s2.add(sq);
    c2 = __fadd_rn(c2, sqe);
  });
  (void)V;
  if (decide_special(r, n, nan, pinf, ninf, out)) return true;
  if (maxdev != 0.0f && (maxdev < kSafeLow || maxdev > kSafeHigh || !isfinite(maxdev))) return false;
  const double S1 = s1.value() + (double)c1;
  const double S2 = s2.value() + (double)c2;
  return combine(r, n, (double)p, S1, S2, out);
}

// float64 input: samples staged as triple floats (hi, mid, lo), exact for
// values inside FP32's exponent range.
struct Triple {
  float h, m, l;
};

template <typename FetchT>
__device__ __forceinline__ bool moments_fp32c_f64(FetchT&& fetch, const Reduce& r, double* out) {
  const int V = r.count;
  long long n = 0;
  bool nan = false, pinf = false, ninf = false, unsafe = false;
  Triple p{0.0f, 0.0f, 0.0f};
  bool have_p = false;
  float maxdev = 0.0f;
  // Blocked float-float sums: 32 terms per inner sum, then an outer sum, so
  // rounding errors accumulate over ~2 * sqrt-like chains instead of V.
  SumFF s1, s2, b1, b2;
  int block = 0;
  for (int i = 0; i < V; ++i) {
    Triple x = fetch(i);
    // NaN / infinity / out-of-range values are staged with x.m as a marker:
    // h holds the float64 classification (NaN, +-inf, or a finite value
    // FP32 cannot split exactly, flagged by m = NaN).
    if (isnan(x.h)) {
      nan = nan || !r.omit;
      continue;
    }
    if (isinf(x.h)) {
      if (r.drop_inf) continue;
      n += 1;
      pinf = pinf || x.h > 0;
      ninf = ninf || x.h < 0;
      continue;
    }
    if (isnan(x.m)) unsafe = true;
    if (!have_p) {
      p = x;
      have_p = true;
    }
    n += 1;
    // d = x - p as float-float: two-sums per component, then renormalize.
    float ah, al, bh, bl;
    two_diff(x.h, p.h, ah, al);
    two_diff(x.m, p.m, bh, bl);
    float cl = __fsub_rn(x.l, p.l);
    float sh = __fadd_rn(ah, bh);
    float bp = __fsub_rn(sh, ah);
    float se = __fadd_rn(__fsub_rn(ah, __fsub_rn(sh, bp)), __fsub_rn(bh, bp));
    se = __fadd_rn(se, __fadd_rn(__fadd_rn(al, bl), cl));
    float dh = __fadd_rn(sh, se);
    float dl = __fsub_rn(se, __fsub_rn(dh, sh));
    maxdev = fmaxf(maxdev, fabsf(dh));
    b1.add(dh, dl);
    float sq = __fmul_rn(dh, dh);
    float sqe = fmaf(dh, dh, -sq);
    sqe = fmaf(__fmul_rn(2.0f, dh), dl, sqe);
    sqe = fmaf(dl, dl, sqe);
    b2.add(sq, sqe);
    if (++block == 32) {
      s1.add(b1.hi, b1.lo);
      s2.add(b2.hi, b2.lo);
      b1 = SumFF{};
      b2 = SumFF{};
      block = 0;
    }
  }
  s1.add(b1.hi, b1.lo);
  s2.add(b2.hi, b2.lo);
  if (decide_special(r, n, nan, pinf, ninf, out)) return true;
  if (unsafe) return false;
  if (maxdev != 0.0f && (maxdev < kSafeLow || maxdev > kSafeHigh || !isfinite(maxdev))) return false;
  double pd = ((double)p.h + (double)p.m) + (double)p.l;
  double S1 = (double)s1.hi + (double)s1.lo;
  double S2 = (double)s2.hi + (double)s2.lo;
  return combine(r, n, pd, S1, S2, out);
}

// Split a float64 into three floats (exact when the value and its tail stay
// in FP32's normal range). Marks values outside that range with m = NaN.
__device__ __forceinline__ Triple split3(double x) {
  if (isnan(x)) return {__uint_as_float(0x7fc00000u), 0.0f, 0.0f};
  if (isinf(x)) return {x > 0 ? __uint_as_float(0x7f800000u) : __uint_as_float(0xff800000u), 0.0f, 0.0f};
  double ax = fabs(x);
  if (ax != 0.0 && (ax > 1.0e30 || ax < 1.0e-20))
    return {(float)(x > 0 ? 1.0f : -1.0f), __uint_as_float(0x7fc00000u), 0.0f};
  float h = __double2float_rn(x);
  double r1 = __dsub_rn(x, (double)h);
  float m = __double2float_rn(r1);
  float l = __double2float_rn(__dsub_rn(r1, (double)m));
  return {h, m, l};
}


// One output tile of the moments kernel; `taps` are shared-memory offsets
// relative to a thread's output.
template <typename T, int PREC>
__device__ __forceinline__ void tile_moments_body(const T* __restrict__ in, T* __restrict__ out,
                                                  const TileArgs& a, long long tile,
                                                  unsigned char* smem_raw, const int32_t* taps,
                                                  const CUtensorMap* tmap = nullptr) {
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const int support = g.kd * t.SH * t.SW;
  long long z, y0, x0;
  net::tile_coords(a, tile, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, (T)a.r.cval, [](T v) { return v; })) return;
  Triple* s3 = reinterpret_cast<Triple*>(s + support);
  // Tap offsets in shared memory (broadcast reads), after the staged values.
  const size_t staged = (size_t)support * sizeof(T) + (PREC == 0 && sizeof(T) == 8 ? (size_t)support * sizeof(Triple) : 0);
  int32_t* taps_s = reinterpret_cast<int32_t*>(
      reinterpret_cast<unsigned char*>(s) + ((staged + 15) & ~(size_t)15));
  for (int i = threadIdx.x; i < a.r.count; i += blockDim.x) taps_s[i] = taps[i];
  taps = taps_s;
  if constexpr (PREC == 0 && sizeof(T) == 8) {
    __syncthreads();
    for (int i = threadIdx.x; i < support; i += blockDim.x) s3[i] = split3((double)s[i]);
  }
  __syncthreads();
  const int tx = threadIdx.x % t.TW;
  const int ty = threadIdx.x / t.TW;
  const long long y = y0 + ty, x = x0 + tx;
  if (ty >= t.TH || y >= g.H || x >= g.W) return;
  const int base = ty * t.SW + tx;
  auto fetch64 = [&](int i) -> double { return (double)s[base + taps[i]]; };
  double result;
  bool done = false;
  if constexpr (PREC == 0) {
    if constexpr (sizeof(T) == 4) {
      auto fetch32 = [&](int i) -> float { return (float)s[base + taps[i]]; };
      if (g.kd * g.kh * g.kw == a.r.count) {
        // A full box: taps in row-major order without the offset table.
        const int plane = t.SH * t.SW;
        auto visit = [&](auto&& f) {
          for (int kz = 0; kz < g.kd; ++kz)
            for (int ky = 0; ky < g.kh; ++ky) {
              const T* row = s + base + kz * plane + ky * t.SW;
#pragma unroll 4
              for (int kx = 0; kx < g.kw; ++kx) f((float)row[kx]);
            }
        };
        done = moments_fp32c_f32(visit, fetch32, a.r, &result);
      } else {
        auto visit = [&](auto&& f) {
#pragma unroll 4
          for (int i = 0; i < a.r.count; ++i) f((float)s[base + taps[i]]);
        };
        done = moments_fp32c_f32(visit, fetch32, a.r, &result);
      }
    } else {
      auto fetch3 = [&](int i) -> Triple { return s3[base + taps[i]]; };
      done = moments_fp32c_f64(fetch3, a.r, &result);
    }
  }
  if (!done) result = moments_exact(fetch64, a.r);
  out[(z * g.H + y) * g.W + x] = canonical(from_f64<T>(result));
}

}  // namespace mom
}  // namespace ndf

// Window moments (mean / var / std) device code shared by the single-image
// and batched kernels. See moments.cu for the two arithmetic paths.
#pragma once

#include "common.cuh"
#include "exact.cuh"
#include "fixed_moments.cuh"
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

// ---------------------------------------------------------------------------
// FP32C path for any footprint: exact fixed-point window sums (the
// arithmetic of fixed_moments.cuh).
//
// Per tile the block finds the support's pivot and bit span and stages every
// sample's deviation X = x - P as an exact 64-bit integer (plus, when the
// support holds NaN or infinities, the sample's 16-bit-field count
// increment); each thread then sums X and X^2 over its window's taps in
// integers (32-bit deviations and 64-bit sums when the span allows, 64 / 128
// bits otherwise) and finishes with fixed_combine. Tiles whose span does not
// fit the integer widths, and windows of 65,535 taps or more, take the
// reference float64 path.
constexpr int kMomentThreads = 256;

template <bool NARROW, bool COUNT, typename Visit>
__device__ __forceinline__ void fixed_sums(Visit&& visit, fixm::i128& s1, fixm::u128& s2,
                                           unsigned long long& cnt) {
  if constexpr (NARROW) {
    long long a1 = 0;
    unsigned long long a2 = 0;
    visit([&](long long x, unsigned long long c) {
      const int xi = (int)x;
      a1 += xi;
      a2 += (unsigned long long)((long long)xi * xi);
      if (COUNT) cnt += c;
    });
    s1 = a1;
    s2 = a2;
  } else {
    fixm::i128 a1 = 0;
    fixm::u128 a2 = 0;
    visit([&](long long x, unsigned long long c) {
      a1 += x;
      a2 += (fixm::u128)((fixm::i128)x * x);
      if (COUNT) cnt += c;
    });
    s1 = a1;
    s2 = a2;
  }
}

// One output tile of the moments kernel; `taps` are shared-memory offsets
// relative to a thread's output. The block has kMomentThreads threads.
template <typename T, int PREC>
__device__ __forceinline__ void tile_moments_body(const T* __restrict__ in, T* __restrict__ out,
                                                  const TileArgs& a, long long tile,
                                                  unsigned char* smem_raw, const int32_t* taps,
                                                  const CUtensorMap* tmap = nullptr) {
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Reduce& r = a.r;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const int support = g.kd * t.SH * t.SW;
  long long z, y0, x0;
  net::tile_coords(a, tile, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, (T)r.cval, [](T v) { return v; })) return;
  // Layout after the staged values (16-byte aligned): deviations X (i64) and
  // count increments (u64) of the FP32C path, then the tap offsets.
  const size_t xs_offset = ((size_t)support * sizeof(T) + 15) & ~(size_t)15;
  long long* xs = reinterpret_cast<long long*>(reinterpret_cast<unsigned char*>(s) + xs_offset);
  unsigned long long* cs = reinterpret_cast<unsigned long long*>(xs + support);
  const size_t staged = xs_offset + (PREC == 0 ? (size_t)support * 16 : 0);
  int32_t* taps_s = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(s) + staged);
  for (int i = threadIdx.x; i < r.count; i += blockDim.x) taps_s[i] = taps[i];
  taps = taps_s;
  __syncthreads();
  const int tx = threadIdx.x % t.TW;
  const int ty = threadIdx.x / t.TW;
  const long long y = y0 + ty, x = x0 + tx;
  const bool active = ty < t.TH && y < g.H && x < g.W;
  const int base = ty * t.SW + tx;
  const bool box = g.kd * g.kh * g.kw == r.count;
  if constexpr (PREC == 0) {
    const int count_bits = 32 - __clz(r.count + 1);
    const fixm::Span<T> sp = fixm::tile_span<T, kMomentThreads>(s, support);
    if (r.count < 65535 && fixm::span_fits(sp, count_bits)) {
      const int lo = sp.lo;
      const fixm::i128 P = fixm::fixed(sp.pivot, lo);
      const bool count = !sp.all_finite;
      for (int e = threadIdx.x; e < support; e += blockDim.x) {
        const T v = s[e];
        xs[e] = isfinite(v) ? (long long)(fixm::fixed(v, lo) - P) : 0ll;
        if (count) cs[e] = exact::sample_counts(v, r.omit, r.drop_inf);
      }
      __syncthreads();
      if (!active) return;
      const int plane = t.SH * t.SW;
      auto visit = [&](auto&& f) {
        if (box) {
          for (int kz = 0; kz < g.kd; ++kz)
            for (int ky = 0; ky < g.kh; ++ky) {
              const int row = base + kz * plane + ky * t.SW;
#pragma unroll 4
              for (int kx = 0; kx < g.kw; ++kx) f(xs[row + kx], count ? cs[row + kx] : 0ull);
            }
        } else {
#pragma unroll 4
          for (int i = 0; i < r.count; ++i) {
            const int o = base + taps[i];
            f(xs[o], count ? cs[o] : 0ull);
          }
        }
      };
      const int bits = fixm::deviation_bits(sp);
      const bool narrow = bits <= 31 && 2 * bits + count_bits <= 63;
      fixm::i128 s1;
      fixm::u128 s2;
      unsigned long long cnt = 0;
      if (narrow) {
        if (count)
          fixed_sums<true, true>(visit, s1, s2, cnt);
        else
          fixed_sums<true, false>(visit, s1, s2, cnt);
      } else {
        if (count)
          fixed_sums<false, true>(visit, s1, s2, cnt);
        else
          fixed_sums<false, false>(visit, s1, s2, cnt);
      }
      if (!count) cnt = (unsigned long long)r.count;
      const unsigned int finite = (unsigned int)(cnt & 0xFFFF), nanc = (unsigned int)((cnt >> 16) & 0xFFFF);
      const unsigned int pos = (unsigned int)((cnt >> 32) & 0xFFFF), neg = (unsigned int)(cnt >> 48);
      double special;
      const long long index = (z * g.H + y) * g.W + x;
      if (decide_special(r, (long long)finite + pos + neg, nanc != 0, pos != 0, neg != 0, &special))
        out[index] = canonical(from_f64<T>(special));
      else
        out[index] = canonical(fixm::fixed_combine<T>(r.kind, r.param, s1, s2, finite, P, sp.e0() + lo));
      return;
    }
  }
  if (!active) return;
  auto fetch64 = [&](int i) -> double { return (double)s[base + taps[i]]; };
  out[(z * g.H + y) * g.W + x] = canonical(from_f64<T>(moments_exact(fetch64, r)));
}

}  // namespace mom
}  // namespace ndf

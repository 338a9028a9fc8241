// Window moments: mean, variance and standard deviation.
//
// Two arithmetic paths:
//  * NDF_MOMENTS_FP64 restates the reference's float64 algorithms operation
//    for operation: the streaming Neumaier mean in tap order with infinity
//    flags and the scaled overflow retry (src/filter_nd.rs:142-158,
//    src/mean.rs:28-113), and dispersion_valid (src/dispersion.rs:5-61).
//    Results are bit-identical to the reference.
//  * NDF_MOMENTS_FP32C (default) shifts every retained sample by the
//    window's pivot (its first retained sample, as dispersion_valid does)
//    and accumulates the deviation sums in FP32 with error-free
//    transformations: two-sum deviations, two-product squares, Neumaier sums
//    (float32 input) or float-float sums over triple-float staged values
//    (float64 input). FP64 runs only in the final combine (mean = p + S1/n,
//    var = (S2 - S1^2/n) / (n - ddof), sqrt). Windows whose deviations leave
//    the range where FP32 squares are safe fall back to the FP64 path.
#include "common.cuh"
#include "plan.h"
#include "staging.cuh"

namespace ndf {
namespace {

constexpr int kThreads = 256;

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
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (kept(v)) sum.add(__ddiv_rn(delta(v), scale));
  }
  double center = __ddiv_rn(sum.total(), (double)n);
  Sum64 squares;
  for (int i = 0; i < V; ++i) {
    double v = fetch(i);
    if (!kept(v)) continue;
    double residual = __dsub_rn(__ddiv_rn(delta(v), scale), center);
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

// float32 input: samples staged as float.
template <typename FetchF>
__device__ __forceinline__ bool moments_fp32c_f32(FetchF&& fetch, const Reduce& r, double* out) {
  const int V = r.count;
  long long n = 0;
  bool nan = false, pinf = false, ninf = false;
  float p = 0.0f, maxdev = 0.0f;
  bool have_p = false;
  Sum32 s1, s2;
  float c1 = 0.0f, c2 = 0.0f;
  for (int i = 0; i < V; ++i) {
    float v = fetch(i);
    if (isnan(v)) {
      nan = nan || !r.omit;
      continue;
    }
    if (isinf(v)) {
      if (r.drop_inf) continue;
      n += 1;
      pinf = pinf || v > 0;
      ninf = ninf || v < 0;
      continue;
    }
    if (!have_p) {
      p = v;
      have_p = true;
    }
    n += 1;
    float dh, dl;
    two_diff(v, p, dh, dl);
    maxdev = fmaxf(maxdev, fabsf(dh));
    s1.add(dh);
    c1 = __fadd_rn(c1, dl);
    float sq = __fmul_rn(dh, dh);
    float sqe = fmaf(dh, dh, -sq);
    sqe = fmaf(__fmul_rn(2.0f, dh), dl, sqe);
    s2.add(sq);
    c2 = __fadd_rn(c2, sqe);
  }
  if (decide_special(r, n, nan, pinf, ninf, out)) return true;
  if (maxdev != 0.0f && (maxdev < kSafeLow || maxdev > kSafeHigh || !isfinite(maxdev))) return false;
  double S1 = ((double)s1.s + (double)s1.c) + (double)c1;
  double S2 = ((double)s2.s + (double)s2.c) + (double)c2;
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
  SumFF s1, s2;
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
    s1.add(dh, dl);
    float sq = __fmul_rn(dh, dh);
    float sqe = fmaf(dh, dh, -sq);
    sqe = fmaf(__fmul_rn(2.0f, dh), dl, sqe);
    sqe = fmaf(dl, dl, sqe);
    s2.add(sq, sqe);
  }
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

__device__ __forceinline__ void tile_coords(const TileArgs& a, long long& z, long long& y0,
                                            long long& x0) {
  long long tile = blockIdx.x;
  long long tx = tile % a.t.tiles_x;
  long long rest = tile / a.t.tiles_x;
  long long ty = rest % a.t.tiles_y;
  z = rest / a.t.tiles_y;
  y0 = ty * a.t.TH;
  x0 = tx * a.t.TW;
}

template <typename T, int PREC>
__global__ void __launch_bounds__(kThreads)
    tile_moments_kernel(const T* __restrict__ in, T* __restrict__ out,
                        const __grid_constant__ TileArgs a, const int32_t* __restrict__ taps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const int support = g.kd * t.SH * t.SW;
  long long z, y0, x0;
  tile_coords(a, z, y0, x0);
  build_maps(maps, g, t, z, y0, x0);
  __syncthreads();
  stage_support(s, maps, in, g, t, (T)a.r.cval, [](T v) { return v; });
  Triple* s3 = reinterpret_cast<Triple*>(s + support);
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
  auto fetch64 = [&](int i) -> double { return (double)s[base + __ldg(taps + i)]; };
  double result;
  bool done = false;
  if constexpr (PREC == 0) {
    if constexpr (sizeof(T) == 4) {
      auto fetch32 = [&](int i) -> float { return (float)s[base + __ldg(taps + i)]; };
      done = moments_fp32c_f32(fetch32, a.r, &result);
    } else {
      auto fetch3 = [&](int i) -> Triple { return s3[base + __ldg(taps + i)]; };
      done = moments_fp32c_f64(fetch3, a.r, &result);
    }
  }
  if (!done) result = moments_exact(fetch64, a.r);
  out[(z * g.H + y) * g.W + x] = canonical(from_f64<T>(result));
}

// Generic N-D gather (rank > 3 or supports beyond shared memory): the FP64
// path, taps mapped per axis as in Window::visit (src/window.rs:232-294).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    generic_moments_kernel(const T* __restrict__ in, T* __restrict__ out,
                           const __grid_constant__ GenericArgs a,
                           const long long* __restrict__ taps) {
  const int rank = a.rank;
  const long long* flat = taps + (long long)a.r.count * rank;
  const double cval = a.r.cval;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < a.n_out;
       o += (long long)gridDim.x * blockDim.x) {
    long long coord[kMaxGenericRank];
    long long rem = o;
    bool interior = true;
    for (int d = 0; d < rank; ++d) {
      coord[d] = rem / a.stride[d];
      rem -= coord[d] * a.stride[d];
      interior = interior && coord[d] + a.low[d] >= 0 && coord[d] + a.high[d] < a.shape[d];
    }
    auto fetch = [&](int i) -> double {
      if (interior) return (double)__ldg(in + o + flat[i]);
      const long long* tap = taps + (long long)i * rank;
      long long src = 0;
      for (int d = 0; d < rank; ++d) {
        long long m;
        if (!map_index(coord[d] + tap[d], a.shape[d], a.mode[d], &m)) return cval;
        src += m * a.stride[d];
      }
      return (double)__ldg(in + src);
    };
    out[o] = canonical(from_f64<T>(moments_exact(fetch, a.r)));
  }
}

template <typename T, int PREC>
cudaError_t launch_tile_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  auto kernel = tile_moments_kernel<T, PREC>;
  cudaError_t e =
      allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  kernel<<<(unsigned)p.tile.t.tiles, kThreads, p.smem_bytes, s>>>(in, out, p.tile, p.d_tile_taps);
  return cudaGetLastError();
}

}  // namespace

size_t tile_moments_smem(const Plan& p, const Tile& t) {
  size_t elem = p.dtype == 0 ? 4 : 8;
  size_t support = (size_t)p.tile.g.kd * t.SH * t.SW;
  size_t bytes = (size_t)(t.SW + t.SH + p.tile.g.kd) * 8 + support * elem;
  if (p.dtype == 1 && p.r.moments == 0) bytes += support * sizeof(Triple);
  return bytes;
}

cudaError_t launch_tile_moments(const Plan& p, const void* in, void* out, cudaStream_t s) {
  const bool fp64 = p.r.moments == 1;
  if (p.dtype == 0)
    return fp64 ? launch_tile_t<float, 1>(p, (const float*)in, (float*)out, s)
                : launch_tile_t<float, 0>(p, (const float*)in, (float*)out, s);
  return fp64 ? launch_tile_t<double, 1>(p, (const double*)in, (double*)out, s)
              : launch_tile_t<double, 0>(p, (const double*)in, (double*)out, s);
}

cudaError_t launch_generic_moments(const Plan& p, const void* in, void* out, cudaStream_t s) {
  long long blocks = (p.n_out + kThreads - 1) / kThreads;
  long long cap = (long long)p.sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (p.dtype == 0)
    generic_moments_kernel<float><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const float*)in, (float*)out, p.generic, p.d_gen_taps);
  else
    generic_moments_kernel<double><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const double*)in, (double*)out, p.generic, p.d_gen_taps);
  return cudaGetLastError();
}

}  // namespace ndf

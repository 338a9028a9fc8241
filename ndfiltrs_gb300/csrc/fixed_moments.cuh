// Exact fixed-point window moments: the arithmetic shared by the sliding
// moments kernel (moments_slide.cu, rectangular windows) and the tile
// moments kernel (moments.cuh, any footprint) in the FP32C mode.
//
// Per tile, a pivot P (the support's first finite sample) and the lowest set
// bit of the support's finite samples turn every deviation x - P into an
// exact signed integer X; window sums of X (128-bit) and X^2 (unsigned
// 128-bit) are exact under addition and subtraction in any order. The mean is
// the exact window sum n P + S1 divided once by n; the variance's numerator
// n S2 - S1^2 is formed exactly in 192 bits, so no cancellation can lose
// bits. Float32 outputs finish in float-float arithmetic on the FP32 pipe;
// float64 outputs use FP64 only for the conversion of the exact integers, the
// division, the power-of-two scaling and the square root.
#pragma once

#include <climits>

#include "exact.cuh"
#include "plan.h"

namespace ndf {
namespace fixm {

using namespace exact;
using i128 = __int128;
using u128 = unsigned __int128;

// |x| as float64 exponent (floor(log2|x|)) from the bits; -1075 for zero.
__device__ __forceinline__ int exponent_of(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  if (b == 0) return -1075;
  const int e = (int)(b >> 52);
  if (e) return e - 1023;
  return -1074 + (63 - __clzll((long long)b));  // subnormal
}

// 2^k as float64 for -1074 <= k <= 1023.
__device__ __forceinline__ double pow2(int k) {
  if (k >= -1022) return __longlong_as_double((long long)(k + 1023) << 52);
  return __longlong_as_double(1ll << (k + 1074));
}

// Exact signed integer value of a finite sample in units of 2^(E0 + lo)
// (the sample's lowest set bit is at or above lo and its top bit below
// lo + 126).
template <typename T>
__device__ __forceinline__ i128 fixed(T v, int lo) {
  unsigned long long m;
  int pos;
  bool neg;
  if (!decompose(v, m, pos, neg)) return 0;
  const i128 x = (i128)((u128)m << (pos - lo));
  return neg ? -x : x;
}

__device__ __forceinline__ double u128_to_double(u128 x) {
  const unsigned long long hi = (unsigned long long)(x >> 64), lo = (unsigned long long)x;
  return (double)hi * 18446744073709551616.0 + (double)lo;
}

__device__ __forceinline__ double i128_to_double(i128 x) {
  return x < 0 ? -u128_to_double((u128)(-x)) : u128_to_double((u128)x);
}

// n * S2 - S1^2 (non-negative) as float64: exact 192-bit integers, one
// rounding in the conversion (to within a few ulps).
__device__ __forceinline__ double spread(u128 s2, i128 s1, unsigned int n) {
  const u128 a = (u128)(s1 < 0 ? -s1 : s1);
  const unsigned long long a0 = (unsigned long long)a, a1 = (unsigned long long)(a >> 64);
  // a^2 = a0^2 + 2 a0 a1 2^64 + a1^2 2^128 as three 64-bit words (+ carries).
  const u128 p00 = (u128)a0 * a0;
  const u128 p01 = (u128)a0 * a1;
  const u128 p11 = (u128)a1 * a1;
  u128 w0 = (u128)(unsigned long long)p00;
  u128 w1 = (p00 >> 64) + (u128)(unsigned long long)p01 * 2;
  u128 w2 = (p01 >> 64) * 2 + p11;
  w1 += w0 >> 64;
  w0 &= 0xFFFFFFFFFFFFFFFFull;
  w2 += w1 >> 64;
  w1 &= 0xFFFFFFFFFFFFFFFFull;
  // n * S2 as three words.
  const u128 q0 = (u128)(unsigned long long)s2 * n;
  const u128 q1 = (u128)(unsigned long long)(s2 >> 64) * n + (q0 >> 64);
  unsigned long long n0 = (unsigned long long)q0, n1 = (unsigned long long)q1;
  unsigned long long n2 = (unsigned long long)(q1 >> 64);
  // Subtract (the difference is >= 0 by Cauchy-Schwarz).
  const unsigned long long b0 = (unsigned long long)w0, b1 = (unsigned long long)w1, b2 = (unsigned long long)w2;
  const unsigned long long d0 = n0 - b0;
  const unsigned long long br0 = n0 < b0;
  const unsigned long long t1 = n1 - b1;
  const unsigned long long d1 = t1 - br0;
  const unsigned long long br1 = (n1 < b1) | (t1 < br0);
  const unsigned long long d2 = n2 - b2 - br1;
  return (double)d2 * 340282366920938463463374607431768211456.0 + (double)d1 * 18446744073709551616.0 +
         (double)d0;
}

// ---------------------------------------------------------------------------
// Float32-output combine without FP64: float-float arithmetic (error-free
// two-product by FMA, Newton-corrected division and square root) on the
// top 48 bits of the exact integers, about 2^-46 relative before the final
// rounding to float.

// floor(log2 |x|) of a float (-150 for zero; 128 for infinities / NaN).
__device__ __forceinline__ int exponent_of(float x) {
  const unsigned int b = __float_as_uint(x) & 0x7fffffffu;
  if (b == 0) return -150;
  const int e = (int)(b >> 23);
  if (e == 255) return 128;
  if (e) return e - 127;
  return -149 + (31 - __clz((int)b));
}

// The top 48 bits of a 192-bit unsigned integer (w2:w1:w0) as float-float
// (hi + lo exact) and the power of two they are in units of.
__device__ __forceinline__ void top48(unsigned long long w2, unsigned long long w1, unsigned long long w0,
                                      float& hi, float& lo, int& e) {
  // Left-aligned to exactly 48 significant bits, so hi holds the top 24 and
  // lo the next 24 (a normalized float-float); small values shift left.
  const int len = w2 ? 128 + bitlen64(w2) : (w1 ? 64 + bitlen64(w1) : bitlen64(w0));
  const int shift = len - 48;
  unsigned long long t;
  if (len == 0) {
    t = 0;
  } else if (shift < 0) {
    t = w0 << (-shift);
  } else if (shift >= 128) {
    t = w2 >> (shift - 128);
  } else if (shift >= 64) {
    const int sh = shift - 64;
    t = sh ? (w1 >> sh) | (w2 << (64 - sh)) : w1;
  } else {
    t = shift ? (w0 >> shift) | (w1 << (64 - shift)) : w0;
  }
  hi = (float)(unsigned int)(t >> 24) * 16777216.0f;
  lo = (float)(unsigned int)(t & 0xFFFFFFull);
  e = len == 0 ? 0 : shift;
}

// (hi + lo) / (dh + dl) as float-float (qh + ql).
__device__ __forceinline__ void ff_div(float hi, float lo, float dh, float dl, float& qh, float& ql) {
  const float q1 = __fdiv_rn(hi, dh);
  const float ph = __fmul_rn(q1, dh);
  const float pl = fmaf(q1, dh, -ph);
  const float r = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(hi, ph), pl), lo), __fmul_rn(q1, dl));
  const float q2 = __fdiv_rn(r, dh);
  qh = __fadd_rn(q1, q2);  // renormalize (|q2| is far below |q1|)
  ql = __fsub_rn(q2, __fsub_rn(qh, q1));
}

// Variance / standard deviation of float32 output from the exact numerator
// n S2 - S1^2 (192-bit, d2:d1:d0, in units of 2^(2 quantum)).
template <int KIND>
__device__ __forceinline__ float spread_f32(unsigned long long d2, unsigned long long d1, unsigned long long d0,
                                            unsigned int finite, long long ddof, int quantum) {
  float hi, lo;
  int e;
  top48(d2, d1, d0, hi, lo, e);
  const unsigned long long den = (unsigned long long)finite * (unsigned long long)(finite - ddof);
  const float dh = (float)den;
  const float dl = (float)((long long)den - (long long)dh);
  float qh, ql;
  ff_div(hi, lo, dh, dl, qh, ql);
  if (KIND == kVar) return scalbnf(__fadd_rn(qh, ql), e + 2 * quantum);
  // sqrt((qh + ql) 2^e) 2^quantum with an even power of two under the root.
  if (e & 1) {
    qh = __fmul_rn(qh, 2.0f);
    ql = __fmul_rn(ql, 2.0f);
    e -= 1;
  }
  const float r0 = __fsqrt_rn(qh);
  float root = r0;
  if (r0 > 0.0f) {
    const float resid = __fadd_rn(fmaf(-r0, r0, qh), ql);
    root = __fadd_rn(r0, __fdiv_rn(resid, __fmul_rn(2.0f, r0)));
  }
  return scalbnf(root, e / 2 + quantum);
}

template <int KIND>
__device__ __forceinline__ float combine_f32(i128 s1, u128 s2, unsigned int finite, long long ddof, float pivot,
                                             int quantum) {
  const float nh = (float)finite;  // exact: finite < 2^16
  if (KIND == kMean) {
    const u128 a = (u128)(s1 < 0 ? -s1 : s1);
    float hi, lo;
    int e;
    top48(0, (unsigned long long)(a >> 64), (unsigned long long)a, hi, lo, e);
    float qh, ql;
    ff_div(hi, lo, nh, 0.0f, qh, ql);
    const int k = e + quantum;
    qh = scalbnf(s1 < 0 ? -qh : qh, k);
    ql = scalbnf(s1 < 0 ? -ql : ql, k);
    // pivot + qh + ql with one final rounding (two-sum of the large parts).
    const float sum = __fadd_rn(pivot, qh);
    const float bp = __fsub_rn(sum, pivot);
    const float err = __fadd_rn(__fsub_rn(pivot, __fsub_rn(sum, bp)), __fsub_rn(qh, bp));
    return __fadd_rn(sum, __fadd_rn(err, ql));
  }
  // n S2 - S1^2 exactly (192 bits), as for the float64 combine.
  const u128 a = (u128)(s1 < 0 ? -s1 : s1);
  const unsigned long long a0 = (unsigned long long)a, a1 = (unsigned long long)(a >> 64);
  const u128 p00 = (u128)a0 * a0, p01 = (u128)a0 * a1, p11 = (u128)a1 * a1;
  u128 w1 = (p00 >> 64) + (u128)(unsigned long long)p01 * 2;
  u128 w2 = (p01 >> 64) * 2 + p11 + (w1 >> 64);
  w1 &= 0xFFFFFFFFFFFFFFFFull;
  const u128 q0 = (u128)(unsigned long long)s2 * finite;
  const u128 q1 = (u128)(unsigned long long)(s2 >> 64) * finite + (q0 >> 64);
  const unsigned long long n0 = (unsigned long long)q0, n1 = (unsigned long long)q1,
                           n2 = (unsigned long long)(q1 >> 64);
  const unsigned long long b0 = (unsigned long long)p00, b1 = (unsigned long long)w1,
                           b2 = (unsigned long long)w2;
  const unsigned long long d0 = n0 - b0, br0 = n0 < b0;
  const unsigned long long t1 = n1 - b1, d1 = t1 - br0, br1 = (n1 < b1) | (t1 < br0);
  const unsigned long long d2 = n2 - b2 - br1;
  return spread_f32<KIND>(d2, d1, d0, finite, ddof, quantum);
}

// The value range of a tile's staged support: its pivot (first finite
// sample), the lowest and highest set bits of its finite samples (units of
// 2^E0), a bound on the exponent of |x - P|, the classes of non-finite
// samples present (bit 0 NaN, bit 1 +inf, bit 2 -inf) and whether every
// sample is finite. Every thread of the block calls it and gets the same
// result.
template <typename T>
struct Span {
  T pivot;
  int lo, top, dev, classes;
  bool all_finite;
  __device__ int e0() const { return sizeof(T) == 4 ? -149 : -1074; }
};

template <typename T, int THREADS>
__device__ Span<T> tile_span(const T* s, int support) {
  constexpr int kWarps = THREADS / 32;
  constexpr int E0 = sizeof(T) == 4 ? -149 : -1074;
  __shared__ int red[4][kWarps];
  __shared__ T pivot_s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int first = INT_MAX;
  for (int e = threadIdx.x; e < support; e += blockDim.x)
    if (isfinite(s[e])) {
      first = e;
      break;
    }
  for (int o = 16; o >= 1; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
  if (lane == 0) red[0][warp] = first;
  __syncthreads();
  if (threadIdx.x == 0) {
    int f = INT_MAX;
    for (int w = 0; w < kWarps; ++w) f = min(f, red[0][w]);
    pivot_s = f == INT_MAX ? (T)0 : s[f];
  }
  __syncthreads();
  Span<T> sp;
  sp.pivot = pivot_s;
  int lo = INT_MAX, top = -1, dev = -1075, nonfinite = 0;
  {
    unsigned long long m;
    int pos;
    bool neg;
    if (threadIdx.x == 0 && decompose(sp.pivot, m, pos, neg)) {
      lo = pos;
      top = pos + bitlen64(m) - 1;
    }
  }
  for (int e = threadIdx.x; e < support; e += blockDim.x) {
    const T v = s[e];
    unsigned long long m;
    int pos;
    bool neg;
    if (decompose(v, m, pos, neg)) {
      lo = min(lo, pos);
      top = max(top, pos + bitlen64(m) - 1);
    }
    if (isfinite(v)) {
      // The rounded difference's exponent plus one bounds the exact one; the
      // float32 difference keeps float32 input off the FP64 pipe.
      if constexpr (sizeof(T) == 4)
        dev = max(dev, exponent_of(__fsub_rn((float)v, (float)sp.pivot)));
      else
        dev = max(dev, exponent_of(__dsub_rn((double)v, (double)sp.pivot)));
    } else {
      nonfinite |= isnan(v) ? 1 : (v > (T)0 ? 2 : 4);
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
    dev = max(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    nonfinite |= __shfl_xor_sync(0xffffffffu, nonfinite, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[0][warp] = lo;
    red[1][warp] = top;
    red[2][warp] = dev;
    red[3][warp] = nonfinite;
  }
  __syncthreads();
  lo = INT_MAX;
  top = -1;
  dev = -1075;
  nonfinite = 0;
  for (int w = 0; w < kWarps; ++w) {
    lo = min(lo, red[0][w]);
    top = max(top, red[1][w]);
    dev = max(dev, red[2][w]);
    nonfinite |= red[3][w];
  }
  __syncthreads();  // red and pivot_s are reused by the next tile
  sp.lo = lo == INT_MAX ? 0 : lo;
  sp.top = top;
  sp.dev = dev;
  sp.classes = nonfinite;
  sp.all_finite = nonfinite == 0;
  (void)E0;
  return sp;
}

// Bits of |X| = |x - P| / 2^(E0 + lo): the rounded difference's exponent
// plus one bounds the exact one.
template <typename T>
__device__ __forceinline__ int deviation_bits(const Span<T>& sp) {
  return sp.dev == -1075 ? 0 : max(0, sp.dev + 2 - (sp.e0() + sp.lo));
}

// Whether the tile's integers fit: |X| in 63 bits, sums of X^2 over a window
// of up to 2^count_bits samples in 127 bits, and the mean's n P + S1 in 127.
template <typename T>
__device__ __forceinline__ bool span_fits(const Span<T>& sp, int count_bits) {
  const int bits = deviation_bits(sp);
  return sp.top - sp.lo <= 108 && bits <= 62 && 2 * bits + count_bits + 2 <= 127;
}

// The mean, variance or standard deviation of a window from its exact sums:
// S1 = sum X, S2 = sum X^2 over `finite` samples, P the pivot in the same
// units 2^quantum (quantum = E0 + lo). The caller has already decided the
// special cases (NaN / infinities / counts).
template <typename T>
__device__ __forceinline__ T fixed_combine(int kind, long long ddof, i128 s1, u128 s2, unsigned int finite,
                                          i128 P, int quantum) {
  if constexpr (sizeof(T) == 4) {
    return kind == kMean  ? combine_f32<kMean>((i128)finite * P + s1, s2, finite, 0, 0.0f, quantum)
           : kind == kVar ? combine_f32<kVar>(s1, s2, finite, ddof, 0.0f, quantum)
                          : combine_f32<kStd>(s1, s2, finite, ddof, 0.0f, quantum);
  } else {
    const double n = (double)finite;
    const double scale = pow2(quantum);
    if (kind == kMean) return __dmul_rn(__ddiv_rn(i128_to_double((i128)finite * P + s1), n), scale);
    const double num = spread(s2, s1, finite);
    const double unscaled = __ddiv_rn(num, __dmul_rn(n, (double)((long long)finite - ddof)));
    // Scale after the square root so that a finite deviation never
    // overflows through its square.
    return kind == kStd ? __dmul_rn(__dsqrt_rn(unscaled), scale) : __dmul_rn(__dmul_rn(unscaled, scale), scale);
  }
}

// fixed_combine for sums held in 64-bit words (|S1| < 2^63, S2 < 2^64): the
// numerator n S2 - S1^2 fits 128 bits, so its upper word is zero and the
// same arithmetic runs on fewer words. Results equal fixed_combine's.
template <typename T>
__device__ __forceinline__ T fixed_combine_narrow(int kind, long long ddof, long long s1, unsigned long long s2,
                                                 unsigned int finite, i128 P, int quantum) {
  if (kind == kMean) return fixed_combine<T>(kind, ddof, (i128)s1, (u128)s2, finite, P, quantum);
  const unsigned long long a = s1 < 0 ? 0ull - (unsigned long long)s1 : (unsigned long long)s1;
  const u128 d = (u128)s2 * finite - (u128)a * a;  // >= 0 (Cauchy-Schwarz)
  const unsigned long long d1 = (unsigned long long)(d >> 64), d0 = (unsigned long long)d;
  if constexpr (sizeof(T) == 4) {
    return kind == kVar ? spread_f32<kVar>(0ull, d1, d0, finite, ddof, quantum)
                        : spread_f32<kStd>(0ull, d1, d0, finite, ddof, quantum);
  } else {
    const double n = (double)finite;
    const double scale = pow2(quantum);
    const double num = (double)0ull * 340282366920938463463374607431768211456.0 + (double)d1 * 18446744073709551616.0 +
                       (double)d0;
    const double unscaled = __ddiv_rn(num, __dmul_rn(n, (double)((long long)finite - ddof)));
    return kind == kStd ? __dmul_rn(__dsqrt_rn(unscaled), scale) : __dmul_rn(__dmul_rn(unscaled, scale), scale);
  }
}

}  // namespace fixm
}  // namespace ndf

// Exact fixed-point arithmetic on floating-point samples, shared by the
// exact rolling mean (boxcar.cu) and the sliding moments (moments_slide.cu).
//
// Every finite float is an integer multiple of its type's smallest subnormal
// 2^E0 (E0 = -149 for float32, -1074 for float64), so a block's samples can be
// held as W-word two's-complement integers above the block's lowest occupied
// bit, where sums and differences are exact.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace ndf {
namespace exact {

template <typename T>
struct Bits;
template <>
struct Bits<float> {
  using U = unsigned int;
  static constexpr int kP = 24, kF = 23, kExpMask = 0xFF, kFull = 5, kWords = 2;
};
template <>
struct Bits<double> {
  using U = unsigned long long;
  static constexpr int kP = 53, kF = 52, kExpMask = 0x7FF, kFull = 34, kWords = 3;
};

template <typename T>
__device__ __forceinline__ typename Bits<T>::U bits_of(T v) {
  if constexpr (sizeof(T) == 4) return __float_as_uint(v);
  else return (unsigned long long)__double_as_longlong(v);
}

template <typename T>
__device__ __forceinline__ T from_bits(typename Bits<T>::U b) {
  if constexpr (sizeof(T) == 4) return __uint_as_float(b);
  else return __longlong_as_double((long long)b);
}

// Window counts, 16 bits each: finite | NaN (propagate policy) << 16 |
// +inf << 32 | -inf << 48 (Counts::sample, src/boxcar.rs:19-36).
template <typename T>
__device__ __forceinline__ unsigned long long sample_counts(T v, bool omit, bool drop_inf) {
  if (isnan(v)) return omit ? 0ull : (1ull << 16);
  if (isinf(v)) return drop_inf ? 0ull : (v > (T)0 ? (1ull << 32) : (1ull << 48));
  return 1ull;
}

// A finite nonzero sample as m * 2^pos (units of the type's smallest
// subnormal) with m odd. Returns false for zero, NaN and infinities.
template <typename T>
__device__ __forceinline__ bool decompose(T v, unsigned long long& m, int& pos, bool& neg) {
  using B = Bits<T>;
  const typename B::U b = bits_of(v);
  const int e = (int)((b >> B::kF) & B::kExpMask);
  if (e == B::kExpMask) return false;
  const unsigned long long frac = (unsigned long long)b & ((1ull << B::kF) - 1);
  m = e ? (frac | (1ull << B::kF)) : frac;
  if (m == 0) return false;
  const int tz = __ffsll((long long)m) - 1;
  m >>= tz;
  pos = (e ? e - 1 : 0) + tz;
  neg = (b >> (sizeof(T) * 8 - 1)) != 0;
  return true;
}

template <int W>
struct Wide {
  unsigned long long w[W];
};

template <int W>
__device__ __forceinline__ void wide_add(Wide<W>& a, const Wide<W>& b) {
  unsigned long long carry = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) {
    const unsigned long long s = a.w[i] + b.w[i];
    const unsigned long long t = s + carry;
    carry = (s < a.w[i]) | (t < s);
    a.w[i] = t;
  }
}

template <int W>
__device__ __forceinline__ void wide_sub(Wide<W>& a, const Wide<W>& b) {
  unsigned long long borrow = 0;
#pragma unroll
  for (int i = 0; i < W; ++i) {
    const unsigned long long d = a.w[i] - b.w[i];
    const unsigned long long t = d - borrow;
    borrow = (a.w[i] < b.w[i]) | (d < borrow);
    a.w[i] = t;
  }
}

// The sample as a W-word two's-complement integer in units of
// 2^(E0 + 64 * low_word); zero for zero and non-finite samples. The tile's
// span guarantees pos >= 64 * low_word and that the value fits.
template <typename T, int W>
__device__ __forceinline__ Wide<W> encode(T v, int low_word) {
  Wide<W> r;
  unsigned long long m;
  int pos;
  bool neg;
  const bool finite = decompose(v, m, pos, neg);
  const int local = finite ? pos - 64 * low_word : 0;
  const int wi = local >> 6, off = local & 63;
  const unsigned long long lo = finite ? m << off : 0ull;
  const unsigned long long hi = (finite && off) ? m >> (64 - off) : 0ull;
#pragma unroll
  for (int i = 0; i < W; ++i) r.w[i] = i == wi ? lo : (i == wi + 1 ? hi : 0ull);
  if (finite && neg) {
    unsigned long long carry = 1;
#pragma unroll
    for (int i = 0; i < W; ++i) {
      r.w[i] = ~r.w[i] + carry;
      carry = (carry && r.w[i] == 0) ? 1ull : 0ull;
    }
  }
  return r;
}

__device__ __forceinline__ int bitlen64(unsigned long long x) { return x ? 64 - __clzll((long long)x) : 0; }

// RN_T(S / n) for the NW-word two's-complement sum S in units of
// 2^(E0 + 64 * low_word) and a count n >= 1, rounded once: with B the bit
// length of |S| and t that of n, q = floor(|S| / (n 2^s)) for
// s = max(B - t - p - 1, 0) has p + 1 or p + 2 bits (p, the precision), so
// its low bits and the remainder decide the rounding exactly; s = 0 is the
// subnormal grid, where no sample has bits below.
template <typename T, int NW>
__device__ __forceinline__ T exact_mean(const unsigned long long (&sum)[NW], int low_word, unsigned int n) {
  using B = Bits<T>;
  constexpr int p = B::kP;
  const bool negative = (sum[NW - 1] >> 63) != 0;
  unsigned long long m[NW];
  unsigned long long carry = 1;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    m[i] = negative ? ~sum[i] + carry : sum[i];
    carry = (negative && carry && m[i] == 0) ? 1ull : 0ull;
  }
  int blocal = 0;
#pragma unroll
  for (int i = 0; i < NW; ++i)
    if (m[i]) blocal = 64 * i + bitlen64(m[i]);
  const typename B::U sign = negative ? (typename B::U)1 << (sizeof(T) * 8 - 1) : 0;
  if (blocal == 0) return from_bits<T>(0);  // exact cancellation gives +0
  const int bits = blocal + 64 * low_word;
  const int t = 32 - __clz((int)n);
  const int s = max(bits - t - p - 1, 0);
  const int sl = s - 64 * low_word;  // shift of the local words
  unsigned __int128 high = 0;
  bool sticky = false;
#pragma unroll
  for (int i = 0; i < NW; ++i) {
    const int sh = 64 * i - sl;  // position of word i in `high`
    if (sh >= 128 || sh <= -64) {
      if (sh <= -64) sticky = sticky || m[i] != 0;
      continue;
    }
    if (sh >= 0) {
      high |= (unsigned __int128)m[i] << sh;
    } else {
      high |= (unsigned __int128)(m[i] >> (-sh));
      sticky = sticky || (m[i] & ((1ull << (-sh)) - 1)) != 0;
    }
  }
  unsigned __int128 q, r;
  if constexpr (sizeof(T) == 4) {
    const unsigned long long h = (unsigned long long)high;  // at most 58 bits
    q = h / n;
    r = h % n;
  } else {
    q = high / n;
    r = high % n;
  }
  const int qbits = (q >> 64) ? 128 - __clzll((long long)(unsigned long long)(q >> 64))
                              : bitlen64((unsigned long long)q);
  const int k = max(qbits - p, 0);
  unsigned long long mant;
  bool up;
  if (k > 0) {
    mant = (unsigned long long)(q >> k);
    const bool guard = ((q >> (k - 1)) & 1) != 0;
    const bool rest = (q & (((unsigned __int128)1 << (k - 1)) - 1)) != 0 || r != 0 || sticky;
    up = guard && (rest || (mant & 1));
  } else {
    mant = (unsigned long long)q;
    const unsigned __int128 twice = 2 * r;
    up = twice > n || (twice == n && (sticky || (mant & 1)));
  }
  const typename B::U out =
      (typename B::U)((((unsigned long long)(s + k)) << (p - 1)) + mant + (up ? 1ull : 0ull)) | sign;
  return from_bits<T>(out);
}


}  // namespace exact
}  // namespace ndf

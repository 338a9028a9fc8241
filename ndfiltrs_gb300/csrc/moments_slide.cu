// Sliding exact moments: mean / var / std over rectangular 1-D / 2-D windows
// (the FP32C arithmetic mode's fast path).
//
// The reference evaluates every window with float64 compensated sums
// (src/mean.rs:7-113, src/dispersion.rs:5-61); this library's FP32C mode
// promises results within 2 ulp (float32) / 1e-12 relative (float64) of the
// exact window moments. This kernel meets that with exact integer sums:
//  * per tile, a pivot P (the support's first finite sample) and the lowest
//    set bit of the support's finite samples turn every deviation x - P into
//    an exact 64-bit integer X; sums of X (128-bit) and X^2 (unsigned
//    128-bit) slide along each support row and then down each column, exact
//    under addition and subtraction, so the work per output does not grow
//    with the window;
//  * n S2 - S1^2 is formed exactly in 192-bit integers (so no cancellation
//    can lose bits); float32 outputs finish in float-float arithmetic on the
//    FP32 pipe, float64 outputs convert it to float64 once and run FP64 only
//    for the division by n (n - ddof), the power-of-two scaling and the
//    square root;
//  * the classification of NaN / infinities / counts is the reference's
//    (decide_special); tiles whose value range does not fit the integer
//    widths compute their outputs with the reference's float64 arithmetic.
#include <algorithm>
#include <climits>

#include "exact.cuh"
#include "moments.cuh"
#include "network.cuh"
#include "plan.h"
#include "staging.cuh"
#include "tma.cuh"

namespace ndf {
namespace {

using namespace exact;
constexpr int kSThreads = 256;
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

struct SlideArgs {
  int count_bits;  // bit length of (window volume + 1)
};

template <typename T>
__global__ void __launch_bounds__(kSThreads)
    moments_slide_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                         const __grid_constant__ SlideArgs sa, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int red[3][kSThreads / 32];
  __shared__ T pivot_s;
  constexpr int E0 = sizeof(T) == 4 ? -149 : -1074;
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Reduce& r = a.r;
  // Layout (offsets from the 16-byte aligned base, each region 16-byte
  // aligned for the 128-bit sums): remap tables | staged samples | row sums
  // of X (i128) | row sums of X^2 (u128) | row counts (u64).
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const size_t sums_offset =
      ((size_t)(t.SW + t.SH + g.kd) * 8 + (size_t)t.SH * t.SW * sizeof(T) + 15) & ~(size_t)15;
  i128* h1 = reinterpret_cast<i128*>(smem_raw + sums_offset);
  u128* h2 = reinterpret_cast<u128*>(h1 + (size_t)t.SH * t.TW);
  unsigned long long* hc = reinterpret_cast<unsigned long long*>(h2 + (size_t)t.SH * t.TW);
  long long z, y0, x0;
  net::tile_coords(a, blockIdx.x, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, &tmap, z, y0, x0, (T)r.cval, [](T v) { return v; })) return;
  __syncthreads();
  const int support = t.SH * t.SW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  // Pivot: the support's first finite sample.
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
    for (int w = 0; w < kSThreads / 32; ++w) f = min(f, red[0][w]);
    pivot_s = f == INT_MAX ? (T)0 : s[f];
  }
  __syncthreads();
  const T pivot = pivot_s;

  // Span: lowest set bit (units E0), top bit of |x| (units E0), and the
  // float64 exponent bound of |x - P| over finite samples.
  int lo = INT_MAX, top = -1, dev = -1075;
  {
    unsigned long long m;
    int pos;
    bool neg;
    if (threadIdx.x == 0 && decompose(pivot, m, pos, neg)) {
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
        dev = max(dev, exponent_of(__fsub_rn((float)v, (float)pivot)));
      else
        dev = max(dev, exponent_of(__dsub_rn((double)v, (double)pivot)));
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    top = max(top, __shfl_xor_sync(0xffffffffu, top, o));
    dev = max(dev, __shfl_xor_sync(0xffffffffu, dev, o));
  }
  __syncthreads();
  if (lane == 0) {
    red[0][warp] = lo;
    red[1][warp] = top;
    red[2][warp] = dev;
  }
  __syncthreads();
  lo = INT_MAX;
  top = -1;
  dev = -1075;
  for (int w = 0; w < kSThreads / 32; ++w) {
    lo = min(lo, red[0][w]);
    top = max(top, red[1][w]);
    dev = max(dev, red[2][w]);
  }
  if (lo == INT_MAX) lo = 0;
  // Bits of |X| = |x - P| / 2^(E0 + lo): the rounded float64 difference's
  // exponent plus one bounds the exact one.
  const int bits = dev == -1075 ? 0 : max(0, dev + 2 - (E0 + lo));
  const bool fits = top - lo <= 125 && bits <= 62 && 2 * bits + sa.count_bits + 2 <= 127;

  const int kw = g.kw, kh = g.kh, TW = t.TW, SW = t.SW;
  const bool omit = r.omit, drop_inf = r.drop_inf;
  if (!fits) {
    // A value range too wide for the integer widths: the reference's float64
    // arithmetic per window (bit-identical to it) over the staged support.
    const int tx = threadIdx.x % TW;
    const int nseg_rows = kSThreads / TW;
    for (int ty = threadIdx.x / TW; ty < t.TH; ty += nseg_rows) {
      const long long gy = y0 + ty, gx = x0 + tx;
      if (gy >= g.H || gx >= g.W) continue;
      const int base = ty * SW + tx;
      auto fetch64 = [&](int i) -> double { return (double)s[base + (i / kw) * SW + i % kw]; };
      out[(z * g.H + gy) * g.W + gx] = canonical(from_f64<T>(mom::moments_exact(fetch64, r)));
    }
    return;
  }
  const i128 P = fixed(pivot, lo);

  // Horizontal sums of every support row, 8 outputs per work item.
  const int nseg = TW / 8;
  for (int item = threadIdx.x; item < t.SH * nseg; item += blockDim.x) {
    const int y = item / nseg;
    const int xs = (item - y * nseg) * 8;
    const T* row = s + (size_t)y * SW + xs;
    i128 s1 = 0;
    u128 s2 = 0;
    unsigned long long cnt = 0;
    auto add = [&](T v, int sign) {
      const long long X = isfinite(v) ? (long long)(fixed(v, lo) - P) : 0ll;
      const u128 sq = (u128)((i128)X * X);
      if (sign > 0) {
        s1 += X;
        s2 += sq;
        cnt += sample_counts(v, omit, drop_inf);
      } else {
        s1 -= X;
        s2 -= sq;
        cnt -= sample_counts(v, omit, drop_inf);
      }
    };
    for (int k = 0; k < kw; ++k) add(row[k], 1);
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
      if (j > 0) {
        add(row[j + kw - 1], 1);
        add(row[j - 1], -1);
      }
      h1[(size_t)y * TW + xs + j] = s1;
      h2[(size_t)y * TW + xs + j] = s2;
      hc[(size_t)y * TW + xs + j] = cnt;
    }
  }
  __syncthreads();

  // Vertical sums down each column, L rows per thread, and the combine.
  const int x = threadIdx.x % TW;
  const int nsegs = kSThreads / TW;
  const int L = t.TH / nsegs;
  const int r0 = (threadIdx.x / TW) * L;
  const long long gx = x0 + x;
  i128 s1 = 0;
  u128 s2 = 0;
  unsigned long long cnt = 0;
  for (int k = 0; k < kh; ++k) {
    s1 += h1[(size_t)(r0 + k) * TW + x];
    s2 += h2[(size_t)(r0 + k) * TW + x];
    cnt += hc[(size_t)(r0 + k) * TW + x];
  }
  const double scale = pow2(E0 + lo);
  for (int rr = 0; rr < L; ++rr) {
    const int row = r0 + rr;
    const long long gy = y0 + row;
    if (gy < g.H && gx < g.W) {
      const unsigned int finite = (unsigned int)(cnt & 0xFFFF), nanc = (unsigned int)((cnt >> 16) & 0xFFFF);
      const unsigned int pos = (unsigned int)((cnt >> 32) & 0xFFFF), neg = (unsigned int)(cnt >> 48);
      double result;
      if (mom::decide_special(r, (long long)finite + pos + neg, nanc != 0, pos != 0, neg != 0, &result)) {
        out[(z * g.H + gy) * g.W + gx] = canonical(from_f64<T>(result));
      } else if constexpr (sizeof(T) == 4) {
        const int quantum = E0 + lo;
        const float v = r.kind == kMean  ? combine_f32<kMean>(s1, s2, finite, 0, (float)pivot, quantum)
                        : r.kind == kVar ? combine_f32<kVar>(s1, s2, finite, r.param, (float)pivot, quantum)
                                         : combine_f32<kStd>(s1, s2, finite, r.param, (float)pivot, quantum);
        out[(z * g.H + gy) * g.W + gx] = canonical(v);
      } else {
        const double n = (double)finite;
        if (r.kind == kMean) {
          result = __dadd_rn((double)pivot, __dmul_rn(__ddiv_rn(i128_to_double(s1), n), scale));
        } else {
          const double num = spread(s2, s1, finite);
          const double unscaled = __ddiv_rn(num, __dmul_rn(n, (double)((long long)finite - r.param)));
          // Scale after the square root so that a finite deviation never
          // overflows through its square.
          result = r.kind == kStd ? __dmul_rn(__dsqrt_rn(unscaled), scale)
                                  : __dmul_rn(__dmul_rn(unscaled, scale), scale);
        }
        out[(z * g.H + gy) * g.W + gx] = canonical(from_f64<T>(result));
      }
    }
    if (rr + 1 < L) {
      const size_t add = (size_t)(row + kh) * TW + x, sub = (size_t)row * TW + x;
      s1 += h1[add] - h1[sub];
      s2 += h2[add] - h2[sub];
      cnt += hc[add] - hc[sub];
    }
  }
}

template <typename T>
size_t tile_smem(const Tile& t, int kd) {
  const size_t sums_offset = ((size_t)(t.SW + t.SH + kd) * 8 + (size_t)t.SH * t.SW * sizeof(T) + 15) & ~(size_t)15;
  return sums_offset + (size_t)t.SH * t.TW * (16 + 16 + 8);
}

template <typename T>
cudaError_t launch_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  auto kernel = moments_slide_kernel<T>;
  cudaError_t e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  SlideArgs sa;
  sa.count_bits = 64 - __builtin_clzll((unsigned long long)p.r.count + 1);
  TileArgs args = p.tile;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, p.tile.t, in, &map, &args, &smem);
  kernel<<<(unsigned)p.tile.t.tiles, kSThreads, smem, s>>>(in, out, args, sa, map);
  return cudaGetLastError();
}

}  // namespace

// Tile shape of the sliding moments kernel (as the exact rolling mean's):
// 32 x TH outputs, TH the largest of 64, 32, 16, 8 within 96 KB of shared
// memory, or 256 x 1 for single-row arrays. False when the window or the
// array does not suit it (footprints, rank 3, counts beyond 16 bits).
bool moments_slide_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1 || !p.footprint.empty()) return false;
  const long long volume = (long long)g.kh * g.kw;
  if (volume + g.kw + g.kh >= 65535) return false;
  auto shape = [&](int tw, int th) {
    Tile t = p.tile.t;
    t.TW = tw;
    t.TH = th;
    t.SW = tw + g.kw - 1;
    t.SH = th + g.kh - 1;
    t.tiles_x = (g.W + tw - 1) / tw;
    t.tiles_y = (g.H + th - 1) / th;
    t.tiles = t.tiles_x * t.tiles_y * g.D;
    return t;
  };
  auto bytes = [&](const Tile& t) {
    return p.dtype == 0 ? tile_smem<float>(t, g.kd) : tile_smem<double>(t, g.kd);
  };
  if (g.H == 1 && g.kh == 1) {
    Tile t = shape(256, 1);
    if (bytes(t) > (size_t)smem_limit) return false;
    p.tile.t = t;
    p.smem_bytes = bytes(t);
    return true;
  }
  const size_t budget = std::min<size_t>(96 * 1024, (size_t)smem_limit);
  for (int th : {64, 32, 16, 8}) {
    Tile t = shape(32, th);
    if (bytes(t) <= budget || (th == 8 && bytes(t) <= (size_t)smem_limit)) {
      p.tile.t = t;
      p.smem_bytes = bytes(t);
      return true;
    }
  }
  return false;
}

cudaError_t launch_moments_slide(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}

}  // namespace ndf

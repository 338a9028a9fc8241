// Exact rectangular means: kind mean_rolling (method="boxcar").
//
// Replaces mean_into and ExactSum (src/boxcar.rs:142-399,
// src/exact_sum.rs:215-349). A window's result is the exact sum of its finite
// samples divided by their count, rounded once to the output type (nearest,
// ties to even); the counts of NaN (propagate policy) and of each signed
// infinity decide NaN / +-inf first (Counts::value, src/boxcar.rs:59-77).
//
// GB300 design:
//  * one thread block per output tile (32 x TH outputs; 256 x 1 for
//    single-row arrays); the block stages its support (one TMA copy for an
//    interior tile) and finds the bit span of the support's finite nonzero
//    samples;
//  * every sample becomes a W-word two's-complement fixed-point integer in
//    units of 2^(E0 + 64 * low_word), E0 being the type's smallest subnormal
//    exponent and low_word the tile's lowest occupied 64-bit word, so sums
//    and differences are exact;
//  * the horizontal window sum of every support row slides along the row
//    (add the entering sample, subtract the leaving one), then each thread
//    slides its column's vertical sum of those row sums down its rows: the
//    work per output does not grow with the window;
//  * the quotient by the count is rounded with one integer division;
//  * a tile whose span needs more than W words is appended to a list that a
//    second kernel finishes with full-width direct sums (5 words for float32,
//    34 for float64, every finite value times any count); that kernel also
//    serves arrays of rank 3 or more and windows whose counts exceed 16 bits.
//
// The band kernel serves wide windows, whose tiles would stage mostly halo:
// one thread block slides down a band of 256 output columns, one output row
// at a time. It keeps the exact vertical sum of every support column (the
// entering row added, the leaving row subtracted), turns the row of column
// sums into exact prefix sums with a block scan, and reads each output's
// window sum as the difference of two prefixes. Sums are modular W-word
// integers, exact because every window sum fits. Bands whose span needs more
// than W words rerun with a wider W (5 words covers every float32), and the
// rest go to the direct kernel.
#include <algorithm>
#include <climits>

#include "network.cuh"
#include "plan.h"
#include "staging.cuh"
#include "tma.cuh"
#include "exact.cuh"

namespace ndf {
namespace {

constexpr int kBThreads = 256;
using namespace exact;

// Counts::value (src/boxcar.rs:59-77) over packed counts; `mean` is only
// called for windows that need it.
template <typename T, typename Mean>
__device__ __forceinline__ T finish(unsigned long long c, const Reduce& r, Mean&& mean) {
  const unsigned int finite = (unsigned int)(c & 0xFFFF), nan = (unsigned int)((c >> 16) & 0xFFFF);
  const unsigned int pos = (unsigned int)((c >> 32) & 0xFFFF), neg = (unsigned int)(c >> 48);
  const unsigned int kept = finite + pos + neg;
  if (nan || kept == 0 || (r.omit && (long long)kept < r.min_count) || (pos && neg)) return nan_of(T());
  if (pos) return from_bits<T>(sizeof(T) == 4 ? (typename Bits<T>::U)0x7f800000u
                                              : (typename Bits<T>::U)0x7ff0000000000000ull);
  if (neg) return from_bits<T>(sizeof(T) == 4 ? (typename Bits<T>::U)0xff800000u
                                              : (typename Bits<T>::U)0xfff0000000000000ull);
  return mean(finite);
}

struct BoxcarArgs {
  int count_bits;          // bit length of (window volume + 1)
  unsigned int* list;      // tiles left to the full-width kernel
  unsigned int* list_len;  // their number
};

template <typename T, int W>
__global__ void __launch_bounds__(kBThreads)
    boxcar_tile_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                       const __grid_constant__ BoxcarArgs b, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int red_lo[kBThreads / 32], red_hi[kBThreads / 32];
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const size_t staged = ((size_t)t.SH * t.SW * sizeof(T) + 15) & ~(size_t)15;
  unsigned long long* hs = reinterpret_cast<unsigned long long*>(reinterpret_cast<unsigned char*>(s) + staged);
  unsigned long long* hc = hs + (size_t)t.SH * W * t.TW;
  long long z, y0, x0;
  net::tile_coords(a, blockIdx.x, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, &tmap, z, y0, x0, (T)a.r.cval, [](T v) { return v; })) return;
  __syncthreads();

  // Bit span of the support's finite nonzero samples.
  const int support = t.SH * t.SW;
  int lo = INT_MAX, hi = -1;
  for (int e = threadIdx.x; e < support; e += blockDim.x) {
    unsigned long long m;
    int pos;
    bool neg;
    if (decompose(s[e], m, pos, neg)) {
      lo = min(lo, pos);
      hi = max(hi, pos + bitlen64(m) - 1);
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red_lo[threadIdx.x >> 5] = lo;
    red_hi[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  lo = INT_MAX;
  hi = -1;
  for (int w = 0; w < kBThreads / 32; ++w) {
    lo = min(lo, red_lo[w]);
    hi = max(hi, red_hi[w]);
  }
  const int low_word = lo == INT_MAX ? 0 : lo >> 6;
  const int need = hi < 0 ? 1 : ((hi + 2 + b.count_bits + 63) >> 6) - low_word;
  if (need > W) {
    if (threadIdx.x == 0) b.list[atomicAdd(b.list_len, 1u)] = blockIdx.x;
    return;
  }

  // Horizontal window sums of every support row, 8 outputs per work item.
  const bool omit = a.r.omit, drop_inf = a.r.drop_inf;
  const int kw = g.kw, kh = g.kh, TW = t.TW, SW = t.SW;
  const int nseg = TW / 8;
  for (int item = threadIdx.x; item < t.SH * nseg; item += blockDim.x) {
    const int y = item / nseg;
    const int xs = (item - y * nseg) * 8;
    const T* row = s + (size_t)y * SW + xs;
    Wide<W> sum = {};
    unsigned long long cnt = 0;
    for (int k = 0; k < kw; ++k) {
      wide_add(sum, encode<T, W>(row[k], low_word));
      cnt += sample_counts(row[k], omit, drop_inf);
    }
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
      if (j > 0) {
        const T enter = row[j + kw - 1], leave = row[j - 1];
        wide_add(sum, encode<T, W>(enter, low_word));
        wide_sub(sum, encode<T, W>(leave, low_word));
        cnt += sample_counts(enter, omit, drop_inf);
        cnt -= sample_counts(leave, omit, drop_inf);
      }
#pragma unroll
      for (int i = 0; i < W; ++i) hs[((size_t)y * W + i) * TW + xs + j] = sum.w[i];
      hc[(size_t)y * TW + xs + j] = cnt;
    }
  }
  __syncthreads();

  // Vertical sums down each column, L rows per thread.
  const int x = threadIdx.x % TW;
  const int nsegs = kBThreads / TW;
  const int L = t.TH / nsegs;
  const int r0 = (threadIdx.x / TW) * L;
  const long long gx = x0 + x;
  auto row_sum = [&](int y, Wide<W>& v, unsigned long long& c) {
#pragma unroll
    for (int i = 0; i < W; ++i) v.w[i] = hs[((size_t)y * W + i) * TW + x];
    c = hc[(size_t)y * TW + x];
  };
  Wide<W> sum = {};
  unsigned long long cnt = 0;
  for (int k = 0; k < kh; ++k) {
    Wide<W> v;
    unsigned long long c;
    row_sum(r0 + k, v, c);
    wide_add(sum, v);
    cnt += c;
  }
  for (int rr = 0; rr < L; ++rr) {
    const int r = r0 + rr;
    const long long gy = y0 + r;
    if (gy < g.H && gx < g.W) {
      const T v = finish<T>(cnt, a.r, [&](unsigned int n) { return exact_mean<T, W>(sum.w, low_word, n); });
      out[(z * g.H + gy) * g.W + gx] = canonical(v);
    }
    if (rr + 1 < L) {
      Wide<W> va, vr;
      unsigned long long ca, cr;
      row_sum(r + kh, va, ca);
      row_sum(r, vr, cr);
      wide_add(sum, va);
      wide_sub(sum, vr);
      cnt += ca - cr;
    }
  }
}

constexpr int kBandWidth = kBThreads;  // outputs per band row, one per thread

struct BandArgs {
  int count_bits;                // bit length of (window volume + 1)
  const unsigned int* in_list;   // bands to run (nullptr: every band)
  const unsigned int* in_len;
  unsigned int* out_list;        // bands whose span needs more than W words
  unsigned int* out_len;
};

// Shared memory of a band: x / y source maps, the column sums (W words and
// the packed counts per support column) and the prefix sums.
template <int W>
__host__ __device__ inline size_t band_smem(const Tile& t) {
  return (size_t)(t.SW + t.SH) * 8 + (size_t)(W + 1) * t.SW * 8 + (size_t)(W + 1) * (t.SW + 1) * 8;
}

template <typename T, int W>
__global__ void __launch_bounds__(kBThreads)
    boxcar_band_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                       const __grid_constant__ BandArgs b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int red_lo[kBThreads / 32], red_hi[kBThreads / 32];
  __shared__ unsigned long long wtot[kBThreads / 32][W + 1];
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long band = blockIdx.x;
  if (b.in_list) {
    if (blockIdx.x >= *b.in_len) return;
    band = b.in_list[blockIdx.x];
  }
  long long z, y0, x0;
  net::tile_coords(a, band, z, y0, x0);
  const int kw = g.kw, kh = g.kh, SW = t.SW;
  const int rows = (int)min((long long)t.TH, g.H - y0);
  const int SH = rows + kh - 1;
  long long* mx = reinterpret_cast<long long*>(smem_raw);
  long long* my = mx + SW;
  unsigned long long* col = reinterpret_cast<unsigned long long*>(my + t.SH);  // [W + 1][SW]
  unsigned long long* pre = col + (size_t)(W + 1) * SW;                        // [W + 1][SW + 1]
  const int SP = SW + 1;
  for (int i = threadIdx.x; i < SW + SH; i += blockDim.x) {
    long long m;
    if (i < SW) {
      mx[i] = map_index(x0 + i - g.ax, g.W, g.mx, &m) ? m : -1;
    } else {
      const int j = i - SW;
      my[j] = map_index(y0 + j - g.ay, g.H, g.my, &m) ? m * g.W : -1;
    }
  }
  __syncthreads();
  const T cval = (T)a.r.cval;
  auto sample = [&](int j, int c) -> T {
    const long long oy = my[j], ox = mx[c];
    return (oy < 0 || ox < 0) ? cval : __ldg(in + oy + ox);
  };

  // Bit span of the band support's finite nonzero samples.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int lo = INT_MAX, hi = -1;
  for (int j = warp; j < SH; j += kBThreads / 32)
    for (int c = lane; c < SW; c += 32) {
      unsigned long long m;
      int pos;
      bool neg;
      if (decompose(sample(j, c), m, pos, neg)) {
        lo = min(lo, pos);
        hi = max(hi, pos + bitlen64(m) - 1);
      }
    }
  for (int o = 16; o >= 1; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    red_lo[warp] = lo;
    red_hi[warp] = hi;
  }
  __syncthreads();
  lo = INT_MAX;
  hi = -1;
  for (int w = 0; w < kBThreads / 32; ++w) {
    lo = min(lo, red_lo[w]);
    hi = max(hi, red_hi[w]);
  }
  const int low_word = lo == INT_MAX ? 0 : lo >> 6;
  const int need = hi < 0 ? 1 : ((hi + 2 + b.count_bits + 63) >> 6) - low_word;
  if (need > W) {
    if (threadIdx.x == 0) b.out_list[atomicAdd(b.out_len, 1u)] = (unsigned int)band;
    return;
  }

  // Each thread owns a contiguous chunk of support columns.
  const bool omit = a.r.omit, drop_inf = a.r.drop_inf;
  const int chunk = (SW + kBThreads - 1) / kBThreads;
  const int c0 = min(SW, (int)threadIdx.x * chunk), c1 = min(SW, c0 + chunk);
  for (int c = c0; c < c1; ++c) {
    Wide<W> v = {};
    unsigned long long n = 0;
    for (int j = 0; j < kh; ++j) {
      const T x = sample(j, c);
      wide_add(v, encode<T, W>(x, low_word));
      n += sample_counts(x, omit, drop_inf);
    }
#pragma unroll
    for (int i = 0; i < W; ++i) col[(size_t)i * SW + c] = v.w[i];
    col[(size_t)W * SW + c] = n;
  }
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i <= W; ++i) pre[(size_t)i * SP] = 0;
  }

  const int x = threadIdx.x;
  const long long gx = x0 + x;
  for (int r = 0; r < rows; ++r) {
    // Chunk total, then an inclusive warp scan of the totals.
    Wide<W> tot = {};
    unsigned long long tn = 0;
    for (int c = c0; c < c1; ++c) {
      Wide<W> v;
#pragma unroll
      for (int i = 0; i < W; ++i) v.w[i] = col[(size_t)i * SW + c];
      wide_add(tot, v);
      tn += col[(size_t)W * SW + c];
    }
    Wide<W> inc = tot;
    unsigned long long incn = tn;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      Wide<W> o;
#pragma unroll
      for (int i = 0; i < W; ++i) o.w[i] = __shfl_up_sync(0xffffffffu, inc.w[i], off);
      const unsigned long long on = __shfl_up_sync(0xffffffffu, incn, off);
      if (lane >= off) {
        wide_add(inc, o);
        incn += on;
      }
    }
    if (lane == 31) {
#pragma unroll
      for (int i = 0; i < W; ++i) wtot[warp][i] = inc.w[i];
      wtot[warp][W] = incn;
    }
    __syncthreads();
    // Exclusive prefix of the chunk: earlier warps, then earlier lanes.
    Wide<W> run = inc;
    unsigned long long runn = incn - tn;
    wide_sub(run, tot);
    for (int w = 0; w < warp; ++w) {
      Wide<W> o;
#pragma unroll
      for (int i = 0; i < W; ++i) o.w[i] = wtot[w][i];
      wide_add(run, o);
      runn += wtot[w][W];
    }
    for (int c = c0; c < c1; ++c) {
      Wide<W> v;
#pragma unroll
      for (int i = 0; i < W; ++i) v.w[i] = col[(size_t)i * SW + c];
      wide_add(run, v);
      runn += col[(size_t)W * SW + c];
#pragma unroll
      for (int i = 0; i < W; ++i) pre[(size_t)i * SP + c + 1] = run.w[i];
      pre[(size_t)W * SP + c + 1] = runn;
    }
    __syncthreads();

    // One output per thread: the difference of two prefixes.
    const long long gy = y0 + r;
    if (gx < g.W) {
      Wide<W> sum, left;
#pragma unroll
      for (int i = 0; i < W; ++i) {
        sum.w[i] = pre[(size_t)i * SP + x + kw];
        left.w[i] = pre[(size_t)i * SP + x];
      }
      wide_sub(sum, left);
      const unsigned long long n = pre[(size_t)W * SP + x + kw] - pre[(size_t)W * SP + x];
      const T v = finish<T>(n, a.r, [&](unsigned int cnt) { return exact_mean<T, W>(sum.w, low_word, cnt); });
      out[gy * g.W + gx] = canonical(v);
    }

    // Slide the column sums down one row.
    if (r + 1 < rows) {
      for (int c = c0; c < c1; ++c) {
        const T enter = sample(r + kh, c), leave = sample(r, c);
        Wide<W> v;
#pragma unroll
        for (int i = 0; i < W; ++i) v.w[i] = col[(size_t)i * SW + c];
        wide_add(v, encode<T, W>(enter, low_word));
        wide_sub(v, encode<T, W>(leave, low_word));
#pragma unroll
        for (int i = 0; i < W; ++i) col[(size_t)i * SW + c] = v.w[i];
        col[(size_t)W * SW + c] += sample_counts(enter, omit, drop_inf) - sample_counts(leave, omit, drop_inf);
      }
    }
  }
}

// Full-width direct sums: every output of the listed tiles (list mode) or
// of the whole array (list == nullptr), gathered through the per-axis
// boundary maps (Window::visit, src/window.rs:232-294).
template <typename T>
__global__ void __launch_bounds__(kBThreads)
    boxcar_direct_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ GenericArgs a,
                         const long long* __restrict__ taps, const __grid_constant__ TileArgs tile,
                         const unsigned int* __restrict__ list, const unsigned int* __restrict__ list_len) {
  constexpr int NW = Bits<T>::kFull;
  const int rank = a.rank;
  const bool omit = a.r.omit, drop_inf = a.r.drop_inf;
  const T cval = (T)a.r.cval;
  const long long per_tile = (long long)tile.t.TW * tile.t.TH;
  const long long total = list ? (long long)(*list_len) * per_tile : a.n_out;
  for (long long item = blockIdx.x * (long long)blockDim.x + threadIdx.x; item < total;
       item += (long long)gridDim.x * blockDim.x) {
    long long o = item;
    if (list) {
      const long long tl = list[item / per_tile];
      const long long within = item % per_tile;
      long long z, y0, x0;
      net::tile_coords(tile, tl, z, y0, x0);
      const long long y = y0 + within / tile.t.TW, x = x0 + within % tile.t.TW;
      if (y >= tile.g.H || x >= tile.g.W) continue;
      o = (z * tile.g.H + y) * tile.g.W + x;
    }
    long long coord[kMaxGenericRank];
    long long rem = o;
    for (int d = 0; d < rank; ++d) {
      coord[d] = rem / a.stride[d];
      rem -= coord[d] * a.stride[d];
    }
    unsigned long long acc[NW];
    for (int i = 0; i < NW; ++i) acc[i] = 0;
    unsigned long long finite = 0, nan = 0, pos = 0, neg = 0;
    for (int i = 0; i < a.r.count; ++i) {
      const long long* tap = taps + (long long)i * rank;
      long long src = 0;
      bool inside = true;
      for (int d = 0; d < rank && inside; ++d) {
        long long m;
        inside = map_index(coord[d] + tap[d], a.shape[d], a.mode[d], &m);
        src += m * a.stride[d];
      }
      const T v = inside ? __ldg(in + src) : cval;
      if (isnan(v)) {
        if (!omit) ++nan;
        continue;
      }
      if (isinf(v)) {
        if (!drop_inf) (v > (T)0 ? pos : neg) += 1;
        continue;
      }
      ++finite;
      unsigned long long mm;
      int p;
      bool negative;
      if (!decompose(v, mm, p, negative)) continue;
      int wi = p >> 6;
      const int off = p & 63;
      const unsigned long long parts[2] = {mm << off, off ? mm >> (64 - off) : 0ull};
      if (!negative) {
        unsigned long long carry = 0;
        for (int j = 0; wi < NW && (j < 2 || carry); ++j, ++wi) {
          const unsigned long long add = j < 2 ? parts[j] : 0ull;
          const unsigned long long s1 = acc[wi] + add;
          const unsigned long long s2 = s1 + carry;
          carry = (s1 < add) | (s2 < s1);
          acc[wi] = s2;
        }
      } else {
        unsigned long long borrow = 0;
        for (int j = 0; wi < NW && (j < 2 || borrow); ++j, ++wi) {
          const unsigned long long sub = j < 2 ? parts[j] : 0ull;
          const unsigned long long d1 = acc[wi] - sub;
          const unsigned long long d2 = d1 - borrow;
          borrow = (acc[wi] < sub) | (d1 < borrow);
          acc[wi] = d2;
        }
      }
    }
    const unsigned long long kept = finite + pos + neg;
    T result;
    if (nan || kept == 0 || (omit && (long long)kept < a.r.min_count) || (pos && neg))
      result = nan_of(T());
    else if (pos)
      result = from_bits<T>(sizeof(T) == 4 ? (typename Bits<T>::U)0x7f800000u
                                           : (typename Bits<T>::U)0x7ff0000000000000ull);
    else if (neg)
      result = from_bits<T>(sizeof(T) == 4 ? (typename Bits<T>::U)0xff800000u
                                           : (typename Bits<T>::U)0xfff0000000000000ull);
    else
      result = exact_mean<T, NW>(acc, 0, (unsigned int)finite);
    out[o] = canonical(result);
  }
}

template <typename T>
size_t tile_smem(const Tile& t, int kd) {
  constexpr int W = Bits<T>::kWords;
  const size_t staged = ((size_t)t.SH * t.SW * sizeof(T) + 15) & ~(size_t)15;
  return (size_t)(t.SW + t.SH + kd) * 8 + staged + (size_t)t.SH * t.TW * (W + 1) * 8;
}

// Bands at W words, bands too wide for that at a wider W, then the direct
// kernel for any left (none for float32, whose 5 words hold every sum).
// Scratch: [len_a, len_b, list_a[bands], list_b[bands]].
template <typename T>
cudaError_t launch_band(const Plan& p, const T* in, T* out, cudaStream_t s) {
  constexpr int W1 = Bits<T>::kWords;
  constexpr int W2 = sizeof(T) == 4 ? 5 : 6;
  const long long bands = p.tile.t.tiles;
  unsigned int* lens = reinterpret_cast<unsigned int*>(p.d_scratch);
  unsigned int* list_a = lens + 2;
  unsigned int* list_b = list_a + bands;
  cudaError_t e = cudaMemsetAsync(lens, 0, 2 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  BandArgs b;
  b.count_bits = 64 - __builtin_clzll((unsigned long long)p.r.count + 1);
  b.in_list = nullptr;
  b.in_len = nullptr;
  b.out_list = list_a;
  b.out_len = lens;
  auto k1 = boxcar_band_kernel<T, W1>;
  auto k2 = boxcar_band_kernel<T, W2>;
  if ((e = allow_max_smem((const void*)k1)) != cudaSuccess) return e;
  if ((e = allow_max_smem((const void*)k2)) != cudaSuccess) return e;
  k1<<<(unsigned)bands, kBThreads, band_smem<W1>(p.tile.t), s>>>(in, out, p.tile, b);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  b.in_list = list_a;
  b.in_len = lens;
  b.out_list = list_b;
  b.out_len = lens + 1;
  k2<<<(unsigned)bands, kBThreads, band_smem<W2>(p.tile.t), s>>>(in, out, p.tile, b);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const long long direct_grid = std::max(1, p.sm_count) * 8ll;
  boxcar_direct_kernel<T><<<(unsigned)direct_grid, kBThreads, 0, s>>>(in, out, p.generic, p.d_gen_taps, p.tile,
                                                                     list_b, lens + 1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  constexpr int W = Bits<T>::kWords;
  if (p.algo == Algo::kBoxcarBand) return launch_band<T>(p, in, out, s);
  const long long direct_grid = std::max(1, p.sm_count) * 8ll;
  if (p.algo == Algo::kBoxcarDirect) {
    boxcar_direct_kernel<T><<<(unsigned)direct_grid, kBThreads, 0, s>>>(in, out, p.generic, p.d_gen_taps, p.tile,
                                                                       nullptr, nullptr);
    return cudaGetLastError();
  }
  unsigned int* list = reinterpret_cast<unsigned int*>(p.d_scratch);
  unsigned int* list_len = list + p.tile.t.tiles;
  cudaError_t e = cudaMemsetAsync(list_len, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  auto kernel = boxcar_tile_kernel<T, W>;
  e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  BoxcarArgs b;
  b.count_bits = 64 - __builtin_clzll((unsigned long long)p.r.count + 1);
  b.list = list;
  b.list_len = list_len;
  TileArgs args = p.tile;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, p.tile.t, in, &map, &args, &smem);
  kernel<<<(unsigned)p.tile.t.tiles, kBThreads, smem, s>>>(in, out, args, b, map);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  boxcar_direct_kernel<T><<<(unsigned)direct_grid, kBThreads, 0, s>>>(in, out, p.generic, p.d_gen_taps, p.tile,
                                                                     list, list_len);
  return cudaGetLastError();
}

}  // namespace

// Tile shape and shared memory of the tiled exact-mean kernel: 32 x TH
// outputs (TH the largest of 64, 32, 16, 8 within 96 KB of shared memory),
// or 256 x 1 for single-row arrays. Returns false when the direct kernel
// must run instead (rank 3 or more, window counts beyond 16 bits, or no tile
// fitting in `smem_limit`).
bool boxcar_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1) return false;
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

// Bands of 256 output columns and TH rows, TH the largest power of two in
// [32, 512] that still gives four bands per SM (else 32). Returns false for
// rank 3, window counts beyond 16 bits, or bands beyond `smem_limit`.
bool boxcar_band_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1) return false;
  const long long volume = (long long)g.kh * g.kw;
  if (volume + g.kw + g.kh >= 65535) return false;
  const long long bands_x = (g.W + kBandWidth - 1) / kBandWidth;
  const long long target = 4ll * std::max(1, p.sm_count);
  int th = 512;
  while (th > 32 && bands_x * ((g.H + th - 1) / th) < target) th /= 2;
  Tile t = p.tile.t;
  t.TW = kBandWidth;
  t.TH = (int)std::min<long long>(th, std::max<long long>(1, g.H));
  t.SW = t.TW + g.kw - 1;
  t.SH = t.TH + g.kh - 1;
  t.tiles_x = bands_x;
  t.tiles_y = (g.H + t.TH - 1) / t.TH;
  t.tiles = t.tiles_x * t.tiles_y;
  const size_t bytes = p.dtype == 0 ? band_smem<5>(t) : band_smem<6>(t);
  if (bytes > (size_t)smem_limit) return false;
  p.tile.t = t;
  p.smem_bytes = bytes;
  return true;
}

cudaError_t launch_boxcar(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}

}  // namespace ndf

// Sliding exact moments: mean / var / std over rectangular 1-D / 2-D windows
// (the FP32C arithmetic mode's fast path).
//
// The reference evaluates every window with float64 compensated sums
// (src/mean.rs:7-113, src/dispersion.rs:5-61); this library's FP32C mode
// promises results within 2 ulp (float32) / 1e-12 relative (float64) of the
// exact window moments. This kernel meets that with exact integer sums:
//  * per tile, a pivot P (the support's first finite sample) and the lowest
//    set bit of the support's finite samples turn every deviation x - P into
//    an exact integer X, written in place of the staged sample (int32 for
//    float32 tiles whose deviations fit 30 bits, int64 for float64 tiles;
//    non-finite samples as marker words);
//  * column sums first: every support column's sums of X and X^2 (64-bit
//    words when every window's sums fit, else 128-bit) slide down the tile
//    one output row at a time, kept in registers across a chunk of rows;
//    the chunk's column sums go to shared memory, where each row item sums
//    kw consecutive columns and slides along the row. Addition and
//    subtraction are exact in any order, so the work per output does not
//    grow with the window;
//  * sample counts: none for tiles without non-finite samples, the count of
//    a tile's single non-finite class packed above the sum of X, or the
//    packed 16-bit count fields of every class as a third sum;
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
#include <cstring>
#include <type_traits>

#include "exact.cuh"
#include "fixed_moments.cuh"
#include "moments.cuh"
#include "network.cuh"
#include "plan.h"
#include "staging.cuh"
#include "tma.cuh"

namespace ndf {
namespace {

using namespace exact;
using namespace fixm;
constexpr int kSThreads = 256;

struct SlideArgs {
  int count_bits;  // bit length of (window volume + 1)
  int rows;        // output rows per chunk (64-bit sums; 128-bit sums take half)
};

// Outputs per row work item: as many as make rows x TW / seg = kSThreads
// items (one per thread), at least one. TW and rows are powers of two.
__host__ __device__ inline int slide_seg(int tw, int rows) {
  return tw * rows / kSThreads > 0 ? tw * rows / kSThreads : 1;
}
__host__ __device__ inline int slide_wide_rows(int rows) { return rows > 1 ? rows / 2 : 1; }

__host__ __device__ inline size_t round16(size_t v) { return (v + 15) & ~(size_t)15; }

// Shared-memory layout of one tile (byte offsets from the 16-byte aligned
// base): remap tables | staged samples (later their deviations) | running
// column sums per support column (kept across chunks) | one chunk of column
// sums, (S1, S2) pairs then counts, row pitch skewed by one entry per eight
// so that the row items' strided reads spread over the banks | the chunk's
// outputs. A TMA staging area may overlay the chunk buffers: they are not
// used before the staged samples are copied out of it.
struct SlideLayout {
  size_t s, state, vbuf, outb, total;
  int pitch;
};

__host__ __device__ inline SlideLayout slide_layout(const Tile& t, int kd, int elem, int rows) {
  SlideLayout l;
  const int wide_rows = slide_wide_rows(rows);
  l.pitch = t.SW + t.SW / 8 + 1;
  l.s = round16((size_t)(t.SW + t.SH + kd) * 8);
  l.state = round16(l.s + (size_t)t.SH * t.SW * elem);
  const size_t state_bytes = t.TH > wide_rows ? (size_t)t.SW * 40 : 0;
  l.vbuf = round16(l.state + state_bytes);
  const size_t chunk = (size_t)l.pitch * (rows * 24 > wide_rows * 40 ? rows * 24 : wide_rows * 40);
  l.outb = round16(l.vbuf + chunk);
  l.total = l.outb + (size_t)rows * t.TW * elem;
  return l;
}

__device__ __forceinline__ int skew(int c) { return c + (c >> 3); }

// The exact window moments of one staged tile, column sums first: each
// support column's running sums of X, X^2 (and the sample counts) slide down
// the tile one output row at a time; a chunk of rows of those column sums
// goes to shared memory, where row items sum kw consecutive columns for
// `seg` consecutive outputs (sliding along the row) and finish each output.
//  XK: 0 = deviations as int32 in place of float32 samples, 1 = as int64 in
//      place of float64 samples (non-finite samples as marker words), 2 =
//      computed from the samples on every use (wide float32 tiles);
//  NARROW: S1 and S2 in 64-bit words (every window's sums fit), else 128;
//  CM: 0 = no non-finite samples (every window counts kh * kw samples),
//      1 = one class of non-finite sample, its window count packed above
//      the sum of X (bit K), 2 = the packed 16-bit count fields of every
//      class (Counts::sample) as a third sum.
template <typename T, int XK, bool NARROW, int CM>
__device__ __forceinline__ void column_walk(unsigned char* base, const SlideLayout& L, const T* s, const TileArgs& a,
                                            const SlideArgs& sa, const Span<T>& sp, i128 P, int bits, long long z,
                                            long long y0, long long x0, T* __restrict__ out) {
  using S1 = typename std::conditional<NARROW, long long, i128>::type;
  using S2 = typename std::conditional<NARROW, unsigned long long, u128>::type;
  using XW = typename std::conditional<XK == 0, int, long long>::type;
  struct __align__(16) Pair {
    S1 a;
    S2 b;
  };
  constexpr int E0 = sizeof(T) == 4 ? -149 : -1074;
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Reduce& r = a.r;
  const int kh = g.kh, kw = g.kw, SW = t.SW, TW = t.TW, TH = t.TH;
  const int rows = NARROW ? sa.rows : slide_wide_rows(sa.rows);
  const int seg0 = slide_seg(TW, sa.rows);
  const int seg = NARROW ? seg0 : (seg0 > 1 ? seg0 / 2 : 1);
  const int pitch = L.pitch;
  S1* st1 = reinterpret_cast<S1*>(base + L.state);
  S2* st2 = reinterpret_cast<S2*>(base + L.state + (size_t)SW * 16);
  unsigned long long* stc = reinterpret_cast<unsigned long long*>(base + L.state + (size_t)SW * 32);
  Pair* vb = reinterpret_cast<Pair*>(base + L.vbuf);
  unsigned long long* vc = reinterpret_cast<unsigned long long*>(base + L.vbuf + (size_t)rows * pitch * sizeof(Pair));
  T* ob = reinterpret_cast<T*>(base + L.outb);
  const XW* xw = reinterpret_cast<const XW*>(s);
  const int lo = sp.lo;
  const int K = bits + sa.count_bits + 1;  // CM 1: bit of the packed count
  const int cls = __ffs(sp.classes) - 1;   // CM 1: the class present
  const unsigned long long code_nan = r.omit ? 0ull : (1ull << 16);
  const unsigned long long code_pos = r.drop_inf ? 0ull : (1ull << 32);
  const unsigned long long code_neg = r.drop_inf ? 0ull : (1ull << 48);
  const unsigned int volume = (unsigned int)(kh * kw);
  const int quantum = E0 + lo;

  // One sample's terms: X (or, CM 1, the packed count for a non-finite
  // sample), X^2 and its counts (CM 2).
  auto term = [&](int e, S1& t1, S2& t2, unsigned long long& tc) {
    if constexpr (XK == 2) {
      const T v = s[e];
      const long long X = isfinite(v) ? (long long)(fixed(v, lo) - P) : 0ll;
      t1 = (S1)X;
      t2 = (S2)((i128)X * X);
      tc = sample_counts(v, r.omit, r.drop_inf);
    } else {
      const XW x = xw[e];
      if constexpr (CM == 0) {
        t1 = (S1)x;
        if constexpr (XK == 0)
          t2 = (S2)(unsigned long long)((long long)x * x);
        else
          t2 = (S2)((i128)x * x);
        tc = 0;
      } else {
        constexpr XW kBound = XK == 0 ? (XW)(-(1 << 30)) : (XW)(-(1ll << 62));
        const bool special = x < kBound;
        const XW X = special ? (XW)0 : x;
        if constexpr (XK == 0)
          t2 = (S2)(unsigned long long)((long long)X * X);
        else
          t2 = (S2)((i128)X * X);
        if constexpr (CM == 1) {
          t1 = special ? ((S1)1 << K) : (S1)X;
          tc = 0;
        } else {
          t1 = (S1)X;
          const int c = (int)(x & 3);
          tc = special ? (c == 0 ? code_nan : (c == 1 ? code_pos : code_neg)) : 1ull;
        }
      }
    }
  };

  // One output from its window sums.
  auto finish = [&](S1 a1, S2 a2, unsigned long long ac) -> T {
    unsigned int finite = volume, nanc = 0, pos = 0, neg = 0;
    if constexpr (CM == 1) {
      const S1 s1 = (S1)((long long)((unsigned long long)a1 << (64 - K)) >> (64 - K));
      const unsigned int k = (unsigned int)((unsigned long long)(a1 - s1) >> K);
      a1 = s1;
      finite = volume - k;
      nanc = cls == 0 && !r.omit ? k : 0u;
      pos = cls == 1 && !r.drop_inf ? k : 0u;
      neg = cls == 2 && !r.drop_inf ? k : 0u;
    } else if constexpr (CM == 2) {
      finite = (unsigned int)(ac & 0xFFFF);
      nanc = (unsigned int)((ac >> 16) & 0xFFFF);
      pos = (unsigned int)((ac >> 32) & 0xFFFF);
      neg = (unsigned int)(ac >> 48);
    }
    double result;
    if (mom::decide_special(r, (long long)finite + pos + neg, nanc != 0, pos != 0, neg != 0, &result))
      return canonical(from_f64<T>(result));
    if constexpr (NARROW)
      return canonical(fixed_combine_narrow<T>(r.kind, r.param, a1, a2, finite, P, quantum));
    else
      return canonical(fixed_combine<T>(r.kind, r.param, (i128)a1, (u128)a2, finite, P, quantum));
  };

  const int chunks = (TH + rows - 1) / rows;
  for (int ch = 0; ch < chunks; ++ch) {
    const int r0 = ch * rows, nr = min(rows, TH - r0);
    // Column sums of the chunk's output rows.
    for (int c = threadIdx.x; c < SW; c += blockDim.x) {
      S1 v1 = 0;
      S2 v2 = 0;
      unsigned long long v3 = 0;
      S1 t1;
      S2 t2;
      unsigned long long tc;
      if (ch == 0) {
        for (int k = 0; k < kh; ++k) {
          term(k * SW + c, t1, t2, tc);
          v1 += t1;
          v2 += t2;
          v3 += tc;
        }
      } else {
        v1 = st1[c];
        v2 = st2[c];
        if constexpr (CM == 2) v3 = stc[c];
      }
#pragma unroll 1
      for (int i = 0; i < nr; ++i) {
        const int y = r0 + i;
        vb[i * pitch + skew(c)] = Pair{v1, v2};
        if constexpr (CM == 2) vc[i * pitch + skew(c)] = v3;
        if (y + 1 < TH) {
          S1 u1;
          S2 u2;
          unsigned long long uc;
          term((y + kh) * SW + c, t1, t2, tc);
          term(y * SW + c, u1, u2, uc);
          v1 += t1 - u1;
          v2 += t2 - u2;
          v3 += tc - uc;
        }
      }
      if (ch + 1 < chunks) {
        st1[c] = v1;
        st2[c] = v2;
        if constexpr (CM == 2) stc[c] = v3;
      }
    }
    __syncthreads();
    // Window sums along the rows and the outputs.
    const int nseg = TW / seg;
    for (int item = threadIdx.x; item < nr * nseg; item += blockDim.x) {
      const int i = item / nseg;
      const int x = (item - i * nseg) * seg;
      const Pair* row = vb + i * pitch;
      const unsigned long long* crow = vc + i * pitch;
      S1 a1 = 0;
      S2 a2 = 0;
      unsigned long long a3 = 0;
      for (int k = 0; k < kw; ++k) {
        const Pair p = row[skew(x + k)];
        a1 += p.a;
        a2 += p.b;
        if constexpr (CM == 2) a3 += crow[skew(x + k)];
      }
#pragma unroll 1
      for (int j = 0; j < seg; ++j) {
        if (j > 0) {
          const Pair pa = row[skew(x + j + kw - 1)], pb = row[skew(x + j - 1)];
          a1 += pa.a - pb.a;
          a2 += pa.b - pb.b;
          if constexpr (CM == 2) a3 += crow[skew(x + j + kw - 1)] - crow[skew(x + j - 1)];
        }
        ob[i * TW + x + j] = finish(a1, a2, a3);
      }
    }
    __syncthreads();
    // The chunk's outputs, row by row (coalesced).
    for (int idx = threadIdx.x; idx < nr * TW; idx += blockDim.x) {
      const int i = idx / TW, xx = idx - i * TW;
      const long long gy = y0 + r0 + i, gx = x0 + xx;
      if (gy < g.H && gx < g.W) out[(z * g.H + gy) * g.W + gx] = ob[idx];
    }
  }
}

// Deviations in place of the staged samples (XK 0: int32 for float32 tiles
// whose deviations fit 30 bits; XK 1: int64 for float64 tiles), non-finite
// samples as marker words below every deviation (the most negative word plus
// the class: 0 NaN, 1 +inf, 2 -inf).
template <typename T, typename XW>
__device__ __forceinline__ void deviations_in_place(T* s, int support, int lo, i128 P, bool small) {
  XW* xw = reinterpret_cast<XW*>(s);
  constexpr XW kMark = sizeof(XW) == 4 ? (XW)INT_MIN : (XW)LLONG_MIN;
  const long long P64 = (long long)P;
  for (int e = threadIdx.x; e < support; e += blockDim.x) {
    const T v = s[e];
    XW x;
    if (!isfinite(v)) {
      x = kMark + (XW)(isnan(v) ? 0 : (v > (T)0 ? 1 : 2));
    } else if (small) {
      // top - lo <= 62: the sample's fixed value fits 63 bits.
      unsigned long long m;
      int pos;
      bool neg;
      long long f = 0;
      if (decompose(v, m, pos, neg)) {
        f = (long long)(m << (pos - lo));
        f = neg ? -f : f;
      }
      x = (XW)(f - P64);
    } else {
      x = (XW)(long long)(fixed(v, lo) - P);
    }
    xw[e] = x;
  }
}

// One output tile (index `tile`) of the sliding moments kernel; `tmap` is
// the launch's tensor map (nullptr: remapped staging only).
template <typename T>
__device__ __forceinline__ void moments_slide_body(const T* __restrict__ in, T* __restrict__ out,
                                                   const TileArgs& a, const SlideArgs& sa, long long tile,
                                                   unsigned char* smem_raw, const CUtensorMap* tmap) {
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Reduce& r = a.r;
  const SlideLayout L = slide_layout(t, g.kd, (int)sizeof(T), sa.rows);
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(smem_raw + L.s);
  long long z, y0, x0;
  net::tile_coords(a, tile, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, (T)r.cval, [](T v) { return v; })) return;
  __syncthreads();
  const int support = t.SH * t.SW;
  const Span<T> sp = tile_span<T, kSThreads>(s, support);
  const int lo = sp.lo;
  const int kw = g.kw, TW = t.TW, SW = t.SW;
  if (!span_fits(sp, sa.count_bits)) {
    // A value range too wide for the integer widths: the reference's float64
    // arithmetic per window (bit-identical to it) over the staged support.
    for (int o = threadIdx.x; o < TW * t.TH; o += blockDim.x) {
      const int ty = o / TW, tx = o - ty * TW;
      const long long gy = y0 + ty, gx = x0 + tx;
      if (gy >= g.H || gx >= g.W) continue;
      const int b = ty * SW + tx;
      auto fetch64 = [&](int i) -> double { return (double)s[b + (i / kw) * SW + i % kw]; };
      out[(z * g.H + gy) * g.W + gx] = canonical(from_f64<T>(mom::moments_exact(fetch64, r)));
    }
    return;
  }
  const i128 P = fixed(sp.pivot, lo);
  const int bits = deviation_bits(sp);
  const bool small = sp.top - lo <= 62;
  // 64-bit sums when every window's sum of X^2 fits (and with it the sum of
  // X); the count of a single non-finite class rides above the sum of X when
  // both fit one word.
  const bool narrow = 2 * bits + sa.count_bits <= 63;
  const int cm = sp.classes == 0 ? 0
                 : (__popc(sp.classes) == 1 && narrow && bits + 2 * sa.count_bits <= 62) ? 1
                                                                                      : 2;
  if constexpr (sizeof(T) == 4) {
    if (bits <= 30 && small) {
      deviations_in_place<T, int>(s, support, lo, P, true);
      __syncthreads();
      if (narrow) {
        if (cm == 0)
          column_walk<T, 0, true, 0>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
        else if (cm == 1)
          column_walk<T, 0, true, 1>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
        else
          column_walk<T, 0, true, 2>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
      } else {
        column_walk<T, 0, false, 2>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
      }
    } else {
      column_walk<T, 2, false, 2>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
    }
  } else {
    deviations_in_place<T, long long>(s, support, lo, P, small);
    __syncthreads();
    if (narrow) {
      if (cm == 0)
        column_walk<T, 1, true, 0>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
      else if (cm == 1)
        column_walk<T, 1, true, 1>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
      else
        column_walk<T, 1, true, 2>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
    } else {
      column_walk<T, 1, false, 2>(smem_raw, L, s, a, sa, sp, P, bits, z, y0, x0, out);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kSThreads)
    moments_slide_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                         const __grid_constant__ SlideArgs sa, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  moments_slide_body<T>(in, out, a, sa, blockIdx.x, smem_raw, &tmap);
}

// Batched float32 images: one persistent launch over the concatenated tile
// lists; a block finds a tile's image by binary search over the images'
// first tiles and keeps its arguments in shared memory until the image
// changes. Staging is the remapped path.
struct SlideTask {
  const float* in;
  float* out;
  long long first_tile;
  TileArgs a;
  SlideArgs sa;
};

__global__ void __launch_bounds__(kSThreads)
    slide_family_kernel(const SlideTask* __restrict__ tasks, int ntasks, long long total_tiles) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ SlideTask task;
  __shared__ int current, found;
  if (threadIdx.x == 0) current = -1;
  __syncthreads();
  for (long long tile = blockIdx.x; tile < total_tiles; tile += gridDim.x) {
    if (threadIdx.x == 0) {
      int lo = 0, hi = ntasks - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].first_tile <= tile)
          lo = mid;
        else
          hi = mid - 1;
      }
      found = lo;
    }
    __syncthreads();
    const int index = found;
    if (index != current) {
      const long long* src = reinterpret_cast<const long long*>(tasks + index);
      long long* dst = reinterpret_cast<long long*>(&task);
      for (int i = threadIdx.x; i < (int)(sizeof(SlideTask) / 8); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      if (threadIdx.x == 0) current = index;
    }
    __syncthreads();
    moments_slide_body<float>(task.in, task.out, task.a, task.sa, tile - task.first_tile, smem_raw, nullptr);
    __syncthreads();
  }
}

int count_bits_of(const Plan& p) { return 64 - __builtin_clzll((unsigned long long)p.r.count + 1); }

template <typename T>
cudaError_t launch_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  auto kernel = moments_slide_kernel<T>;
  cudaError_t e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  SlideArgs sa{count_bits_of(p), p.slide_rows};
  TileArgs args = p.tile;
  CUtensorMap map{};
  // The TMA staging area overlays the chunk buffers (see SlideLayout).
  size_t smem = slide_layout(p.tile.t, p.tile.g.kd, (int)sizeof(T), p.slide_rows).vbuf;
  if (tma_prepare(p, p.tile.t, in, &map, &args, &smem))
    smem = std::max(smem, p.smem_bytes);
  else
    smem = p.smem_bytes;
  kernel<<<(unsigned)p.tile.t.tiles, kSThreads, smem, s>>>(in, out, args, sa, map);
  return cudaGetLastError();
}

}  // namespace

// Tile shape and chunk rows of the sliding moments kernel, in the order
// measured fastest on the GB300 (4096^2 float32 / float64): 64 x 32 outputs
// in chunks of 16 rows for most windows (31 x 31: 0.53 ms; 9 x 9: 0.36 ms;
// 31 x 31 float64: 1.87 ms); 128 x 16 in chunks of 8 for flat windows whose
// width is at least four times their height (7 x 51: 0.48 ms; 1 x 31:
// 0.35 ms); 128 x 64 / 64 x 64 in chunks of 16 for windows of 48 rows and
// columns or more (65 x 65: 1.02 ms; 101 x 101: 1.88 ms); then smaller
// tiles down to 32 x 8 when shared memory is short. Single-row arrays take
// 1024 x 1 tiles. False when the window or the array does not suit the
// kernel (footprints, rank 3, counts beyond 16 bits, supports beyond shared
// memory).
bool moments_slide_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1 || !p.footprint.empty()) return false;
  const long long volume = (long long)g.kh * g.kw;
  if (volume + g.kw + g.kh >= 65535) return false;
  const int elem = p.dtype == 0 ? 4 : 8;
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
  auto take = [&](int tw, int th, int rows) {
    const Tile t = shape(tw, th);
    const size_t bytes = slide_layout(t, g.kd, elem, rows).total;
    if (bytes > (size_t)smem_limit) return false;
    p.tile.t = t;
    p.slide_rows = rows;
    p.smem_bytes = bytes;
    return true;
  };
  if (g.H == 1 && g.kh == 1) return take(1024, 1, 1);
  if (g.kw >= 4 * g.kh && g.kh <= 16 && take(128, 16, 8)) return true;
  if (g.kh >= 48 && g.kw >= 48 && (take(128, 64, 16) || take(64, 64, 16))) return true;
  static const int order[][3] = {{64, 32, 16}, {64, 64, 16}, {128, 32, 8}, {32, 64, 32},
                                 {32, 32, 32}, {32, 16, 16}, {32, 8, 8}};
  for (const auto& o : order)
    if (take(o[0], o[1], o[2])) return true;
  return false;
}

cudaError_t launch_moments_slide(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}

namespace {

int slide_family_variant(const Plan& p) { return p.algo == Algo::kMomentsSlide && p.dtype == 0 ? 0 : -1; }

long long slide_family_tiles(const Plan& p) { return p.tile.t.tiles; }

long long slide_family_slot_bytes(const Plan&) { return 0; }

void slide_family_write_task(const Plan& p, const void* in, void* out, long long first_tile, void* task) {
  SlideTask t{};
  t.in = (const float*)in;
  t.out = (float*)out;
  t.first_tile = first_tile;
  t.a = p.tile;
  t.a.r = p.r;
  t.a.tma_bw = 0;
  t.sa.count_bits = count_bits_of(p);
  t.sa.rows = p.slide_rows;
  std::memcpy(task, &t, sizeof(t));
}

const void* slide_family_kernel_of(int) { return (const void*)slide_family_kernel; }

cudaError_t slide_family_launch(int, const void* d_tasks, int ntasks, long long tiles, unsigned char*, long long,
                                size_t smem, int grid, cudaStream_t s) {
  void* args[] = {(void*)&d_tasks, &ntasks, &tiles};
  return cudaLaunchKernel((const void*)slide_family_kernel, dim3(grid), dim3(kSThreads), args, smem, s);
}

}  // namespace

const FamilyOps& slide_family_ops() {
  static const FamilyOps ops{sizeof(SlideTask), slide_family_variant, slide_family_tiles, slide_family_slot_bytes,
                             slide_family_write_task, slide_family_kernel_of, slide_family_launch};
  return ops;
}

}  // namespace ndf

// Register sorting networks and their epilogues, shared by the tile
// selection kernels (select.cu, box.cu).
#pragma once

#include <utility>

#include "common.cuh"
#include "plan.h"
#include "staging.cuh"

namespace ndf {
namespace net {

constexpr int kThreads = 256;

template <int N>
struct TapTable {
  int32_t off[N];
};

template <typename K>
__device__ __forceinline__ void cmpx(K& a, K& b) {
  K lo = a < b ? a : b;
  K hi = a < b ? b : a;
  a = lo;
  b = hi;
}

// Batcher odd-even merge sort over N (a power of two) wires, generated at
// compile time as a comparator table and applied by a fold expression, so
// every wire index is a constant expression and the keys stay in registers.
template <int N, int PSTART = 1>
struct Batcher {
  static constexpr bool same_block(int lo, int hi, int p) { return lo / (2 * p) == hi / (2 * p); }
  static constexpr int count() {
    int c = 0;
    for (int p = PSTART; p < N; p <<= 1)
      for (int k = p; k >= 1; k >>= 1)
        for (int j = k % p; j + k < N; j += 2 * k)
          for (int i = 0; i < k && i + j + k < N; ++i)
            if (same_block(i + j, i + j + k, p)) ++c;
    return c;
  }
  static constexpr int kCount = count();
  struct Table {
    short lo[kCount];
    short hi[kCount];
  };
  static constexpr Table table() {
    Table t{};
    int c = 0;
    for (int p = PSTART; p < N; p <<= 1)
      for (int k = p; k >= 1; k >>= 1)
        for (int j = k % p; j + k < N; j += 2 * k)
          for (int i = 0; i < k && i + j + k < N; ++i)
            if (same_block(i + j, i + j + k, p)) {
              t.lo[c] = (short)(i + j);
              t.hi[c] = (short)(i + j + k);
              ++c;
            }
    return t;
  }
  static constexpr Table kTable = table();
};

template <int N, int PSTART, int I, typename K>
__device__ __forceinline__ void cmpx_at(K (&a)[N]) {
  constexpr int lo = Batcher<N, PSTART>::kTable.lo[I];
  constexpr int hi = Batcher<N, PSTART>::kTable.hi[I];
  cmpx(a[lo], a[hi]);
}

template <int N, int PSTART, typename K, int... Is>
__device__ __forceinline__ void apply_network(K (&a)[N], std::integer_sequence<int, Is...>) {
  (cmpx_at<N, PSTART, Is>(a), ...);
}

template <int N, typename K>
__device__ __forceinline__ void batcher_sort(K (&a)[N]) {
  apply_network<N, 1>(a, std::make_integer_sequence<int, Batcher<N, 1>::kCount>{});
}

// Merge of two sorted halves a[0, N/2) and a[N/2, N): the last level of the
// Batcher network.
template <int N, typename K>
__device__ __forceinline__ void batcher_merge(K (&a)[N]) {
  apply_network<N, N / 2>(a, std::make_integer_sequence<int, Batcher<N, N / 2>::kCount>{});
}

constexpr int pow2_at_least(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Register pick a[idx] for a runtime idx < BOUND.
template <int BOUND, int N, typename K>
__device__ __forceinline__ K pick(const K (&a)[N], int idx) {
  K v = a[0];
#pragma unroll
  for (int i = 1; i < BOUND; ++i) v = (i == idx) ? a[i] : v;
  return v;
}

template <typename T>
__device__ __forceinline__ T median_of_two(T lower, T upper) {
  if constexpr (sizeof(T) == 4) {
    return midpoint_f32(lower, upper);
  } else {
    return midpoint(lower, upper);
  }
}

// Epilogue of the register network: the statistic from sorted keys.
// MODE 0: any selection kind, runtime policy. MODE 1: median kinds only.
template <typename T, int N, int VFIX, int MODE, typename K>
__device__ __forceinline__ T network_finish(const K (&k)[N], int nv, const Reduce& r) {
  using KO = KeyOf<T>;
  const int V = VFIX > 0 ? VFIX : r.count;
  const bool missing = r.omit ? (nv < r.min_count) : (nv != V);
  if (missing || nv == 0) return nan_of(T());
  if (MODE == 1) {
    if (VFIX > 0 && !r.omit) {
      // Propagate with a fixed tap count: compile-time ranks.
      if (VFIX & 1) return KO::value(k[VFIX / 2]);
      return median_of_two(KO::value(k[VFIX / 2 - 1]), KO::value(k[VFIX / 2]));
    }
    constexpr int B = (VFIX > 0 ? VFIX : N) / 2 + 1;
    if constexpr (VFIX >= 9 && VFIX % 2 == 1) {
      // With at most 4 dropped samples (odd VFIX) the middle ranks lie in
      // [VFIX/2 - 2, VFIX/2]: a 3-way pick instead of a B-way one.
      constexpr int L = VFIX / 2 - 2;
      if (nv >= VFIX - 4) {
        const int hi = nv / 2 - L;  // 0, 1 or 2
        const K c0 = k[L], c1 = k[L + 1], c2 = k[L + 2];
        const K a_hi = hi == 0 ? c0 : (hi == 1 ? c1 : c2);
        if (nv & 1) return KO::value(a_hi);
        const K a_lo = hi == 1 ? c0 : c1;  // even nv: hi is 1 or 2
        return median_of_two(KO::value(a_lo), KO::value(a_hi));
      }
    }
    if (nv & 1) return KO::value(pick<B>(k, nv / 2));
    return median_of_two(KO::value(pick<B>(k, nv / 2 - 1)), KO::value(pick<B>(k, nv / 2)));
  }
  constexpr int A = (VFIX > 0 && VFIX < N) ? VFIX : N;
  switch (r.kind) {
    case kMin:
      return KO::value(k[0]);
    case kMax:
      return KO::value(pick<A>(k, nv - 1));
    case kRank:
    case kRankHistogram:
      if (r.param >= nv) return nan_of(T());
      return KO::value(pick<A>(k, (int)r.param));
    case kPercentile: {
      if (r.q_is_max) return KO::value(pick<A>(k, nv - 1));
      const PctSplit ps = pct_split(r, nv);
      return pct_value<T>(ps, KO::value(pick<A>(k, ps.lower)), KO::value(pick<A>(k, ps.upper)));
    }
    default:
      if (nv & 1) return KO::value(pick<A>(k, nv / 2));
      return median_of_two(KO::value(pick<A>(k, nv / 2 - 1)), KO::value(pick<A>(k, nv / 2)));
  }
}

__device__ __forceinline__ void tile_coords(const TileArgs& a, long long tile, long long& z,
                                            long long& y0, long long& x0) {
  long long tx = tile % a.t.tiles_x;
  long long rest = tile / a.t.tiles_x;
  long long ty = rest % a.t.tiles_y;
  z = rest / a.t.tiles_y;
  y0 = ty * a.t.TH;
  x0 = tx * a.t.TW;
}

// One output tile of the register-network kernel. `tap(i)` returns the
// shared-memory offset of tap i relative to a thread's output.
template <typename T, int N, int VFIX, int MODE, typename Tap>
__device__ __forceinline__ void tile_network_body(const T* __restrict__ in, T* __restrict__ out,
                                                  const TileArgs& a, long long tile,
                                                  unsigned char* smem_raw, Tap tap,
                                                  const CUtensorMap* tmap = nullptr) {
  using K = typename KeyOf<T>::K;
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  K* s = reinterpret_cast<K*>(maps + (t.SW + t.SH + g.kd));
  long long z, y0, x0;
  tile_coords(a, tile, z, y0, x0);
  const bool drop_inf = a.r.drop_inf;
  const K outside = sample_key<T>((T)a.r.cval, drop_inf);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, outside,
                  [&](T v) { return sample_key<T>(v, drop_inf); }))
    return;
  __syncthreads();

  const int tx = threadIdx.x % t.TW;
  const int ty = threadIdx.x / t.TW;
  const long long y = y0 + ty, x = x0 + tx;
  if (ty >= t.TH || y >= g.H || x >= g.W) return;
  const K* base = s + ty * t.SW + tx;
  const int V = VFIX > 0 ? VFIX : a.r.count;
  K k[N];
#pragma unroll
  for (int i = 0; i < N; ++i) k[i] = i < V ? base[tap(i)] : KeyOf<T>::kSentinel;
  int nv = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) nv += (i < V && k[i] != KeyOf<T>::kSentinel) ? 1 : 0;
  batcher_sort<N>(k);
  T result = network_finish<T, N, VFIX, MODE>(k, nv, a.r);
  out[(z * g.H + y) * g.W + x] = canonical(result);
}

// ---------------------------------------------------------------------------
// Bit-serial radix select: the k-th smallest retained key (k < nv). Bits
// shared by every retained key (from their AND and OR) are skipped.
template <typename K, typename Fetch>
__device__ __forceinline__ K radix_select(Fetch&& fetch, int V, long long k, K and_v, K or_v) {
  K diff = and_v ^ or_v;
  if (diff == 0) return and_v;
  const int bits = sizeof(K) * 8;
  int top = bits - 1 - (sizeof(K) == 8 ? __clzll((long long)diff) : __clz((int)diff));
  K mask = top + 1 >= bits ? K(0) : ~((K(1) << (top + 1)) - 1);
  K prefix = and_v & mask;
  for (int b = top; b >= 0; --b) {
    K bit = K(1) << b;
    K m = mask | bit;
    long long c = 0;
    for (int i = 0; i < V; ++i) c += ((fetch(i) & m) == prefix) ? 1 : 0;
    if (k >= c) {
      k -= c;
      prefix |= bit;
    }
    mask = m;
  }
  return prefix;
}

struct KeyStats {
  int nv;
};

template <typename T, typename K, typename Fetch>
__device__ __forceinline__ T radix_finish(Fetch&& fetch, const Reduce& r) {
  using KO = KeyOf<T>;
  const K sent = KO::kSentinel;
  const int V = r.count;
  int nv = 0;
  K and_v = sent, or_v = 0, kmin = sent, kmax = 0;
  for (int i = 0; i < V; ++i) {
    K key = fetch(i);
    if (key != sent) {
      nv += 1;
      and_v &= key;
      or_v |= key;
      kmin = key < kmin ? key : kmin;
      kmax = key > kmax ? key : kmax;
    }
  }
  const bool missing = r.omit ? (nv < r.min_count) : (nv != V);
  if (missing || nv == 0) return nan_of(T());
  auto sel = [&](long long kk) { return radix_select<K>(fetch, V, kk, and_v, or_v); };
  switch (r.kind) {
    case kMin:
      return KO::value(kmin);
    case kMax:
      return KO::value(kmax);
    case kRank:
    case kRankHistogram:
      if (r.param >= nv) return nan_of(T());
      return KO::value(sel(r.param));
    case kPercentile: {
      if (r.q_is_max) return KO::value(kmax);
      const PctSplit ps = pct_split(r, nv);
      const T lo = KO::value(sel(ps.lower));
      const T hi = ps.upper == ps.lower ? lo : KO::value(sel(ps.upper));
      return pct_value<T>(ps, lo, hi);
    }
    default:
      if (nv & 1) return KO::value(sel(nv / 2));
      return median_of_two(KO::value(sel(nv / 2 - 1)), KO::value(sel(nv / 2)));
  }
}

// One output tile of the radix-select kernel; `taps` are shared-memory
// offsets relative to a thread's output.
template <typename T>
__device__ __forceinline__ void tile_radix_body(const T* __restrict__ in, T* __restrict__ out,
                                                const TileArgs& a, long long tile,
                                                unsigned char* smem_raw, const int32_t* taps) {
  using K = typename KeyOf<T>::K;
  const Geom3& g = a.g;
  const Tile& t = a.t;
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  K* s = reinterpret_cast<K*>(maps + (t.SW + t.SH + g.kd));
  long long z, y0, x0;
  tile_coords(a, tile, z, y0, x0);
  build_maps(maps, g, t, z, y0, x0);
  __syncthreads();
  const bool drop_inf = a.r.drop_inf;
  const K outside = sample_key<T>((T)a.r.cval, drop_inf);
  stage_support(s, maps, in, g, t, outside, [&](T v) { return sample_key<T>(v, drop_inf); });
  __syncthreads();
  const int tx = threadIdx.x % t.TW;
  const int ty = threadIdx.x / t.TW;
  const long long y = y0 + ty, x = x0 + tx;
  if (ty >= t.TH || y >= g.H || x >= g.W) return;
  const K* base = s + ty * t.SW + tx;
  auto fetch = [&](int i) -> K { return base[taps[i]]; };
  T result = radix_finish<T, K>(fetch, a.r);
  out[(z * g.H + y) * g.W + x] = canonical(result);
}

}  // namespace net
}  // namespace ndf

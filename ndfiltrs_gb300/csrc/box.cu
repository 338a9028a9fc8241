// Box-window pair kernel (see tile_box_kernel): 3x3, 5x5 and 7x7 windows in
// 2-D arrays, two vertically adjacent outputs per thread sharing the sort of
// their common rows.
#include <cstring>

#include "network.cuh"

namespace ndf {
namespace {
using namespace net;

// ---------------------------------------------------------------------------
// Box windows (KH x KW, compile-time) in 2-D: each thread computes vertically
// adjacent output pairs. The two windows share KH - 1 rows: those keys are
// sorted once, each private row is sorted separately, and each output merges
// the shared sorted run with its private run (the last Batcher level). With a
// fixed tile width every tap offset is a compile-time shared-memory
// immediate.
constexpr int kBoxTW = 32;
constexpr int kBoxPairs = 2;  // pairs per thread: tile height 16 * kBoxPairs

// The key of rank R (0-based) in the union of two sorted runs `a` and `b`,
// NB of b's keys in play: R + 1 smallest keys split as p from a and q from
// b, and the rank-R key is the smallest over splits of the larger last
// element, min over q of max(a[R - q], b[q - 1]) (q = 0: a[R]). Dropped
// samples sit at the runs' ends as the largest key and never win for
// R below the retained count. 2 NB + 1 operations instead of a merge.
template <int R, int NB, int P, typename K>
__device__ __forceinline__ K union_rank(const K (&a)[P], const K (&b)[P]) {
  static_assert(R < P, "rank beyond the first run");
  K best = a[R];
#pragma unroll
  for (int q = 1; q <= NB; ++q) {
    if (q > R + 1) break;
    const K t = (R - q >= 0) ? (a[R - q > 0 ? R - q : 0] > b[q - 1] ? a[R - q > 0 ? R - q : 0] : b[q - 1])
                             : b[q - 1];
    best = t < best ? t : best;
  }
  return best;
}

// The window median (Reduction::finish for the median kinds,
// src/reduction.rs:78-130) from the shared and private sorted runs: the
// reducers midpoint for even counts, NaN when the window has too few
// retained samples (omit) or any dropped one (propagate). With at most four
// dropped samples the middle ranks lie in [V/2 - 2, V/2]; otherwise the runs
// are merged.
template <typename T, int V, int NB, int P, typename K>
__device__ __forceinline__ T box_median(const K (&sh)[P], const K (&pv)[P], int nv, const Reduce& r) {
  using KO = KeyOf<T>;
  const bool missing = r.omit ? (nv < r.min_count) : (nv != V);
  if (missing || nv == 0) return nan_of(T());
  if (!r.omit) {
    if constexpr (V & 1) return KO::value(union_rank<V / 2, NB>(sh, pv));
    else return median_of_two(KO::value(union_rank<V / 2 - 1, NB>(sh, pv)), KO::value(union_rank<V / 2, NB>(sh, pv)));
  }
  if constexpr (V >= 9 && (V & 1)) {
    constexpr int L = V / 2 - 2;
    if (nv >= V - 4) {
      const K c0 = union_rank<L, NB>(sh, pv), c1 = union_rank<L + 1, NB>(sh, pv), c2 = union_rank<L + 2, NB>(sh, pv);
      const int hi = nv / 2 - L;  // 0, 1 or 2
      const K a_hi = hi == 0 ? c0 : (hi == 1 ? c1 : c2);
      if (nv & 1) return KO::value(a_hi);
      const K a_lo = hi == 1 ? c0 : c1;  // even nv: hi is 1 or 2
      return median_of_two(KO::value(a_lo), KO::value(a_hi));
    }
  }
  K m[2 * P];
#pragma unroll
  for (int i = 0; i < P; ++i) {
    m[i] = sh[i];
    m[P + i] = pv[i];
  }
  batcher_merge<2 * P>(m);
  return network_finish<T, 2 * P, V, 1>(m, nv, r);
}

// One output tile (index `tile`) of the box pair kernel; `tmap` is the
// launch's tensor map (nullptr: remapped staging only).
template <typename T, int KH, int KW, int MODE>
__device__ __forceinline__ void tile_box_body(const T* __restrict__ in, T* __restrict__ out, const TileArgs& a,
                                              long long tile, unsigned char* smem_raw, const CUtensorMap* tmap) {
  using K = typename KeyOf<T>::K;
  constexpr K kSent = KeyOf<T>::kSentinel;
  constexpr int SW = kBoxTW + KW - 1;
  constexpr int SHARED = (KH - 1) * KW;
  constexpr int P = pow2_at_least(SHARED > KW ? SHARED : KW);
  constexpr int V = KH * KW;
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

  const int tx = threadIdx.x % kBoxTW;
  const int tr = threadIdx.x / kBoxTW;
  const long long x = x0 + tx;
  if (x >= g.W) return;
#pragma unroll 1
  for (int pair = 0; pair < kBoxPairs; ++pair) {
    const int row0 = 2 * (tr + (kThreads / kBoxTW) * pair);
    const long long y = y0 + row0;
    if (y >= g.H) break;
    const K* base = s + row0 * SW + tx;
    K sh[P], pa[P], pb[P];
    int n_sh = 0, n_a = 0, n_b = 0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      sh[i] = i < SHARED ? base[(1 + i / KW) * SW + i % KW] : kSent;
      pa[i] = i < KW ? base[i] : kSent;
      pb[i] = i < KW ? base[KH * SW + i] : kSent;
      n_sh += (i < SHARED && sh[i] != kSent) ? 1 : 0;
      n_a += (i < KW && pa[i] != kSent) ? 1 : 0;
      n_b += (i < KW && pb[i] != kSent) ? 1 : 0;
    }
    batcher_sort<P>(sh);
    batcher_sort<P>(pa);
    batcher_sort<P>(pb);
    if constexpr (MODE == 1) {
      out[(z * g.H + y) * g.W + x] = canonical(box_median<T, V, KW>(sh, pa, n_sh + n_a, a.r));
      if (y + 1 < g.H)
        out[(z * g.H + y + 1) * g.W + x] = canonical(box_median<T, V, KW>(sh, pb, n_sh + n_b, a.r));
      continue;
    }
    {
      K m[2 * P];
#pragma unroll
      for (int i = 0; i < P; ++i) {
        m[i] = sh[i];
        m[P + i] = pa[i];
      }
      batcher_merge<2 * P>(m);
      out[(z * g.H + y) * g.W + x] = canonical(network_finish<T, 2 * P, V, MODE>(m, n_sh + n_a, a.r));
    }
    if (y + 1 < g.H) {
      K m[2 * P];
#pragma unroll
      for (int i = 0; i < P; ++i) {
        m[i] = sh[i];
        m[P + i] = pb[i];
      }
      batcher_merge<2 * P>(m);
      out[(z * g.H + y + 1) * g.W + x] = canonical(network_finish<T, 2 * P, V, MODE>(m, n_sh + n_b, a.r));
    }
  }
}

template <typename T, int KH, int KW, int MODE>
__global__ void __launch_bounds__(kThreads)
    tile_box_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                    const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tile_box_body<T, KH, KW, MODE>(in, out, a, blockIdx.x, smem_raw, &tmap);
}

// Batched images (float32) of one box size and epilogue: one persistent
// launch over the concatenated tile lists; a block finds a tile's image by
// binary search over the images' first tiles and keeps its arguments in
// shared memory until the image changes. Staging is the remapped path.
struct BoxTask {
  const float* in;
  float* out;
  long long first_tile;
  TileArgs a;
};

template <int KH, int KW, int MODE>
__global__ void __launch_bounds__(kThreads)
    box_family_kernel(const BoxTask* __restrict__ tasks, int ntasks, long long total_tiles) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ BoxTask task;
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
      for (int i = threadIdx.x; i < (int)(sizeof(BoxTask) / 8); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      if (threadIdx.x == 0) current = index;
    }
    __syncthreads();
    tile_box_body<float, KH, KW, MODE>(task.in, task.out, task.a, tile - task.first_tile, smem_raw, nullptr);
    __syncthreads();
  }
}

template <typename T, int KH, int KW>
cudaError_t launch_box(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork;
  auto kernel = median ? tile_box_kernel<T, KH, KW, 1> : tile_box_kernel<T, KH, KW, 0>;
  cudaError_t e =
      allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  TileArgs args = p.tile;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, p.tile.t, in, &map, &args, &smem);
  kernel<<<(unsigned)p.tile.t.tiles, kThreads, smem, s>>>(in, out, args, map);
  return cudaGetLastError();
}

}  // namespace

bool box_supported(int dtype, int kh, int kw) {
  if (kh == 3 && kw == 3) return true;
  if (kh == 5 && kw == 5) return true;
  return dtype == 0 && kh == 7 && kw == 7;
}

Tile box_tile(const Geom3& g) {
  Tile t{};
  t.TW = kBoxTW;
  t.TH = 16 * kBoxPairs;
  t.SW = t.TW + g.kw - 1;
  t.SH = t.TH + g.kh - 1;
  t.tiles_x = (g.W + t.TW - 1) / t.TW;
  t.tiles_y = (g.H + t.TH - 1) / t.TH;
  t.tiles = t.tiles_x * t.tiles_y * g.D;
  return t;
}

cudaError_t launch_tile_box(const Plan& p, const void* in, void* out, cudaStream_t s) {
  const int kh = p.tile.g.kh, kw = p.tile.g.kw;
  if (p.dtype == 0) {
    const float* i = (const float*)in;
    float* o = (float*)out;
    if (kh == 3 && kw == 3) return launch_box<float, 3, 3>(p, i, o, s);
    if (kh == 5 && kw == 5) return launch_box<float, 5, 5>(p, i, o, s);
    if (kh == 7 && kw == 7) return launch_box<float, 7, 7>(p, i, o, s);
  } else {
    const double* i = (const double*)in;
    double* o = (double*)out;
    if (kh == 3 && kw == 3) return launch_box<double, 3, 3>(p, i, o, s);
    if (kh == 5 && kw == 5) return launch_box<double, 5, 5>(p, i, o, s);
  }
  return cudaErrorInvalidValue;
}

namespace {

// Variants: 2 * size index (3x3, 5x5, 7x7) + median epilogue.
int box_family_variant(const Plan& p) {
  if (p.algo != Algo::kTileBox || p.dtype != 0) return -1;
  const Geom3& g = p.tile.g;
  const int size = g.kh == 3 && g.kw == 3 ? 0 : g.kh == 5 && g.kw == 5 ? 1 : g.kh == 7 && g.kw == 7 ? 2 : -1;
  if (size < 0) return -1;
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork;
  return 2 * size + (median ? 1 : 0);
}

long long box_family_tiles(const Plan& p) { return p.tile.t.tiles; }

long long box_family_slot_bytes(const Plan&) { return 0; }

void box_family_write_task(const Plan& p, const void* in, void* out, long long first_tile, void* task) {
  BoxTask t{};
  t.in = (const float*)in;
  t.out = (float*)out;
  t.first_tile = first_tile;
  t.a = p.tile;
  t.a.r = p.r;
  t.a.tma_bw = 0;
  std::memcpy(task, &t, sizeof(t));
}

const void* box_family_kernel_of(int v) {
  static const void* const table[] = {
      (const void*)box_family_kernel<3, 3, 0>, (const void*)box_family_kernel<3, 3, 1>,
      (const void*)box_family_kernel<5, 5, 0>, (const void*)box_family_kernel<5, 5, 1>,
      (const void*)box_family_kernel<7, 7, 0>, (const void*)box_family_kernel<7, 7, 1>};
  return table[v];
}

cudaError_t box_family_launch(int v, const void* d_tasks, int ntasks, long long tiles, unsigned char*, long long,
                              size_t smem, int grid, cudaStream_t s) {
  void* args[] = {(void*)&d_tasks, &ntasks, &tiles};
  return cudaLaunchKernel(box_family_kernel_of(v), dim3(grid), dim3(kThreads), args, smem, s);
}

}  // namespace

const FamilyOps& box_family_ops() {
  static const FamilyOps ops{sizeof(BoxTask), box_family_variant, box_family_tiles, box_family_slot_bytes,
                             box_family_write_task, box_family_kernel_of, box_family_launch};
  return ops;
}

}  // namespace ndf

// Separable sliding minimum / maximum for rectangular 1-D / 2-D windows.
//
// Replaces extrema_into (src/extrema.rs:124-437; van Herk / Gil-Werman):
// results equal direct selection bit for bit (total order, the invalid-value
// policies, min_count), because a window's minimum is the minimum of its
// column minima and every comparison runs on order-preserving keys.
//
// GB300 design: one thread block per 32 x TH output tile. The block stages
// its support (one TMA copy for an interior tile) as keys: retained samples
// keep their key (complemented for the maximum, so both run as a minimum),
// dropped samples (NaN, and infinities under ignore_inf) take the all-ones
// key. Pass 1 runs down each support column: prefix and suffix minima within
// blocks of kh rows give every window's column minimum as
// min(suffix[r], prefix[r + kh - 1]) (three comparisons per sample for any
// kh), and a sliding sum counts the retained samples. Pass 2 does the same
// along each output row over kw columns. The per-output cost does not grow
// with the window.
#include <algorithm>

#include "network.cuh"
#include "plan.h"
#include "staging.cuh"
#include "tma.cuh"

namespace ndf {
namespace {

constexpr int kEThreads = 256;

template <typename T>
struct Layout {
  using K = typename KeyOf<T>::K;
  size_t maps, keys, pre, vmin, vcnt, pcnt, total;
};

template <typename T>
__host__ __device__ inline Layout<T> layout(const Tile& t, int kd) {
  using K = typename KeyOf<T>::K;
  Layout<T> l;
  auto a16 = [](size_t v) { return (v + 15) & ~(size_t)15; };
  l.maps = 0;
  l.keys = a16((size_t)(t.SW + t.SH + kd) * 8);       // SH x SW keys (suffix minima in place)
  l.pre = a16(l.keys + (size_t)t.SH * t.SW * sizeof(K));  // SH x SW prefix minima
  l.vmin = a16(l.pre + (size_t)t.SH * t.SW * sizeof(K));  // TH x SW column minima
  l.vcnt = a16(l.vmin + (size_t)t.TH * t.SW * sizeof(K)); // TH x SW column counts
  l.pcnt = a16(l.vcnt + (size_t)t.TH * t.SW * 4);         // TH x (SW + 1) row prefix counts
  l.total = a16(l.pcnt + (size_t)t.TH * (t.SW + 1) * 4);
  return l;
}

template <typename T, bool MAXIMUM>
__global__ void __launch_bounds__(kEThreads)
    extrema_tile_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ TileArgs a,
                        const __grid_constant__ CUtensorMap tmap) {
  using KO = KeyOf<T>;
  using K = typename KO::K;
  constexpr K kNone = KO::kSentinel;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Layout<T> l = layout<T>(t, g.kd);
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  K* keys = reinterpret_cast<K*>(smem_raw + l.keys);
  K* pre = reinterpret_cast<K*>(smem_raw + l.pre);
  K* vmin = reinterpret_cast<K*>(smem_raw + l.vmin);
  unsigned int* vcnt = reinterpret_cast<unsigned int*>(smem_raw + l.vcnt);
  unsigned int* pcnt = reinterpret_cast<unsigned int*>(smem_raw + l.pcnt);
  long long z, y0, x0;
  net::tile_coords(a, blockIdx.x, z, y0, x0);
  const bool drop_inf = a.r.drop_inf;
  auto conv = [&](T v) -> K {
    const K k = sample_key<T>(v, drop_inf);
    return (MAXIMUM && k != kNone) ? ~k : k;
  };
  const K outside = conv((T)a.r.cval);
  if (!stage_tile(keys, maps, smem_raw, in, a, &tmap, z, y0, x0, outside, conv)) return;
  __syncthreads();

  const int kh = g.kh, kw = g.kw, SW = t.SW, SH = t.SH, TH = t.TH, TW = t.TW;
  // Pass 1: down each support column.
  for (int c = threadIdx.x; c < SW; c += blockDim.x) {
    // Retained counts of every window's column part (sliding sum).
    unsigned int cnt = 0;
    for (int k = 0; k < kh; ++k) cnt += keys[k * SW + c] != kNone;
    for (int r = 0; r < TH; ++r) {
      vcnt[r * SW + c] = cnt;
      if (r + 1 < TH) cnt += (unsigned int)(keys[(r + kh) * SW + c] != kNone) -
                             (unsigned int)(keys[r * SW + c] != kNone);
    }
    // Prefix minima within blocks of kh rows.
    K run = kNone;
    for (int r = 0; r < SH; ++r) {
      const K k = keys[r * SW + c];
      run = (r % kh == 0) ? k : (k < run ? k : run);
      pre[r * SW + c] = run;
    }
    // Suffix minima within blocks, in place.
    run = kNone;
    for (int r = SH - 1; r >= 0; --r) {
      const K k = keys[r * SW + c];
      run = (r == SH - 1 || r % kh == kh - 1) ? k : (k < run ? k : run);
      keys[r * SW + c] = run;
    }
    for (int r = 0; r < TH; ++r) {
      const K s = keys[r * SW + c], p = pre[(r + kh - 1) * SW + c];
      vmin[r * SW + c] = s < p ? s : p;
    }
  }
  __syncthreads();

  // Pass 2: along each output row (prefix / suffix minima over blocks of kw
  // columns reuse the pass-1 arrays; prefix counts for the window sums).
  K* pre2 = pre;
  K* suf2 = keys;
  for (int item = threadIdx.x; item < TH; item += blockDim.x) {
    const int r = item;
    unsigned int acc = 0;
    pcnt[r * (SW + 1)] = 0;
    K run = kNone;
    for (int x = 0; x < SW; ++x) {
      acc += vcnt[r * SW + x];
      pcnt[r * (SW + 1) + x + 1] = acc;
      const K k = vmin[r * SW + x];
      run = (x % kw == 0) ? k : (k < run ? k : run);
      pre2[r * SW + x] = run;
    }
    run = kNone;
    for (int x = SW - 1; x >= 0; --x) {
      const K k = vmin[r * SW + x];
      run = (x == SW - 1 || x % kw == kw - 1) ? k : (k < run ? k : run);
      suf2[r * SW + x] = run;
    }
  }
  __syncthreads();

  const Reduce& red = a.r;
  for (int o = threadIdx.x; o < TW * TH; o += blockDim.x) {
    const int r = o / TW, x = o - r * TW;
    const long long gy = y0 + r, gx = x0 + x;
    if (gy >= g.H || gx >= g.W) continue;
    const K s = suf2[r * SW + x], p = pre2[r * SW + x + kw - 1];
    const K m = s < p ? s : p;
    const unsigned int n = pcnt[r * (SW + 1) + x + kw] - pcnt[r * (SW + 1) + x];
    const bool missing = red.omit ? ((long long)n < red.min_count) : ((int)n != red.count);
    const T v = (missing || n == 0) ? nan_of(T()) : KO::value(MAXIMUM ? ~m : m);
    out[(z * g.H + gy) * g.W + gx] = canonical(v);
  }
}

template <typename T>
cudaError_t launch_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const bool maximum = p.r.kind == kMax;
  auto kernel = maximum ? extrema_tile_kernel<T, true> : extrema_tile_kernel<T, false>;
  cudaError_t e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  TileArgs args = p.tile;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, p.tile.t, in, &map, &args, &smem);
  kernel<<<(unsigned)p.tile.t.tiles, kEThreads, smem, s>>>(in, out, args, map);
  return cudaGetLastError();
}

}  // namespace

// 32 x TH output tiles (TH the largest of 64, 32, 16, 8 whose shared memory
// fits in 100 KB, else in `smem_limit`), or 256 x 1 for single-row arrays.
// False for footprints, rank 3 and supports that do not fit.
bool extrema_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1 || !p.footprint.empty()) return false;
  if (p.r.kind != kMin && p.r.kind != kMax) return false;
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
    return p.dtype == 0 ? layout<float>(t, g.kd).total : layout<double>(t, g.kd).total;
  };
  if (g.H == 1 && g.kh == 1) {
    Tile t = shape(256, 1);
    if (bytes(t) > (size_t)smem_limit) return false;
    p.tile.t = t;
    p.smem_bytes = bytes(t);
    return true;
  }
  const size_t budget = std::min<size_t>(100 * 1024, (size_t)smem_limit);
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

cudaError_t launch_extrema(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}

}  // namespace ndf

// Separable sliding minimum / maximum for rectangular 1-D / 2-D windows.
//
// Replaces extrema_into (src/extrema.rs:124-437; van Herk / Gil-Werman):
// results equal direct selection bit for bit (total order, the invalid-value
// policies, min_count), because a window's minimum is the minimum of its
// column minima and every comparison runs on order-preserving keys.
//
// GB300 design, two kernels:
//  * extrema_pass_kernel (the default): two launches of one column pass.
//    Each block takes a strip of 32 columns and R rows, stages those rows
//    plus the window halo (through the boundary mode) as keys, runs van Herk
//    down every column in blocks of the window length (prefix and suffix
//    minima, three comparisons per sample for any window) with all threads
//    busy on (column, block) pairs, and writes its strip transposed. The
//    first launch reduces along the rows of the image into a transposed key
//    array, the second reduces along the original columns and transposes
//    back, so both read and write whole 128-byte lines.
//  * extrema_tile_kernel: one block per 32 x TH output tile doing both
//    passes in shared memory (an autotuner alternative).
// Keys: retained samples keep their key (complemented for the maximum, so
// both run as a minimum), dropped samples take the all-ones key, and under
// the propagate policy a NaN takes key 0, which wins every minimum: such a
// window's minimum is 0 exactly when it holds a NaN. Retained counts ride
// along only when min_count > 1.
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

constexpr int kStrip = 32;       // columns per block of the column pass
constexpr int kPitch = kStrip + 1;  // shared-memory row pitch (conflict-free transposes)

struct PassArgs {
  long long rows, cols;  // source array: `rows` along the pass, `cols` contiguous
  int k, anchor, mode;   // window length, anchor and boundary mode along the pass
  int R;                 // output rows per block
  long long strips;      // blocks per row of blocks
  int prior;             // window length of the previous pass (its outside count)
  Reduce r;
};

template <typename K, bool COUNT>
__host__ __device__ inline size_t pass_smem(int R, int k) {
  const size_t sh = (size_t)R + k - 1;
  return sh * kPitch * (2 * sizeof(K) + (COUNT ? 4 : 0)) + 16;
}

// One column pass: sliding minimum over `k` rows of every column of a
// 32-column strip, written transposed (dst is cols x rows). FIRST reads the
// samples of type T and writes keys (and 16-bit counts); the second pass
// reads keys and writes the filtered values.
template <typename T, bool MAXIMUM, bool COUNT, bool FIRST>
__global__ void __launch_bounds__(kEThreads)
    extrema_pass_kernel(const void* __restrict__ src, const unsigned short* __restrict__ src_n,
                        void* __restrict__ dst, unsigned short* __restrict__ dst_n,
                        const __grid_constant__ PassArgs a) {
  using KO = KeyOf<T>;
  using K = typename KO::K;
  constexpr K kNone = KO::kSentinel;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = a.k, R = a.R;
  const long long c0 = (blockIdx.x % a.strips) * kStrip;
  const long long r0 = (blockIdx.x / a.strips) * (long long)R;
  const int rows = (int)min((long long)R, a.rows - r0);
  const int SH = rows + k - 1;
  const size_t plane = (size_t)(R + k - 1) * kPitch;
  K* keys = reinterpret_cast<K*>(smem_raw);  // suffix minima in place, then results
  K* pre = keys + plane;
  unsigned short* cnt = reinterpret_cast<unsigned short*>(pre + plane);  // suffix counts in place
  unsigned short* cpre = cnt + plane;
  const bool omit = a.r.omit, drop_inf = a.r.drop_inf;
  auto conv = [&](T v) -> K {
    if (isnan(v)) return omit ? kNone : (K)0;
    if (drop_inf && isinf(v)) return kNone;
    const K key = KO::key(v);
    return MAXIMUM ? (K)~key : key;
  };
  const T cval = (T)a.r.cval;
  const K outside = conv(cval);
  const unsigned short outside_n =
      (unsigned short)((isnan(cval) || (drop_inf && isinf(cval))) ? 0 : (FIRST ? 1 : a.prior));

  // Stage: one warp per support row, one lane per column.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long col = c0 + lane;
  for (int j = warp; j < SH; j += kEThreads / 32) {
    long long m;
    const bool inside = map_index(r0 + j - a.anchor, a.rows, a.mode, &m);
    K key = outside;
    unsigned short n = outside_n;
    if (inside && col < a.cols) {
      const size_t at = (size_t)m * a.cols + col;
      if constexpr (FIRST) {
        key = conv(__ldg(reinterpret_cast<const T*>(src) + at));
        n = key == kNone ? 0 : 1;
      } else {
        key = __ldg(reinterpret_cast<const K*>(src) + at);
        if constexpr (COUNT) n = __ldg(src_n + at);
      }
    }
    keys[j * kPitch + lane] = key;
    if constexpr (COUNT) cnt[j * kPitch + lane] = n;
  }
  __syncthreads();

  // Prefix and suffix minima (and counts) within blocks of k rows, one
  // (column, block) pair per work item.
  const int nb = (SH + k - 1) / k;
  for (int item = threadIdx.x; item < kStrip * nb; item += kEThreads) {
    const int c = item % kStrip, b = item / kStrip;
    const int j0 = b * k, j1 = min(SH, j0 + k);
    K run = kNone;
    unsigned int rn = 0;
    for (int j = j0; j < j1; ++j) {
      const K key = keys[j * kPitch + c];
      run = j == j0 ? key : (key < run ? key : run);
      pre[j * kPitch + c] = run;
      if constexpr (COUNT) {
        rn = (j == j0 ? 0u : rn) + cnt[j * kPitch + c];
        cpre[j * kPitch + c] = (unsigned short)rn;
      }
    }
    rn = 0;
    for (int j = j1 - 1; j >= j0; --j) {
      const K key = keys[j * kPitch + c];
      run = j == j1 - 1 ? key : (key < run ? key : run);
      keys[j * kPitch + c] = run;
      if constexpr (COUNT) {
        rn += cnt[j * kPitch + c];
        cnt[j * kPitch + c] = (unsigned short)rn;
      }
    }
  }
  __syncthreads();
  for (int item = threadIdx.x; item < kStrip * rows; item += kEThreads) {
    const int c = item % kStrip, r = item / kStrip;
    const K s = keys[r * kPitch + c], p = pre[(r + k - 1) * kPitch + c];
    keys[r * kPitch + c] = s < p ? s : p;
    if constexpr (COUNT) {
      const unsigned int tail = cpre[(r + k - 1) * kPitch + c];
      cnt[r * kPitch + c] = (unsigned short)(r % k == 0 ? tail : tail + cnt[r * kPitch + c]);
    }
  }
  __syncthreads();

  // Transposed store: one warp per column, lanes along the rows.
  for (int c = warp; c < kStrip; c += kEThreads / 32) {
    if (c0 + c >= a.cols) break;
    const size_t base = (size_t)(c0 + c) * a.rows + r0;
    for (int r = lane; r < rows; r += 32) {
      const K m = keys[r * kPitch + c];
      if constexpr (FIRST) {
        reinterpret_cast<K*>(dst)[base + r] = m;
        if constexpr (COUNT) dst_n[base + r] = cnt[r * kPitch + c];
      } else {
        bool missing = m == kNone || m == (K)0;
        if constexpr (COUNT) missing = missing || (long long)cnt[r * kPitch + c] < a.r.min_count;
        const T v = missing ? nan_of(T()) : KO::value(MAXIMUM ? (K)~m : m);
        reinterpret_cast<T*>(dst)[base + r] = canonical(v);
      }
    }
  }
}

// Rows per block of a pass over a window of length k: the largest of 128,
// 64, 32 whose shared memory stays within 64 KB (four blocks per SM), else
// 32 within `limit`; 0 when nothing fits.
template <typename K, bool COUNT>
int pass_rows(int k, int limit) {
  for (int R : {128, 64, 32})
    if (pass_smem<K, COUNT>(R, k) <= (size_t)std::min(limit, 64 * 1024)) return R;
  return pass_smem<K, COUNT>(32, k) <= (size_t)limit ? 32 : 0;
}

template <typename T, bool MAXIMUM, bool COUNT>
cudaError_t launch_passes_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  using K = typename KeyOf<T>::K;
  const Geom3& g = p.tile.g;
  const long long n = g.H * g.W;
  K* keys = reinterpret_cast<K*>(p.d_scratch);
  unsigned short* counts = COUNT ? reinterpret_cast<unsigned short*>(keys + n) : nullptr;
  auto k1 = extrema_pass_kernel<T, MAXIMUM, COUNT, true>;
  auto k2 = extrema_pass_kernel<T, MAXIMUM, COUNT, false>;
  cudaError_t e;
  if ((e = allow_max_smem((const void*)k1)) != cudaSuccess) return e;
  if ((e = allow_max_smem((const void*)k2)) != cudaSuccess) return e;
  PassArgs a;
  a.r = p.r;
  // Along the rows of the image (its y axis) into the transposed keys.
  a.rows = g.H;
  a.cols = g.W;
  a.k = g.kh;
  a.anchor = g.ay;
  a.mode = g.my;
  a.R = p.ext_rows[0];
  a.strips = (g.W + kStrip - 1) / kStrip;
  a.prior = 1;
  long long blocks = a.strips * ((a.rows + a.R - 1) / a.R);
  k1<<<(unsigned)blocks, kEThreads, pass_smem<K, COUNT>(a.R, a.k), s>>>(in, nullptr, keys, counts, a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // Along the original x axis, transposing back.
  a.rows = g.W;
  a.cols = g.H;
  a.k = g.kw;
  a.anchor = g.ax;
  a.mode = g.mx;
  a.R = p.ext_rows[1];
  a.strips = (g.H + kStrip - 1) / kStrip;
  a.prior = g.kh;
  blocks = a.strips * ((a.rows + a.R - 1) / a.R);
  k2<<<(unsigned)blocks, kEThreads, pass_smem<K, COUNT>(a.R, a.k), s>>>(keys, counts, out, nullptr, a);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_passes(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const bool maximum = p.r.kind == kMax, count = p.r.omit && p.r.min_count > 1;
  if (maximum) return count ? launch_passes_t<T, true, true>(p, in, out, s) : launch_passes_t<T, true, false>(p, in, out, s);
  return count ? launch_passes_t<T, false, true>(p, in, out, s) : launch_passes_t<T, false, false>(p, in, out, s);
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

// Rows per block of the two column passes and the transposed key array
// (plus 16-bit counts when min_count > 1) they exchange. False for
// footprints, rank 3 and windows whose passes do not fit.
bool extrema_passes_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  if (p.ndim > 2 || g.D != 1 || !p.footprint.empty()) return false;
  if (p.r.kind != kMin && p.r.kind != kMax) return false;
  const bool count = p.r.omit && p.r.min_count > 1;
  if (count && (long long)g.kh * g.kw > 65535) return false;
  auto rows = [&](int k) {
    if (p.dtype == 0) return count ? pass_rows<uint32_t, true>(k, smem_limit) : pass_rows<uint32_t, false>(k, smem_limit);
    return count ? pass_rows<unsigned long long, true>(k, smem_limit)
                 : pass_rows<unsigned long long, false>(k, smem_limit);
  };
  const int r1 = rows(g.kh), r2 = rows(g.kw);
  if (r1 == 0 || r2 == 0) return false;
  p.ext_rows[0] = r1;
  p.ext_rows[1] = r2;
  p.scratch_bytes = (size_t)(g.H * g.W) * ((p.dtype == 0 ? 4 : 8) + (count ? 2 : 0));
  return true;
}

cudaError_t launch_extrema(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.algo == Algo::kExtremaPasses) {
    if (p.dtype == 0) return launch_passes<float>(p, (const float*)in, (float*)out, s);
    return launch_passes<double>(p, (const double*)in, (double*)out, s);
  }
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}

}  // namespace ndf

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
};

// The exact sliding sums of one tile and its outputs: horizontal sums of X,
// X^2 and the sample counts along every support row (8 outputs per work
// item), then vertical sums down each output column (L rows per thread) and
// the combine. NARROW keeps S1 and S2 in 64-bit words (the caller has checked
// that every window's sums fit), otherwise 128-bit words; the row sums live
// in shared memory at `sums`.
template <typename T, bool NARROW>
__device__ __forceinline__ void slide_sums(const T* s, const TileArgs& a, const Span<T>& sp, i128 P,
                                           const SlideArgs& sa, unsigned char* sums, long long z, long long y0,
                                           long long x0, T* __restrict__ out) {
  using S1 = typename std::conditional<NARROW, long long, i128>::type;
  using S2 = typename std::conditional<NARROW, unsigned long long, u128>::type;
  constexpr int E0 = sizeof(T) == 4 ? -149 : -1074;
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const Reduce& r = a.r;
  const int kw = g.kw, kh = g.kh, TW = t.TW, SW = t.SW;
  const bool omit = r.omit, drop_inf = r.drop_inf;
  const int lo = sp.lo;
  S1* h1 = reinterpret_cast<S1*>(sums);
  S2* h2 = reinterpret_cast<S2*>(h1 + (size_t)t.SH * t.TW);
  unsigned long long* hc = reinterpret_cast<unsigned long long*>(h2 + (size_t)t.SH * t.TW);
  const long long P64 = (long long)P;
  // X = x - P in units of 2^(E0 + lo); zero for non-finite samples.
  auto deviation = [&](T v) -> long long {
    if constexpr (NARROW) {
      unsigned long long m;
      int pos;
      bool neg;
      if (!decompose(v, m, pos, neg)) return isfinite(v) ? -P64 : 0ll;  // zero, or not finite
      const long long f = (long long)(m << (pos - lo));
      return (neg ? -f : f) - P64;
    } else {
      return isfinite(v) ? (long long)(fixed(v, lo) - P) : 0ll;
    }
  };

  // Horizontal sums of every support row, 8 outputs per work item.
  const int nseg = TW / 8;
  for (int item = threadIdx.x; item < t.SH * nseg; item += blockDim.x) {
    const int y = item / nseg;
    const int xs = (item - y * nseg) * 8;
    const T* row = s + (size_t)y * SW + xs;
    S1 s1 = 0;
    S2 s2 = 0;
    unsigned long long cnt = 0;
    auto add = [&](T v, int sign) {
      const long long X = deviation(v);
      S2 sq;
      if constexpr (NARROW)
        sq = (unsigned long long)(X * X);
      else
        sq = (u128)((i128)X * X);
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
  S1 s1 = 0;
  S2 s2 = 0;
  unsigned long long cnt = 0;
  for (int k = 0; k < kh; ++k) {
    s1 += h1[(size_t)(r0 + k) * TW + x];
    s2 += h2[(size_t)(r0 + k) * TW + x];
    cnt += hc[(size_t)(r0 + k) * TW + x];
  }
  const int quantum = E0 + lo;
  for (int rr = 0; rr < L; ++rr) {
    const int row = r0 + rr;
    const long long gy = y0 + row;
    if (gy < g.H && gx < g.W) {
      const unsigned int finite = (unsigned int)(cnt & 0xFFFF), nanc = (unsigned int)((cnt >> 16) & 0xFFFF);
      const unsigned int pos = (unsigned int)((cnt >> 32) & 0xFFFF), neg = (unsigned int)(cnt >> 48);
      double result;
      if (mom::decide_special(r, (long long)finite + pos + neg, nanc != 0, pos != 0, neg != 0, &result))
        out[(z * g.H + gy) * g.W + gx] = canonical(from_f64<T>(result));
      else
        out[(z * g.H + gy) * g.W + gx] =
            canonical(fixed_combine<T>(r.kind, r.param, (i128)s1, (u128)s2, finite, P, quantum));
    }
    if (rr + 1 < L) {
      const size_t add = (size_t)(row + kh) * TW + x, sub = (size_t)row * TW + x;
      s1 += h1[add] - h1[sub];
      s2 += h2[add] - h2[sub];
      cnt += hc[add] - hc[sub];
    }
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
  // Layout (offsets from the 16-byte aligned base, each region 16-byte
  // aligned for the 128-bit sums): remap tables | staged samples | row sums
  // of X | row sums of X^2 | row counts (u64), the sums 128-bit (wide tiles)
  // or 64-bit (narrow tiles) each.
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  T* s = reinterpret_cast<T*>(maps + (t.SW + t.SH + g.kd));
  const size_t sums_offset =
      ((size_t)(t.SW + t.SH + g.kd) * 8 + (size_t)t.SH * t.SW * sizeof(T) + 15) & ~(size_t)15;
  long long z, y0, x0;
  net::tile_coords(a, tile, z, y0, x0);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, (T)r.cval, [](T v) { return v; })) return;
  __syncthreads();
  const int support = t.SH * t.SW;
  const Span<T> sp = tile_span<T, kSThreads>(s, support);
  const T pivot = sp.pivot;
  const int lo = sp.lo;
  const bool fits = span_fits(sp, sa.count_bits);

  const int kw = g.kw, TW = t.TW, SW = t.SW;
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
  // Narrow tiles (deviations within 31 bits and their window sums within 64
  // bits, the usual case for float32 data of moderate range) keep every sum
  // in 64-bit words; wide tiles in 128-bit words. Both are exact.
  const int bits = deviation_bits(sp);
  if (sp.top - lo <= 62 && bits <= 31 && 2 * bits + sa.count_bits <= 63)
    slide_sums<T, true>(s, a, sp, P, sa, smem_raw + sums_offset, z, y0, x0, out);
  else
    slide_sums<T, false>(s, a, sp, P, sa, smem_raw + sums_offset, z, y0, x0, out);
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
  int pad;
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
  t.sa.count_bits = 64 - __builtin_clzll((unsigned long long)p.r.count + 1);
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

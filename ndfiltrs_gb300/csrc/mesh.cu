// Mesh background: per-mesh robust background / RMS, fill of invalid meshes,
// median filter of the mesh grid, and full-resolution maps.
//
// Replaces MeshBackground (src/background.rs:417-923) with its statistics
// (src/background.rs:924-1152), the natural spline (src/background.rs:349-397,
// 858-921, 1154-1212) and the SExtractor-compatible interpolation
// (src/background/sep_interpolation.rs). Every float64 operation is the
// reference's, in its order (explicitly rounded intrinsics on the device, a
// host compiled without contraction; fused multiply-adds exactly where the
// reference writes mul_add), so results equal the reference bit for bit.
//
// GB300 design:
//  * mesh_stats_kernel: one 128-thread block per mesh gathers the mesh's
//    finite, unmasked samples as order-preserving 64-bit keys into shared
//    memory (global scratch for meshes beyond 8192 samples), bitonic-sorts
//    them and runs the SExtractor or sigma-clip sequence with the whole
//    block. The reference accumulates Neumaier sums in sorted order; the
//    block sums the terms exactly in fixed point, in parallel, and proves
//    from the exact sum and a bound on the compensation's rounding that the
//    sequential sum rounds to the same double (thread 0 runs the sequential
//    sum in the rare case it cannot), so the float64 chains of one mesh no
//    longer run one sample at a time; medians, MADs and clipping bounds are
//    binary searches over the sorted samples;
//  * fill, median filter and the global medians run on the host over the
//    small mesh grid;
//  * the maps: the natural spline is a tensor product, one axis per pass
//    (second derivatives by the Thomas algorithm per mesh line, then four
//    weighted terms per output); the last pass writes the output dtype with
//    one block per output line. The SExtractor form runs one block per output
//    row. Both are a handful of float64 operations per output pixel.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/ndfiltrs_gb300.h"
#include "common.cuh"
#include "hostpool.h"
#include "moments.cuh"
#include "plan.h"

namespace ndf {
namespace {

constexpr int kMThreads = 128;
constexpr long long kMeshSmemBytes = 64 * 1024;  // sort buffer a block keeps in shared memory
constexpr double kNuq = 0.6744897501960817;  // Phi^-1(0.75)
constexpr int kMaxMeshRank = 8;

struct MeshArgs {
  int ndim;
  long long shape[kMaxMeshRank], box[kMaxMeshRank], mesh_shape[kMaxMeshRank];
  long long mesh_len;
  long long capacity;  // keys per block in `scratch` (0: shared memory)
  long long box_volume;
  int estimator, center, spread, statistic, mode_estimator, rms, valid_count, valid_base;
  long long maxiters;
  double pearson, lower, upper, min_valid_fraction;
};

struct MeshOut {
  double* background;
  double* rms;
  long long* finite;
  long long* retained;
  unsigned char* valid;
};

__device__ __forceinline__ unsigned long long mkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double mval(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

// A mesh's sorted samples: element i is p[i] (float64 bits).
struct SV {
  const unsigned long long* p;
  __device__ __forceinline__ double operator[](long long i) const { return __longlong_as_double((long long)p[i]); }
  __device__ __forceinline__ SV at(long long k) const { return {p + k}; }
};

// Block state of the statistics: per-warp partial sums and a broadcast slot.
struct MeshShared {
  W3 part[kMThreads / 32];
  int low[kMThreads / 32];
  double value;
};

// Thread 0's `v` in every thread of the block.
__device__ double broadcast(double v, MeshShared& sh) {
  if (threadIdx.x == 0) sh.value = v;
  __syncthreads();
  v = sh.value;
  __syncthreads();
  return v;
}

// median_sorted, src/background.rs:950-963.
__device__ double m_median(SV v, long long n) {
  if (n % 2 == 1) return v[n / 2];
  const double a = v[n / 2 - 1], b = v[n / 2];
  const double mid = __ddiv_rn(__dadd_rn(a, b), 2.0);
  return finite64(mid) ? mid : __dadd_rn(__ddiv_rn(a, 2.0), __ddiv_rn(b, 2.0));
}

// The reference's sequential Neumaier sum of term(0..n-1), every |term|
// below 2^H (a term that is not gives the sequential sum): the block adds
// the terms exactly (ExactSum, in any order) and proves the rounding; thread
// 0 runs the sequential sum when the proof fails. Called by every thread of
// the block with the same arguments; returns the same value in all.
template <typename Term>
__device__ double block_sum(Term&& term, long long n, int H, MeshShared& sh) {
  ExactSum e(H);
  if (n < (1ll << 31))
    for (long long i = threadIdx.x; i < n; i += blockDim.x) e.add(term(i));
  else
    e.ok = false;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long b0 = __shfl_down_sync(0xffffffffu, e.s.w0, off);
    const unsigned long long b1 = __shfl_down_sync(0xffffffffu, e.s.w1, off);
    const unsigned long long b2 = __shfl_down_sync(0xffffffffu, e.s.w2, off);
    add3(e.s, b0, b1, b2);
  }
  e.low = __reduce_min_sync(0xffffffffu, e.low);
  if ((threadIdx.x & 31) == 0) {
    sh.part[threadIdx.x >> 5] = e.s;
    sh.low[threadIdx.x >> 5] = e.low;
  }
  e.ok = !__syncthreads_or(!e.ok);
  e.s = sh.part[0];
  e.low = sh.low[0];
#pragma unroll
  for (int w = 1; w < kMThreads / 32; ++w) {
    add3(e.s, sh.part[w].w0, sh.part[w].w1, sh.part[w].w2);
    e.low = min(e.low, sh.low[w]);
  }
  __syncthreads();
  double result;
  if (e.result(n, &result)) return result;
  double sequential = 0.0;
  if (threadIdx.x == 0) {
    Sum64 sum;
    for (long long i = 0; i < n; ++i) sum.add(term(i));
    sequential = sum.total();
  }
  return broadcast(sequential, sh);
}

// mean_of, src/background.rs:965-978 (mean_valid on overflow).
__device__ double m_mean(SV v, long long n, MeshShared& sh) {
  const int H = bound_exponent(fmax(abs64(v[0]), abs64(v[n - 1])));
  const double total = block_sum([&](long long i) { return v[i]; }, n, H, sh);
  if (finite64(total)) return __ddiv_rn(total, (double)n);
  double mean = 0.0;
  if (threadIdx.x == 0) {
    Reduce r{};
    r.count = (int)n;
    mean = mom::mean_exact([&](int i) { return v[i]; }, r);
  }
  return broadcast(mean, sh);
}

// std_about, src/background.rs:1000-1015. Every scaled deviation is at most
// 1 in magnitude (the extremes of sorted samples set the scale and rounding
// is monotone), so the squares lie below 2^1.
__device__ double m_std(SV v, long long n, double mean, MeshShared& sh) {
  if (n == 0) return nan_of(0.0);
  const double scale = fmax(abs64(__dsub_rn(v[0], mean)), abs64(__dsub_rn(v[n - 1], mean)));
  if (scale == 0.0) return 0.0;
  if (!finite64(scale)) return nan_of(0.0);
  const Divisor by = make_divisor(scale);
  const double squares = block_sum(
      [&](long long i) {
        const double d = div_by(__dsub_rn(v[i], mean), by);
        return __dmul_rn(d, d);
      },
      n, 1, sh);
  return __dmul_rn(scale, __dsqrt_rn(__ddiv_rn(squares, (double)n)));
}

// mad_std, src/background.rs:1017-1022: the median of |v - median| over
// sorted v, divided by Phi^-1(0.75). The deviations ascend on both sides of
// the first sample at or above the median, so the two middle ranks of their
// union come from a binary search over the split between the two sides.
__device__ double m_mad_std(SV v, long long n, double median) {
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long mid = (lo + hi) / 2;
    if (__dsub_rn(v[mid], median) < 0.0) lo = mid + 1; else hi = mid;
  }
  const long long right = lo, na = right, nb = n - right;
  auto A = [&](long long t) { return abs64(__dsub_rn(v[right - 1 - t], median)); };
  auto B = [&](long long t) { return abs64(__dsub_rn(v[right + t], median)); };
  // Rank r (0-based) of the union: p from A and r + 1 - p from B, the
  // smallest p with no smaller key of A left out.
  auto rank = [&](long long r) {
    long long a = r + 1 - nb > 0 ? r + 1 - nb : 0, b = r + 1 < na ? r + 1 : na;
    while (a < b) {
      const long long p = (a + b) / 2, q = r + 1 - p;
      if (p < na && q > 0 && A(p) < B(q - 1)) a = p + 1; else b = p;
    }
    const long long q = r + 1 - a;
    if (a == 0) return B(q - 1);
    if (q == 0) return A(a - 1);
    return fmax(A(a - 1), B(q - 1));
  };
  const double a = rank((n - 1) / 2), b = rank(n / 2);
  const double mad = n % 2 == 1 ? b : (finite64(__ddiv_rn(__dadd_rn(a, b), 2.0))
                                           ? __ddiv_rn(__dadd_rn(a, b), 2.0)
                                           : __dadd_rn(__ddiv_rn(a, 2.0), __ddiv_rn(b, 2.0)));
  return __ddiv_rn(mad, kNuq);
}

// within, src/background.rs:1024-1032 (two binary searches).
__device__ void m_within(SV v, long long r0, long long r1, double low, double high, long long& lo,
                         long long& hi) {
  long long a = r0, b = r1;
  while (a < b) {
    const long long m = (a + b) / 2;
    if (v[m] < low) a = m + 1; else b = m;
  }
  lo = a;
  a = r0;
  b = r1;
  while (a < b) {
    const long long m = (a + b) / 2;
    if (v[m] <= high) a = m + 1; else b = m;
  }
  hi = a > lo ? a : lo;
}

// clip_sorted, src/background.rs:1034-1069.
__device__ void m_clip(SV v, long long& r0, long long& r1, double lower, double upper, long long maxiters,
                       int center, int spread, MeshShared& sh) {
  long long iteration = 0;
  while (r1 - r0 >= 1 && (maxiters < 0 || iteration < maxiters)) {
    const SV kept = v.at(r0);
    const long long n = r1 - r0;
    const double middle = center == 0 ? m_mean(kept, n, sh) : m_median(kept, n);
    double width;
    if (spread == 0)
      width = m_std(kept, n, center == 0 ? middle : m_mean(kept, n, sh), sh);
    else
      width = m_mad_std(kept, n, center == 1 ? middle : m_median(kept, n));
    long long lo, hi;
    m_within(v, r0, r1, __dsub_rn(middle, __dmul_rn(lower, width)), __dadd_rn(middle, __dmul_rn(upper, width)),
             lo, hi);
    ++iteration;
    if (lo == r0 && hi == r1) break;
    r0 = lo;
    r1 = hi;
  }
}

__device__ double m_mode(double mean, double median, double sd, int estimator, double pearson) {
  const double difference = __dsub_rn(median, mean);
  const double pearson_mode = __dadd_rn(median, __dmul_rn(__dsub_rn(pearson, 1.0), difference));
  if (estimator == kModeMmm) return pearson_mode;
  if (estimator == kModeIraf) return mean < median ? mean : pearson_mode;
  if (sd == 0.0) return mean;
  if (__ddiv_rn(abs64(difference), sd) >= 0.3) return median;
  return pearson_mode;
}

// finish_stats with sextractor_stats / clipped_stats, src/background.rs:652-705,
// 1071-1152. Every thread of the block runs it with the same values; thread
// 0 writes the mesh's results.
__device__ void m_finish(SV v, long long n, long long volume, const MeshArgs& a, const MeshOut& o, long long mesh,
                         MeshShared& sh) {
  double background = nan_of(0.0), rms = nan_of(0.0);
  long long retained = 0;
  if (n > 0) {
    if (a.estimator == 0) {
      const double mean = m_mean(v, n, sh);
      const double sd = m_std(v, n, mean, sh);
      long long f0, f1;
      m_within(v, 0, n, __dsub_rn(mean, __dmul_rn(2.0, sd)), __dadd_rn(mean, __dmul_rn(2.0, sd)), f0, f1);
      if (f0 != f1) {
        const double mean2 = m_mean(v.at(f0), f1 - f0, sh);
        const double sd2 = m_std(v.at(f0), f1 - f0, mean2, sh);
        long long s0, s1;
        m_within(v, 0, n, __dsub_rn(mean2, __dmul_rn(5.0, sd2)), __dadd_rn(mean2, __dmul_rn(5.0, sd2)), s0, s1);
        m_clip(v, s0, s1, 3.0, 3.0, 100, 1, 0, sh);
        if (s0 != s1) {
          const SV k = v.at(s0);
          const long long c = s1 - s0;
          const double mean3 = m_mean(k, c, sh);
          const double sd3 = m_std(k, c, mean3, sh);
          background = m_mode(mean3, m_median(k, c), sd3, kModeSex, a.pearson);
          rms = sd3;
          retained = c;
        }
      }
    } else {
      long long r0 = 0, r1 = n;
      m_clip(v, r0, r1, a.lower, a.upper, a.maxiters, a.center, a.spread, sh);
      retained = r1 - r0;
      if (retained > 0) {
        const SV k = v.at(r0);
        const double mean = m_mean(k, retained, sh);
        const double median = m_median(k, retained);
        const bool need_std = a.statistic == 2 || a.rms == 0;
        const double sd = need_std ? m_std(k, retained, mean, sh) : 0.0;
        if (a.statistic == 0)
          background = mean;
        else if (a.statistic == 1)
          background = median;
        else
          background = m_mode(mean, median, sd, a.mode_estimator, a.pearson);
        rms = a.rms == 0 ? sd : m_mad_std(k, retained, median);
      }
    }
  }
  if (threadIdx.x != 0) return;
  const long long count = a.valid_count == 0 ? n : retained;
  const long long base = a.valid_base == 0 ? volume : a.box_volume;
  const bool valid = count > 0 && (double)count >= __dmul_rn(a.min_valid_fraction, (double)base) &&
                     finite64(background) && finite64(rms);
  o.background[mesh] = valid ? background : nan_of(0.0);
  o.rms[mesh] = valid ? rms : nan_of(0.0);
  o.finite[mesh] = n;
  o.retained[mesh] = n > 0 ? retained : 0;
  o.valid[mesh] = valid ? 1 : 0;
}

// One block per mesh (grid-stride over meshes): gather the finite, unmasked
// samples as order-preserving 64-bit keys, bitonic-sort them, turn them back
// into float64 samples in place and run the statistics with the whole block.
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    mesh_stats_kernel(const T* __restrict__ in, const unsigned char* __restrict__ mask,
                      const __grid_constant__ MeshArgs a, unsigned long long* __restrict__ scratch, MeshOut o) {
  extern __shared__ __align__(16) unsigned long long skeys[];
  __shared__ unsigned int count;
  __shared__ MeshShared sh;
  unsigned long long* keys = a.capacity > 0 ? scratch + blockIdx.x * a.capacity : skeys;
  const int ndim = a.ndim;
  for (long long mesh = blockIdx.x; mesh < a.mesh_len; mesh += gridDim.x) {
    long long start[kMaxMeshRank], extent[kMaxMeshRank];
    long long rest = mesh, volume = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      const long long k = rest % a.mesh_shape[d];
      rest /= a.mesh_shape[d];
      start[d] = k * a.box[d];
      extent[d] = min(start[d] + a.box[d], a.shape[d]) - start[d];
      volume *= extent[d];
    }
    if (threadIdx.x == 0) count = 0;
    __syncthreads();
    for (long long p = threadIdx.x; p < volume; p += blockDim.x) {
      long long q = p, offset = 0, stride = 1;
      for (int d = ndim - 1; d >= 0; --d) {
        offset += (start[d] + q % extent[d]) * stride;
        q /= extent[d];
        stride *= a.shape[d];
      }
      const double v = (double)__ldg(in + offset);
      if (finite64(v) && !(mask && mask[offset])) keys[atomicAdd(&count, 1u)] = mkey(v);
    }
    __syncthreads();
    const unsigned int n = count;
    unsigned int padded = 1;
    while (padded < n) padded <<= 1;
    for (unsigned int i = n + threadIdx.x; i < padded; i += blockDim.x) keys[i] = ~0ull;
    __syncthreads();
    // Bitonic sort, ascending: each stage's padded / 2 compare-exchanges
    // (i, i + j), i with bit j clear, spread over the block.
    for (unsigned int k = 2; k <= padded; k <<= 1) {
      for (unsigned int j = k >> 1; j > 0; j >>= 1) {
        for (unsigned int p = threadIdx.x; p < padded / 2; p += blockDim.x) {
          const unsigned int i = 2 * p - (p & (j - 1));
          const unsigned long long x = keys[i], y = keys[i + j];
          if ((x > y) == ((i & k) == 0)) {
            keys[i] = y;
            keys[i + j] = x;
          }
        }
        __syncthreads();
      }
    }
    for (unsigned int i = threadIdx.x; i < n; i += blockDim.x)
      keys[i] = (unsigned long long)__double_as_longlong(mval(keys[i]));
    __syncthreads();
    m_finish(SV{keys}, n, volume, a, o, mesh, sh);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Natural spline passes.

struct SplineTap {
  long long seg;
  double a, b, c, d;
};

// Second derivatives along `nodes` for the `inner` interleaved columns of
// each of `outer` blocks (columns_second_derivatives, src/background.rs:1187-1212).
__global__ void spline_second_kernel(const double* __restrict__ cur, const double* __restrict__ pivots,
                                     double* __restrict__ second, long long outer, long long nodes, long long inner) {
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= outer * inner) return;
  const long long o = col / inner, j = col % inner;
  const double* b = cur + o * nodes * inner + j;
  double* s = second + o * nodes * inner + j;
  for (long long i = 0; i < nodes; ++i) s[i * inner] = 0.0;
  if (nodes < 3) return;
  for (long long i = 1; i + 1 < nodes; ++i) {
    const double rhs = __dmul_rn(6.0, __dadd_rn(__dsub_rn(b[(i - 1) * inner], __dmul_rn(2.0, b[i * inner])),
                                                b[(i + 1) * inner]));
    s[i * inner] = __dmul_rn(__dsub_rn(rhs, s[(i - 1) * inner]), pivots[i]);
  }
  for (long long i = nodes - 3; i >= 1; --i)
    s[i * inner] = __dsub_rn(s[i * inner], __dmul_rn(pivots[i], s[(i + 1) * inner]));
}

__device__ __forceinline__ double tap_eval(const SplineTap& t, const double* y, const double* m, long long stride) {
  return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(t.a, y[t.seg * stride]), __dmul_rn(t.b, y[(t.seg + 1) * stride])),
                             __dmul_rn(t.c, m[t.seg * stride])),
                   __dmul_rn(t.d, m[(t.seg + 1) * stride]));
}

// A non-last axis: next[(o, p), j] from the taps of output index p.
__global__ void spline_expand_kernel(const double* __restrict__ cur, const double* __restrict__ second,
                                     const SplineTap* __restrict__ taps, double* __restrict__ next, long long outer,
                                     long long length, long long nodes, long long inner) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= outer * length * inner) return;
  const long long j = idx % inner, row = idx / inner;
  const long long o = row / length, p = row % length;
  const long long base = o * nodes * inner;
  if (nodes < 2) {
    next[idx] = cur[base + j];
    return;
  }
  next[idx] = tap_eval(taps[p], cur + base + j, second + base + j, inner);
}

// The last axis: one block per line; the line's second derivatives in
// shared memory, then every output of the line in the output dtype.
template <typename T>
__global__ void spline_last_kernel(const double* __restrict__ cur, const double* __restrict__ pivots,
                                   const SplineTap* __restrict__ taps, T* __restrict__ out, long long lines,
                                   long long nodes, long long length) {
  extern __shared__ double m[];
  for (long long line = blockIdx.x; line < lines; line += gridDim.x) {
    const double* y = cur + line * nodes;
    if (threadIdx.x == 0) {
      for (long long i = 0; i < nodes; ++i) m[i] = 0.0;
      if (nodes >= 3) {
        for (long long i = 1; i + 1 < nodes; ++i) {
          const double rhs = __dmul_rn(6.0, __dadd_rn(__dsub_rn(y[i - 1], __dmul_rn(2.0, y[i])), y[i + 1]));
          m[i] = __dmul_rn(__dsub_rn(rhs, m[i - 1]), pivots[i]);
        }
        for (long long i = nodes - 3; i >= 1; --i) m[i] = __dsub_rn(m[i], __dmul_rn(pivots[i], m[i + 1]));
      }
    }
    __syncthreads();
    for (long long p = threadIdx.x; p < length; p += blockDim.x) {
      const double v = nodes < 2 ? y[0] : tap_eval(taps[p], y, m, 1);
      if constexpr (sizeof(T) == 4)
        out[line * length + p] = __double2float_rn(v);
      else
        out[line * length + p] = v;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void fill_kernel(T* __restrict__ out, long long n, double value) {
  const T v = sizeof(T) == 4 ? (T)__double2float_rn(value) : (T)value;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = v;
}

// Broadcast one float64 row to every row of the output.
template <typename T>
__global__ void rows_kernel(const double* __restrict__ row, T* __restrict__ out, long long rows, long long width) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows * width;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = row[i % width];
    out[i] = sizeof(T) == 4 ? (T)__double2float_rn(v) : (T)v;
  }
}

// ---------------------------------------------------------------------------
// SExtractor-compatible interpolation (sep_interpolation.rs:111-209): one
// block per output row.

struct SepRow {
  long long i;  // upper mesh row of the interval
  double b, ca, cb;
};

struct SepWeight {
  double fraction, left_curve, right_curve;
};

template <typename T>
__global__ void sep_rows_kernel(const double* __restrict__ values, const double* __restrict__ y_coeff,
                                const double* __restrict__ x_pivots, const SepRow* __restrict__ rows,
                                const SepWeight* __restrict__ first, const SepWeight* __restrict__ later,
                                const int* __restrict__ pix_interval, const int* __restrict__ pix_weight,
                                T* __restrict__ out, long long ny, long long nx, long long columns, double scale,
                                int have_x) {
  extern __shared__ double sh[];
  double* line = sh;
  double* xc = sh + columns;
  for (long long y = blockIdx.x; y < ny; y += gridDim.x) {
    const SepRow r = rows[y];
    const double* top = values + r.i * columns;
    const double* bottom = top + columns;
    const double* ct = y_coeff + r.i * columns;
    const double* cbot = ct + columns;
    for (long long j = threadIdx.x; j < columns; j += blockDim.x) {
      const double linear = __fma_rn(r.b, __dsub_rn(bottom[j], top[j]), top[j]);
      line[j] = __fma_rn(r.cb, cbot[j], __fma_rn(r.ca, ct[j], linear));
      xc[j] = 0.0;
    }
    __syncthreads();
    if (have_x && threadIdx.x == 0) {
      for (long long i = 1; i + 1 < columns; ++i) {
        const double difference = __dsub_rn(__dsub_rn(line[i + 1], line[i]), __dsub_rn(line[i], line[i - 1]));
        xc[i] = __dmul_rn(__fma_rn(3.0, difference, __dmul_rn(-0.5, xc[i - 1])), x_pivots[i]);
      }
      for (long long i = columns - 2; i >= 1; --i)
        xc[i] = __ddiv_rn(__fma_rn(__dmul_rn(-0.5, x_pivots[i]), xc[i + 1], xc[i]), 6.0);
    }
    __syncthreads();
    for (long long p = threadIdx.x; p < nx; p += blockDim.x) {
      double v;
      if (have_x) {
        const int i = pix_interval[p];
        const SepWeight w = (i == 0 ? first : later)[pix_weight[p]];
        const double left = line[i], right = line[i + 1];
        const double slope = __dsub_rn(right, left);
        const double linear = __fma_rn(w.fraction, slope, left);
        v = __fma_rn(w.right_curve, xc[i + 1], __fma_rn(w.left_curve, xc[i], linear));
      } else {
        v = line[0];
      }
      v = __dmul_rn(v, scale);
      out[y * nx + p] = sizeof(T) == 4 ? (T)__double2float_rn(v) : (T)v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Host side.

struct Rules {
  ndf_mesh_config c;
  std::vector<long long> shape, box, filter, mesh_shape;
  long long len = 1, mesh_len = 1, box_volume = 1;
};

int validate(const uint64_t* shape, const uint64_t* box_size, const uint64_t* filter_size, int ndim,
             const ndf_mesh_config* config, Rules& r) {
  if (ndim <= 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "shape must have at least one axis");
  if (!shape || !box_size || !filter_size || !config)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "box and filter sizes need one entry per axis");
  if (ndim > kMaxMeshRank) return fail(NDF_ERR_UNSUPPORTED, "mesh backgrounds support up to 8 dimensions");
  for (int a = 0; a < ndim; ++a)
    if (box_size[a] == 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "box sizes must be positive");
  for (int a = 0; a < ndim; ++a)
    if (filter_size[a] % 2 == 0) return fail(NDF_ERR_INVALID_CONFIGURATION, "filter sizes must be odd and positive");
  const ndf_mesh_config& c = *config;
  // MeshConfig::validate, src/background.rs:230-289.
  if (!(std::isfinite(c.pearson) && c.pearson >= 1.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "pearson must be finite and at least one");
  if (c.estimator == NDF_MESH_ESTIMATOR_SIGMA_CLIP &&
      (!std::isfinite(c.sigma_lower) || !std::isfinite(c.sigma_upper) || c.sigma_lower < 0.0 || c.sigma_upper < 0.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "clipping limits must be finite and nonnegative");
  if (!(c.min_valid_fraction >= 0.0 && c.min_valid_fraction <= 1.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "minimum valid fraction must be between zero and one");
  if (c.fill == NDF_MESH_FILL_IDW && (c.idw_neighbors == 0 || !std::isfinite(c.idw_power) || c.idw_power < 0.0))
    return fail(NDF_ERR_INVALID_CONFIGURATION,
                "inverse-distance fill needs at least one neighbor and a finite nonnegative power");
  if (c.threshold_kind != NDF_MESH_THRESHOLD_ALL && !std::isfinite(c.threshold))
    return fail(NDF_ERR_INVALID_CONFIGURATION, "filter threshold must be finite");
  if (c.interpolation == NDF_MESH_INTERP_SEXTRACTOR && ndim != 2)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "SExtractor interpolation needs a 2-D shape");
  r.c = c;
  for (int a = 0; a < ndim; ++a) {
    r.shape.push_back((long long)shape[a]);
    r.box.push_back((long long)box_size[a]);
    r.filter.push_back((long long)filter_size[a]);
    r.mesh_shape.push_back(((long long)shape[a] + (long long)box_size[a] - 1) / (long long)box_size[a]);
    r.len *= r.shape.back();
    r.mesh_len *= r.mesh_shape.back();
    if (box_size[a] > (uint64_t)(1ll << 62) / (uint64_t)r.box_volume)
      return fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
    r.box_volume *= (long long)box_size[a];
  }
  return NDF_OK;
}

double median_sorted_host(const double* v, size_t n) {
  if (n % 2 == 1) return v[n / 2];
  const double a = v[n / 2 - 1], b = v[n / 2];
  const double mid = (a + b) / 2.0;
  return std::isfinite(mid) ? mid : a / 2.0 + b / 2.0;
}

uint64_t host_key(double v) {
  uint64_t b;
  std::memcpy(&b, &v, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// median_of, src/background.rs:940-948.
double median_of(std::vector<double> v) {
  if (v.empty()) return NAN;
  for (double x : v)
    if (std::isnan(x)) return NAN;
  std::sort(v.begin(), v.end(), [](double a, double b) { return host_key(a) < host_key(b); });
  return median_sorted_host(v.data(), v.size());
}

struct NeumaierHost {
  double value = 0.0, correction = 0.0;
  void add(double x) {
    const double next = value + x;
    if (std::fabs(value) >= std::fabs(x))
      correction += (value - next) + x;
    else
      correction += (x - next) + value;
    value = next;
  }
  double total() const { return value + correction; }
};

void unravel(long long flat, const std::vector<long long>& dims, long long* index) {
  for (size_t a = dims.size(); a-- > 0;) {
    index[a] = flat % dims[a];
    flat /= dims[a];
  }
}

// body(i) for every i in [0, count), spread over host threads when `work`
// (a rough operation count) is large enough to pay for them.
template <typename Body>
void parallel_for(long long count, long long work, Body&& body) {
  long long threads = host_thread_count();
  threads = std::min({threads, count, std::max(1ll, work / 200000)});
  if (threads <= 1) {
    for (long long i = 0; i < count; ++i) body(i);
    return;
  }
  std::atomic<long long> next{0};
  auto run = [&] {
    for (long long i = next.fetch_add(1); i < count; i = next.fetch_add(1)) body(i);
  };
  std::vector<std::thread> pool;
  for (long long t = 1; t < threads; ++t) pool.emplace_back(run);
  run();
  for (std::thread& t : pool) t.join();
}

// fill_invalid / replacement, src/background.rs:715-798: each invalid mesh takes the mean
// of its nearest valid meshes ('nearest') or the inverse-distance weighted
// mean of the valid meshes within its idw_neighbors-th smallest distance
// ('idw'), summed in (distance, index) order. The invalid meshes are
// independent: they run on host threads, and 'idw' selects the cut-off
// distance with nth_element and sorts only the meshes within it.
void fill_invalid(std::vector<double>& bg, std::vector<double>& rms, const std::vector<unsigned char>& valid,
                  const Rules& r) {
  const long long n = r.mesh_len;
  const size_t ndim = r.mesh_shape.size();
  std::vector<long long> good, bad;
  for (long long i = 0; i < n; ++i) (valid[i] ? good : bad).push_back(i);
  if (bad.empty() || good.empty()) return;
  std::vector<long long> gi(good.size() * ndim);
  for (size_t s = 0; s < good.size(); ++s) unravel(good[s], r.mesh_shape, &gi[s * ndim]);
  std::vector<double> values(bad.size()), spreads(bad.size());
  parallel_for((long long)bad.size(), (long long)(bad.size() * good.size()), [&](long long j) {
    std::vector<long long> idx(ndim);
    unravel(bad[j], r.mesh_shape, idx.data());
    std::vector<std::pair<uint64_t, long long>> d(good.size());
    for (size_t s = 0; s < good.size(); ++s) {
      uint64_t d2 = 0;
      for (size_t a = 0; a < ndim; ++a) {
        const long long diff = idx[a] - gi[s * ndim + a];
        const uint64_t ad = (uint64_t)(diff < 0 ? -diff : diff);
        d2 += ad * ad;
      }
      d[s] = {d2, good[s]};
    }
    double value, spread;
    if (r.c.fill == NDF_MESH_FILL_NEAREST) {
      uint64_t nearest = UINT64_MAX;
      for (const auto& e : d) nearest = std::min(nearest, e.first);
      NeumaierHost v, s;
      size_t count = 0;
      for (const auto& e : d)
        if (e.first == nearest) {
          v.add(bg[e.second]);
          s.add(rms[e.second]);
          ++count;
        }
      value = v.total() / (double)count;
      spread = s.total() / (double)count;
    } else {
      const size_t kth = std::min<size_t>(r.c.idw_neighbors, d.size()) - 1;
      std::vector<uint64_t> distances(d.size());
      for (size_t s = 0; s < d.size(); ++s) distances[s] = d[s].first;
      std::nth_element(distances.begin(), distances.begin() + (long long)kth, distances.end());
      const uint64_t last = distances[kth];
      std::vector<std::pair<uint64_t, long long>> near;
      for (const auto& e : d)
        if (e.first <= last) near.push_back(e);
      std::sort(near.begin(), near.end());
      NeumaierHost weighted, weighted_rms, total;
      for (const auto& e : near) {
        const double weight = 1.0 / std::pow(std::sqrt((double)e.first), r.c.idw_power);
        weighted.add(weight * bg[e.second]);
        weighted_rms.add(weight * rms[e.second]);
        total.add(weight);
      }
      value = weighted.total() / total.total();
      spread = weighted_rms.total() / total.total();
    }
    values[j] = value;
    spreads[j] = spread;
  });
  for (size_t j = 0; j < bad.size(); ++j) {
    bg[bad[j]] = values[j];
    rms[bad[j]] = spreads[j];
  }
}

void median_filter(std::vector<double>& bg, std::vector<double>& rms, const Rules& r) {
  bool all_one = true;
  for (long long f : r.filter) all_one = all_one && f == 1;
  if (all_one || r.mesh_len == 0) return;
  const size_t ndim = r.mesh_shape.size();
  std::vector<double> ob(bg), orms(rms), wb, wr;
  std::vector<long long> idx(ndim), low(ndim), high(ndim);
  for (long long flat = 0; flat < r.mesh_len; ++flat) {
    unravel(flat, r.mesh_shape, idx.data());
    for (size_t a = 0; a < ndim; ++a) {
      const long long k = idx[a], n = r.mesh_shape[a], half = r.filter[a] / 2;
      if (r.c.filter_edge == NDF_MESH_EDGE_SHRINK) {
        const long long h = std::min(std::min(half, k), n - 1 - k);
        low[a] = k - h;
        high[a] = k + h;
      } else {
        low[a] = std::max(k - half, 0ll);
        high[a] = std::min(k + half, n - 1);
      }
    }
    wb.clear();
    wr.clear();
    long long volume = 1;
    for (size_t a = 0; a < ndim; ++a) volume *= high[a] - low[a] + 1;
    for (long long pos = 0; pos < volume; ++pos) {
      long long rest = pos, offset = 0, stride = 1;
      for (size_t a = ndim; a-- > 0;) {
        const long long width = high[a] - low[a] + 1;
        offset += (low[a] + rest % width) * stride;
        rest /= width;
        stride *= r.mesh_shape[a];
      }
      wb.push_back(bg[offset]);
      wr.push_back(rms[offset]);
    }
    const double median = median_of(wb);
    bool replace = true;
    if (r.c.threshold_kind == NDF_MESH_THRESHOLD_DEVIATION) replace = std::fabs(median - bg[flat]) >= r.c.threshold;
    if (r.c.threshold_kind == NDF_MESH_THRESHOLD_ABOVE) replace = bg[flat] > r.c.threshold;
    if (replace) {
      ob[flat] = median;
      orms[flat] = median_of(wr);
    }
  }
  bg.swap(ob);
  rms.swap(orms);
}

SplineTap make_tap(double u, long long nodes) {
  if (nodes < 2) return {0, 1.0, 0.0, 0.0, 0.0};
  const double fl = std::floor(u);
  long long seg = fl > 0.0 ? (long long)fl : 0;
  seg = std::min(seg, nodes - 2);
  const double t = u - (double)seg;
  const double a = 1.0 - t;
  return {seg, a, t, (a * a * a - a) / 6.0, (t * t * t - t) / 6.0};
}

std::vector<double> natural_pivots(long long nodes) {
  std::vector<double> p((size_t)std::max(nodes, 0ll), 0.0);
  double previous = 0.0;
  for (long long i = 1; i + 1 < nodes; ++i) {
    p[i] = 1.0 / (4.0 - previous);
    previous = p[i];
  }
  return p;
}

inline double legacy_phase(double v) { return (double)(float)v; }

std::vector<double> sep_pivots(long long nodes) {
  std::vector<double> p((size_t)nodes, 0.0);
  for (long long i = 1; i + 1 < nodes; ++i) p[i] = 1.0 / (2.0 - 0.25 * p[i - 1]);
  return p;
}

void sep_coefficients(const double* values, const std::vector<double>& pivots, long long lanes, double* coeff) {
  const long long n = (long long)pivots.size();
  for (long long i = 1; i + 1 < n; ++i)
    for (long long j = 0; j < lanes; ++j) {
      const double left = values[(i - 1) * lanes + j], middle = values[i * lanes + j],
                   right = values[(i + 1) * lanes + j];
      const double difference = (right - middle) - (middle - left);
      coeff[i * lanes + j] = std::fma(3.0, difference, -0.5 * coeff[(i - 1) * lanes + j]) * pivots[i];
    }
  for (long long i = n - 2; i >= 1; --i) {
    const double multiplier = -0.5 * pivots[i];
    for (long long j = 0; j < lanes; ++j)
      coeff[i * lanes + j] = std::fma(multiplier, coeff[(i + 1) * lanes + j], coeff[i * lanes + j]) / 6.0;
  }
}

// Device buffers released at scope exit.
struct DevBuffers {
  std::vector<void*> ptrs;
  template <typename P>
  cudaError_t alloc(P** p, size_t bytes) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, bytes ? bytes : 1);
    if (e == cudaSuccess) ptrs.push_back(v);
    *p = reinterpret_cast<P*>(v);
    return e;
  }
  ~DevBuffers() {
    for (void* p : ptrs) cudaFree(p);
  }
};

template <typename T>
int interpolate_spline(const std::vector<double>& mesh, const Rules& r, T* d_out, cudaStream_t s, int sm_count) {
  DevBuffers buf;
  const size_t ndim = r.shape.size();
  double* cur = nullptr;
  cudaError_t e = buf.alloc(&cur, mesh.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(cur, mesh.data(), mesh.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "mesh spline upload");
  for (size_t axis = 0; axis < ndim; ++axis) {
    long long outer = 1, inner = 1;
    for (size_t a = 0; a < axis; ++a) outer *= r.shape[a];
    for (size_t a = axis + 1; a < ndim; ++a) inner *= r.mesh_shape[a];
    const long long nodes = r.mesh_shape[axis], length = r.shape[axis];
    std::vector<SplineTap> taps((size_t)length);
    for (long long p = 0; p < length; ++p)
      taps[p] = make_tap(((double)p + 0.5) / (double)r.box[axis] - 0.5, nodes);
    const std::vector<double> pivots = natural_pivots(nodes);
    SplineTap* d_taps = nullptr;
    double* d_pivots = nullptr;
    e = buf.alloc(&d_taps, taps.size() * sizeof(SplineTap));
    if (e == cudaSuccess) e = buf.alloc(&d_pivots, pivots.size() * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_taps, taps.data(), taps.size() * sizeof(SplineTap), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !pivots.empty())
      e = cudaMemcpyAsync(d_pivots, pivots.data(), pivots.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh spline tables");
    if (axis + 1 == ndim) {
      const long long blocks = std::min(outer, (long long)std::max(1, sm_count) * 16);
      const size_t smem = (size_t)std::max(nodes, 1ll) * sizeof(double);
      auto k = spline_last_kernel<T>;
      if ((e = allow_max_smem((const void*)k)) != cudaSuccess) return cuda_fail(e, "mesh spline");
      k<<<(unsigned)std::max(blocks, 1ll), 256, smem, s>>>(cur, d_pivots, d_taps, d_out, outer, nodes, length);
      e = cudaGetLastError();
      if (e != cudaSuccess) return cuda_fail(e, "mesh spline");
      // The temporaries are freed at scope exit: wait for the kernels first.
      e = cudaStreamSynchronize(s);
      return e == cudaSuccess ? NDF_OK : cuda_fail(e, "mesh spline");
    }
    double* second = nullptr;
    double* next = nullptr;
    e = buf.alloc(&second, (size_t)(outer * nodes * inner) * sizeof(double));
    if (e == cudaSuccess) e = buf.alloc(&next, (size_t)(outer * length * inner) * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "mesh spline buffers");
    const long long cols = outer * inner;
    spline_second_kernel<<<(unsigned)((cols + 255) / 256), 256, 0, s>>>(cur, d_pivots, second, outer, nodes, inner);
    const long long items = outer * length * inner;
    spline_expand_kernel<<<(unsigned)((items + 255) / 256), 256, 0, s>>>(cur, second, d_taps, next, outer, length,
                                                                         nodes, inner);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mesh spline");
    cur = next;
  }
  return NDF_OK;
}

template <typename T>
int interpolate_sep(const std::vector<double>& mesh, const Rules& r, T* d_out, cudaStream_t s, int sm_count) {
  DevBuffers buf;
  const long long ny = r.shape[0], nx = r.shape[1], height = r.box[0], width = r.box[1];
  const long long rows = r.mesh_shape[0], columns = r.mesh_shape[1];
  const long long blocks = std::max(1ll, std::min(ny, (long long)std::max(1, sm_count) * 16));
  if (mesh.size() == 1) {
    fill_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(d_out, ny * nx, mesh[0]);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NDF_OK : cuda_fail(e, "mesh fill");
  }
  double peak = 0.0;
  for (double v : mesh) peak = std::fmax(peak, std::fabs(v));
  uint64_t pb;
  std::memcpy(&pb, &peak, 8);
  pb &= 0x7ff0000000000000ull;
  double exp_part;
  std::memcpy(&exp_part, &pb, 8);
  const double scale = std::fmax(exp_part, 2.2250738585072014e-308);
  const double inverse_scale = 1.0 / scale;
  std::vector<double> values(mesh.size());
  for (size_t i = 0; i < mesh.size(); ++i) values[i] = mesh[i] * inverse_scale;
  const bool have_x = columns > 1;
  std::vector<long long> lengths;
  std::vector<SepWeight> first, later;
  std::vector<int> pix_interval((size_t)nx, 0), pix_weight((size_t)nx, 0);
  if (have_x) {
    const double step = legacy_phase(1.0 / legacy_phase((double)width));
    auto weights = [&](double b, long long length) {
      std::vector<SepWeight> w;
      for (long long i = 0; i < length; ++i) {
        const double a = 1.0 - b;
        w.push_back({b, a * std::fma(a, a, -1.0), b * std::fma(b, b, -1.0)});
        b = legacy_phase(b + step);
      }
      return w;
    };
    const long long intervals = width == 1 ? 1 : columns - 1;
    long long start = 0;
    for (long long i = 1; i <= intervals; ++i) {
      const long long end = i == intervals ? nx : i * width + width / 2;
      lengths.push_back(end - start);
      start = end;
    }
    first = weights(legacy_phase(0.5 * step - 0.5), lengths[0]);
    long long longest = 0;
    for (size_t i = 1; i < lengths.size(); ++i) longest = std::max(longest, lengths[i]);
    later = weights(width % 2 == 0 ? 0.5 * step : 0.0, longest);
    long long pos = 0;
    for (size_t i = 0; i < lengths.size(); ++i)
      for (long long k = 0; k < lengths[i]; ++k, ++pos) {
        pix_interval[pos] = (int)i;
        pix_weight[pos] = (int)k;
      }
  }
  cudaError_t e = cudaSuccess;
  if (rows == 1 && have_x) {
    // One mesh row: a piecewise linear profile (zero curvature terms).
    std::vector<double> profile((size_t)nx);
    for (long long p = 0; p < nx; ++p) {
      const int i = pix_interval[p];
      const SepWeight& w = (i == 0 ? first : later)[pix_weight[p]];
      const double left = values[i], right = values[i + 1];
      const double linear = std::fma(w.fraction, right - left, left);
      profile[p] = std::fma(w.right_curve, 0.0, std::fma(w.left_curve, 0.0, linear)) * scale;
    }
    double* d_profile = nullptr;
    e = buf.alloc(&d_profile, profile.size() * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_profile, profile.data(), profile.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh sep profile");
    rows_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(d_profile, d_out, ny, nx);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? NDF_OK : cuda_fail(e, "mesh sep profile");
  }
  std::vector<double> y_coeff(mesh.size(), 0.0);
  sep_coefficients(values.data(), sep_pivots(rows), columns, y_coeff.data());
  const std::vector<double> x_pivots = have_x ? sep_pivots(columns) : std::vector<double>(1, 0.0);
  const double phase_height = legacy_phase((double)height);
  std::vector<SepRow> row_table((size_t)ny);
  for (long long y = 0; y < ny; ++y) {
    const double box_coordinate = legacy_phase(legacy_phase((double)y) / phase_height);
    const double z = legacy_phase(box_coordinate - 0.5);
    const long long i = std::min(z > 0.0 ? (long long)z : 0ll, rows - 2);
    const double b = z - (double)i, a = 1.0 - b;
    row_table[y] = {i, b, std::fma(a * a, a, -a), std::fma(b * b, b, -b)};
  }
  double *d_values, *d_ycoeff, *d_xpiv;
  SepRow* d_rows;
  SepWeight *d_first, *d_later;
  int *d_pi, *d_pw;
  auto up = [&](auto** dst, const auto& vec) {
    using E = typename std::decay_t<decltype(vec)>::value_type;
    cudaError_t err = buf.alloc(dst, std::max<size_t>(vec.size(), 1) * sizeof(E));
    if (err == cudaSuccess && !vec.empty())
      err = cudaMemcpyAsync(*dst, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice, s);
    return err;
  };
  if ((e = up(&d_values, values)) != cudaSuccess || (e = up(&d_ycoeff, y_coeff)) != cudaSuccess ||
      (e = up(&d_xpiv, x_pivots)) != cudaSuccess || (e = up(&d_rows, row_table)) != cudaSuccess ||
      (e = up(&d_first, first)) != cudaSuccess || (e = up(&d_later, later)) != cudaSuccess ||
      (e = up(&d_pi, pix_interval)) != cudaSuccess || (e = up(&d_pw, pix_weight)) != cudaSuccess)
    return cuda_fail(e, "mesh sep tables");
  const size_t smem = (size_t)columns * 2 * sizeof(double);
  auto k = sep_rows_kernel<T>;
  if ((e = allow_max_smem((const void*)k)) != cudaSuccess) return cuda_fail(e, "mesh sep");
  k<<<(unsigned)blocks, 256, smem, s>>>(d_values, d_ycoeff, d_xpiv, d_rows, d_first, d_later, d_pi, d_pw, d_out, ny,
                                        nx, columns, scale, have_x ? 1 : 0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? NDF_OK : cuda_fail(e, "mesh sep");
}

template <typename T>
int interpolate(const std::vector<double>& mesh, const Rules& r, T* d_out, cudaStream_t s, int sm_count) {
  if (r.len == 0) return NDF_OK;
  bool constant = true;
  for (double v : mesh) constant = constant && v == mesh[0];
  if (constant) {
    const long long blocks = std::max(1ll, std::min((r.len + 255) / 256, (long long)std::max(1, sm_count) * 16));
    fill_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(d_out, r.len, mesh[0]);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NDF_OK : cuda_fail(e, "mesh fill");
  }
  if (r.c.interpolation == NDF_MESH_INTERP_SEXTRACTOR) return interpolate_sep(mesh, r, d_out, s, sm_count);
  return interpolate_spline(mesh, r, d_out, s, sm_count);
}

template <typename T>
int run_device(const T* d_in, const uint8_t* d_mask, const Rules& r, T* d_bg, T* d_rms, double* mesh_bg,
               double* mesh_rms, uint8_t* mesh_valid, int64_t* finite_count, int64_t* retained_count,
               double* globals, cudaStream_t s) {
  int device = 0, sm_count = 0, smem_optin = 0;
  int rc = device_ready(&device, &sm_count, &smem_optin);
  if (rc != NDF_OK) return rc;
  const long long m = r.mesh_len;
  std::vector<double> bg((size_t)m, NAN), rms((size_t)m, NAN);
  std::vector<long long> fin((size_t)m, 0), ret((size_t)m, 0);
  std::vector<unsigned char> valid((size_t)m, 0);
  if (r.len > 0 && m > 0) {
    DevBuffers buf;
    MeshArgs a{};
    a.ndim = (int)r.shape.size();
    for (int d = 0; d < a.ndim; ++d) {
      a.shape[d] = r.shape[d];
      a.box[d] = r.box[d];
      a.mesh_shape[d] = r.mesh_shape[d];
    }
    a.mesh_len = m;
    a.box_volume = r.box_volume;
    a.estimator = r.c.estimator;
    a.center = r.c.center;
    a.spread = r.c.spread;
    a.statistic = r.c.statistic;
    a.mode_estimator = r.c.mode_estimator;
    a.rms = r.c.rms;
    a.valid_count = r.c.valid_count;
    a.valid_base = r.c.valid_base;
    a.maxiters = r.c.maxiters < 0 ? -1 : r.c.maxiters;
    a.pearson = r.c.pearson;
    a.lower = r.c.sigma_lower;
    a.upper = r.c.sigma_upper;
    a.min_valid_fraction = r.c.min_valid_fraction;
    // Largest mesh volume, padded to a power of two for the sort.
    long long largest = 1;
    for (int d = 0; d < a.ndim; ++d) largest *= std::min(r.box[d], r.shape[d]);
    long long padded = 1;
    while (padded < largest) padded <<= 1;
    // One block per mesh when the sort fits in shared memory; otherwise the
    // blocks share a bounded global workspace and stride over the meshes.
    long long blocks = std::min(m, (long long)INT_MAX);
    unsigned long long* scratch = nullptr;
    size_t smem = 0;
    if (padded * 8 <= std::min((long long)smem_optin, kMeshSmemBytes)) {
      smem = (size_t)padded * 8;
      a.capacity = 0;
    } else {
      a.capacity = padded;
      blocks = std::min({m, (long long)std::max(1, sm_count) * 16, std::max(1ll, (1ll << 30) / (padded * 8))});
      cudaError_t e = buf.alloc(&scratch, (size_t)(blocks * padded) * 8);
      if (e != cudaSuccess) return fail(NDF_ERR_MEMORY, "unable to allocate mesh workspace");
    }
    MeshOut o;
    cudaError_t e = buf.alloc(&o.background, (size_t)m * 8);
    if (e == cudaSuccess) e = buf.alloc(&o.rms, (size_t)m * 8);
    if (e == cudaSuccess) e = buf.alloc(&o.finite, (size_t)m * 8);
    if (e == cudaSuccess) e = buf.alloc(&o.retained, (size_t)m * 8);
    if (e == cudaSuccess) e = buf.alloc(&o.valid, (size_t)m);
    if (e != cudaSuccess) return fail(NDF_ERR_MEMORY, "unable to allocate mesh workspace");
    auto k = mesh_stats_kernel<T>;
    if ((e = allow_max_smem((const void*)k)) != cudaSuccess) return cuda_fail(e, "mesh statistics");
    k<<<(unsigned)blocks, kMThreads, smem, s>>>(d_in, d_mask, a, scratch, o);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(bg.data(), o.background, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rms.data(), o.rms, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fin.data(), o.finite, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ret.data(), o.retained, (size_t)m * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(valid.data(), o.valid, (size_t)m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "mesh statistics");
  }
  fill_invalid(bg, rms, valid, r);
  median_filter(bg, rms, r);
  for (long long i = 0; i < m; ++i) {
    if (mesh_bg) mesh_bg[i] = bg[i];
    if (mesh_rms) mesh_rms[i] = rms[i];
    if (mesh_valid) mesh_valid[i] = valid[i];
    if (finite_count) finite_count[i] = fin[i];
    if (retained_count) retained_count[i] = ret[i];
  }
  if (globals) {
    globals[0] = median_of(bg);
    globals[1] = median_of(rms);
  }
  rc = interpolate(bg, r, d_bg, s, sm_count);
  if (rc != NDF_OK) return rc;
  return interpolate(rms, r, d_rms, s, sm_count);
}

}  // namespace
}  // namespace ndf

using namespace ndf;

extern "C" {

int ndf_mesh_background_device(const void* d_in, const uint8_t* d_mask, int32_t dtype, int32_t ndim,
                               const uint64_t* shape, const uint64_t* box_size, const uint64_t* filter_size,
                               const ndf_mesh_config* config, void* d_background, void* d_rms,
                               double* mesh_background, double* mesh_rms, uint8_t* mesh_valid,
                               int64_t* mesh_finite_count, int64_t* mesh_retained_count, double* globals,
                               void* stream) {
  Rules r;
  int rc = validate(shape, box_size, filter_size, ndim, config, r);
  if (rc != NDF_OK) return rc;
  if (dtype != NDF_FLOAT32 && dtype != NDF_FLOAT64)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "array dtype must be float32 or float64");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (dtype == NDF_FLOAT32)
    return run_device((const float*)d_in, d_mask, r, (float*)d_background, (float*)d_rms, mesh_background, mesh_rms,
                      mesh_valid, mesh_finite_count, mesh_retained_count, globals, s);
  return run_device((const double*)d_in, d_mask, r, (double*)d_background, (double*)d_rms, mesh_background,
                    mesh_rms, mesh_valid, mesh_finite_count, mesh_retained_count, globals, s);
}

int ndf_mesh_background(const void* h_in, const uint8_t* h_mask, int32_t dtype, int32_t ndim, const uint64_t* shape,
                        const uint64_t* box_size, const uint64_t* filter_size, const ndf_mesh_config* config,
                        void* h_background, void* h_rms, double* mesh_background, double* mesh_rms,
                        uint8_t* mesh_valid, int64_t* mesh_finite_count, int64_t* mesh_retained_count,
                        double* globals) {
  Rules r;
  int rc = validate(shape, box_size, filter_size, ndim, config, r);
  if (rc != NDF_OK) return rc;
  if (dtype != NDF_FLOAT32 && dtype != NDF_FLOAT64)
    return fail(NDF_ERR_INVALID_CONFIGURATION, "array dtype must be float32 or float64");
  int device = 0, sm_count = 0, smem_optin = 0;
  rc = device_ready(&device, &sm_count, &smem_optin);
  if (rc != NDF_OK) return rc;
  const size_t bytes = (size_t)r.len * (dtype == NDF_FLOAT32 ? 4 : 8);
  DevBuffers buf;
  void *d_in = nullptr, *d_bg = nullptr, *d_rms = nullptr;
  uint8_t* d_mask = nullptr;
  cudaError_t e = buf.alloc(&d_in, bytes);
  if (e == cudaSuccess) e = buf.alloc(&d_bg, bytes);
  if (e == cudaSuccess) e = buf.alloc(&d_rms, bytes);
  if (e == cudaSuccess && h_mask) e = buf.alloc(&d_mask, (size_t)r.len);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(NDF_ERR_MEMORY, "unable to allocate filtering workspace");
  }
  // Fresh pageable maps fault their pages one at a time inside a copy: touch
  // them on the host pool while the upload and the pipeline run.
  std::thread prefault([&] {
    for (void* h : {h_background, h_rms}) {
      cudaPointerAttributes attr{};
      if (cudaPointerGetAttributes(&attr, h) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if (attr.type == cudaMemoryTypeUnregistered) prefault_pages(h, bytes);
    }
  });
  if (bytes) e = cudaMemcpy(d_in, h_in, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && h_mask && r.len) e = cudaMemcpy(d_mask, h_mask, (size_t)r.len, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    rc = ndf_mesh_background_device(d_in, h_mask ? d_mask : nullptr, dtype, ndim, shape, box_size, filter_size,
                                    config, d_bg, d_rms, mesh_background, mesh_rms, mesh_valid, mesh_finite_count,
                                    mesh_retained_count, globals, nullptr);
  prefault.join();
  if (e != cudaSuccess) return cuda_fail(e, "mesh upload");
  if (rc != NDF_OK) return rc;
  if (bytes) {
    e = cudaMemcpy(h_background, d_bg, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_rms, d_rms, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mesh download");
  }
  return NDF_OK;
}

}  // extern "C"

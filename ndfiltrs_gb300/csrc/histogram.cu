// Sliding rank-histogram median and rank for rectangular 1-D/2-D windows
// (method="histogram"; also the large-window path of "direct").
//
// Replaces order_statistic_into / Geometry::block / Histogram
// (src/histogram.rs:93-631). As in the reference, each block of outputs
// ranks its support (the block plus the window halo, through the boundary
// modes) so that every retained sample gets a unique block-local rank; a
// window is then a set of ranks, kept as a bit histogram, and a k-th
// order statistic is the k-th set bit. Results equal direct selection bit
// for bit: equal keys are interchangeable, so the tie order of the ranks
// does not matter.
//
// GB300 design:
//  * one thread block per output tile (persistent grid over tiles);
//  * ranking: a block-level LSD radix sort of the support's keys (8-bit
//    digits, warp match_any ranking for stability, digits on which every
//    retained key agrees are skipped) through a per-block scratch slot in
//    global memory (L2-resident); rank codes are u16 (support <= 65534);
//  * sliding: each half-warp (16 lanes) owns a strip of output columns and
//    walks it in boustrophedon order, so a warp advances two windows per
//    step; a vertical step removes one support row segment (kw codes) and
//    adds another, spread over the 16 lanes with shared-memory atomics on the
//    half-warp's private bitset; a selection scans 512 ranks per step from a
//    tracked pivot (the previous window's order statistic) and ends with a
//    5-step select in the final word. Tile widths are multiples of 32 columns,
//    so every half-warp's columns lie inside the tile's support.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/ndfiltrs_gb300.h"
#include "common.cuh"
#include "plan.h"

namespace ndf {

int fail(int code, const std::string& message);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kHThreads = 512;
constexpr int kHWarps = kHThreads / 32;
constexpr uint16_t kOmitted = 0xFFFF;
constexpr uint16_t kPropagated = 0xFFFE;
constexpr int kMaxSupport = 65534;

struct HistArgs {
  Geom3 g;
  int TW, TH, SW, SH, S;
  int plane;                // SH * SW: one support plane (the support is kd planes)
  long long tiles_x, tiles_yx, tiles;
  int cols_per_warp;        // columns walked by each half-warp segment
  int words;                // per-segment bit histogram: 32-bit words
  long long slot_bytes;     // scratch bytes per block slot
  int digit_bits;           // radix digit width of the block sort (8 or 11)
  Reduce r;
  // Footprint windows: support-linear offsets (y * SW + x) of the taps
  // (nf), of the top and bottom ends of every vertical run of taps (nv
  // each) and of the left and right ends of every horizontal run (nh
  // each), in that order. Unused (nullptr) for rectangular windows.
  const uint16_t* lists;
  int nf, nv, nh;
};

// A block's sort slot: ping-pong keys and 16-bit payloads (support indices).
template <typename K>
struct Slot {
  K* keys_a;
  K* keys_b;
  uint16_t* pay_a;
  uint16_t* pay_b;
};

__host__ __device__ inline long long align16(long long v) { return (v + 15) & ~15ll; }

template <typename K>
__host__ __device__ inline long long slot_bytes_for(int S) {
  return 2 * align16((long long)S * sizeof(K)) + 2 * align16((long long)S * 2);
}

template <typename K>
__device__ inline Slot<K> slot_at(unsigned char* base, int S) {
  Slot<K> s;
  long long off = 0;
  s.keys_a = reinterpret_cast<K*>(base + off);
  off += align16((long long)S * sizeof(K));
  s.keys_b = reinterpret_cast<K*>(base + off);
  off += align16((long long)S * sizeof(K));
  s.pay_a = reinterpret_cast<uint16_t*>(base + off);
  off += align16((long long)S * 2);
  s.pay_b = reinterpret_cast<uint16_t*>(base + off);
  return s;
}

// Accesses to the sort slots in global memory with an L2 evict-last policy.
// A block rewrites its slot on every radix pass; together the slots hold
// (grid) x S x 12 bytes (67 MB for 152 blocks of 36,864 samples), which fits
// in the 126 MB L2, and the hint keeps them there against the input stream
// (read with evict-first loads), so the ping-pong does not reach DRAM.
__device__ __forceinline__ unsigned long long keep_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_keep(uint32_t* a, uint32_t v, unsigned long long p) {
  asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(a), "r"(v), "l"(p) : "memory");
}
__device__ __forceinline__ void st_keep(unsigned long long* a, unsigned long long v, unsigned long long p) {
  asm volatile("st.global.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(a), "l"(v), "l"(p) : "memory");
}
__device__ __forceinline__ void st_keep(uint16_t* a, uint16_t v, unsigned long long p) {
  asm volatile("st.global.L2::cache_hint.b16 [%0], %1, %2;" ::"l"(a), "h"(v), "l"(p) : "memory");
}
__device__ __forceinline__ uint32_t ld_keep(const uint32_t* a, unsigned long long p) {
  uint32_t v;
  asm volatile("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_keep(const unsigned long long* a, unsigned long long p) {
  unsigned long long v;
  asm volatile("ld.global.L2::cache_hint.b64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint16_t ld_keep(const uint16_t* a, unsigned long long p) {
  uint16_t v;
  asm volatile("ld.global.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(a), "l"(p) : "memory");
  return v;
}

// Shared-memory words of the sort's counter tables for `nd` digits: one
// table of nd counters per warp plus the nd digit totals.
__host__ __device__ inline long long sort_table_words(int nd) { return (long long)(kHWarps + 1) * nd; }

// One stable counting pass over `nd`-valued digits. `table` holds
// kHWarps x nd counters, `totals` nd. Each warp owns a contiguous segment
// and ranks its 32-key chunks in order with match_any, so equal digits keep
// their order. Loads are batched (kBatch keys per lane in registers) so a
// pass costs one memory round trip per batch rather than one per chunk.
constexpr int kBatch = 16;

template <typename K, typename Digit>
__device__ void radix_pass(const K* src_k, const uint16_t* src_p, K* dst_k, uint16_t* dst_p, int S,
                           unsigned int* table, unsigned int* totals, int nd, Digit digit,
                           unsigned long long keep) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < kHWarps * nd; i += blockDim.x) table[i] = 0;
  __syncthreads();
  const int chunk = (((S + kHWarps - 1) / kHWarps) + 31) & ~31;
  const int begin = warp * chunk;
  const int end = min(S, begin + chunk);
  unsigned int* wt = table + warp * nd;
  for (int b = begin; b < end; b += 32 * kBatch) {
    K keys[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int i = b + j * 32 + lane;
      keys[j] = i < end ? ld_keep(src_k + i, keep) : K(0);
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j)
      if (b + j * 32 + lane < end) atomicAdd(&wt[digit(keys[j])], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nd; d += blockDim.x) {
    unsigned int sum = 0;
    for (int w = 0; w < kHWarps; ++w) sum += table[w * nd + d];
    totals[d] = sum;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // Exclusive scan of the nd totals by one warp (nd / 32 per lane).
    const int per = nd >> 5;
    unsigned int run = 0;
    for (int j = 0; j < per; ++j) {
      const unsigned int t = totals[lane * per + j];
      totals[lane * per + j] = run;
      run += t;
    }
    unsigned int inc = run;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    const unsigned int excl = inc - run;
    for (int j = 0; j < per; ++j) totals[lane * per + j] += excl;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < nd; d += blockDim.x) {
    unsigned int run = totals[d];
    for (int w = 0; w < kHWarps; ++w) {
      const unsigned int c = table[w * nd + d];
      table[w * nd + d] = run;
      run += c;
    }
  }
  __syncthreads();
  for (int b = begin; b < end; b += 32 * kBatch) {
    K keys[kBatch];
    uint16_t pays[kBatch];
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const int i = b + j * 32 + lane;
      keys[j] = i < end ? ld_keep(src_k + i, keep) : K(0);
      pays[j] = i < end ? ld_keep(src_p + i, keep) : uint16_t(0);
    }
#pragma unroll
    for (int j = 0; j < kBatch; ++j) {
      const bool valid = b + j * 32 + lane < end;
      const int d = valid ? (int)digit(keys[j]) : nd + lane;
      const unsigned int peers = __match_any_sync(0xffffffffu, d);
      const int before = __popc(peers & ((1u << lane) - 1u));
      unsigned int pos = 0;
      if (valid) pos = wt[d] + before;
      __syncwarp();
      if (valid && lane == 31 - __clz(peers)) wt[d] += __popc(peers);
      __syncwarp();
      if (valid) {
        st_keep(dst_k + pos, keys[j], keep);
        st_keep(dst_p + pos, pays[j], keep);
      }
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int select_in_word32(unsigned int word, int k) {
  int position = 0;
#pragma unroll
  for (int width = 16; width >= 1; width >>= 1) {
    int low = __popc(word & ((1u << width) - 1u));
    if (k >= low) {
      k -= low;
      word >>= width;
      position += width;
    }
  }
  return position;
}

// Each half-warp (16 lanes, a "segment") owns one bit histogram of the
// ranks in its window, so a warp advances two windows per step. The segment
// tracks the rank `m` of its last selected order statistic and the number
// `lt` of window samples ranked below it, kept up to date by every histogram
// update. A selection walks from m word by word (every lane loads the same
// word, so the walk costs what one thread's would); the next window's order
// statistic is usually a few window samples away, within a word or two. A
// walk longer than kSeqWords words continues as a parallel scan of 16 words
// per iteration (sixteen sequential words measured 2-5% faster than four,
// and four faster than one or two, from 13 x 13 to 65 x 65 windows; 32 no
// faster than 16). Every loop
// that contains warp-synchronous operations runs until both segments of the
// warp are done, so the two halves stay converged.
constexpr int kSeg = 16;
constexpr int kSegs = kHThreads / kSeg;
constexpr unsigned int kFull = 0xffffffffu;
constexpr int kSeqWords = 16;

struct SegHist {
  unsigned int* words;
  int nwords;
  int m;      // tracked rank (the last order statistic selected)
  int lt;     // window samples ranked below m
  int count;  // retained samples in the window
  int nan;    // propagated NaN samples in the window
};

__device__ __forceinline__ int seg_lane() { return threadIdx.x & (kSeg - 1); }

__device__ __forceinline__ unsigned int seg_ballot(bool p) {
  return (__ballot_sync(kFull, p) >> (threadIdx.x & kSeg)) & 0xFFFFu;
}

__device__ __forceinline__ int seg_sum(int v) {
#pragma unroll
  for (int o = kSeg / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(kFull, v, o, kSeg);
  return v;
}

__device__ __forceinline__ unsigned int seg_scan(unsigned int v) {
  const int hl = seg_lane();
#pragma unroll
  for (int o = 1; o < kSeg; o <<= 1) {
    const unsigned int t = __shfl_up_sync(kFull, v, o, kSeg);
    if (hl >= o) v += t;
  }
  return v;
}

template <typename V>
__device__ __forceinline__ V seg_bcast(V v, int src) {
  return __shfl_sync(kFull, v, src, kSeg);
}

// Parallel continuation of a walk. Forward: the rem-th (0-based) set bit at
// or above word wi. Backward: the rem-th (1-based) set bit counting down
// from the top of word wi. `active` false takes part for convergence only
// and returns r unchanged.
__device__ __noinline__ int seg_scan_select(const SegHist& h, int wi, int rem, bool fwd, bool active, int r) {
  const int hl = seg_lane();
  bool found = !active;
  for (int guard = 0; guard < 8192; ++guard) {
    if (!__any_sync(kFull, !found)) break;
    const int widx = fwd ? wi + hl : wi - hl;
    const unsigned int word = (widx >= 0 && widx < h.nwords) ? h.words[widx] : 0u;
    const unsigned int pc = __popc(word);
    const unsigned int incl = seg_scan(pc);
    const int total = (int)seg_bcast(incl, kSeg - 1);
    const unsigned int ball = seg_ballot(fwd ? (int)incl > rem : (int)incl >= rem);
    const int L = ball ? __ffs(ball) - 1 : 0;
    const unsigned int w = seg_bcast(word, L);
    const int excl = (int)seg_bcast(incl - pc, L);
    if (!found) {
      if (ball) {
        const int within = rem - excl;
        r = ((fwd ? wi + L : wi - L) << 5) + select_in_word32(w, fwd ? within : __popc(w) - within);
        found = true;
      } else {
        rem -= total;
        wi = fwd ? wi + kSeg : wi - kSeg;
        if (wi < 0 || wi >= h.nwords) found = true;  // no such bit: leave r
      }
    }
  }
  return r;
}

// Rank of the k-th (0-based) retained sample of the segment's window; the
// tracked rank moves to it. `active` false leaves the state untouched.
__device__ __forceinline__ int seg_select(SegHist& h, int k, bool active) {
  int r = 0, wi = 0, rem = 0;
  bool fwd = true, done = !active;
  if (active) {
    int d = k - h.lt;
    wi = h.m >> 5;
    const int bit = h.m & 31;
    if (d >= 0) {
      unsigned int w = h.words[wi] & (~0u << bit);
      int pc = __popc(w);
#pragma unroll 1
      for (int s = 0; d >= pc && s < kSeqWords; ++s) {
        d -= pc;
        ++wi;
        w = wi < h.nwords ? h.words[wi] : 0u;
        pc = __popc(w);
      }
      if (d < pc) {
        r = (wi << 5) + select_in_word32(w, d);
        done = true;
      } else {
        rem = d - pc;
        ++wi;
      }
    } else {
      int e = -d;
      unsigned int w = h.words[wi] & ((1u << bit) - 1u);
      int pc = __popc(w);
#pragma unroll 1
      for (int s = 0; e > pc && s < kSeqWords; ++s) {
        e -= pc;
        --wi;
        w = wi >= 0 ? h.words[wi] : 0u;
        pc = __popc(w);
      }
      if (e <= pc) {
        r = (wi << 5) + select_in_word32(w, pc - e);
        done = true;
      } else {
        rem = e - pc;
        --wi;
        fwd = false;
      }
    }
  }
  if (__any_sync(kFull, !done)) r = seg_scan_select(h, wi, rem, fwd, !done, r);
  if (active) {
    h.m = r;
    h.lt = k;
  }
  return r;
}

// Rank of the first retained sample above `rank` (the next order statistic).
__device__ __forceinline__ int seg_next(const SegHist& h, int rank, bool active) {
  int r = rank, wi = 0;
  bool done = !active;
  if (active) {
    wi = rank >> 5;
    unsigned int w = h.words[wi] & ~((2u << (rank & 31)) - 1u);
#pragma unroll 1
    for (int s = 0; w == 0u && s < kSeqWords; ++s) {
      ++wi;
      w = wi < h.nwords ? h.words[wi] : 0u;
    }
    if (w) {
      r = (wi << 5) + __ffs(w) - 1;
      done = true;
    } else {
      ++wi;
    }
  }
  if (__any_sync(kFull, !done)) r = seg_scan_select(h, wi, 0, true, !done, r);
  return r;
}

// Per-step bookkeeping of a lane: retained, below-m and propagated-NaN
// deltas.
struct StepDelta {
  int kept = 0, below = 0, nans = 0;
};

template <bool PROPAGATE>
__device__ __forceinline__ void update(const SegHist& h, int c, int sign, StepDelta& d) {
  const bool valid = c < (int)kPropagated;
  // Unconditional: a dropped code XORs zero into a word of the segment's own
  // bitset (the lane's, within its bounds), so the update has no branch (and
  // no reconvergence) around its atomic.
  atomicXor(&h.words[valid ? (c >> 5) : min(seg_lane(), h.nwords - 1)], valid ? 1u << (c & 31) : 0u);
  d.kept += valid ? sign : 0;
  d.below += c < h.m ? sign : 0;  // codes below m are retained (dropped codes are the largest)
  if (PROPAGATE) d.nans += c == (int)kPropagated ? sign : 0;
}

// Apply a step's deltas. Under the omit policy the retained and below-m
// deltas share one reduction in two 16-bit halves biased by 1024 per lane,
// valid while a lane handles fewer than 512 codes (`narrow`).
template <bool PROPAGATE>
__device__ __forceinline__ void finish_update(SegHist& h, const StepDelta& d, bool narrow) {
  if (PROPAGATE || !narrow) {
    h.count += seg_sum(d.kept);
    h.lt += seg_sum(d.below);
    if (PROPAGATE) h.nan += seg_sum(d.nans);
  } else {
    const int packed = (d.kept + 1024) | ((d.below + 1024) << 16);
    const unsigned int sum = (unsigned int)seg_sum(packed);
    h.count += (int)(sum & 0xFFFFu) - kSeg * 1024;
    h.lt += (int)(sum >> 16) - kSeg * 1024;
  }
  __syncwarp();
}

// Remove the codes of one face and add those of another (n codes each,
// `stride` apart, in shared memory).
template <bool PROPAGATE>
__device__ __forceinline__ void step(const uint16_t* codes, int remove_start, int add_start, int n,
                                     int stride, SegHist& h) {
  const int hl = seg_lane();
  StepDelta d;
  // The same trip count in every lane (lanes past the face's end update a
  // dropped code, a no-op), so the loop never diverges.
  const int iters = (n + kSeg - 1) / kSeg;
  for (int it = 0, i = hl; it < iters; ++it, i += kSeg) {
    const bool in = i < n;
    const int rc = in ? codes[remove_start + i * stride] : (int)kOmitted;
    const int ac = in ? codes[add_start + i * stride] : (int)kOmitted;
    update<PROPAGATE>(h, rc, -1, d);
    update<PROPAGATE>(h, ac, +1, d);
  }
  finish_update<PROPAGATE>(h, d, n <= 8 * 1024);
}

// Add every code of a kh x kw box (the first window of a segment's walk).
template <bool PROPAGATE>
__device__ __forceinline__ void add_box(const uint16_t* codes, int start, int kh, int kw, int SW,
                                       SegHist& h) {
  const int hl = seg_lane();
  for (int ky = 0; ky < kh; ++ky) {
    StepDelta d;
    for (int i = hl; i < kw; i += kSeg) update<PROPAGATE>(h, codes[start + ky * SW + i], +1, d);
    finish_update<PROPAGATE>(h, d, kw <= 8 * 1024);
  }
}

// Footprint windows: remove the codes at rbase + rlist[i] and add those at
// abase + alist[i] (n each).
template <bool PROPAGATE>
__device__ __forceinline__ void step_lists(const uint16_t* codes, int rbase, const uint16_t* rlist,
                                           int abase, const uint16_t* alist, int n, SegHist& h) {
  const int hl = seg_lane();
  StepDelta d;
  const int iters = (n + kSeg - 1) / kSeg;
  for (int it = 0, i = hl; it < iters; ++it, i += kSeg) {
    const bool in = i < n;
    const int rc = in ? codes[rbase + rlist[i]] : (int)kOmitted;
    const int ac = in ? codes[abase + alist[i]] : (int)kOmitted;
    update<PROPAGATE>(h, rc, -1, d);
    update<PROPAGATE>(h, ac, +1, d);
  }
  finish_update<PROPAGATE>(h, d, n <= 8 * 1024);
}

// Footprint windows: add every tap of the window whose origin is `base`.
template <bool PROPAGATE>
__device__ __forceinline__ void add_taps(const uint16_t* codes, int base, const uint16_t* taps, int n,
                                        SegHist& h) {
  const int hl = seg_lane();
  StepDelta d;
  for (int i = hl; i < n; i += kSeg) update<PROPAGATE>(h, codes[base + taps[i]], +1, d);
  finish_update<PROPAGATE>(h, d, false);
}

// The ranks a window's statistic is read from: lo (and hi for an even
// median or an interpolated percentile), the retained count, and whether
// the window has a value at all.
struct Ranks {
  int lo = 0, hi = 0, n = 0;
  bool valid = false, two = false;
};

// Select the ranks of the segment's window. Every branch on per-segment data
// calls the same sequence of selections, so the warp stays converged.
__device__ __forceinline__ Ranks hist_ranks(SegHist& h, const HistArgs& a) {
  const Reduce& r = a.r;
  Ranks o;
  o.n = h.count;
  const bool valid = !((!r.omit && h.nan > 0) || (r.omit && h.count < r.min_count) || h.count == 0);
  const int last = max(h.count - 1, 0);
  switch (r.kind) {
    case kRank:
    case kRankHistogram: {
      const bool ok = valid && r.param < h.count;
      o.lo = o.hi = seg_select(h, ok ? (int)r.param : 0, ok);
      o.valid = ok;
      return o;
    }
    case kMin:
      o.lo = o.hi = seg_select(h, 0, valid);
      o.valid = valid;
      return o;
    case kMax:
      o.lo = o.hi = seg_select(h, last, valid);
      o.valid = valid;
      return o;
    case kPercentile: {
      if (r.q_is_max) {
        o.lo = o.hi = seg_select(h, last, valid);
        o.valid = valid;
        return o;
      }
      const PctSplit ps = pct_split(r, max(h.count, 1));
      o.lo = seg_select(h, valid ? ps.lower : 0, valid);
      o.two = ps.upper != ps.lower;
      o.hi = seg_next(h, o.lo, valid && o.two);
      o.valid = valid;
      return o;
    }
    default: {
      const bool even = (h.count & 1) == 0;
      const int k = even ? h.count / 2 - 1 : h.count / 2;
      o.lo = seg_select(h, valid ? k : 0, valid);
      o.hi = seg_next(h, o.lo, valid && even);
      o.two = even;
      o.valid = valid;
      return o;
    }
  }
}

// The statistic of a window from its ranks' keys (kl = sorted[lo],
// kh = sorted[hi]).
template <typename T>
__device__ __forceinline__ T hist_value(const Ranks& o, const HistArgs& a, typename KeyOf<T>::K kl,
                                        typename KeyOf<T>::K kh) {
  using KO = KeyOf<T>;
  if (!o.valid) return nan_of(T());
  const T vlo = KO::value(kl);
  switch (a.r.kind) {
    case kPercentile: {
      if (a.r.q_is_max) return vlo;
      const PctSplit ps = pct_split(a.r, max(o.n, 1));
      return pct_value<T>(ps, vlo, o.two ? KO::value(kh) : vlo);
    }
    case kRank:
    case kRankHistogram:
    case kMin:
    case kMax:
      return vlo;
    default:
      if (!o.two) return vlo;
      if constexpr (sizeof(T) == 4) {
        return midpoint_f32(vlo, KO::value(kh));
      } else {
        return midpoint(vlo, KO::value(kh));
      }
  }
}

// Outputs of a walk, one per lane of the segment: the ranks are selected in
// order (one window after another) and parked in lane i % 16; every 16
// outputs the batch's keys are loaded (one independent load per lane), and
// the previous batch's values are computed and stored, so the loads' latency
// overlaps the next 16 windows.
template <typename T>
struct OutPipe {
  using K = typename KeyOf<T>::K;
  Ranks next;             // ranks parked in this lane
  long long next_at = -1; // its output index (-1: none / not stored)
  Ranks held;             // the previous batch: ranks and loaded keys
  long long held_at = -1;
  K kl = 0, kh = 0;

  __device__ __forceinline__ void park(const Ranks& o, long long at, int slot) {
    if (seg_lane() == slot) {
      next = o;
      next_at = at;
    }
  }
  __device__ __forceinline__ void complete(const HistArgs& a, T* __restrict__ out) {
    if (held_at >= 0) out[held_at] = canonical(hist_value<T>(held, a, kl, kh));
    held_at = -1;
  }
  // Complete the held batch, then load the parked one's keys and hold it.
  __device__ __forceinline__ void rotate(const HistArgs& a, const K* sorted, T* __restrict__ out) {
    complete(a, out);
    if (next_at >= 0) {
      kl = next.valid ? sorted[next.lo] : K(0);
      kh = next.valid && next.two ? sorted[next.hi] : kl;
    }
    held = next;
    held_at = next_at;
    next_at = -1;
  }
};

// A segment's boustrophedon walk over columns [c_begin, c_begin + ncols)
// of its tile; columns at or beyond `tw_eff` are computed for convergence
// but not stored. A window's origin is its top-left support position
// o = row * SW + c. Rectangular windows (FP false) move whole support row or
// column segments; footprint windows (FP true) move the run ends in `lists`:
// down removes o + top[i] and adds o + SW + bottom[i], up removes
// o + bottom[i] and adds o - SW + top[i], right removes o + left[i] and adds
// o + 1 + right[i].
template <typename T, bool PROPAGATE, bool FP>
__device__ __forceinline__ void walk(const uint16_t* codes, const uint16_t* lists, int c_begin,
                                     int ncols, int tw_eff, int th_eff, int kh, int kw, int SW,
                                     long long y0, long long x0, const Geom3& g, const HistArgs& a,
                                     const typename KeyOf<T>::K* sorted, T* __restrict__ out,
                                     SegHist& h) {
  const uint16_t* top = lists + a.nf;
  const uint16_t* bottom = top + a.nv;
  const uint16_t* left = bottom + a.nv;
  const uint16_t* right = left + a.nh;
  if (FP)
    add_taps<PROPAGATE>(codes, c_begin, lists, a.nf, h);
  else
    add_box<PROPAGATE>(codes, c_begin, kh, kw, SW, h);
  OutPipe<T> pipe;
  int slot = 0;
  int row = 0;
  int dir = 1;
  for (int j = 0; j < ncols; ++j) {
    const int c = c_begin + j;
    for (int i = 0; i < th_eff; ++i) {
      const Ranks o = hist_ranks(h, a);
      pipe.park(o, c < tw_eff ? (y0 + row) * g.W + x0 + c : -1, slot);
      if (++slot == kSeg) {
        pipe.rotate(a, sorted, out);
        slot = 0;
      }
      if (i + 1 < th_eff) {
        const int o = row * SW + c;
        if (dir > 0) {
          if (FP)
            step_lists<PROPAGATE>(codes, o, top, o + SW, bottom, a.nv, h);
          else
            step<PROPAGATE>(codes, o, o + kh * SW, kw, 1, h);
          ++row;
        } else {
          if (FP)
            step_lists<PROPAGATE>(codes, o, bottom, o - SW, top, a.nv, h);
          else
            step<PROPAGATE>(codes, o + (kh - 1) * SW, o - SW, kw, 1, h);
          --row;
        }
      }
    }
    if (j + 1 < ncols) {
      const int o = row * SW + c;
      if (FP)
        step_lists<PROPAGATE>(codes, o, left, o + 1, right, a.nh, h);
      else
        step<PROPAGATE>(codes, o, o + kw, kh, SW, h);
    }
    dir = -dir;
  }
  pipe.rotate(a, sorted, out);
  pipe.complete(a, out);
}

// One output tile (index `tile` of the plan's tile list) of the sliding
// rank-histogram filter: gather the support, rank it, slide. `scratch_slot`
// is the calling block's sort slot; `smem` the dynamic shared memory, whose
// footprint-list region the caller has filled for FP windows.
template <typename T, bool SDEC, bool FP>
__device__ __forceinline__ void histogram_tile(const T* __restrict__ in, T* __restrict__ out, const HistArgs& a,
                                               long long tile, unsigned char* scratch_slot, unsigned char* smem) {
  using K = typename KeyOf<T>::K;
  const K kSent = KeyOf<T>::kSentinel;
  __shared__ K red_and[kHWarps], red_or[kHWarps];
  __shared__ int red_sent[kHWarps];
  const Geom3& g = a.g;
  const int S = a.S;
  // Shared memory: rank codes [S] u16 | footprint lists (FP) | decode table
  // [S] keys (SDEC) | work (radix tables during the sort, half-warp
  // histograms while sliding).
  uint16_t* codes_s = reinterpret_cast<uint16_t*>(smem);
  const long long list_bytes = FP ? align16((long long)(a.nf + 2 * a.nv + 2 * a.nh) * 2) : 0;
  uint16_t* lists_s = reinterpret_cast<uint16_t*>(smem + align16((long long)a.S * 2));
  K* decode_s = reinterpret_cast<K*>(smem + align16((long long)a.S * 2) + list_bytes);
  unsigned int* work = reinterpret_cast<unsigned int*>(
      smem + align16((long long)a.S * 2) + list_bytes + (SDEC ? align16((long long)a.S * sizeof(K)) : 0));
  const int nd = 1 << a.digit_bits;
  unsigned int* table = work;
  unsigned int* totals = work + kHWarps * nd;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Slot<K> slot = slot_at<K>(scratch_slot, S);
  const unsigned long long keep = keep_policy();
  const bool drop_inf = a.r.drop_inf;
  const K outside = sample_key<T>((T)a.r.cval, drop_inf);
  const long long z = tile / a.tiles_yx;
  const long long tyx = tile - z * a.tiles_yx;
  const long long y0 = (tyx / a.tiles_x) * a.TH;
  const long long x0 = (tyx % a.tiles_x) * a.TW;
  // Gather the support as keys (payload = support index), mapping each
  // coordinate through the boundary modes.
  K k_and = kSent, k_or = 0;
  int sent = 0;
  for (int e = threadIdx.x; e < S; e += blockDim.x) {
    const int sz = e / a.plane;
    const int ep = e - sz * a.plane;
    const int sy = ep / a.SW;
    const int sx = ep - sy * a.SW;
    long long mz, my, mx;
    const bool inside = map_index(z + sz - g.az, g.D, g.mz, &mz) &&
                        map_index(y0 + sy - g.ay, g.H, g.my, &my) &&
                        map_index(x0 + sx - g.ax, g.W, g.mx, &mx);
    const K key = inside ? sample_key<T>(__ldcs(in + (mz * g.H + my) * g.W + mx), drop_inf) : outside;
    st_keep(slot.keys_a + e, key, keep);
    st_keep(slot.pay_a + e, (uint16_t)e, keep);
    if (key != kSent) {
      k_and &= key;
      k_or |= key;
    } else {
      ++sent;
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    k_and &= __shfl_xor_sync(0xffffffffu, k_and, o);
    k_or |= __shfl_xor_sync(0xffffffffu, k_or, o);
    sent += __shfl_xor_sync(0xffffffffu, sent, o);
  }
  if (lane == 0) {
    red_and[warp] = k_and;
    red_or[warp] = k_or;
    red_sent[warp] = sent;
  }
  __syncthreads();
  k_and = kSent;
  k_or = 0;
  sent = 0;
  for (int w = 0; w < kHWarps; ++w) {
    k_and &= red_and[w];
    k_or |= red_or[w];
    sent += red_sent[w];
  }
  // Sort keys (LSD over the bits on which the retained keys differ). The
  // dropped samples' all-ones keys take part like any other key: an LSD
  // sort orders the retained keys among themselves whatever lies between
  // them, and a dropped sample's position is never set in a histogram.
  K* src_k = slot.keys_a;
  K* dst_k = slot.keys_b;
  uint16_t* src_p = slot.pay_a;
  uint16_t* dst_p = slot.pay_b;
  const K varying = sent == S ? K(0) : (k_and ^ k_or);
  if (varying != 0) {
    const int bits = (int)sizeof(K) * 8;
    const int lo = sizeof(K) == 8 ? __ffsll((long long)varying) - 1 : __ffs((int)varying) - 1;
    const int hi = bits - 1 - (sizeof(K) == 8 ? __clzll((long long)varying) : __clz((int)varying));
    const K mask = (K)(nd - 1);
    for (int shift = lo; shift <= hi; shift += a.digit_bits) {
      radix_pass(src_k, src_p, dst_k, dst_p, S, table, totals, nd,
                 [shift, mask](K key) { return (unsigned int)((key >> shift) & mask); }, keep);
      K* tk = src_k;
      src_k = dst_k;
      dst_k = tk;
      uint16_t* tp = src_p;
      src_p = dst_p;
      dst_p = tp;
    }
  }
  const uint16_t dropped = a.r.omit ? kOmitted : kPropagated;
  for (int pos = threadIdx.x; pos < S; pos += blockDim.x) {
    const K key = ld_keep(src_k + pos, keep);
    codes_s[ld_keep(src_p + pos, keep)] = key == kSent ? dropped : (uint16_t)pos;
    if (SDEC) decode_s[pos] = key;
  }
  __syncthreads();
  const K* sorted = SDEC ? decode_s : src_k;

  // Slide: each half-warp walks its columns in boustrophedon order.
  const int th_eff = (int)min((long long)a.TH, g.H - y0);
  const int tw_eff = (int)min((long long)a.TW, g.W - x0);
  const int seg = threadIdx.x / kSeg;
  SegHist h;
  h.words = work + seg * a.words;
  h.nwords = a.words;
  h.m = 0;
  h.lt = 0;
  h.count = 0;
  h.nan = 0;
  for (int i = seg_lane(); i < a.words; i += kSeg) h.words[i] = 0u;
  __syncwarp();
  const int kh = g.kh, kw = g.kw, SW = a.SW;
  // Both halves of a warp have columns iff the warp's first column is in
  // the tile's valid width; whole warps beyond it sit out.
  const int warp_first = (threadIdx.x / 32) * 2 * a.cols_per_warp;
  T* plane_out = out + z * g.H * g.W;
  if (warp_first < tw_eff) {
    if (!a.r.omit)
      walk<T, true, FP>(codes_s, lists_s, seg * a.cols_per_warp, a.cols_per_warp, tw_eff, th_eff, kh,
                        kw, SW, y0, x0, g, a, sorted, plane_out, h);
    else
      walk<T, false, FP>(codes_s, lists_s, seg * a.cols_per_warp, a.cols_per_warp, tw_eff, th_eff, kh,
                         kw, SW, y0, x0, g, a, sorted, plane_out, h);
  }
  __syncthreads();
}

// Copy a footprint window's run lists into their shared-memory region (made
// visible by the first barrier of the next tile).
__device__ __forceinline__ void load_lists(const HistArgs& a, unsigned char* smem) {
  uint16_t* lists_s = reinterpret_cast<uint16_t*>(smem + align16((long long)a.S * 2));
  const int n = a.nf + 2 * a.nv + 2 * a.nh;
  for (int i = threadIdx.x; i < n; i += blockDim.x) lists_s[i] = a.lists[i];
}

template <typename T, bool SDEC, bool FP>
__global__ void __launch_bounds__(kHThreads, 1)
    histogram_kernel(const T* __restrict__ in, T* __restrict__ out, const __grid_constant__ HistArgs a,
                     unsigned char* scratch) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (FP) load_lists(a, smem);
  unsigned char* slot = scratch + (long long)blockIdx.x * a.slot_bytes;
  for (long long tile = blockIdx.x; tile < a.tiles; tile += gridDim.x)
    histogram_tile<T, SDEC, FP>(in, out, a, tile, slot, smem);
}

// Batched images (float32): one persistent launch walks the concatenated
// tile lists of every image of a family (same SDEC / FP variant); a block
// finds a tile's image by binary search over the images' first tiles and
// keeps that image's arguments in shared memory until the image changes.
struct HistTask {
  const float* in;
  float* out;
  long long first_tile;
  HistArgs a;
};

template <bool SDEC, bool FP>
__global__ void __launch_bounds__(kHThreads, 1)
    histogram_family_kernel(const HistTask* __restrict__ tasks, int ntasks, long long total_tiles,
                            unsigned char* scratch, long long slot_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ HistTask task;
  __shared__ int current, found;
  if (threadIdx.x == 0) current = -1;
  __syncthreads();
  unsigned char* slot = scratch + (long long)blockIdx.x * slot_bytes;
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
      for (int i = threadIdx.x; i < (int)(sizeof(HistTask) / 8); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      if (FP) load_lists(task.a, smem);
      if (threadIdx.x == 0) current = index;
    }
    __syncthreads();
    histogram_tile<float, SDEC, FP>(task.in, task.out, task.a, tile - task.first_tile, slot, smem);
  }
}

struct HistChoice {
  int TW = 0, TH = 0;
  bool sdec = false;
  size_t smem = 0;
};

constexpr size_t kSmemBudget = 225 * 1024;

// Run-list entries of a footprint window (0 for a rectangular one).
struct Runs {
  int nf = 0, nv = 0, nh = 0;
  bool footprint = false;
  int entries() const { return footprint ? nf + 2 * nv + 2 * nh : 0; }
};

// Bytes of the work region (the sort's 8-bit-digit tables, or the
// segments' bit histograms while sliding, whichever is larger).
size_t work_bytes_for(int S) {
  const size_t sort = (size_t)sort_table_words(256) * 4;
  const size_t hist = (size_t)kSegs * ((S + 31) / 32) * 4;
  return std::max(sort, hist);
}

// The sort uses 11-bit digits (three passes cover 32 varying bits) when
// their tables fit in the work region, else 8-bit digits.
int digit_bits_for(int S) { return work_bytes_for(S) >= (size_t)sort_table_words(2048) * 4 ? 11 : 8; }

size_t smem_bytes_for(int S, bool sdec, size_t key_bytes, int list_entries) {
  size_t codes = (size_t)align16((long long)S * 2);
  size_t lists = (size_t)align16((long long)list_entries * 2);
  size_t decode = sdec ? (size_t)align16((long long)S * (long long)key_bytes) : 0;
  return codes + lists + decode + work_bytes_for(S);
}

// Count the taps and the vertical and horizontal runs (within each plane)
// of a kd x kh x kw footprint mask (row-major).
Runs count_runs(const std::vector<uint8_t>& mask, int kd, int kh, int kw) {
  Runs r;
  r.footprint = true;
  for (int zz = 0; zz < kd; ++zz)
    for (int y = 0; y < kh; ++y)
      for (int x = 0; x < kw; ++x) {
        const size_t at = ((size_t)zz * kh + y) * kw + x;
        if (!mask[at]) continue;
        ++r.nf;
        if (y == 0 || !mask[at - kw]) ++r.nv;
        if (x == 0 || !mask[at - 1]) ++r.nh;
      }
  return r;
}

// Pick the output tile by a cost model in units of one histogram update per
// output: vertical steps (2 kw), the first window of each warp's walk, the
// column moves, the block sort (about 8 units per support sample) and a
// global decode when the sorted keys do not fit in shared memory.
// The tile of a sliding-histogram plan: by the cost model, or the given
// tw x th when it fits (an autotuner candidate; 0 when it does not).
HistChoice choose_tile(const Geom3& g, size_t key_bytes, const Runs& runs = Runs{}, int force_tw = 0,
                       int force_th = 0) {
  HistChoice best;
  if ((long long)g.kw > kMaxSupport || (long long)g.kh > kMaxSupport || (long long)g.kd > kMaxSupport)
    return best;
  // Windows deeper than one plane walk their (kd-plane) faces through the
  // run lists.
  if (g.kd > 1 && !runs.footprint) return best;
  double best_cost = 1e300;
  auto consider = [&](int tw, int th) {
    long long S = (long long)g.kd * (tw + g.kw - 1) * (th + g.kh - 1);
    if (S > kMaxSupport) return;
    for (int sdec = 1; sdec >= 0; --sdec) {
      size_t smem = smem_bytes_for((int)S, sdec != 0, key_bytes, runs.entries());
      if (smem > kSmemBudget) continue;
      const double cpw = (tw + kSegs - 1) / kSegs;
      const double outputs = (double)tw * th;
      const double vertical = runs.footprint ? runs.nv : g.kw;
      const double horizontal = runs.footprint ? runs.nh : g.kh;
      const double taps = runs.footprint ? runs.nf : (double)g.kh * g.kw;
      double cost = 2.0 * vertical + taps / (cpw * th) + 2.0 * horizontal / th +
                    8.0 * (double)S / outputs + (sdec ? 0.0 : 12.0);
      if (smem * 2 <= kSmemBudget) cost *= 0.9;  // two resident blocks per SM
      if (cost < best_cost) {
        best_cost = cost;
        best.TW = tw;
        best.TH = th;
        best.sdec = sdec != 0;
        best.smem = smem;
      }
      return;
    }
  };
  if (force_tw > 0) {
    consider(force_tw, force_th);
    return best;
  }
  if (g.H == 1 && g.kh == 1) {
    for (int tw : {8192, 4096, 2048, 1024, 512, 256, 128, 64, 32})
      if (tw <= 32 || tw / 2 < g.W) consider(tw, 1);
    return best;
  }
  for (int tw : {128, 64, 32}) {
    if (tw > 32 && tw / 2 >= g.W) continue;
    for (int th : {256, 192, 128, 96, 64, 48, 32, 16, 8, 4, 2, 1}) {
      if (th > 1 && th / 2 >= g.H) continue;
      consider(tw, th);
    }
  }
  return best;
}

HistArgs make_args_core(const Geom3& g, int TW, int TH, int dtype, const Reduce& r) {
  HistArgs a{};
  a.g = g;
  a.TW = TW;
  a.TH = TH;
  a.SW = a.TW + a.g.kw - 1;
  a.SH = a.TH + a.g.kh - 1;
  a.plane = a.SW * a.SH;
  a.S = a.g.kd * a.plane;
  a.tiles_x = (a.g.W + a.TW - 1) / a.TW;
  a.tiles_yx = a.tiles_x * ((a.g.H + a.TH - 1) / a.TH);
  a.tiles = a.tiles_yx * a.g.D;
  a.cols_per_warp = (a.TW + kSegs - 1) / kSegs;  // columns per half-warp segment
  a.words = (a.S + 31) / 32;
  a.slot_bytes = dtype == 0 ? slot_bytes_for<uint32_t>(a.S) : slot_bytes_for<unsigned long long>(a.S);
  a.digit_bits = digit_bits_for(a.S);
  a.r = r;
  a.lists = nullptr;
  a.nf = a.g.kh * a.g.kw;
  a.nv = a.g.kw;
  a.nh = a.g.kh;
  return a;
}

HistArgs make_args(const Plan& p) {
  HistArgs a{};
  a.g = p.tile.g;
  a.TW = p.hist_block_w;
  a.TH = p.hist_block_h;
  a.SW = a.TW + a.g.kw - 1;
  a.SH = a.TH + a.g.kh - 1;
  a.plane = a.SW * a.SH;
  a.S = a.g.kd * a.plane;
  a.tiles_x = (a.g.W + a.TW - 1) / a.TW;
  a.tiles_yx = a.tiles_x * ((a.g.H + a.TH - 1) / a.TH);
  a.tiles = a.tiles_yx * a.g.D;
  a.cols_per_warp = (a.TW + kSegs - 1) / kSegs;  // columns per half-warp segment
  a.words = (a.S + 31) / 32;
  a.slot_bytes = p.dtype == 0 ? slot_bytes_for<uint32_t>(a.S) : slot_bytes_for<unsigned long long>(a.S);
  a.digit_bits = digit_bits_for(a.S);
  a.r = p.r;
  if (p.hist_footprint) {
    a.lists = p.d_hist_lists;
    a.nf = p.hist_nf;
    a.nv = p.hist_nv;
    a.nh = p.hist_nh;
  } else {
    a.lists = nullptr;
    a.nf = a.g.kh * a.g.kw;
    a.nv = a.g.kw;
    a.nh = a.g.kh;
  }
  return a;
}

template <typename T>
void* kernel_for(bool sdec, bool fp = false) {
  if (fp) return sdec ? (void*)histogram_kernel<T, true, true> : (void*)histogram_kernel<T, false, true>;
  return sdec ? (void*)histogram_kernel<T, true, false> : (void*)histogram_kernel<T, false, false>;
}

template <typename T>
cudaError_t launch_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  HistArgs a = make_args(p);
  long long slots = (long long)(p.scratch_bytes / (size_t)a.slot_bytes);
  long long grid = std::min<long long>(a.tiles, slots);
  if (grid < 1) return cudaErrorInvalidValue;
  unsigned char* scratch = (unsigned char*)p.d_scratch;
  const unsigned blocks = (unsigned)grid;
  if (p.hist_footprint) {
    if (p.hist_sdec)
      histogram_kernel<T, true, true><<<blocks, kHThreads, p.smem_bytes, s>>>(in, out, a, scratch);
    else
      histogram_kernel<T, false, true><<<blocks, kHThreads, p.smem_bytes, s>>>(in, out, a, scratch);
  } else {
    if (p.hist_sdec)
      histogram_kernel<T, true, false><<<blocks, kHThreads, p.smem_bytes, s>>>(in, out, a, scratch);
    else
      histogram_kernel<T, false, false><<<blocks, kHThreads, p.smem_bytes, s>>>(in, out, a, scratch);
  }
  return cudaGetLastError();
}

}  // namespace

namespace {

// The footprint of a plan as a kd x kh x kw mask in the tile's (z, y, x)
// orientation, from the taps' box positions (all ones for a box).
std::vector<uint8_t> footprint_mask(const Plan& p) {
  const Geom3& g = p.tile.g;
  std::vector<uint8_t> mask((size_t)g.kd * g.kh * g.kw, 0);
  for (int i = 0; i < p.r.count; ++i) {
    const int* bt = &p.box_taps[(size_t)i * 3];
    mask[((size_t)bt[0] * g.kh + bt[1]) * g.kw + bt[2]] = 1;
  }
  return mask;
}

// Run lists for footprint windows and for every window deeper than one
// plane (a 3-D box is walked as a footprint); none for 1-D/2-D boxes.
Runs runs_of(const Plan& p) {
  const Geom3& g = p.tile.g;
  if (p.footprint.empty() && g.kd == 1) return Runs{};
  if ((long long)g.kd * g.kh * g.kw > (1ll << 24)) return Runs{};  // too large to list
  return count_runs(footprint_mask(p), g.kd, g.kh, g.kw);
}

}  // namespace

bool histogram_supported(const Plan& p) {
  if (p.ndim > 3 || p.r.count < 1) return false;
  const int k = p.r.kind;
  if (k != kMedian && k != kMedianNetwork && k != kMedianHistogram && k != kRank &&
      k != kRankHistogram && k != kMin && k != kMax && k != kPercentile)
    return false;
  HistChoice c = choose_tile(p.tile.g, p.dtype == 0 ? 4 : 8, runs_of(p));
  return c.TW > 0;
}

void histogram_configure(Plan& p, int tw, int th) {
  const Runs runs = runs_of(p);
  HistChoice c = choose_tile(p.tile.g, p.dtype == 0 ? 4 : 8, runs, tw, th);
  p.hist_block_w = c.TW;
  p.hist_block_h = c.TH;
  p.hist_sdec = c.sdec;
  p.hist_footprint = runs.footprint;
  p.hist_nf = runs.nf;
  p.hist_nv = runs.nv;
  p.hist_nh = runs.nh;
  p.hist_lists.clear();
  if (runs.footprint && c.TW > 0) {
    // Support-linear offsets (zz * plane + y * SW + x) of the taps and of
    // the run ends; below the support size, so they fit 16 bits.
    const Geom3& g = p.tile.g;
    const int SW = c.TW + g.kw - 1;
    const int plane = SW * (c.TH + g.kh - 1);
    const std::vector<uint8_t> mask = footprint_mask(p);
    auto at = [&](int zz, int y, int x) {
      return y >= 0 && y < g.kh && x >= 0 && x < g.kw && mask[((size_t)zz * g.kh + y) * g.kw + x] != 0;
    };
    std::vector<uint16_t> taps, top, bottom, left, right;
    for (int zz = 0; zz < g.kd; ++zz)
      for (int y = 0; y < g.kh; ++y)
        for (int x = 0; x < g.kw; ++x) {
          if (!at(zz, y, x)) continue;
          const uint16_t off = (uint16_t)(zz * plane + y * SW + x);
          taps.push_back(off);
          if (!at(zz, y - 1, x)) top.push_back(off);
          if (!at(zz, y + 1, x)) bottom.push_back(off);
          if (!at(zz, y, x - 1)) left.push_back(off);
          if (!at(zz, y, x + 1)) right.push_back(off);
        }
    // A step removes one list and adds the other; the pairing of entries
    // does not matter, only that both lists of an axis have one entry per run.
    p.hist_lists = taps;
    p.hist_lists.insert(p.hist_lists.end(), top.begin(), top.end());
    p.hist_lists.insert(p.hist_lists.end(), bottom.begin(), bottom.end());
    p.hist_lists.insert(p.hist_lists.end(), left.begin(), left.end());
    p.hist_lists.insert(p.hist_lists.end(), right.begin(), right.end());
  }
  HistArgs a = make_args(p);
  p.hist_blocks_x = a.tiles_x;
  p.hist_blocks_y = a.tiles / a.tiles_x;
}

size_t histogram_smem(const Plan& p) {
  HistArgs a = make_args(p);
  return smem_bytes_for(a.S, p.hist_sdec, p.dtype == 0 ? 4 : 8, (int)p.hist_lists.size());
}

// Scratch slots for the block sort: one per resident block (occupancy x
// SMs), capped by the number of tiles.
cudaError_t histogram_allocate(Plan& p) {
  HistArgs a = make_args(p);
  void* kernel = p.dtype == 0 ? kernel_for<float>(p.hist_sdec, p.hist_footprint)
                              : kernel_for<double>(p.hist_sdec, p.hist_footprint);
  cudaError_t e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  if (p.hist_footprint) {
    e = cudaMalloc(&p.d_hist_lists, p.hist_lists.size() * sizeof(uint16_t));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(p.d_hist_lists, p.hist_lists.data(), p.hist_lists.size() * sizeof(uint16_t),
                   cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kHThreads, p.smem_bytes);
  if (e != cudaSuccess) return e;
  long long slots = std::min<long long>(a.tiles, (long long)std::max(per_sm, 1) * p.sm_count);
  p.scratch_bytes = (size_t)slots * (size_t)a.slot_bytes;
  return cudaMalloc(&p.d_scratch, p.scratch_bytes);
}

namespace {

int hist_family_variant(const Plan& p) {
  if (p.algo != Algo::kHistogram || p.dtype != 0) return -1;
  return (p.hist_sdec ? 1 : 0) + (p.hist_footprint ? 2 : 0);
}

long long hist_family_tiles(const Plan& p) { return make_args(p).tiles; }

long long hist_family_slot_bytes(const Plan& p) { return make_args(p).slot_bytes; }

void hist_family_write_task(const Plan& p, const void* in, void* out, long long first_tile, void* task) {
  HistTask t{};
  t.in = (const float*)in;
  t.out = (float*)out;
  t.first_tile = first_tile;
  t.a = make_args(p);
  std::memcpy(task, &t, sizeof(t));
}

const void* hist_family_kernel(int v) {
  switch (v) {
    case 0: return (const void*)histogram_family_kernel<false, false>;
    case 1: return (const void*)histogram_family_kernel<true, false>;
    case 2: return (const void*)histogram_family_kernel<false, true>;
    default: return (const void*)histogram_family_kernel<true, true>;
  }
}

cudaError_t hist_family_launch(int v, const void* d_tasks, int ntasks, long long tiles, unsigned char* scratch,
                               long long slot_bytes, size_t smem, int grid, cudaStream_t s) {
  void* args[] = {(void*)&d_tasks, &ntasks, &tiles, &scratch, &slot_bytes};
  return cudaLaunchKernel(hist_family_kernel(v), dim3(grid), dim3(kHThreads), args, smem, s);
}

}  // namespace

const FamilyOps& histogram_family_ops() {
  static const FamilyOps ops{sizeof(HistTask), hist_family_variant, hist_family_tiles, hist_family_slot_bytes,
                             hist_family_write_task, hist_family_kernel, hist_family_launch};
  return ops;
}

cudaError_t launch_histogram(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0) return launch_t<float>(p, (const float*)in, (float*)out, s);
  return launch_t<double>(p, (const double*)in, (double*)out, s);
}


// ---------------------------------------------------------------------------
// Allocation-free variant of the histogram kernel.
//
// Some callers cannot let a library allocate device memory: code that runs
// while a CUDA stream is being captured (cudaMalloc is not allowed there),
// frameworks that own all device memory through their own pool, and real-time
// pipelines where an allocation's implicit device synchronization is not
// acceptable. For them, ndf_histogram_filter_noalloc takes the caller's
// device input and output and keeps its only scratch (the per-block sort
// slots) in the file-scope array below, so it never calls cudaMalloc,
// cudaFree or any allocating routine.
//
// Limits and sharing:
//  * the array holds kNoAllocScratchBytes (16 MiB) on every GPU that loads
//    the library, until the process exits;
//  * the number of concurrently working thread blocks is the number of sort
//    slots that fit in it (a slot is 2 x S keys + 2 x S u32 payloads for a
//    support of S samples), capped by the device's resident capacity; a
//    support whose slot does not fit is rejected with NDF_ERR_MEMORY;
//  * every call shares the array and it keeps the last call's contents; the
//    kernel writes every slot word before reading it, so nothing needs
//    clearing; calls that overlap on the GPU (other streams, other host
//    threads) race on it and must be serialized by the caller;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture;
//  * the address is kept for the life of the process: do not use the entry
//    point on a device after cudaDeviceReset (or another teardown of its
//    primary context), which can move the array.

constexpr size_t kNoAllocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;

struct NoAllocDevices {
  std::mutex lock;
  void* address[kMaxDevices] = {};
};

NoAllocDevices& noalloc_devices() {
  static NoAllocDevices d;
  return d;
}

// Device address of g_noalloc_scratch on the current device (set-up once
// per device, with that device current).
cudaError_t noalloc_scratch(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  NoAllocDevices& d = noalloc_devices();
  std::lock_guard<std::mutex> guard(d.lock);
  if (!d.address[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    d.address[device] = ptr;
  }
  *out = d.address[device];
  return cudaSuccess;
}

int noalloc_fail(int code, const char* message) {
  return fail(code, message);
}

// a * b into *out; false when the product does not fit in 64 bits.
bool mul_fits(unsigned long long a, unsigned long long b, unsigned long long* out) {
  if (a != 0 && b > ~0ull / a) return false;
  *out = a * b;
  return true;
}

}  // namespace
}  // namespace ndf

extern "C" int ndf_histogram_filter_noalloc(const void* d_in, void* d_out, int32_t dtype, int32_t ndim,
                                            const uint64_t* shape, const uint64_t* size,
                                            const int64_t* origin, const int32_t* modes, double cval,
                                            int32_t kind, int32_t omit_nan, int32_t ignore_inf,
                                            uint64_t min_count, uint64_t parameter, double percentile,
                                            void* stream) {
  using namespace ndf;
  if (dtype != NDF_FLOAT32 && dtype != NDF_FLOAT64)
    return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION, "array dtype must be float32 or float64");
  if (ndim < 1 || ndim > 2)
    return noalloc_fail(NDF_ERR_UNSUPPORTED, "the allocation-free histogram filter takes 1-D or 2-D arrays");
  if (!shape || !size || !origin || !modes)
    return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION, "missing shape, size, origin or mode");
  if (kind != kMedian && kind != kMedianNetwork && kind != kMedianHistogram && kind != kRank &&
      kind != kRankHistogram && kind != kMin && kind != kMax && kind != kPercentile)
    return noalloc_fail(NDF_ERR_UNSUPPORTED, "the allocation-free histogram filter computes order statistics");
  long long shp[2] = {1, 1}, sz[2] = {1, 1}, org[2] = {0, 0};
  int md[2] = {kNearest, kNearest};
  const int pad = 2 - ndim;
  unsigned long long volume = 1, n_out = 1;
  for (int a = 0; a < ndim; ++a) {
    if (modes[a] < 0 || modes[a] > 4) return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION, "unsupported boundary mode");
    if (size[a] == 0) return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION, "window sizes must be positive");
    if (size[a] > 65534 || shape[a] > (1ull << 40))
      return noalloc_fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
    const long long length = (long long)size[a];
    if (origin[a] < -(length / 2) || origin[a] > (length - 1) / 2)
      return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION,
                          "origin must satisfy -(size // 2) <= origin <= (size - 1) // 2");
    shp[a + pad] = (long long)shape[a];
    sz[a + pad] = length;
    org[a + pad] = origin[a];
    md[a + pad] = modes[a];
    if (!mul_fits(volume, size[a], &volume) || !mul_fits(n_out, shape[a], &n_out))
      return noalloc_fail(NDF_ERR_OVERFLOW, "shape or index arithmetic overflowed");
  }
  if (omit_nan && (min_count == 0 || min_count > volume))
    return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION,
                        "min_count must be between 1 and the number of window elements");
  if (kind == kPercentile && (!std::isfinite(percentile) || percentile < 0.0 || percentile > 100.0))
    return noalloc_fail(NDF_ERR_INVALID_CONFIGURATION, "percentile must be finite and between zero and 100");
  if (n_out == 0) return NDF_OK;
  if (!d_in || !d_out) return noalloc_fail(NDF_ERR_LENGTH_MISMATCH, "missing input or output buffer");
  Geom3 g{};
  g.D = 1;
  g.H = shp[0];
  g.W = shp[1];
  g.kd = 1;
  g.kh = (int)sz[0];
  g.kw = (int)sz[1];
  g.az = 0;
  g.ay = (int)(sz[0] / 2 + org[0]);
  g.ax = (int)(sz[1] / 2 + org[1]);
  g.mz = kNearest;
  g.my = md[0];
  g.mx = md[1];
  Reduce r{};
  r.kind = kind;
  r.omit = omit_nan != 0;
  r.drop_inf = r.omit && ignore_inf != 0;
  r.count = (int)std::min<unsigned long long>(volume, 1ull << 30);
  r.min_count = r.omit ? (long long)min_count : 1;
  r.param = (long long)std::min<uint64_t>(parameter, (uint64_t)(1ull << 62));
  r.q = percentile;
  r.q_fraction = percentile / 100.0;
  r.q_is_max = percentile == 100.0;
  r.pct = nullptr;
  r.cval = dtype == NDF_FLOAT32 ? (double)(float)cval : cval;
  HistChoice c = choose_tile(g, dtype == 0 ? 4 : 8);
  if (c.TW == 0) return noalloc_fail(NDF_ERR_UNSUPPORTED, "window too large for the histogram kernel");
  HistArgs a = make_args_core(g, c.TW, c.TH, dtype, r);
  if ((size_t)a.slot_bytes > kNoAllocScratchBytes)
    return noalloc_fail(NDF_ERR_MEMORY,
                        "the window's sort slot exceeds the 16 MiB allocation-free scratch");
  int device = 0, sm_count = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return noalloc_fail(NDF_ERR_NO_DEVICE, "no usable CUDA device");
  }
  const size_t smem = smem_bytes_for(a.S, c.sdec, dtype == 0 ? 4 : 8, 0);
  if (smem > (size_t)optin) return noalloc_fail(NDF_ERR_UNSUPPORTED, "window too large for shared memory");
  void* scratch = nullptr;
  e = noalloc_scratch(device, &scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  const void* kernel = dtype == 0 ? kernel_for<float>(c.sdec) : kernel_for<double>(c.sdec);
  e = allow_max_smem(kernel);
  int per_sm = 1;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kHThreads, smem);
  if (e != cudaSuccess) return cuda_fail(e, "histogram (allocation-free) set-up");
  long long slots = (long long)(kNoAllocScratchBytes / (size_t)a.slot_bytes);
  long long grid = std::min<long long>(std::min<long long>(a.tiles, slots),
                                       (long long)std::max(per_sm, 1) * sm_count);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == 0) {
    if (c.sdec)
      histogram_kernel<float, true, false><<<(unsigned)grid, kHThreads, smem, s>>>(
          (const float*)d_in, (float*)d_out, a, (unsigned char*)scratch);
    else
      histogram_kernel<float, false, false><<<(unsigned)grid, kHThreads, smem, s>>>(
          (const float*)d_in, (float*)d_out, a, (unsigned char*)scratch);
  } else {
    if (c.sdec)
      histogram_kernel<double, true, false><<<(unsigned)grid, kHThreads, smem, s>>>(
          (const double*)d_in, (double*)d_out, a, (unsigned char*)scratch);
    else
      histogram_kernel<double, false, false><<<(unsigned)grid, kHThreads, smem, s>>>(
          (const double*)d_in, (double*)d_out, a, (unsigned char*)scratch);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "histogram (allocation-free)");
  return NDF_OK;
}

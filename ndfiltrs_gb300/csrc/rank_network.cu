// Ranked register networks (float32): order statistics over windows of 33 to
// 128 taps (footprints such as rings, 3-D boxes, boxes beyond the box-pair
// kernel), two windows per thread.
//
// The register network of tile_network_kernel (network.cuh) spends almost all
// of its time on 32-bit min / max pairs, one ALU-pipe instruction per key per
// comparator. Here a tile of 64 x TH outputs first ranks its staged support:
// the retained keys are compacted in support order and sorted by a block LSD
// radix sort in shared memory (8-bit digits, only over the bits on which the
// retained keys differ; stable, so equal keys keep their support order: lanes
// with equal digits are found by ballots), and
// every retained sample gets a 16-bit code, its position in that order, while
// dropped samples get 0xFFFF. The codes of outputs x and x + 32 of a tile row
// are packed into one 32-bit word, and the Batcher network runs on the packed
// words with min.u16x2 / max.u16x2: one instruction per comparator for both
// windows. The selected codes index the sorted keys. Equal keys are
// interchangeable, so the result equals direct selection bit for bit (the
// reference ranks a block's support the same way for its histogram,
// src/histogram.rs:302-486; the statistic is Reduction::finish,
// src/reduction.rs:78-130).
#include <algorithm>
#include <cstring>
#include <utility>

#include "network.cuh"
#include "plan.h"
#include "staging.cuh"
#include "tma.cuh"

namespace ndf {
namespace {

using namespace net;

constexpr int kRThreads = 256;
constexpr int kRWarps = kRThreads / 32;
constexpr int kRankTW = 64;  // outputs per tile row: pairs (x, x + 32)
constexpr uint16_t kDrop = 0xFFFF;
constexpr int kMaxRankSupport = 65534;

// Radix digits of the ranking sort: kDigitBits per pass; with more than 8
// bits two 16-bit counters share a word (a support has at most 65,534
// samples, so no count or offset reaches 2^16).
constexpr int kDigitBits = 8;
constexpr unsigned int kDigits = 1u << kDigitBits;
constexpr bool kPacked = kDigitBits > 8;
constexpr int kTableWords = kPacked ? (int)kDigits / 2 : (int)kDigits;  // per warp
constexpr int kPerThread = (int)kDigits / kRThreads;

__device__ __forceinline__ unsigned int word_of(unsigned int d) { return kPacked ? d >> 1 : d; }
__device__ __forceinline__ unsigned int half_of(unsigned int d) { return kPacked ? (d & 1u) * 16u : 0u; }
__device__ __forceinline__ unsigned int counter(const unsigned int* row, unsigned int d) {
  return kPacked ? (row[d >> 1] >> ((d & 1u) * 16u)) & 0xFFFFu : row[d];
}

// The lanes of `active` whose digit equals this lane's, from one ballot per
// digit bit (cheaper here than the match instruction).
__device__ __forceinline__ unsigned int same_digit(unsigned int active, unsigned int dg) {
  unsigned int peers = active;
#pragma unroll
  for (int b = 0; b < kDigitBits; ++b) {
    const bool set = (dg >> b) & 1u;
    const unsigned int bal = __ballot_sync(active, set);
    peers &= set ? bal : ~bal;
  }
  return peers;
}

// Two 16-bit codes; the comparator orders both halves at once.
struct Pair16 {
  uint32_t v;
};

__device__ __forceinline__ void cmpx(Pair16& a, Pair16& b) {
  uint32_t lo, hi;
  asm("min.u16x2 %0, %1, %2;" : "=r"(lo) : "r"(a.v), "r"(b.v));
  asm("max.u16x2 %0, %1, %2;" : "=r"(hi) : "r"(a.v), "r"(b.v));
  a.v = lo;
  b.v = hi;
}

// The Batcher network over N wires on packed codes. With a fixed tap count
// VF the wires from VF up hold the dropped code (all ones) throughout: every
// comparator whose upper wire is among them leaves both wires unchanged and
// is left out here (the inline min / max are opaque to the compiler's
// constant folding).
template <int N, int VF, int I>
__device__ __forceinline__ void cmpx_fixed(Pair16 (&a)[N]) {
  constexpr int lo = Batcher<N, 1>::kTable.lo[I];
  constexpr int hi = Batcher<N, 1>::kTable.hi[I];
  if constexpr (VF == 0 || hi < VF) cmpx(a[lo], a[hi]);
}

template <int N, int VF, int... Is>
__device__ __forceinline__ void sort_pairs(Pair16 (&a)[N], std::integer_sequence<int, Is...>) {
  (cmpx_fixed<N, VF, Is>(a), ...);
}

// Shared-memory layout of a tile (byte offsets from the 16-byte aligned
// base): remap tables | staged keys S x 4 | second key buffer S x 4 | index
// buffers 2 x S x 2 | codes S x 2 | radix counters. After the sort the
// sorted keys are in the first key buffer, and the second key buffer and the
// index buffers (contiguous, 8 S bytes) hold the packed code pairs with their
// retained flags. A TMA staging area overlays everything after the staged
// keys (unused until the staged keys are copied out of it).
struct RankLayout {
  size_t s, kb, ia, codes, table, total;
};

__host__ __device__ inline RankLayout rank_layout(const Tile& t, int kd) {
  RankLayout l;
  const size_t S = (size_t)kd * t.SH * t.SW;
  l.s = (((size_t)(t.SW + t.SH + kd) * 8) + 15) & ~(size_t)15;
  l.kb = (l.s + S * 4 + 15) & ~(size_t)15;
  l.ia = (l.kb + S * 4 + 15) & ~(size_t)15;
  l.codes = (l.ia + S * 4 + 15) & ~(size_t)15;
  l.table = (l.codes + S * 2 + 15) & ~(size_t)15;
  l.total = l.table + (size_t)kRWarps * kTableWords * 4;
  return l;
}

// Rank the staged keys s[0, S) (dropped samples keyed 0xFFFFFFFF). Returns
// the retained count R; codes[e] is sample e's position among the retained
// keys in sorted order, or kDrop; the R sorted keys end in s (*sorted). kb
// is a second key buffer, ia and ib S-entry index buffers, table kRWarps x
// kTableWords counters.
__device__ int rank_support(uint32_t* s, uint32_t* kb, uint16_t* ia, uint16_t* ib, uint16_t* codes,
                            unsigned int* table, int S, const uint32_t** sorted) {
  __shared__ unsigned int warp_n[kRWarps];
  __shared__ uint32_t red_and[kRWarps], red_or[kRWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned int below = (1u << lane) - 1u;

  // Compaction in support order: warp w takes positions [w C, (w + 1) C).
  const int C = (S + kRWarps * 32 - 1) / (kRWarps * 32) * 32;
  const int begin = warp * C, end = min(S, begin + C);
  unsigned int n = 0;
  uint32_t kand = 0xFFFFFFFFu, kor = 0u;
  for (int base = begin; base < end; base += 32) {
    const int e = base + lane;
    const uint32_t key = e < end ? s[e] : 0xFFFFFFFFu;
    const bool keep = key != 0xFFFFFFFFu;
    n += __popc(__ballot_sync(0xffffffffu, keep));
    if (keep) {
      kand &= key;
      kor |= key;
    }
  }
  for (int o = 16; o >= 1; o >>= 1) {
    kand &= __shfl_xor_sync(0xffffffffu, kand, o);
    kor |= __shfl_xor_sync(0xffffffffu, kor, o);
  }
  if (lane == 0) {
    warp_n[warp] = n;
    red_and[warp] = kand;
    red_or[warp] = kor;
  }
  __syncthreads();
  unsigned int off = 0, R = 0;
  kand = 0xFFFFFFFFu;
  kor = 0u;
  for (int w = 0; w < kRWarps; ++w) {
    if (w < warp) off += warp_n[w];
    R += warp_n[w];
    kand &= red_and[w];
    kor |= red_or[w];
  }
  for (int base = begin; base < end; base += 32) {
    const int e = base + lane;
    const uint32_t key = e < end ? s[e] : 0xFFFFFFFFu;
    const bool keep = key != 0xFFFFFFFFu;
    const unsigned int b = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const unsigned int pos = off + __popc(b & below);
      kb[pos] = key;
      ib[pos] = (uint16_t)e;
    } else if (e < end) {
      codes[e] = kDrop;
    }
    off += __popc(b);
  }
  __syncthreads();

  // LSD passes over the bits on which the retained keys differ.
  uint32_t* src_k = kb;
  uint16_t* src_i = ib;
  uint32_t* dst_k = s;
  uint16_t* dst_i = ia;
  const uint32_t varying = kand ^ kor;
  if (R > 1 && varying != 0u) {
    const int lo = __ffs((int)varying) - 1;
    const int hi = 31 - __clz((int)varying);
    const int C2 = ((int)R + kRWarps * 32 - 1) / (kRWarps * 32) * 32;
    const int b2 = warp * C2, e2 = min((int)R, b2 + C2);
    unsigned int* mine = table + warp * kTableWords;
    for (int shift = lo; shift <= hi; shift += kDigitBits) {
      for (int w = lane; w < kTableWords; w += 32) mine[w] = 0u;
      __syncwarp();
      for (int base = b2; base < e2; base += 32) {
        const int e = base + lane;
        if (e < e2) {
          const unsigned int dg = (src_k[e] >> shift) & (kDigits - 1u);
          atomicAdd(&mine[word_of(dg)], 1u << half_of(dg));
        }
      }
      __syncthreads();
      // Exclusive offsets in (digit, warp) order; thread t owns digits
      // [t kPerThread, (t + 1) kPerThread), in pairs when counters are packed.
      {
        const int d0 = threadIdx.x * kPerThread;
        unsigned int col[kPerThread];
        unsigned int total = 0;
#pragma unroll
        for (int j = 0; j < kPerThread; ++j) {
          col[j] = 0;
          for (int w = 0; w < kRWarps; ++w) col[j] += counter(table + w * kTableWords, d0 + j);
          total += col[j];
        }
        unsigned int incl = total;
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (lane == 31) warp_n[warp] = incl;
        __syncthreads();
        unsigned int run = incl - total;
        for (int w = 0; w < warp; ++w) run += warp_n[w];
        unsigned int first[kPerThread];
#pragma unroll
        for (int j = 0; j < kPerThread; ++j) {
          first[j] = run;
          run += col[j];
        }
        for (int w = 0; w < kRWarps; ++w) {
          unsigned int* row = table + w * kTableWords;
          unsigned int next[kPerThread];
#pragma unroll
          for (int j = 0; j < kPerThread; ++j) next[j] = first[j] + counter(row, d0 + j);
#pragma unroll
          for (int j = 0; j < kPerThread; j += (kPacked ? 2 : 1)) {
            if constexpr (kPacked)
              row[(d0 + j) >> 1] = first[j] | (first[j + 1] << 16);
            else
              row[d0 + j] = first[j];
          }
#pragma unroll
          for (int j = 0; j < kPerThread; ++j) first[j] = next[j];
        }
      }
      __syncthreads();
      // Stable scatter: each warp walks its segment in order, 32 keys at a
      // time; equal digits within a group keep their lane order.
      for (int base = b2; base < e2; base += 32) {
        const int e = base + lane;
        const bool in = e < e2;
        const unsigned int active = __ballot_sync(0xffffffffu, in);
        if (in) {
          const uint32_t key = src_k[e];
          const unsigned int dg = (key >> shift) & (kDigits - 1u);
          const unsigned int peers = same_digit(active, dg);
          const unsigned int pos = counter(mine, dg) + __popc(peers & below);
          dst_k[pos] = key;
          dst_i[pos] = src_i[e];
          __syncwarp(active);
          // Atomic: with packed counters two digits of the group can share a word.
          if (lane == 31 - __clz((int)peers)) atomicAdd(&mine[word_of(dg)], (unsigned int)__popc(peers) << half_of(dg));
        }
        __syncwarp();
      }
      __syncthreads();
      uint32_t* tk = src_k;
      src_k = dst_k;
      dst_k = tk;
      uint16_t* ti = src_i;
      src_i = dst_i;
      dst_i = ti;
    }
  }
  // Codes of the retained samples; the sorted keys end in s.
  const bool move = src_k != s;
  for (int p = threadIdx.x; p < (int)R; p += blockDim.x) {
    codes[src_i[p]] = (uint16_t)p;
    if (move) s[p] = src_k[p];
  }
  __syncthreads();
  *sorted = s;
  return (int)R;
}

// The statistic of one half (H = 0: output x, H = 1: output x + 32) of the
// sorted packed codes, nv retained samples; as network_finish.
template <int N, int VFIX, int MODE, int H>
__device__ __forceinline__ float finish_half(const Pair16 (&k)[N], int nv, const Reduce& r,
                                             const uint32_t* __restrict__ sorted) {
  using KO = KeyOf<float>;
  auto val = [&](Pair16 p) -> float { return KO::value(sorted[H == 0 ? (p.v & 0xFFFFu) : (p.v >> 16)]); };
  const int V = VFIX > 0 ? VFIX : r.count;
  const bool missing = r.omit ? (nv < r.min_count) : (nv != V);
  if (missing || nv == 0) return nan_of(0.0f);
  if (MODE == 1) {
    if (VFIX > 0 && !r.omit) {
      if (VFIX & 1) return val(k[VFIX / 2]);
      return median_of_two(val(k[VFIX / 2 - 1]), val(k[VFIX / 2]));
    }
    if constexpr (VFIX >= 9) {
      // With at most 4 dropped samples the middle ranks lie in [L, VFIX / 2].
      constexpr int L = (VFIX - 5) / 2;
      if (nv >= VFIX - 4) {
        const int lo = (nv - 1) / 2 - L, hi = nv / 2 - L;
        const Pair16 a_hi = pick<VFIX / 2 - L + 1>(*reinterpret_cast<const Pair16(*)[VFIX / 2 - L + 1]>(&k[L]), hi);
        if (nv & 1) return val(a_hi);
        const Pair16 a_lo = pick<VFIX / 2 - L + 1>(*reinterpret_cast<const Pair16(*)[VFIX / 2 - L + 1]>(&k[L]), lo);
        return median_of_two(val(a_lo), val(a_hi));
      }
    }
    constexpr int B = (VFIX > 0 ? VFIX : N) / 2 + 1;
    if (nv & 1) return val(pick<B>(k, nv / 2));
    return median_of_two(val(pick<B>(k, nv / 2 - 1)), val(pick<B>(k, nv / 2)));
  }
  constexpr int A = (VFIX > 0 && VFIX < N) ? VFIX : N;
  switch (r.kind) {
    case kMin:
      return val(k[0]);
    case kMax:
      return val(pick<A>(k, nv - 1));
    case kRank:
    case kRankHistogram:
      if (r.param >= nv) return nan_of(0.0f);
      return val(pick<A>(k, (int)r.param));
    case kPercentile: {
      if (r.q_is_max) return val(pick<A>(k, nv - 1));
      const PctSplit ps = pct_split(r, nv);
      return pct_value<float>(ps, val(pick<A>(k, ps.lower)), val(pick<A>(k, ps.upper)));
    }
    default:
      if (nv & 1) return val(pick<A>(k, nv / 2));
      return median_of_two(val(pick<A>(k, nv / 2 - 1)), val(pick<A>(k, nv / 2)));
  }
}

// Resident blocks per SM the register allocation must allow: three for the
// median networks up to 80 wires (at most 80 registers; ring(4, 6) needs
// 77), two for the general selections (whose run-time picks spill
// kilobytes at 80 registers) and 96 wires, else one.
template <int N, int MODE>
constexpr int rank_min_blocks() {
  return (N <= 80 && MODE == 1) ? 3 : (N <= 96 ? 2 : 1);
}

// One output tile (index `tile`) of the ranked network kernel; off(i) is tap
// i's offset in the staged support (a kernel parameter, which the compiler
// uses as a constant operand, or a volatile read of shared memory so that
// the offsets are read where they are used instead of being held in
// registers), `tmap` the launch's tensor map (nullptr: remapped staging only).
template <int N, int VFIX, int MODE, typename Off>
__device__ __forceinline__ void rank_network_body(const float* __restrict__ in, float* __restrict__ out,
                                                  const TileArgs& a, Off off, long long tile,
                                                  unsigned char* smem_raw, const CUtensorMap* tmap) {
  const Geom3& g = a.g;
  const Tile& t = a.t;
  const RankLayout L = rank_layout(t, g.kd);
  long long* maps = reinterpret_cast<long long*>(smem_raw);
  uint32_t* s = reinterpret_cast<uint32_t*>(smem_raw + L.s);
  uint32_t* kb = reinterpret_cast<uint32_t*>(smem_raw + L.kb);
  const int S = g.kd * t.SH * t.SW;
  uint16_t* ia = reinterpret_cast<uint16_t*>(smem_raw + L.ia);
  uint16_t* ib = ia + S;
  uint16_t* codes = reinterpret_cast<uint16_t*>(smem_raw + L.codes);
  unsigned int* table = reinterpret_cast<unsigned int*>(smem_raw + L.table);
  long long z, y0, x0;
  tile_coords(a, tile, z, y0, x0);
  const bool drop_inf = a.r.drop_inf;
  const uint32_t outside = sample_key<float>((float)a.r.cval, drop_inf);
  if (!stage_tile(s, maps, smem_raw, in, a, tmap, z, y0, x0, outside,
                  [&](float v) { return sample_key<float>(v, drop_inf); }))
    return;
  __syncthreads();
  const uint32_t* sorted = nullptr;
  rank_support(s, kb, ia, ib, codes, table, S, &sorted);
  // Per support position j: the packed codes of (j, j + 32) and their
  // retained flags, one 8-byte entry over the free key and index buffers.
  uint2* pv = reinterpret_cast<uint2*>(smem_raw + L.kb);
  for (int j = threadIdx.x; j < S; j += blockDim.x) {
    const uint32_t c0 = codes[j], c1 = j + 32 < S ? codes[j + 32] : kDrop;
    pv[j] = make_uint2(c0 | (c1 << 16), (c0 != kDrop ? 1u : 0u) | (c1 != kDrop ? 0x10000u : 0u));
  }
  __syncthreads();
  const int V = VFIX > 0 ? VFIX : a.r.count;
  for (int p = threadIdx.x; p < 32 * t.TH; p += blockDim.x) {
    const int ty = p >> 5, tx = p & 31;
    const long long y = y0 + ty, x = x0 + tx;
    if (y >= g.H || x >= g.W) continue;
    const int base = ty * t.SW + tx;
    Pair16 k[N];
    uint32_t cnt = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (i < V) {
        const uint2 e = pv[base + off(i)];
        k[i].v = e.x;
        cnt += e.y;
      } else {
        k[i].v = 0xFFFFFFFFu;
      }
    }
    sort_pairs<N, VFIX>(k, std::make_integer_sequence<int, Batcher<N, 1>::kCount>{});
    float* row = out + (z * g.H + y) * g.W;
    row[x] = canonical(finish_half<N, VFIX, MODE, 0>(k, (int)(cnt & 0xFFFFu), a.r, sorted));
    if (x + 32 < g.W) row[x + 32] = canonical(finish_half<N, VFIX, MODE, 1>(k, (int)(cnt >> 16), a.r, sorted));
  }
}

template <int N, int VFIX, int MODE>
__global__ void __launch_bounds__(kRThreads, rank_min_blocks<N, MODE>())
    rank_network_kernel(const float* __restrict__ in, float* __restrict__ out, const __grid_constant__ TileArgs a,
                        const __grid_constant__ TapTable<N> taps, const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  rank_network_body<N, VFIX, MODE>(in, out, a, [&](int i) { return taps.off[i]; }, blockIdx.x, smem_raw, &tmap);
}

// Batched float32 images: one persistent launch per (width, tap count,
// mode) over the concatenated tile lists; a block finds a tile's image by
// binary search over the images' first tiles and keeps its arguments and
// tap offsets in shared memory until the image changes. Staging is the
// remapped path.
struct RankTask {
  const float* in;
  float* out;
  long long first_tile;
  TileArgs a;
  int32_t off[kMaxNetwork32];
};

// The family kernels read the tap offsets from shared memory; with a
// run-time tap count the 80-wire median then spills about 600 bytes at the
// three-block cap, so only its fixed-count form keeps three blocks.
template <int N, int VFIX, int MODE>
__global__ void __launch_bounds__(kRThreads, (N <= 80 && MODE == 1 && VFIX > 0) ? 3 : (N <= 96 ? 2 : 1))
    rank_family_kernel(const RankTask* __restrict__ tasks, int ntasks, long long total_tiles) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ RankTask task;
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
      for (int i = threadIdx.x; i < (int)(sizeof(RankTask) / 8); i += blockDim.x) dst[i] = src[i];
      __syncthreads();
      if (threadIdx.x == 0) current = index;
    }
    __syncthreads();
    const volatile int32_t* off = task.off;
    rank_network_body<N, VFIX, MODE>(task.in, task.out, task.a, [off](int i) { return (int)off[i]; },
                                     tile - task.first_tile, smem_raw, nullptr);
    __syncthreads();
  }
}

template <int N, int VFIX, int MODE>
cudaError_t launch_rank(const Plan& p, const float* in, float* out, cudaStream_t s) {
  TapTable<N> taps{};
  const TileArgs& a = p.tile;
  for (int i = 0; i < N; ++i) {
    if (i < p.r.count) {
      const int* bt = &p.box_taps[(size_t)i * 3];
      taps.off[i] = (bt[0] * a.t.SH + bt[1]) * a.t.SW + bt[2];
    } else {
      taps.off[i] = 0;
    }
  }
  auto kernel = rank_network_kernel<N, VFIX, MODE>;
  cudaError_t e = allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  TileArgs args = a;
  CUtensorMap map{};
  // The TMA staging area overlays the buffers after the staged keys.
  size_t smem = rank_layout(a.t, a.g.kd).kb;
  if (tma_prepare(p, a.t, in, &map, &args, &smem))
    smem = std::max(smem, p.smem_bytes);
  else
    smem = p.smem_bytes;
  kernel<<<(unsigned)a.t.tiles, kRThreads, smem, s>>>(in, out, args, taps, map);
  return cudaGetLastError();
}

template <int N>
cudaError_t dispatch_rank(const Plan& p, const float* in, float* out, cudaStream_t s) {
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork || p.r.kind == kMedianHistogram;
  if (!median) return launch_rank<N, 0, 0>(p, in, out, s);
  if (N == 80 && p.r.count == 68) return launch_rank<80, 68, 1>(p, in, out, s);
  return launch_rank<N, 0, 1>(p, in, out, s);
}

}  // namespace

// Tile of the ranked network kernel: 64 x TH outputs, TH the largest of
// 64, 48, 32, 16, 8 whose shared memory still lets as many blocks reside on
// an SM as the kernel's registers do (rank_min_blocks), else the largest
// within the device limit: a taller tile ranks fewer support samples per
// output. False for float64, single-row arrays, 3-D windows (a tile would
// rank kd planes of support for one plane of outputs), widths below 48 or
// supports beyond 16-bit codes.
bool rank_network_configure(Plan& p, int smem_limit) {
  const Geom3& g = p.tile.g;
  const int width = network_width_for(p.dtype, p.r.count);
  if (p.dtype != 0 || width < 48 || g.H == 1 || g.kd > 1) return false;
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork || p.r.kind == kMedianHistogram;
  const int blocks = (width <= 80 && median) ? 3 : (width <= 96 ? 2 : 1);
  constexpr size_t kSmPerSm = 233472, kReserved = 1024;  // bytes per SM, reserved per block
  const size_t budget = std::min<size_t>(kSmPerSm / blocks - kReserved, (size_t)smem_limit);
  for (size_t limit : {budget, (size_t)smem_limit}) {
    for (int th : {64, 48, 32, 16, 8}) {
      Tile t = p.tile.t;
      t.TW = kRankTW;
      t.TH = th;
      t.SW = kRankTW + g.kw - 1;
      t.SH = th + g.kh - 1;
      t.tiles_x = (g.W + kRankTW - 1) / kRankTW;
      t.tiles_y = (g.H + th - 1) / th;
      t.tiles = t.tiles_x * t.tiles_y * g.D;
      if ((long long)g.kd * t.SH * t.SW > kMaxRankSupport) continue;
      const size_t bytes = rank_layout(t, g.kd).total;
      if (bytes > limit) continue;
      p.tile.t = t;
      p.smem_bytes = bytes;
      p.network = width;
      return true;
    }
  }
  return false;
}

cudaError_t launch_rank_network(const Plan& p, const void* in, void* out, cudaStream_t s) {
  const float* fin = (const float*)in;
  float* fout = (float*)out;
  switch (p.network) {
    case 48:
      return dispatch_rank<48>(p, fin, fout, s);
    case 64:
      return dispatch_rank<64>(p, fin, fout, s);
    case 80:
      return dispatch_rank<80>(p, fin, fout, s);
    case 96:
      return dispatch_rank<96>(p, fin, fout, s);
    case 112:
      return dispatch_rank<112>(p, fin, fout, s);
    case 128:
      return dispatch_rank<128>(p, fin, fout, s);
    default:
      return cudaErrorInvalidValue;
  }
}

namespace {

// Batch family variants: (width, fixed tap count, mode).
constexpr int kRankVariants[][3] = {{48, 0, 0},  {48, 0, 1},  {64, 0, 0},  {64, 0, 1},  {80, 0, 0},
                                    {80, 0, 1},  {80, 68, 1}, {96, 0, 0},  {96, 0, 1},  {112, 0, 0},
                                    {112, 0, 1}, {128, 0, 0}, {128, 0, 1}};
constexpr int kNumRankVariants = (int)(sizeof(kRankVariants) / sizeof(kRankVariants[0]));

int rank_family_variant(const Plan& p) {
  if (p.algo != Algo::kTileRank || p.dtype != 0) return -1;
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork || p.r.kind == kMedianHistogram;
  const int vfix = median && p.network == 80 && p.r.count == 68 ? 68 : 0;
  for (int v = 0; v < kNumRankVariants; ++v)
    if (kRankVariants[v][0] == p.network && kRankVariants[v][1] == vfix && kRankVariants[v][2] == (median ? 1 : 0))
      return v;
  return -1;
}

long long rank_family_tiles(const Plan& p) { return p.tile.t.tiles; }

long long rank_family_slot_bytes(const Plan&) { return 0; }

void rank_family_write_task(const Plan& p, const void* in, void* out, long long first_tile, void* task) {
  RankTask t{};
  t.in = (const float*)in;
  t.out = (float*)out;
  t.first_tile = first_tile;
  t.a = p.tile;
  t.a.r = p.r;
  t.a.tma_bw = 0;
  for (int i = 0; i < p.r.count && i < kMaxNetwork32; ++i) {
    const int* bt = &p.box_taps[(size_t)i * 3];
    t.off[i] = (bt[0] * p.tile.t.SH + bt[1]) * p.tile.t.SW + bt[2];
  }
  std::memcpy(task, &t, sizeof(t));
}

const void* rank_family_kernel_of(int variant) {
  switch (variant) {
    case 0: return (const void*)rank_family_kernel<48, 0, 0>;
    case 1: return (const void*)rank_family_kernel<48, 0, 1>;
    case 2: return (const void*)rank_family_kernel<64, 0, 0>;
    case 3: return (const void*)rank_family_kernel<64, 0, 1>;
    case 4: return (const void*)rank_family_kernel<80, 0, 0>;
    case 5: return (const void*)rank_family_kernel<80, 0, 1>;
    case 6: return (const void*)rank_family_kernel<80, 68, 1>;
    case 7: return (const void*)rank_family_kernel<96, 0, 0>;
    case 8: return (const void*)rank_family_kernel<96, 0, 1>;
    case 9: return (const void*)rank_family_kernel<112, 0, 0>;
    case 10: return (const void*)rank_family_kernel<112, 0, 1>;
    case 11: return (const void*)rank_family_kernel<128, 0, 0>;
    default: return (const void*)rank_family_kernel<128, 0, 1>;
  }
}

cudaError_t rank_family_launch(int variant, const void* d_tasks, int ntasks, long long tiles, unsigned char*, long long,
                               size_t smem, int grid, cudaStream_t s) {
  void* args[] = {(void*)&d_tasks, &ntasks, &tiles};
  return cudaLaunchKernel(rank_family_kernel_of(variant), dim3(grid), dim3(kRThreads), args, smem, s);
}

}  // namespace

const FamilyOps& rank_family_ops() {
  static const FamilyOps ops{sizeof(RankTask), rank_family_variant, rank_family_tiles, rank_family_slot_bytes,
                             rank_family_write_task, rank_family_kernel_of, rank_family_launch};
  return ops;
}

}  // namespace ndf

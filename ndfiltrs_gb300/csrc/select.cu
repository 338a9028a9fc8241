// Exact order statistics on the GPU: median (direct / sortnet), rank, min,
// max and percentile.
//
// * tile_network: the window's keys sit in registers and a Batcher
//   odd-even merge network sorts them (replaces Network::new/apply,
//   src/median_network.rs:116-209, and the per-output selection of
//   Reduction::finish, src/reduction.rs:78-130). The network width is a
//   compile-time constant (8, 16, 32, then multiples of 16); padding wires
//   hold the sentinel key, so the compiler folds their comparators away, and
//   comparators whose outputs no
//   rank of the reduction can reach are removed as dead code (the backward
//   liveness pruning of the reference's Network::new).
// * tile_radix: windows too wide for a register network run a bit-serial
//   radix select over the staged keys.
// * generic: arrays of rank > 3 (or supports that do not fit in shared
//   memory) gather every tap through the boundary maps from global memory.
//
// Dropped samples (NaN, and infinities under ignore_inf) take the sentinel
// key, the largest key, so a sorted window holds its `nv` retained samples
// first. Propagate windows are NaN when nv != V.
#include "network.cuh"
#include "select_launch.cuh"

namespace ndf {

cudaError_t launch_network_wide(const Plan& p, const void* in, void* out, cudaStream_t s);

namespace {
using namespace net;
using namespace netlaunch;

template <typename T>
__global__ void __launch_bounds__(kThreads)
    tile_radix_kernel(const T* __restrict__ in, T* __restrict__ out,
                      const __grid_constant__ TileArgs a, const int32_t* __restrict__ taps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tile_radix_body<T>(in, out, a, blockIdx.x, smem_raw, taps);
}

// ---------------------------------------------------------------------------
// Generic N-D gather: one thread per output, taps mapped per axis
// (Window::prepare / visit_mapped, src/window.rs:254-294).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    generic_select_kernel(const T* __restrict__ in, T* __restrict__ out,
                          const __grid_constant__ GenericArgs a,
                          const long long* __restrict__ taps) {
  using K = typename KeyOf<T>::K;
  const int rank = a.rank;
  const long long* flat = taps + (long long)a.r.count * rank;
  const bool drop_inf = a.r.drop_inf;
  const T cval = (T)a.r.cval;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < a.n_out;
       o += (long long)gridDim.x * blockDim.x) {
    long long coord[kMaxGenericRank];
    long long rem = o;
    bool interior = true;
    for (int d = 0; d < rank; ++d) {
      coord[d] = rem / a.stride[d];
      rem -= coord[d] * a.stride[d];
      interior = interior && coord[d] + a.low[d] >= 0 && coord[d] + a.high[d] < a.shape[d];
    }
    auto fetch = [&](int i) -> K {
      if (interior) return sample_key<T>(__ldg(in + o + flat[i]), drop_inf);
      const long long* tap = taps + (long long)i * rank;
      long long src = 0;
      for (int d = 0; d < rank; ++d) {
        long long m;
        if (!map_index(coord[d] + tap[d], a.shape[d], a.mode[d], &m))
          return sample_key<T>(cval, drop_inf);
        src += m * a.stride[d];
      }
      return sample_key<T>(__ldg(in + src), drop_inf);
    };
    out[o] = canonical(radix_finish<T, K>(fetch, a.r));
  }
}

// ---------------------------------------------------------------------------
// Host launchers.

template <typename T>
cudaError_t launch_tile_select_t(const Plan& p, const T* in, T* out, cudaStream_t s) {
  if (p.algo == Algo::kTileBox) return launch_tile_box(p, in, out, s);
  if (p.algo == Algo::kTileNetwork) {
    switch (p.network) {
      case 8:
        return dispatch_network_mode<T, 8>(p, in, out, s);
      case 16:
        return dispatch_network_mode<T, 16>(p, in, out, s);
      case 32:
        return dispatch_network_mode<T, 32>(p, in, out, s);
      case 48:
        return dispatch_network_mode<T, 48>(p, in, out, s);
      case 64:
        return dispatch_network_mode<T, 64>(p, in, out, s);
      default:
        // Widths 80 to 128 (float32 keys only).
        if constexpr (sizeof(T) == 4) return launch_network_wide(p, in, out, s);
        return cudaErrorInvalidValue;
    }
  }
  auto kernel = tile_radix_kernel<T>;
  cudaError_t e =
      allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  kernel<<<(unsigned)p.tile.t.tiles, kThreads, p.smem_bytes, s>>>(in, out, p.tile, p.d_tile_taps);
  return cudaGetLastError();
}

}  // namespace

// Network width for `count` taps: 8, 16 or 32, then multiples of 16 up to the
// key type's register limit. A width that is not a power of two is the
// power-of-two network with its top wires removed (they would hold the
// sentinel, so their comparators are no-ops), e.g. 849 comparators for 80
// wires against 1471 for 128.
int network_width_for(int dtype, int count) {
  int limit = dtype == 0 ? kMaxNetwork32 : kMaxNetwork64;
  if (count > limit) return 0;
  if (count <= 32) {
    int n = 8;
    while (n < count) n <<= 1;
    return n;
  }
  return (count + 15) / 16 * 16;
}

size_t tile_select_smem(const Plan& p, const Tile& t) {
  size_t key = p.dtype == 0 ? 4 : 8;
  return (size_t)(t.SW + t.SH + p.tile.g.kd) * 8 + (size_t)p.tile.g.kd * t.SH * t.SW * key;
}

cudaError_t launch_tile_select(const Plan& p, const void* in, void* out, cudaStream_t s) {
  if (p.dtype == 0)
    return launch_tile_select_t<float>(p, (const float*)in, (float*)out, s);
  return launch_tile_select_t<double>(p, (const double*)in, (double*)out, s);
}

cudaError_t launch_generic_select(const Plan& p, const void* in, void* out, cudaStream_t s) {
  long long blocks = (p.n_out + kThreads - 1) / kThreads;
  long long cap = (long long)p.sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (p.dtype == 0)
    generic_select_kernel<float><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const float*)in, (float*)out, p.generic, p.d_gen_taps);
  else
    generic_select_kernel<double><<<(unsigned)blocks, kThreads, 0, s>>>(
        (const double*)in, (double*)out, p.generic, p.d_gen_taps);
  return cudaGetLastError();
}

}  // namespace ndf

// Tile network kernels and their launchers, shared by select.cu (network
// widths up to 64) and select_wide.cu (widths 80 to 128), which compile in
// parallel.
#pragma once

#include "network.cuh"

namespace ndf {
namespace netlaunch {
using namespace net;

// Minimum resident blocks per SM the compiler must allow for: the 80-wire
// median network (68- to 80-tap windows such as ring(4, 6) and 3 x 5 x 5)
// fits three 256-thread blocks in 80 registers with a 72-byte spill, which
// raises occupancy from two blocks (89 registers); wider networks spill
// kilobytes under such a cap and keep one.
template <int N, int MODE>
constexpr int network_min_blocks() {
  return (N == 80 && MODE == 1) ? 3 : 1;
}

template <typename T, int N, int VFIX, int MODE>
__global__ void __launch_bounds__(kThreads, network_min_blocks<N, MODE>())
    tile_network_kernel(const T* __restrict__ in, T* __restrict__ out,
                        const __grid_constant__ TileArgs a, const __grid_constant__ TapTable<N> taps,
                        const __grid_constant__ CUtensorMap tmap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  tile_network_body<T, N, VFIX, MODE>(in, out, a, blockIdx.x, smem_raw,
                                      [&](int i) { return taps.off[i]; }, &tmap);
}

template <typename T, int N, int VFIX, int MODE>
cudaError_t launch_network(const Plan& p, const T* in, T* out, cudaStream_t s) {
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
  auto kernel = tile_network_kernel<T, N, VFIX, MODE>;
  cudaError_t e =
      allow_max_smem((const void*)kernel);
  if (e != cudaSuccess) return e;
  TileArgs args = a;
  CUtensorMap map{};
  size_t smem = p.smem_bytes;
  tma_prepare(p, a.t, in, &map, &args, &smem);
  kernel<<<(unsigned)a.t.tiles, kThreads, smem, s>>>(in, out, args, taps, map);
  return cudaGetLastError();
}

template <typename T, int N>
cudaError_t dispatch_network_mode(const Plan& p, const T* in, T* out, cudaStream_t s) {
  const bool median = p.r.kind == kMedian || p.r.kind == kMedianNetwork ||
                      p.r.kind == kMedianHistogram;
  if (!median) return launch_network<T, N, 0, 0>(p, in, out, s);
  if constexpr (sizeof(T) == 4) {
    // Fixed tap counts of the hot configurations: 3x3, 5x5 and 7x7 boxes,
    // the 68-tap ring(4, 6) and the 3 x 5 x 5 box (the compiler then drops
    // the comparators of the padding wires).
    if (N == 16 && p.r.count == 9) return launch_network<T, 16, 9, 1>(p, in, out, s);
    if (N == 32 && p.r.count == 25) return launch_network<T, 32, 25, 1>(p, in, out, s);
    if (N == 64 && p.r.count == 49) return launch_network<T, 64, 49, 1>(p, in, out, s);
    if (N == 80 && p.r.count == 68) return launch_network<T, 80, 68, 1>(p, in, out, s);
    if (N == 80 && p.r.count == 75) return launch_network<T, 80, 75, 1>(p, in, out, s);
  }
  return launch_network<T, N, 0, 1>(p, in, out, s);
}

}  // namespace netlaunch
}  // namespace ndf

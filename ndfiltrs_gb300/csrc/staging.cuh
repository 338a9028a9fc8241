// Halo-tile staging: one thread block copies the samples that its output
// tile's windows read (the tile plus the window halo, through the boundary
// modes) into shared memory, converted by `conv` (a key or the value).
//
// This replaces the reference's per-tap gather and boundary remapping
// (Window::gather / visit_mapped, src/window.rs:211-294, and map_index,
// src/boundary.rs:29-71): the remapping runs once per staged sample instead
// of once per tap, and interior rows are read with coalesced loads.
#pragma once

#include "common.cuh"
#include "plan.h"

namespace ndf {

// Per-axis source offsets of the support, or -1 outside a constant boundary.
// Layout in shared memory: [SW] x offsets, [SH] y offsets (times W),
// [kd] z offsets (times H*W).
__device__ __forceinline__ void build_maps(long long* maps, const Geom3& g, const Tile& t,
                                           long long z, long long y0, long long x0) {
  long long* mx = maps;
  long long* my = maps + t.SW;
  long long* mz = my + t.SH;
  for (int i = threadIdx.x; i < t.SW + t.SH + g.kd; i += blockDim.x) {
    long long m;
    if (i < t.SW) {
      mx[i] = map_index(x0 + i - g.ax, g.W, g.mx, &m) ? m : -1;
    } else if (i < t.SW + t.SH) {
      int j = i - t.SW;
      my[j] = map_index(y0 + j - g.ay, g.H, g.my, &m) ? m * g.W : -1;
    } else {
      int j = i - t.SW - t.SH;
      mz[j] = map_index(z + j - g.az, g.D, g.mz, &m) ? m * g.H * g.W : -1;
    }
  }
}

// Stage kd x SH x SW samples; rows are spread over warps, columns over
// lanes, so interior rows load with coalesced 128-byte transactions.
template <typename T, typename S, typename Conv>
__device__ __forceinline__ void stage_support(S* smem, const long long* maps,
                                              const T* __restrict__ in, const Geom3& g,
                                              const Tile& t, S outside, Conv conv) {
  const long long* mx = maps;
  const long long* my = maps + t.SW;
  const long long* mz = my + t.SH;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int warps = blockDim.x >> 5;
  const int rows = g.kd * t.SH;
  for (int row = warp; row < rows; row += warps) {
    int sz = row / t.SH;
    int sy = row - sz * t.SH;
    long long oz = mz[sz], oy = my[sy];
    S* dst = smem + (size_t)row * t.SW;
    if (oz < 0 || oy < 0) {
      for (int sx = lane; sx < t.SW; sx += 32) dst[sx] = outside;
      continue;
    }
    const T* src = in + oz + oy;
    for (int sx = lane; sx < t.SW; sx += 32) {
      long long ox = mx[sx];
      dst[sx] = ox < 0 ? outside : conv(__ldg(src + ox));
    }
  }
}

}  // namespace ndf

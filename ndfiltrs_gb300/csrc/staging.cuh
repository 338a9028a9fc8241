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
#include "tma.cuh"

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

// Stage a tile's support: one TMA copy for an interior tile when the launch
// enabled TMA (a.tma_bw > 0), else the boundary-remapped loads above. Uses
// `maps` (the remap tables) only on the remapped path. Returns false, in
// every thread, when the TMA wait timed out; the caller then returns without
// writing outputs. The caller synchronizes the block after a true return.
template <typename T, typename S, typename Conv>
__device__ __forceinline__ bool stage_tile(S* s, long long* maps, unsigned char* smem_raw,
                                           const T* __restrict__ in, const TileArgs& a,
                                           const CUtensorMap* tmap, long long z, long long y0,
                                           long long x0, S outside, Conv conv) {
  const Geom3& g = a.g;
  const Tile& t = a.t;
  constexpr int kAlign = 16 / (int)sizeof(T);
  const long long xs = x0 - g.ax, ys = y0 - g.ay, zs = z - g.az;
  const long long xa = xs >= 0 ? xs - xs % kAlign : -1;
  const bool interior = a.tma_bw > 0 && xa >= 0 && ys >= 0 && zs >= 0 && xa + a.tma_bw <= g.W &&
                        ys + t.SH <= g.H && zs + g.kd <= g.D;
  if (!interior) {
    build_maps(maps, g, t, z, y0, x0);
    __syncthreads();
    stage_support(s, maps, in, g, t, outside, conv);
    return true;
  }
  __shared__ __align__(8) unsigned long long bar;
  // The staging area starts at the first 128-byte aligned shared address at
  // or after tma_offset (the launch reserves 127 bytes of slack for it).
  const unsigned int base = tma::smem_addr(smem_raw + a.tma_offset);
  T* raw = reinterpret_cast<T*>(smem_raw + a.tma_offset + ((128u - (base & 127u)) & 127u));
  if (threadIdx.x == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int bytes = (unsigned int)((size_t)a.tma_bw * t.SH * g.kd * sizeof(T));
    tma::mbar_arrive_expect_tx(&bar, bytes);
    if (a.tma_rank == 2)
      tma::load_2d(raw, tmap, &bar, (int)xa, (int)ys);
    else
      tma::load_3d(raw, tmap, &bar, (int)xa, (int)ys, (int)zs);
  }
  const bool ok = __syncthreads_and(tma::mbar_wait(&bar, 0, kWaitLimitNs, a.status) ? 1 : 0) != 0;
  if (!ok) {
    // The copy was issued and may still land: wait once more (bounded) so
    // that the block does not retire while the copy can write shared memory
    // that the next block on this SM would own. If the second wait runs out
    // too the block returns anyway (a wait never spins without a limit); the
    // status word already makes the call report NDF_ERR_TIMEOUT.
    if (threadIdx.x == 0) tma::mbar_wait(&bar, 0, kWaitLimitNs, nullptr);
    __syncthreads();
    return false;
  }
  const int r = (int)(xs - xa);
  const int rows = g.kd * t.SH;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  for (int row = warp; row < rows; row += warps) {
    const T* src = raw + (size_t)row * a.tma_bw + r;
    S* dst = s + (size_t)row * t.SW;
    for (int sx = lane; sx < t.SW; sx += 32) dst[sx] = conv(src[sx]);
  }
  return true;
}

}  // namespace ndf

// Tensor Memory Accelerator (TMA) staging of interior halo tiles and the
// bounded mbarrier wait that every TMA copy completes on.
//
// An interior tile (its whole support inside the array, so no boundary
// remapping) is copied global -> shared by ONE cp.async.bulk.tensor 2-D/3-D
// load issued by one thread; the block waits on an mbarrier whose
// transaction count the copy completes. TMA needs the innermost coordinate
// times the element size to be a multiple of 16 bytes, so the copy starts at
// the support's first column rounded down to 16 bytes and is `bw` elements
// wide (a multiple of 16 bytes covering the rounding); the staging pass then
// reads the support from offset r = x_start - x_aligned. Edge tiles keep the
// per-sample boundary-remapped loads of staging.cuh.
//
// Every wait is bounded (1 s of %globaltimer by default): a wait that runs
// out sets the status word that the host reads after its next synchronization
// (NDF_ERR_TIMEOUT), drains the issued copy with a second bounded wait, and
// the block returns without writing outputs.
#pragma once

#include <cuda.h>

#include "plan.h"

namespace ndf {

constexpr unsigned int kStatusTimeout = 1u;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;

namespace tma {

__device__ __forceinline__ unsigned int smem_addr(const void* p) {
  return (unsigned int)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Make the initialized barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned int phase) {
  unsigned int done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return done != 0;
}

// Wait for `phase` of the barrier for at most `limit_ns`; on timeout record
// kStatusTimeout in `status` (a host-mapped word) and return false.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned int phase,
                                          unsigned long long limit_ns, volatile unsigned int* status) {
  if (mbar_try_wait(bar, phase)) return true;
  const unsigned long long start = globaltimer();
  while (!mbar_try_wait(bar, phase)) {
    if (globaltimer() - start > limit_ns) {
      if (status) *status = kStatusTimeout;
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void load_2d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x,
                                        int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x,
                                        int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace tma

// Host side (tma.cu).

// Tensor map and launch fields for TMA staging of the plan's interior tiles
// with tile `t` over input `in`. Returns false (TMA off: a.tma_bw = 0) when
// TMA is disabled, the array is 1-D, the input or its rows are not 16-byte
// aligned, a box dimension exceeds 256, or the staging area does not fit in
// shared memory; `smem` grows by the staging area otherwise.
bool tma_prepare(const Plan& p, const Tile& t, const void* in, CUtensorMap* map, TileArgs* a, size_t* smem);

// Host-mapped status word of the current process (kernels write
// kStatusTimeout into it); nullptr when it cannot be allocated.
unsigned int* status_word_device();
// Read and clear the status word on the host (after a synchronization).
unsigned int status_take();

}  // namespace ndf

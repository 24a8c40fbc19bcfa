// tma.cuh -- Tensor Memory Accelerator plumbing for the staged stencil
// kernels: a 4-D tiled tensor map over an IDX4S gridfunction array
// ([gf][i2][i1][i0], i0 fastest), and the device side -- mbarrier set-up,
// one-thread bulk tensor loads into shared memory that complete on an
// mbarrier, and a bounded wait.
//
// Alignment rules the host checks before it takes this path: the array
// base is 16-byte aligned, every stride (n0, n0*n1, n0*n1*n2 elements) is a
// multiple of 16 bytes, the box's innermost extent is a multiple of 16 bytes,
// and every load starts at an i0 coordinate whose byte offset is a multiple
// of 16 (the kernels start boxes at multiples of their 16-point tile width).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace nrgpu {

// ------------------------------------------------------------------ host
// Encodes a tiled map of `ngf` gridfunctions of n0 x n1 x n2 elements of
// `esize` bytes (4 or 8) at `base`, with a box of bx x by x bz x 1.
// Returns false (and leaves *map untouched) if an alignment rule fails or
// the driver refuses the map.
bool tma_map_gridfunctions(CUtensorMap *map, const void *base, int esize, int n0, int n1, int n2, int ngf, int bx,
                           int by, int bz);

// --------------------------------------------------------------- device
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the initialised barriers visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier shared-memory accesses before async-proxy
// accesses it issues next (a buffer refilled by TMA after it was read).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Bulk tensor load of box (c0, c1, c2, c3) of `map` into dst; completes
// `bytes` transaction bytes on `bar`.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Prefetch of box (c0, c1, c2, c3) of `map` into L2 (no shared memory, no
// completion to wait for): starts the DRAM reads of boxes needed later.
__device__ __forceinline__ void tma_prefetch_l2_4d(const CUtensorMap *map, int c0, int c1, int c2, int c3) {
  asm volatile("cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
                   (unsigned long long)map),
               "r"(c0), "r"(c1), "r"(c2), "r"(c3)
               : "memory");
}

// Plain L2 prefetch of the line holding p (global memory).
__device__ __forceinline__ void prefetch_l2(const void *p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for phase `parity` of `bar` to complete; gives up after about
// 2^31 SM cycles (about one second) and returns false.  No wait in these
// kernels is unbounded.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > (1LL << 31)) return false;
  }
  return true;
}

}  // namespace nrgpu

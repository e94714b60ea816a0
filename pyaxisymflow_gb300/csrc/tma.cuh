// mbarrier and TMA (cp.async.bulk.tensor) helpers shared by the tensor-core
// GEMM and the stencil kernels, plus the host-side encoder of a plain
// (unswizzled) 2-D box.
//
// Every wait is bounded by a wall-clock limit: on expiry the waiting thread
// records an error code in a device word and returns false, so a kernel can
// drain its copies and exit instead of spinning forever.
#pragma once

#include <cuda.h>
#include <cstdint>

#include "axi_common.cuh"

namespace axi_tma {

constexpr unsigned long long WAIT_NS = 1000000000ull;  // 1 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier shared-memory accesses (generic proxy) before
// later TMA writes (async proxy) to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase. False on timeout (error recorded) or when
// another thread of the grid has already failed. The error word (an L2 round
// trip) and the clock are read once every 64 polls, so a phase that completes
// while the thread waits is seen at the next poll; each try_wait suspends for
// at most a hardware time limit, which keeps the loop bounded.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (unsigned int i = 1;; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63u) == 0) {
      if (*reinterpret_cast<volatile int*>(err) != 0) return false;
      if (globaltimer() - t0 > WAIT_NS) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}

// Bounded wait that ignores the error word: used to drain copies still in
// flight before a failing block exits (its shared memory must outlive them).
__device__ __forceinline__ bool mbar_wait_drain(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = globaltimer();
  while (!mbar_try_wait(bar, parity))
    if (globaltimer() - t0 > WAIT_NS) return false;
  return true;
}

// L2 prefetch of a box (no shared memory, no barrier); c0 as for a load.
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int c0, int c1) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1)
               : "memory");
}

// Box load: c0 is the innermost (contiguous) coordinate. Out-of-range
// elements of the box are filled with zeros; c0 * element size must be a
// multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Host: the driver's cuTensorMapEncodeTiled (null when unavailable).
void* encode_tiled_fn();

// Host: map of a row-major (rows, cols) array of elem_bytes-sized floats for
// box_rows x box_cols boxes without swizzle, zero fill out of range. Checks
// the 16-byte rules (base, row stride, box row). Returns an AXI status.
int encode_box(CUtensorMap* map, const void* base, int elem_bytes, int rows, int cols,
               int box_rows, int box_cols);

}  // namespace axi_tma

// Bulk asynchronous copies (global -> shared) completed on an mbarrier, in
// inline PTX for sm_103a. Used to stream contiguous tiles of particle state
// into shared memory while the previous tile is being computed.
//
// Every wait is bounded by a clock budget: a wait that runs out records
// kStatusTimeout in the engine status word and reports failure, so a stuck
// copy can never hang the GPU.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace tdem {
namespace bulk {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
}

// Make barrier initialisation visible to the async proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// 1-D bulk copy; both addresses 16-byte aligned, size a multiple of 16 bytes.
__device__ __forceinline__ void copy_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0u;
}

// Non-blocking probe of phase `parity` of `bar`.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0u;
}

// Wait for phase `parity` of `bar` for at most `budget` SM clock cycles. A
// budget of 0 makes the wait one non-blocking probe (try_wait itself may
// suspend until the phase completes), which tests of the failure path use.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long budget) {
  if (budget <= 0) return mbar_test_wait(bar, parity);
  const long long start = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - start > budget) return false;
  }
  return true;
}

// Per-thread asynchronous copies (cp.async, 16 bytes, L2 only) into shared
// memory, in commit groups that complete in order. A thread waits only for
// its own groups, so a thread that reads back only what it copied needs no
// block barrier. The copies are plain loads that always complete.
__device__ __forceinline__ void cp16(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst_smem)), "l"(src_gmem) : "memory");
}

// 8-byte variant (through L1: the 16-byte L2-only form has no smaller size).
__device__ __forceinline__ void cp8(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst_smem)), "l"(src_gmem) : "memory");
}

// 4-byte variant.
__device__ __forceinline__ void cp4(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst_smem)), "l"(src_gmem) : "memory");
}

// Bulk prefetch of [src, src + bytes) into L2 (16-byte aligned, bytes a
// multiple of 16, inside the array).
__device__ __forceinline__ void prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Wait until at most N of this thread's most recent groups are pending.
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace bulk
}  // namespace tdem

// pps_mbarrier.cuh -- shared-memory barriers and bulk copies (inline PTX) used
// by the kernels that stage data through the Tensor Memory Accelerator or hand
// buffers to the tensor cores.
//
// Every wait here is bounded: mbar_wait_bounded gives up after a time limit
// (read from %globaltimer) or when another thread of the block has given up,
// so a copy or an MMA that never completes ends the launch with a status the
// host reads, never a hang.
#pragma once
#include <cstdint>

namespace pps {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
// makes initialised barriers visible to the async proxy (bulk copies, MMA commits)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.release.cta.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(mbar)
               : "memory");
}
// one arrival that also announces `bytes` of transactions (bulk copies) the
// phase waits for
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.release.cta.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(
                   mbar),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait for the phase of `parity` to complete: false when `limit_ns`
// passed or another thread set *abort_flag (the clock and the flag are looked
// at every 64 polls); a thread that gives up sets *abort_flag itself
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity, volatile int* abort_flag,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(mbar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try_wait(mbar, parity)) return true;
    if ((i & 63u) == 0 && (*abort_flag || globaltimer() - t0 > limit_ns)) {
      *abort_flag = 1;
      return false;
    }
  }
}
// bulk copy (TMA, no tensor map) of `bytes` from global to this CTA's shared
// memory, completing as transactions on `mbar`.  Both addresses 16-byte
// aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

}  // namespace pps

// Inline-PTX helpers for bulk asynchronous copies global -> shared memory
// (cp.async.bulk, and cp.async.bulk.tensor through a tensor map) completing on
// an mbarrier, and the bounded mbarrier wait of the staged kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {
namespace tma {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t mb, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mb), "r"(count) : "memory");
}
// makes the initialised barrier visible to the async proxy (the copy engine)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(uint32_t mb) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(mb) : "memory");
}
// the single arrival of a phase, announcing the bytes its copies deliver
__device__ __forceinline__ void mbar_arrive_tx(uint32_t mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(mb), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase with the given parity to complete; gives up after
// `limit` polls (each poll suspends the thread for a hardware-chosen time)
// and returns false.
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity, int limit) {
  for (int i = 0; i < limit; i++)
    if (mbar_try_wait(mb, parity)) return true;
  return false;
}

// contiguous copy: dst and src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mb) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mb)
               : "memory");
}
// one box of a rank-5 tensor map (unused trailing dimensions have extent 1)
__device__ __forceinline__ void tensor_load5(uint32_t dst, const CUtensorMap* tm, int c0, int c1, int c2, int c3, int c4,
                                             uint32_t mb) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(dst),
      "l"(tm), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(mb)
      : "memory");
}
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* tm) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(tm) : "memory");
}

}  // namespace tma
}  // namespace pg

// Kernel unit of the batched persistent launch (batch_kernel.cuh), float batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f32(const BatchLaunch& q, int grid, int smem, cudaStream_t s, bool r8) {
  if (r8)
    k_batch<false, true><<<grid, BATCH_THREADS, smem, s>>>(q);
  else
    k_batch<false, false><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f32(bool r8) {
  return r8 ? (const void*)k_batch<false, true> : (const void*)k_batch<false, false>;
}

}  // namespace pg

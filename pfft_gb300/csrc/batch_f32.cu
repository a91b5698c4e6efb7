// Kernel unit of the batched persistent launch (batch_kernel.cuh), float batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f32(const BatchLaunch& q, int grid, int smem, cudaStream_t s, int r8) {
  if (r8)
    k_batch<false, 1><<<grid, BATCH_THREADS, smem, s>>>(q);
  else
    k_batch<false, 0><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f32(int r8) { return r8 ? (const void*)k_batch<false, 1> : (const void*)k_batch<false, 0>; }

}  // namespace pg

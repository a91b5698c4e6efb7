// Kernel unit of the batched persistent launch (batch_kernel.cuh), float batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f32(const BatchLaunch& q, int grid, int smem, cudaStream_t s) {
  k_batch<false><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f32() { return (const void*)k_batch<false>; }

}  // namespace pg

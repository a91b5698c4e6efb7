// Kernel unit of the batched persistent launch (batch_kernel.cuh), double batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64(const BatchLaunch& q, int grid, int smem, cudaStream_t s) {
  k_batch<true><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64() { return (const void*)k_batch<true>; }

}  // namespace pg

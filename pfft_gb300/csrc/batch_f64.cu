// Kernel unit of the batched persistent launch (batch_kernel.cuh), double batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64(const BatchLaunch& q, int grid, int smem, cudaStream_t s, int r8) {
  switch (r8) {
    case 1: k_batch<true, 1><<<grid, BATCH_THREADS, smem, s>>>(q); break;
    case 2: k_batch<true, 2><<<grid, BATCH_THREADS, smem, s>>>(q); break;
    case 3: k_batch<true, 3><<<grid, BATCH_THREADS, smem, s>>>(q); break;
    default: k_batch<true, 0><<<grid, BATCH_THREADS, smem, s>>>(q); break;
  }
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64(int r8) {
  switch (r8) {
    case 1: return (const void*)k_batch<true, 1>;
    case 2: return (const void*)k_batch<true, 2>;
    case 3: return (const void*)k_batch<true, 3>;
  }
  return (const void*)k_batch<true, 0>;
}

}  // namespace pg

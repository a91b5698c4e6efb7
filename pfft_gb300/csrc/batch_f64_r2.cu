// Kernel unit of the batched persistent launch (batch_kernel.cuh): double
// batches, kernel variant R8 = 2 (one variant per unit so that they compile
// in parallel).
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64_r2(const BatchLaunch& q, int grid, int smem, cudaStream_t s) {
  k_batch<true, 2><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64_r2() { return (const void*)k_batch<true, 2>; }

}  // namespace pg

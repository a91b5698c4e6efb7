// Kernel unit of the batched persistent launch (batch_kernel.cuh): double
// batches, kernel variant R8 = 1 (one variant per unit so that they compile
// in parallel).
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64_r1(const BatchLaunch& q, int grid, int smem, cudaStream_t s) {
  k_batch<true, 1><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64_r1() { return (const void*)k_batch<true, 1>; }

}  // namespace pg

// Kernel unit of the batched persistent launch (batch_kernel.cuh): double
// batches, kernel variant R8 = 4 (one variant per unit so that they compile
// in parallel).
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64_r4(const BatchLaunch& q, int grid, int smem, cudaStream_t s) {
  k_batch<true, 4><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64_r4() { return (const void*)k_batch<true, 4>; }

}  // namespace pg

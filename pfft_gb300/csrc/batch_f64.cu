// Kernel unit of the batched persistent launch (batch_kernel.cuh), double batches.
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64(const BatchLaunch& q, int grid, int smem, cudaStream_t s, bool r8) {
  if (r8)
    k_batch<true, true><<<grid, BATCH_THREADS, smem, s>>>(q);
  else
    k_batch<true, false><<<grid, BATCH_THREADS, smem, s>>>(q);
  return (int)cudaGetLastError();
}

const void* batch_kernel_f64(bool r8) {
  return r8 ? (const void*)k_batch<true, true> : (const void*)k_batch<true, false>;
}

}  // namespace pg

// Double batches of the batched persistent launch: dispatch to the kernel
// variant units batch_f64_r0.cu .. batch_f64_r4.cu (k_batch's R8).
#include "batch_kernel.cuh"

namespace pg {

int batch_launch_f64_r0(const BatchLaunch& q, int grid, int smem, cudaStream_t s);
int batch_launch_f64_r1(const BatchLaunch& q, int grid, int smem, cudaStream_t s);
int batch_launch_f64_r2(const BatchLaunch& q, int grid, int smem, cudaStream_t s);
int batch_launch_f64_r3(const BatchLaunch& q, int grid, int smem, cudaStream_t s);
const void* batch_kernel_f64_r0();
const void* batch_kernel_f64_r1();
const void* batch_kernel_f64_r2();
const void* batch_kernel_f64_r3();
int batch_launch_f64_r4(const BatchLaunch& q, int grid, int smem, cudaStream_t s);
const void* batch_kernel_f64_r4();

int batch_launch_f64(const BatchLaunch& q, int grid, int smem, cudaStream_t s, int r8) {
  switch (r8) {
    case 1: return batch_launch_f64_r1(q, grid, smem, s);
    case 2: return batch_launch_f64_r2(q, grid, smem, s);
    case 3: return batch_launch_f64_r3(q, grid, smem, s);
    case 4: return batch_launch_f64_r4(q, grid, smem, s);
  }
  return batch_launch_f64_r0(q, grid, smem, s);
}

const void* batch_kernel_f64(int r8) {
  switch (r8) {
    case 1: return batch_kernel_f64_r1();
    case 2: return batch_kernel_f64_r2();
    case 3: return batch_kernel_f64_r3();
    case 4: return batch_kernel_f64_r4();
  }
  return batch_kernel_f64_r0();
}

}  // namespace pg

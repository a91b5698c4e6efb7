// Ghost-cell exchange that allocates nothing.
//
// pfft_exchange works through a plan, and creating that plan allocates device
// scratch memory (cudaMalloc) for the copy of the compact block.  Some callers
// cannot allocate at the point where they need the halo: code running inside
// a memory-pool budget that forbids new device allocations, code that must not
// synchronise the device (cudaMalloc/cudaFree may), or long-running solvers
// that pre-size every buffer at start-up.  pfft_gb300_exchange_noalloc gives
// them the same periodic-wrap exchange with no allocation at all: the copy of
// the compact block goes to a fixed-size scratch array that lives in this
// library's device image (a file-scope __device__ array), so every GPU that
// loads this code holds PG_NOALLOC_SCRATCH_BYTES of device memory until the
// process exits.
#include <cuda_runtime.h>
#include <stddef.h>
#include <mutex>
#include "../../include/pfft_gb300.h"

#define PG_NOALLOC_SCRATCH_BYTES (32u << 20)  // 32 MiB
#define PG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[PG_NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of the scratch array, looked up once per device.  In host
// code the name g_noalloc_scratch is only a stand-in for the device symbol,
// never a usable pointer.
std::mutex g_mu;
void* g_scratch_dev[PG_NOALLOC_MAX_DEVICES] = {nullptr};

int scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= PG_NOALLOC_MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return (int)e;
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return 0;
}

template <class T>
__global__ void k_noalloc_gather(const T* __restrict__ src, T* __restrict__ box, long long n0, long long n1,
                                 long long n2, long long b0, long long b1, long long b2, long long g1, long long g2,
                                 long long tuple, long long ncell) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
    long long r = c;
    long long k2 = r % g2;
    r /= g2;
    long long k1 = r % g1;
    long long k0 = r / g1;
    long long j0 = (k0 - b0) % n0, j1 = (k1 - b1) % n1, j2 = (k2 - b2) % n2;
    if (j0 < 0) j0 += n0;
    if (j1 < 0) j1 += n1;
    if (j2 < 0) j2 += n2;
    const T* s = src + ((j0 * n1 + j1) * n2 + j2) * tuple;
    T* d = box + c * tuple;
    for (long long h = 0; h < tuple; h++) d[h] = s[h];
  }
}

}  // namespace

extern "C" int pfft_gb300_exchange_noalloc(int precision, const ptrdiff_t* n, const ptrdiff_t* gc_below,
                                           const ptrdiff_t* gc_above, ptrdiff_t tuple, void* data, void* stream) {
  if (!n || !gc_below || !gc_above || !data || tuple < 1 || (precision != 0 && precision != 1))
    return (int)cudaErrorInvalidValue;
  long long cells = 1, box = 1, ng[3];
  for (int t = 0; t < 3; t++) {
    if (n[t] < 1 || gc_below[t] < 0 || gc_above[t] < 0) return (int)cudaErrorInvalidValue;
    ng[t] = gc_below[t] + n[t] + gc_above[t];
    cells *= n[t];
    box *= ng[t];
  }
  const size_t esz = precision ? sizeof(double) : sizeof(float);
  const size_t block_bytes = (size_t)cells * (size_t)tuple * esz;
  if (block_bytes > PG_NOALLOC_SCRATCH_BYTES) return (int)cudaErrorMemoryAllocation;
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, data) != cudaSuccess) {
    cudaGetLastError();
    return (int)cudaErrorInvalidValue;
  }
  if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged) return (int)cudaErrorInvalidValue;
  void* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(scratch, data, block_bytes, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return (int)e;
  long long blocks = (box + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (precision)
    k_noalloc_gather<double><<<(unsigned)blocks, 256, 0, s>>>((const double*)scratch, (double*)data, n[0], n[1], n[2],
                                                              gc_below[0], gc_below[1], gc_below[2], ng[1], ng[2],
                                                              tuple, box);
  else
    k_noalloc_gather<float><<<(unsigned)blocks, 256, 0, s>>>((const float*)scratch, (float*)data, n[0], n[1], n[2],
                                                             gc_below[0], gc_below[1], gc_below[2], ng[1], ng[2],
                                                             tuple, box);
  return (int)cudaGetLastError();
}

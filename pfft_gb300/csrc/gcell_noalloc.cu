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
#include <limits.h>
#include <mutex>
#include "../../include/pfft_gb300.h"

#define PG_NOALLOC_SCRATCH_BYTES (32u << 20)  // 32 MiB
#define PG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[PG_NOALLOC_SCRATCH_BYTES];

namespace {

// Per-device set-up, done once with that device current: the device address
// of the scratch array (in host code the name g_noalloc_scratch is only a
// stand-in for the device symbol, never a usable pointer) and the number of
// SMs, which caps the grid.  pfft_cleanup() forgets both (noalloc_forget),
// so that a process which resets a device (cudaDeviceReset rebuilds the
// context and may move the array) and then calls pfft_cleanup looks the
// address up again.
std::mutex g_mu;
void* g_scratch_dev[PG_NOALLOC_MAX_DEVICES] = {nullptr};
int g_sms[PG_NOALLOC_MAX_DEVICES] = {0};

int setup_current_device(int dev, void** out, int* sms) {
  if (dev < 0 || dev >= PG_NOALLOC_MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return (int)e;
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    g_scratch_dev[dev] = p;
    g_sms[dev] = n > 0 ? n : 1;
  }
  *out = g_scratch_dev[dev];
  *sms = g_sms[dev];
  return 0;
}

// a * b into *r unless it leaves [0, limit]
bool mul_within(unsigned long long a, unsigned long long b, unsigned long long limit, unsigned long long* r) {
  unsigned long long p;
  if (__builtin_mul_overflow(a, b, &p) || p > limit) return false;
  *r = p;
  return true;
}

}  // namespace

namespace pg {
void noalloc_forget() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (int d = 0; d < PG_NOALLOC_MAX_DEVICES; d++) {
    g_scratch_dev[d] = nullptr;
    g_sms[d] = 0;
  }
}
}  // namespace pg

// The buffer check of pfft_gb300_exchange_noalloc, on the attributes of the
// pointer: device memory of the current device, or managed memory.  A
// device pointer of another GPU is refused (the gather would address that
// GPU's memory from this one without peer access).  Exported for the CPU
// tests of the rule; not part of the public header.
extern "C" int pg_noalloc_buffer_check(int mem_type, int ptr_device, int current_device) {
  if (mem_type == (int)cudaMemoryTypeManaged) return 0;
  if (mem_type != (int)cudaMemoryTypeDevice) return (int)cudaErrorInvalidValue;
  return ptr_device == current_device ? 0 : (int)cudaErrorInvalidDevice;
}

namespace {

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
  const size_t esz = precision ? sizeof(double) : sizeof(float);
  const unsigned long long lim = PG_NOALLOC_SCRATCH_BYTES;
  // every product is checked: the block against the scratch size, the box
  // against the range of the kernel's 64-bit cell index
  unsigned long long cells = 1, box = 1, block_bytes = 0;
  long long ng[3];
  for (int t = 0; t < 3; t++) {
    if (n[t] < 1 || gc_below[t] < 0 || gc_above[t] < 0) return (int)cudaErrorInvalidValue;
    unsigned long long e;
    if (__builtin_add_overflow((unsigned long long)gc_below[t], (unsigned long long)n[t], &e) ||
        __builtin_add_overflow(e, (unsigned long long)gc_above[t], &e) || e > (unsigned long long)LLONG_MAX)
      return (int)cudaErrorInvalidValue;
    ng[t] = (long long)e;
    if (!mul_within(cells, (unsigned long long)n[t], lim, &cells)) return (int)cudaErrorMemoryAllocation;
    if (!mul_within(box, e, (unsigned long long)LLONG_MAX, &box)) return (int)cudaErrorInvalidValue;
  }
  unsigned long long scal = 0, boxscal = 0;
  if (!mul_within(cells, (unsigned long long)tuple, lim, &scal) || !mul_within(scal, esz, lim, &block_bytes))
    return (int)cudaErrorMemoryAllocation;
  if (!mul_within(box, (unsigned long long)tuple, (unsigned long long)LLONG_MAX, &boxscal))
    return (int)cudaErrorInvalidValue;
  int cur = 0;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return (int)e;
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, data) != cudaSuccess) {
    cudaGetLastError();
    return (int)cudaErrorInvalidValue;
  }
  int rc = pg_noalloc_buffer_check((int)pa.type, pa.device, cur);
  if (rc) return rc;
  void* scratch = nullptr;
  int sms = 0;
  rc = setup_current_device(cur, &scratch, &sms);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  e = cudaMemcpyAsync(scratch, data, (size_t)block_bytes, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return (int)e;
  unsigned long long blocks = (box + 255) / 256;
  const unsigned long long cap = (unsigned long long)sms * 32;
  if (blocks > cap) blocks = cap;
  if (precision)
    k_noalloc_gather<double><<<(unsigned)blocks, 256, 0, s>>>((const double*)scratch, (double*)data, n[0], n[1], n[2],
                                                              gc_below[0], gc_below[1], gc_below[2], ng[1], ng[2],
                                                              tuple, (long long)box);
  else
    k_noalloc_gather<float><<<(unsigned)blocks, 256, 0, s>>>((const float*)scratch, (float*)data, n[0], n[1], n[2],
                                                             gc_below[0], gc_below[1], gc_below[2], ng[1], ng[2],
                                                             tuple, (long long)box);
  return (int)cudaGetLastError();
}

// Batched strided 1-D transform pass (see pass.h).
//
// Shared-memory Stockham autosort FFT, mixed radix.  A stage of radix R with
// Ns = product of the earlier radices maps, for j < M/R and k = j mod Ns,
//   x[j + r*M/R] * W_{Ns*R}^{k*r}  --DFT_R-->  y[(j-k)*R + k + r*Ns]
// so after the last stage the line is in natural order.  Radices 2,3,4,5,8,16
// have dedicated butterflies, small odd primes (7, 11, 13) use a register DFT
// with table twiddles, and any other prime uses a shared-memory ping-pong stage.
#include <stdlib.h>
#include <string.h>
#include <atomic>
#include "pass_tile.cuh"

namespace pg {

// The dynamic shared-memory limit is raised once per kernel, device and size
// (an attribute call costs microseconds; small transforms launch often).
template <const void* (*KFN)()>
static int ensure_smem_attr(int bytes) {
  static std::atomic<int> done[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (done[dev].load(std::memory_order_relaxed) >= bytes) return 0;
  cudaError_t e = cudaFuncSetAttribute(KFN(), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return (int)e;
  int cur = done[dev].load();
  while (cur < bytes && !done[dev].compare_exchange_weak(cur, bytes)) {
  }
  return 0;
}
template <class A, int SIGN>
static const void* kptr() {
  return (const void*)k_pass<A, SIGN>;
}
template <class A, int SIGN>
static const void* kptr_small() {
  return (const void*)k_pass_small<A, SIGN>;
}

template <class A>
static int launch_t(const PassParams& p, cudaStream_t stream) {
  long long grid = (p.nlines + p.L - 1) / p.L;
  if (grid <= 0) return 0;
  if (grid > 2147483647LL) return (int)cudaErrorInvalidConfiguration;
  const bool small = pass_is_small(p);
  int rc;
  if (p.sign < 0) {
    if (small) {
      if ((rc = ensure_smem_attr<kptr_small<A, -1>>(p.smem_bytes))) return rc;
      k_pass_small<A, -1><<<(unsigned)grid, p.threads, p.smem_bytes, stream>>>(p);
    } else {
      if ((rc = ensure_smem_attr<kptr<A, -1>>(p.smem_bytes))) return rc;
      k_pass<A, -1><<<(unsigned)grid, p.threads, p.smem_bytes, stream>>>(p);
    }
  } else {
    if (small) {
      if ((rc = ensure_smem_attr<kptr_small<A, 1>>(p.smem_bytes))) return rc;
      k_pass_small<A, 1><<<(unsigned)grid, p.threads, p.smem_bytes, stream>>>(p);
    } else {
      if ((rc = ensure_smem_attr<kptr<A, 1>>(p.smem_bytes))) return rc;
      k_pass<A, 1><<<(unsigned)grid, p.threads, p.smem_bytes, stream>>>(p);
    }
  }
  return (int)cudaGetLastError();
}

int launch_fast_pass(const PassParams& p, int arith, cudaStream_t stream);

static int g_kernel_path = -1;  // 0 generic only, 1 fast kernel where it applies
int kernel_path() {
  if (g_kernel_path < 0) {
    const char* e = getenv("PFFT_GB300_KERNEL");
    g_kernel_path = (e && strcmp(e, "generic") == 0) ? 0 : 1;
  }
  return g_kernel_path;
}
void set_kernel_path(int v) { g_kernel_path = v; }

int launch_pass(const PassParams& p, int arith, cudaStream_t stream) {
  if (kernel_path() == 1 && p.kpath == 0) {
    int rc = launch_fast_pass(p, arith, stream);
    if (rc != -1) return rc;
  }
  switch (arith) {
    case ARITH_F32: return launch_t<ArF32>(p, stream);
    case ARITH_F64: return launch_t<ArF64>(p, stream);
    case ARITH_DF: return launch_t<ArDF>(p, stream);
  }
  return (int)cudaErrorInvalidValue;
}

}  // namespace pg

namespace {
__global__ void k_df_roundtrip(const double* in, double* out, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = pg::df_to_double_sel(pg::df_from_double(in[i]));
}
// pairs (hi, lo): the fast float-float -> double conversion against the full
// one.  Counts: [0] values the fast path took, [1] its results that differ.
__global__ void k_df_fast(const float2* in, long long n, unsigned long long* counts) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bool ok;
  const pg::df d{in[i].x, in[i].y};
  const double f = pg::df_to_double_fast(d, ok), g = pg::df_to_double(d);
  if (ok) {
    atomicAdd(counts, 1ull);
    if (__double_as_longlong(f) != __double_as_longlong(g)) atomicAdd(counts + 1, 1ull);
  }
}
}  // namespace

// Test hook: out[i] = the double -> float-float -> double conversion of in[i]
// used by the double API's kernels.
extern "C" int pfft_gb300_selftest_df_roundtrip(const double* in, double* out, long long n, void* stream) {
  if (n <= 0) return 0;
  k_df_roundtrip<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(in, out, n);
  return (int)cudaGetLastError();
}

// Test hook: agreement of the float-float -> double fast path with the full
// routine (device arrays; counts = two zeroed device words, see k_df_fast).
extern "C" int pfft_gb300_selftest_df_fast(const float* pairs, long long n, unsigned long long* counts, void* stream) {
  if (n <= 0) return 0;
  k_df_fast<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>((const float2*)pairs, n, counts);
  return (int)cudaGetLastError();
}

// Dispatcher of the register-resident radix-8 pass kernel (fft_fast.cuh).
#include <atomic>
#include <mutex>
#include <string.h>
#include <cudaTypedefs.h>
#include "fft_fast.cuh"
#include "fft_mixed.cuh"
#include "core.h"

namespace pg {

static int g_staged = -1;  // 0 off, 1 per-pass choice, 2 wherever the layout allows
static std::atomic<long long> g_staged_launches{0};
int staged_mode() {
  if (g_staged < 0) {
    const char* e = getenv("PFFT_GB300_STAGED");
    g_staged = (e && strcmp(e, "0") == 0) ? 0 : (e && strcmp(e, "2") == 0) ? 2 : 1;
  }
  return g_staged;
}
void set_staged_mode(int v) { g_staged = (v >= 0 && v <= 2) ? v : 1; }
long long staged_launches() { return g_staged_launches.load(); }

namespace fast {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  });
  return fn;
}

int sm_count() {
  static int n[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 1;
  if (!n[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n[dev] = v > 0 ? v : 1;
  }
  return n[dev];
}

// one error word per device, zeroed when allocated
static int* g_err[64] = {nullptr};
static std::mutex g_err_mu;
int* staged_err_word() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (!g_err[dev]) {
    int* p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) {
      cudaFree(p);
      return nullptr;
    }
    g_err[dev] = p;
  }
  return g_err[dev];
}

}  // namespace fast

int* staged_err_word_if_any() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(fast::g_err_mu);
  return fast::g_err[dev];
}

namespace fast {
bool staged_setup(const FastArgs& a, int N, int L, int esz, bool row_in, CUtensorMap* tm) {
  if (!staged_mode() || a.nlines <= 0 || ((uintptr_t)a.src & 15)) return false;
  // default: float column passes (measured: the float-float kernels are
  // bound by instruction issue and lose a resident CTA per SM to the staging
  // area; row passes load whole lines with full coalescing already)
  if (staged_mode() == 1 && (a.staged == 2 || (a.staged == 0 && (esz != 8 || row_in)))) return false;
  if (row_in) {
    // every line's copy starts on a 16-byte boundary and is N * esz bytes
    if (a.sIa != 1 || (N * esz) % 16) return false;
    for (int b = 0; b < a.nb; b++)
      if ((a.bsI[b] * esz) % 16) return false;
    memset(tm, 0, sizeof *tm);
    g_staged_launches++;
    return true;
  }
  // column tiles: L adjacent lines along batch dimension 0, never straddling it
  if (a.nb < 1 || a.nb > 4 || a.bsI[0] != 1 || a.bext[0] % L || (L * esz) % 16 || L * esz / 4 > 256) return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return false;
  const int words = esz / 4;
  cuuint64_t dims[5], strides[4];
  cuuint32_t box[5], estr[5] = {1, 1, 1, 1, 1};
  dims[0] = (cuuint64_t)a.bext[0] * words;
  dims[1] = (cuuint64_t)N;
  strides[0] = (cuuint64_t)a.sIa * esz;
  box[0] = (cuuint32_t)(L * words);
  box[1] = (cuuint32_t)(N < 256 ? N : 256);
  for (int d = 2; d < 5; d++) {
    const int b = d - 1;
    if (b < a.nb) {
      dims[d] = (cuuint64_t)a.bext[b];
      strides[d - 1] = (cuuint64_t)a.bsI[b] * esz;
    } else {
      dims[d] = 1;
      strides[d - 1] = strides[d - 2];
    }
    box[d] = 1;
  }
  for (int d = 0; d < 4; d++)
    if (strides[d] % 16 || strides[d] >= (1ull << 40)) return false;
  for (int d = 0; d < 5; d++)
    if (dims[d] > (1ull << 32)) return false;
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 5, (void*)a.src, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  g_staged_launches++;
  return true;
}

// Twiddle tables of a pass on the radix-8 (pow2) or mixed-radix kernel: the
// FFT's table (stage-major for radix-8, natural for mixed-radix; float-float
// packed and of the FFT's direction: the DCTs run 10 forward, 01 inverse) and
// the DCT's 4N-point rotation table (natural; forward for FP32).
static bool fast_tables(const PassParams& p, int arith, bool pow2, const void** tw, const void** tw2) {
  cudaError_t e;
  const bool dct = p.mode == MODE_RE10 || p.mode == MODE_RE01;
  const int fsign = p.mode == MODE_RE10 ? -1 : (p.mode == MODE_RE01 ? 1 : p.sign);
  if (arith == ARITH_F64) {  // 64-bit fixed point (FX): stage-major (radix-8) or natural (mixed radix)
    *tw = twiddle_table(p.N, pow2 ? (fsign < 0 ? TW_FX_FWD_STG : TW_FX_BWD_STG) : (fsign < 0 ? TW_FX_FWD : TW_FX_BWD), &e);
    if (dct) *tw2 = twiddle_table(p.M, fsign < 0 ? TW_FX_FWD : TW_FX_BWD, &e);
  } else if (arith == ARITH_DF) {
    *tw = twiddle_table(p.N, pow2 ? (fsign < 0 ? TW_DFP_FWD_STG : TW_DFP_BWD_STG) : (fsign < 0 ? TW_DFP_FWD : TW_DFP_BWD),
                        &e);
    if (dct) *tw2 = twiddle_table(p.M, fsign < 0 ? TW_DFP_FWD : TW_DFP_BWD, &e);
  } else {
    *tw = pow2 ? twiddle_table(p.N, TW_F32_STG, &e) : twiddle_table(p.N, ARITH_F32, &e);
    if (dct) *tw2 = twiddle_table(p.M, ARITH_F32, &e);
  }
  return *tw && (!dct || *tw2);
}

bool fast_args(const PassParams& p, int arith, FastArgs* a, bool* row_in, bool* row_out) {
  const bool dct = p.mode == MODE_RE10 || p.mode == MODE_RE01;
  if ((p.mode != MODE_C2C && p.mode != MODE_R2C && p.mode != MODE_C2R && !dct) || p.nst == 0) return false;
  if (p.M != (dct ? 4 * p.N : p.N) || p.Ni > p.N || p.No > p.N) return false;
  if (p.wmode && !((p.wmode == 1 && p.mode == MODE_C2R) || (p.wmode == 2 && p.mode == MODE_R2C))) return false;
  const int N = p.N;
  const bool pow2 = N >= 16 && N <= 4096 && !(N & (N - 1));
  const bool plain = p.mode == MODE_C2C && p.Zi == 0 && p.Ni == N && p.Zo == 0 && p.No == N && !p.wmode;
  // the mixed-radix kernel reads and writes plain c2c lines only
  if (!pow2 && (!mixed_supported(N) || !plain)) return false;
  if ((p.mode == MODE_RE10 || p.mode == MODE_RE01) && N > 512) return false;
  // double plans (native FP64 storage and arithmetic class): 64-bit fixed
  // point (PassParams::quant == 2) on the radix-8 kernel's power-of-two c2c,
  // r2c, c2r, REDFT10 and REDFT01 lines with any window or adjoint weight,
  // and on the mixed-radix kernel's plain c2c lines; every other pass of such
  // a plan runs the general kernel in FP64
  if (arith == ARITH_F64 && p.quant != 2) return false;
  if (arith != ARITH_F32 && arith != ARITH_DF && arith != ARITH_F64) return false;
  if (p.ashI.en || p.ashO.en) return false;
  if (p.nb > PG_MAX_BATCH) return false;
  for (int b = 0; b < p.nb; b++)
    if (p.bshI[b].en || p.bshO[b].en) return false;
  a->src = p.src;
  a->dst = p.dst;
  a->tw = p.tw;
  a->sIa = p.sIa;
  a->sOa = p.sOa;
  a->nb = p.nb;
  for (int b = 0; b < p.nb; b++) {
    a->bext[b] = p.bext[b];
    a->bsI[b] = p.bsI[b];
    a->bsO[b] = p.bsO[b];
  }
  a->nlines = p.nlines;
  a->conj_in = p.conj_in;
  a->conj_out = p.conj_out;
  a->in_df = p.in_df;
  a->out_df = p.out_df;
  a->mode = p.mode == MODE_C2C ? 0 : p.mode == MODE_R2C ? 1 : p.mode == MODE_C2R ? 2 : p.mode == MODE_RE10 ? 3 : 4;
  a->tw2 = nullptr;
  if (!fast_tables(p, arith, pow2, &a->tw, &a->tw2)) return false;
  a->fx_in = arith == ARITH_F64 ? p.fx_in : 0;
  a->fx_out = arith == ARITH_F64 ? p.fx_out : 0;
  a->lexp_in = p.lexp_in;
  a->lexp_out = p.lexp_out;
  a->lexp_in_n = p.lexp_in_n;
  for (int b = 0; b < PG_MAX_BATCH; b++) {
    a->gin_np[b] = p.gin_np[b];
    a->gin_bofs[b] = p.gin_bofs[b];
  }
  for (int q = 0; q < 2 * PG_MAX_BATCH; q++) {
    a->gin_pext[q] = p.gin_pext[q];
    a->gin_pcoef[q] = p.gin_pcoef[q];
  }
  a->gin_k = p.gin_k;
  a->gout_off = p.gout_off;
  // paired real lines: batch dimension 0 halved, its odd lines the partners
  a->pair = 0;
  if (p.pair && arith == ARITH_F64 && !p.fx_in && !p.fx_out && p.nb >= 1 && p.bext[0] % 2 == 0 &&
      (p.mode == MODE_R2C || p.mode == MODE_C2R || p.mode == MODE_RE10 || p.mode == MODE_RE01)) {
    a->pair = 1;
    a->pairI = p.bsI[0];
    a->pairO = p.bsO[0];
    a->bext[0] = p.bext[0] / 2;
    a->bsI[0] = 2 * p.bsI[0];
    a->bsO[0] = 2 * p.bsO[0];
    a->nlines = p.nlines / 2;
  }
  a->Zi = p.Zi;
  a->Ni = p.Ni;
  a->Zo = p.Zo;
  a->No = p.No;
  a->plain = plain ? 1 : 0;
  a->wmode = p.wmode;
  *row_in = p.sIa == 1;
  *row_out = p.sOa == 1;
  // column mapping needs adjacent lines on that side
  if (!*row_in && !(p.nb > 0 && p.bsI[0] == 1)) return false;
  if (!*row_out && !(p.nb > 0 && p.bsO[0] == 1)) return false;
  if (a->mode >= 3 && *row_in != *row_out) return false;  // DCT kernels: one orientation
  return true;
}
}  // namespace fast

// Builds the tables a radix-8 / mixed-radix pass and its reverse direction
// use (plans build them when created, so that executing allocates nothing).
bool fast_pass_tables(const PassParams& p, int arith) {
  fast::FastArgs a;
  bool ri, ro;
  PassParams q = p;
  for (int sign : {-1, 1}) {
    q.sign = sign;
    fast::fast_args(q, arith, &a, &ri, &ro);
  }
  return true;
}

bool fast_pass_eligible(const PassParams& p, int arith) {
  fast::FastArgs a;
  bool ri, ro;
  return kernel_path() == 1 && p.kpath == 0 && fast::fast_args(p, arith, &a, &ri, &ro);
}

// Returns -1 when the pass is not covered by the fast kernel.
int launch_fast_pass(const PassParams& p, int arith, cudaStream_t stream) {
  using namespace fast;
  FastArgs a;
  bool row_in, row_out;
  if (!fast_args(p, arith, &a, &row_in, &row_out)) return -1;
  const int N = p.N;
  const bool big = N >= 1024;
  a.fastL = p.fastL;
  a.staged = p.staged;
  // the FFT direction: the pass's, except for the DCTs (10 forward, 01 inverse)
  const int sign = a.mode == 3 ? -1 : (a.mode == 4 ? 1 : p.sign);
  if (a.mode == 4 && arith == ARITH_F64 && a.pair)  // paired REDFT01
    return sign > 0 ? launch_dct_pinv<FX, 1>(N, a, row_in, row_out, stream) : -1;
  if (a.mode >= 3 && arith == ARITH_F64)
    return sign < 0 ? launch_dct<FX, -1>(N, a, row_in, row_out, stream) : launch_dct<FX, 1>(N, a, row_in, row_out, stream);
  if (a.mode >= 3)
    return arith == ARITH_F32 ? (sign < 0 ? launch_dct<F32, -1>(N, a, row_in, row_out, stream)
                                          : launch_dct<F32, 1>(N, a, row_in, row_out, stream))
                              : (sign < 0 ? launch_dct<FDD, -1>(N, a, row_in, row_out, stream)
                                          : launch_dct<FDD, 1>(N, a, row_in, row_out, stream));
  if (N & (N - 1)) {  // 3 * 2^a or 5 * 2^a: mixed-radix kernel
    const bool three = N % 3 == 0;
    if (arith == ARITH_F64)  // 64-bit fixed point
      return sign < 0 ? (three ? launch_mixed_three<FX, -1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<FX, -1>(N, a, row_in, row_out, stream))
                        : (three ? launch_mixed_three<FX, 1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<FX, 1>(N, a, row_in, row_out, stream));
    if (arith == ARITH_F32)
      return sign < 0 ? (three ? launch_mixed_three<F32, -1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<F32, -1>(N, a, row_in, row_out, stream))
                        : (three ? launch_mixed_three<F32, 1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<F32, 1>(N, a, row_in, row_out, stream));
    if (p.quant)  // block-quantised float-float butterflies
      return sign < 0 ? (three ? launch_mixed_three<FQ, -1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<FQ, -1>(N, a, row_in, row_out, stream))
                        : (three ? launch_mixed_three<FQ, 1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<FQ, 1>(N, a, row_in, row_out, stream));
    return sign < 0 ? (three ? launch_mixed_three<FDD, -1>(N, a, row_in, row_out, stream)
                               : launch_mixed_five<FDD, -1>(N, a, row_in, row_out, stream))
                      : (three ? launch_mixed_three<FDD, 1>(N, a, row_in, row_out, stream)
                               : launch_mixed_five<FDD, 1>(N, a, row_in, row_out, stream));
  }
  if (!a.plain) {  // r2c / c2r / windows / weights: the general-I/O instantiations
    if (arith == ARITH_F64 && a.pair && a.mode == 2)  // paired c2r
      return sign < 0 ? launch_gio_pinv<FX, -1>(N, a, row_in, row_out, stream)
                      : launch_gio_pinv<FX, 1>(N, a, row_in, row_out, stream);
    if (arith == ARITH_F64)
      return sign < 0 ? launch_gio<FX, -1>(N, a, row_in, row_out, stream) : launch_gio<FX, 1>(N, a, row_in, row_out, stream);
    return arith == ARITH_F32 ? (sign < 0 ? launch_gio<F32, -1>(N, a, row_in, row_out, stream)
                                          : launch_gio<F32, 1>(N, a, row_in, row_out, stream))
                              : (sign < 0 ? launch_gio<FDD, -1>(N, a, row_in, row_out, stream)
                                          : launch_gio<FDD, 1>(N, a, row_in, row_out, stream));
  }
  if (arith == ARITH_F32) {
    if (sign < 0)
      return big ? launch_large<F32, -1>(N, a, row_in, row_out, stream) : launch_small<F32, -1>(N, a, row_in, row_out, stream);
    return big ? launch_large<F32, 1>(N, a, row_in, row_out, stream) : launch_small<F32, 1>(N, a, row_in, row_out, stream);
  }
  if (arith == ARITH_F64) {  // 64-bit fixed-point radix-8 stages (plain c2c)
    if (sign < 0)
      return big ? launch_large<FX, -1>(N, a, row_in, row_out, stream) : launch_small<FX, -1>(N, a, row_in, row_out, stream);
    return big ? launch_large<FX, 1>(N, a, row_in, row_out, stream) : launch_small<FX, 1>(N, a, row_in, row_out, stream);
  }
  if (p.quant) {  // block-quantised float-float radix-8 stages
    if (sign < 0)
      return big ? launch_large<FQ, -1>(N, a, row_in, row_out, stream) : launch_small<FQ, -1>(N, a, row_in, row_out, stream);
    return big ? launch_large<FQ, 1>(N, a, row_in, row_out, stream) : launch_small<FQ, 1>(N, a, row_in, row_out, stream);
  }
  if (sign < 0)
    return big ? launch_large<FDD, -1>(N, a, row_in, row_out, stream) : launch_small<FDD, -1>(N, a, row_in, row_out, stream);
  return big ? launch_large<FDD, 1>(N, a, row_in, row_out, stream) : launch_small<FDD, 1>(N, a, row_in, row_out, stream);
}

}  // namespace pg

// Dispatcher of the register-resident radix-8 pass kernel (fft_fast.cuh).
#include "fft_fast.cuh"
#include "fft_mixed.cuh"
#include "core.h"

namespace pg {

namespace fast {
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
  if (arith != ARITH_F32 && arith != ARITH_DF) return false;
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
  if (dct) {  // Makhoul: the FFT runs on N points; the pre/post rotation uses the 4N table
    cudaError_t e;
    a->tw2 = p.tw;
    a->tw = twiddle_table(p.N, arith, &e);
    if (!a->tw) return false;
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
  // the FFT direction: the pass's, except for the DCTs (10 forward, 01 inverse)
  const int sign = a.mode == 3 ? -1 : (a.mode == 4 ? 1 : p.sign);
  if (a.mode >= 3)
    return arith == ARITH_F32 ? (sign < 0 ? launch_dct<F32, -1>(N, a, row_in, row_out, stream)
                                          : launch_dct<F32, 1>(N, a, row_in, row_out, stream))
                              : (sign < 0 ? launch_dct<FDD, -1>(N, a, row_in, row_out, stream)
                                          : launch_dct<FDD, 1>(N, a, row_in, row_out, stream));
  if (N & (N - 1)) {  // 3 * 2^a or 5 * 2^a: mixed-radix kernel
    const bool three = N % 3 == 0;
    if (arith == ARITH_F32)
      return sign < 0 ? (three ? launch_mixed_three<F32, -1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<F32, -1>(N, a, row_in, row_out, stream))
                        : (three ? launch_mixed_three<F32, 1>(N, a, row_in, row_out, stream)
                                 : launch_mixed_five<F32, 1>(N, a, row_in, row_out, stream));
    return sign < 0 ? (three ? launch_mixed_three<FDD, -1>(N, a, row_in, row_out, stream)
                               : launch_mixed_five<FDD, -1>(N, a, row_in, row_out, stream))
                      : (three ? launch_mixed_three<FDD, 1>(N, a, row_in, row_out, stream)
                               : launch_mixed_five<FDD, 1>(N, a, row_in, row_out, stream));
  }
  if (!a.plain)  // r2c / c2r / windows / weights: the general-I/O instantiations
    return arith == ARITH_F32 ? (sign < 0 ? launch_gio<F32, -1>(N, a, row_in, row_out, stream)
                                          : launch_gio<F32, 1>(N, a, row_in, row_out, stream))
                              : (sign < 0 ? launch_gio<FDD, -1>(N, a, row_in, row_out, stream)
                                          : launch_gio<FDD, 1>(N, a, row_in, row_out, stream));
  if (arith == ARITH_F32) {
    if (sign < 0)
      return big ? launch_large<F32, -1>(N, a, row_in, row_out, stream) : launch_small<F32, -1>(N, a, row_in, row_out, stream);
    return big ? launch_large<F32, 1>(N, a, row_in, row_out, stream) : launch_small<F32, 1>(N, a, row_in, row_out, stream);
  }
  if (sign < 0)
    return big ? launch_large<FDD, -1>(N, a, row_in, row_out, stream) : launch_small<FDD, -1>(N, a, row_in, row_out, stream);
  return big ? launch_large<FDD, 1>(N, a, row_in, row_out, stream) : launch_small<FDD, 1>(N, a, row_in, row_out, stream);
}

}  // namespace pg

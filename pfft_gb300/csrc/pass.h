// One "pass" = a batched 1-D transform along one axis of a strided array,
// staged through shared memory: gather a tile of lines (with zero-embedding),
// run a mixed-radix Stockham FFT of length M in shared memory, scatter the
// tile (with truncation).  Layout permutations (PFFT's TRANSPOSED_IN/OUT
// layouts), r2c/c2r Hermitian handling, r2r symmetric extensions, conjugation
// and the (-1)^k index-shift signs are all folded into the gather/scatter.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace pg {

enum ArithId { ARITH_F32 = 0, ARITH_F64 = 1, ARITH_DF = 2 };
// Twiddle table kinds besides the arithmetic ids (one table per length and
// kind, twiddle.cpp):
//   TW_DFP_FWD / _BWD: packed float-float tables of the mixed-radix kernel
//     and of the DCT rotations, entry m = W_M^(+-m) in natural order;
//   TW_F32_STG, TW_DFP_FWD_STG / _BWD_STG: the radix-8 kernel's tables in
//     stage-major order (fast_tw_count entries): radix-8 stage s (Ns = 8^s)
//     holds W_N^(k r N/(8 Ns)) at Ns - 8 + (r-1) Ns + k (r = 1..7,
//     k < Ns), the final radix-q stage (q = 2, 4) holds W_N^(j r) at
//     P - 8 + (r-1) N/q + j (P the last power of 8 dividing N), so a warp's
//     threads (consecutive k or j) read consecutive entries.
// Packed tables are stored as two arrays of float4: all high parts, then all
// low parts (FDD::W).
//   TW_FX_FWD_STG / _BWD_STG: the radix-8 kernel's stage-major tables for the
//     64-bit fixed-point arithmetic (FX::W): three arrays of int2, Re w,
//     Im w - Re w and Re w + Im w, each scaled by 2^62 (w / 4 in units of
//     2^-64) and split as hi * 2^32 + lo with lo in [-2^31, 2^31).
enum TwiddleKind {
  TW_DFP_FWD = 16,
  TW_DFP_BWD = 17,
  TW_F32_STG = 18,
  TW_DFP_FWD_STG = 19,
  TW_DFP_BWD_STG = 20,
  TW_FX_FWD_STG = 21,
  TW_FX_BWD_STG = 22,
  TW_FX_FWD = 23,  // the same format in natural order (the DCTs' length-4N rotations)
  TW_FX_BWD = 24
};
// entries of a stage-major table for a power-of-two N >= 16
inline int fast_tw_count(int N) {
  int p8 = 8;
  while (p8 * 8 <= N) p8 *= 8;
  const int q = N / p8;
  return p8 - 8 + (q - 1) * (N / q);
}

// How the logical length-N input line is turned into the length-M complex
// sequence in shared memory, and how the output line is read back.
enum PassMode {
  MODE_C2C = 0,   // complex in, complex out, M == N
  MODE_R2C = 1,   // real in, complex out (bins 0..N/2), M == N
  MODE_C2R = 2,   // complex half spectrum in, real out, M == N
  MODE_RE00 = 3,  // FFTW_REDFT00, M = 2(N-1)
  MODE_RE01 = 4,  // FFTW_REDFT01, M = 4N
  MODE_RE10 = 5,  // FFTW_REDFT10, M = 4N
  MODE_RE11 = 6,  // FFTW_REDFT11, M = 8N
  MODE_RO00 = 7,  // FFTW_RODFT00, M = 2(N+1)
  MODE_RO01 = 8,  // FFTW_RODFT01, M = 4N
  MODE_RO10 = 9,  // FFTW_RODFT10, M = 4N
  MODE_RO11 = 10, // FFTW_RODFT11, M = 8N
  MODE_R2HC = 11, // FFTW_R2HC, M = N
  MODE_HC2R = 12, // FFTW_HC2R, M = N (backward)
  MODE_DHT = 13,  // FFTW_DHT, M = N
  MODE_COPYR = 14 // real identity (skipped r2r axis), M = N
};

// (-1)^k sign pattern of PFFT's SHIFTED flags along one axis:
// factor(i) = (en && i+start < thresh) ? ((i+start odd) ? -extra : extra) : 1
struct ShiftSign {
  int en;
  int start;
  int thresh;
  int extra;
};

#define PG_MAX_BATCH 8
#define PG_MAX_STAGES 24

struct PassParams {
  const void* src;
  void* dst;
  const void* tw;      // twiddle table W_M^m, m < M, in the policy's sm_t format
  int mode;
  int sign;            // -1 forward, +1 backward (the complex FFT direction)
  int N;               // logical transform length along the axis
  int M;               // complex FFT length run in shared memory
  int Ni, Zi;          // input count and its offset in the logical sequence
  int No, Zo;          // output count and the logical offset it starts at
  long long sIa, sOa;  // element strides along the axis (input / output)
  int nb;              // batch dims (fastest first)
  long long bext[PG_MAX_BATCH];
  long long bsI[PG_MAX_BATCH];
  long long bsO[PG_MAX_BATCH];
  ShiftSign bshI[PG_MAX_BATCH];  // per batch dim sign (load side)
  ShiftSign bshO[PG_MAX_BATCH];  // per batch dim sign (store side)
  ShiftSign ashI, ashO;          // axis sign (load / store side)
  long long nlines;
  int L;        // lines per CTA
  int LS;       // shared-memory line stride (elements)
  int nst;      // number of stages
  int radix[PG_MAX_STAGES];
  int pingpong; // 1 if a generic (large prime) stage needs a second buffer
  int conj_in, conj_out;
  int wmode;    // adjoint weights: 1 = halve interior half-spectrum bins on load
                // (C2R), 2 = double interior bins on store (R2C)
  int in_contig, out_contig;  // axis has unit stride on that side
  int in_df, out_df;  // double API: complex array held as float-float pairs (intermediates)
  int threads;
  int smem_bytes;
  int kpath;    // 0: register-resident radix-8 kernel where it applies, 1: general kernel
  int fastL;    // radix-8 kernel lines per CTA (0: default for the length)
  int staged;   // staged variant of the radix-8 kernel (plain c2c passes): 0 default
                // (float column passes), 1 on where the layout allows, 2 off
  // double plans, 64-bit fixed point kept between two radix-8 passes (FX):
  // fx_out stores the mantissas (int64 pairs, the 16 bytes of a complex
  // double) and one exponent per line into lexp_out[gout_off + line]; fx_in
  // reads them, the exponent of an element being that of its line in the
  // previous pass: lexp_in[sum over this pass's batch dimensions b of the
  // pieces of (idx_b + gin_bofs[b]) + k * gin_k], k the position along this
  // pass's axis.  Batch dimension b is split into gin_np[b] pieces (mixed
  // radix, fastest first, extents gin_pext, coefficients gin_pcoef, listed
  // dimension after dimension): the previous pass's dimensions it crosses.
  int fx_in, fx_out;
  const int* lexp_in;
  int* lexp_out;
  long long lexp_in_n;  // entries of lexp_in (bound of every lookup)
  int gin_np[PG_MAX_BATCH];
  long long gin_pext[2 * PG_MAX_BATCH], gin_pcoef[2 * PG_MAX_BATCH];
  long long gin_bofs[PG_MAX_BATCH];
  long long gin_k, gout_off;
  int quant;    // double API, plain c2c passes of the radix-8 and mixed-radix
                // kernels: float-float plans (ARITH_DF) with block-quantised high
                // words (1) instead of TwoSum additions (0); double plans
                // (ARITH_F64): 2 = the radix-8 kernel's 64-bit fixed-point
                // arithmetic (fft_fast.cuh, FX) on the power-of-two passes
  // FX r2c, c2r, REDFT10 and REDFT01 passes: two real lines (adjacent along
  // batch dimension 0, whose extent is even) transformed as the real and
  // imaginary parts of one complex line; the forward kinds separate the
  // spectra after the transform, the inverse kinds (kernels of their own)
  // combine them before it (host-set when the pass qualifies; fast_args
  // halves batch dimension 0)
  int pair;
};

// Launch one pass on `stream`.  Returns a cudaError_t value.
int launch_pass(const PassParams& p, int arith, cudaStream_t stream);
// 1: use the register-resident kernel where it applies (default), 0: generic only
int kernel_path();
// true when launch_pass runs this pass on the register-resident radix-8 kernel
bool fast_pass_eligible(const PassParams& p, int arith);
// builds the twiddle tables of a radix-8 / mixed-radix pass, both directions
bool fast_pass_tables(const PassParams& p, int arith);
void set_kernel_path(int v);
// staged persistent variant of the radix-8 kernel for plain c2c passes:
// 1 per pass as PassParams::staged says (default), 2 wherever the layout
// allows, 0 off (PFFT_GB300_STAGED=0/1/2)
int staged_mode();
void set_staged_mode(int v);
long long staged_launches();  // staged launches so far in this process
int* staged_err_word_if_any();  // the current device's error word, or null if none was made

// Shared-memory element size of a policy.
inline int arith_sm_bytes(int arith) { return arith == ARITH_F32 ? 8 : 16; }

}  // namespace pg

// Register-resident radix-8 pass for power-of-two c2c lines (16..4096).
//
// The generic pass (fft_pass.cu) stages every stage through shared memory and
// handles every mode.  This kernel covers the hot case - a plain c2c line
// transform with no embedding, truncation or index-shift signs - with:
//   * each thread owning one radix-8 butterfly per stage (N/8 threads a line),
//     eight complex values held in registers;
//   * stage 1 loading straight from global memory and the last stage storing
//     straight to global memory, both coalesced (consecutive threads walk the
//     contiguous direction: along the line for rows, across lines for
//     columns); only the stages in between exchange through shared memory
//     (one buffer, two barriers per exchange);
//   * a shared-memory layout (pad, lsp_of) that keeps the stage exchanges
//     free of bank conflicts;
//   * for the double API, float-float arithmetic with unnormalised additions
//     (TwoSum on the high parts, plain sums of the low parts); values cross
//     the shared-memory exchanges unnormalised (an unevaluated sum hi + lo
//     whose low part is a sum of rounding errors: its own rounding error is
//     2^-24 |lo|, below 2^-45 of the operands' magnitude), and are
//     renormalised only when written to global memory.
// A length N = 8^a * q (q = 1, 2, 4) runs a radix-8 stages and one radix-q stage.
#pragma once
#include <limits.h>
#include <algorithm>
#include <type_traits>
#include "arith.cuh"
#include "pass.h"
#include "tma.cuh"

namespace pg {

namespace fast {

// ---- arithmetic -----------------------------------------------------------------
struct F32 {
  typedef float2 S;   // shared / twiddle element
  typedef float2 G;   // global element
  typedef float2 C;
  static __device__ __forceinline__ C add(C a, C b) { return make_float2(a.x + b.x, a.y + b.y); }
  static __device__ __forceinline__ C sub(C a, C b) { return make_float2(a.x - b.x, a.y - b.y); }
  static __device__ __forceinline__ C mul(C a, S w) {
    return make_float2(__fmaf_rn(a.x, w.x, -a.y * w.y), __fmaf_rn(a.x, w.y, a.y * w.x));
  }
  static __device__ __forceinline__ C scal(C a, float c) { return make_float2(a.x * c, a.y * c); }
  static __device__ __forceinline__ C neg(C a) { return make_float2(-a.x, -a.y); }
  static __device__ __forceinline__ C swap_neg_re(C a) { return make_float2(-a.y, a.x); }  // *i
  static __device__ __forceinline__ C swap_neg_im(C a) { return make_float2(a.y, -a.x); }  // *(-i)
  static __device__ __forceinline__ C renorm(C a) { return a; }
  static __device__ __forceinline__ C tw0(C a) { return a; }
  static __device__ __forceinline__ C ld(const G* p) { return *p; }
  static __device__ __forceinline__ void st(G* p, C v) { *p = v; }
  static __device__ __forceinline__ C lds(const S& s) { return s; }
  static __device__ __forceinline__ S sts(C v) { return v; }
  static __device__ __forceinline__ S twc(S w, int sign) { return sign < 0 ? w : make_float2(w.x, -w.y); }
  // twiddles: the forward table W_M^m, conjugated for SIGN > 0
  typedef float2 W;
  static __device__ __forceinline__ W ldw(const void* base, int idx, int) { return __ldg((const W*)base + idx); }
  template <int SIGN>
  static __device__ __forceinline__ W twd(W w) {
    return twc(w, SIGN);
  }
  static __device__ __forceinline__ C conj(C a) { return make_float2(a.x, -a.y); }
  static __device__ __forceinline__ float c8() { return 0.70710678118654752440f; }
};

// lazily-normalised float-float
struct DD {
  float hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  float s = __fadd_rn(a.hi, b.hi);
  float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return {s, __fadd_rn(__fadd_rn(a.lo, b.lo), e)};
}
__device__ __forceinline__ DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DD dd_sub(DD a, DD b) { return dd_add(a, dd_neg(b)); }
__device__ __forceinline__ DD dd_norm(DD a) {
  float s = __fadd_rn(a.hi, a.lo);
  return {s, __fsub_rn(a.lo, __fsub_rn(s, a.hi))};
}
// a * c with c a normalised constant
__device__ __forceinline__ DD dd_mulc(DD a, DD c) {
  float p = __fmul_rn(a.hi, c.hi);
  float e = __fmaf_rn(a.hi, c.hi, -p);
  e = __fmaf_rn(a.hi, c.lo, e);
  e = __fmaf_rn(a.lo, c.hi, e);
  return {p, e};
}
// a*b - c*d (b, d normalised)
__device__ __forceinline__ DD dd_mms(DD a, DD b, DD c, DD d) {
  float p1 = __fmul_rn(a.hi, b.hi);
  float e1 = __fmaf_rn(a.hi, b.hi, -p1);
  float p2 = __fmul_rn(c.hi, d.hi);
  float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  float s = __fsub_rn(p1, p2);
  float bb = __fsub_rn(s, p1);
  float e = __fsub_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fadd_rn(p2, bb));
  e = __fadd_rn(e, __fsub_rn(e1, e2));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(-c.hi, d.lo, e);
  e = __fmaf_rn(-c.lo, d.hi, e);
  return {s, e};
}

// Packed two-lane FP32 arithmetic (FADD2 / FMUL2 / FFMA2, sm_100 and
// later): one instruction does the same operation on both floats of a pair,
// so float-float complex arithmetic on the pairs (re, im) issues half the
// instructions of its scalar form.  Negated operands are written as negated
// pairs for the compiler to fold into the instruction.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Float-float complex, packed: h = (re.hi, im.hi), l = (re.lo, im.lo).
// Twiddles come from direction-specific tables (twiddle table kinds
// TW_DFP_*) of two float4 per entry, w = wr + i wi:
//   h = (wr.hi, wr.hi, -wi.hi, wi.hi), l = (wr.lo, wr.lo, -wi.lo, wi.lo),
// the pairs of (re, im) = a (wr, wr) + swap(a) (-wi, wi), so no pair is built
// at run time but the swapped operand; all h of a table come first, then
// all l, so that a warp reading consecutive entries reads contiguous memory.
struct FDD {
  typedef float4 S;   // shared memory: (re.hi, im.hi, re.lo, im.lo)
  typedef double2 G;
  struct W {
    float4 h, l;
  };
  struct C {
    float2 h, l;
  };
  // TwoSum on the high pairs, plain sums of the low pairs (unnormalised)
  static __device__ __forceinline__ C add(C a, C b) {
    const float2 s = add2(a.h, b.h);
    const float2 bb = sub2(s, a.h);
    const float2 e = add2(sub2(a.h, sub2(s, bb)), sub2(b.h, bb));
    return {s, add2(add2(a.l, b.l), e)};
  }
  // a + (-b) with the same steps
  static __device__ __forceinline__ C sub(C a, C b) {
    const float2 s = sub2(a.h, b.h);
    const float2 bb = sub2(s, a.h);
    const float2 e = sub2(sub2(a.h, sub2(s, bb)), add2(b.h, bb));
    return {s, add2(sub2(a.l, b.l), e)};
  }
  static __device__ __forceinline__ C mul(C a, const W& w) {
    const float2 sh = make_float2(a.h.y, a.h.x), sl = make_float2(a.l.y, a.l.x);
    const float2 wr = make_float2(w.h.x, w.h.y), wi = make_float2(w.h.z, w.h.w);
    const float2 wrl = make_float2(w.l.x, w.l.y), wil = make_float2(w.l.z, w.l.w);
    const float2 P = mul2(a.h, wr);         // (x wr, y wr)
    const float2 nEP = fma2(a.h, neg2(wr), P);  // minus its rounding error, exact
    const float2 Q = mul2(sh, wi);          // (-y wi, x wi)
    const float2 nEQ = fma2(sh, neg2(wi), Q);
    const float2 s = add2(P, Q);
    const float2 bb = sub2(s, P);
    float2 e = add2(sub2(P, sub2(s, bb)), sub2(Q, bb));
    e = sub2(sub2(e, nEP), nEQ);
    e = fma2(a.h, wrl, e);
    e = fma2(a.l, wr, e);
    e = fma2(sh, wil, e);
    e = fma2(sl, wi, e);
    return {s, e};
  }
  // product with a real float-float constant, per component (scalar FMAs
  // take the constant as an immediate)
  static __device__ __forceinline__ C scal(C a, DD c) {
    const DD x = dd_mulc(DD{a.h.x, a.l.x}, c), y = dd_mulc(DD{a.h.y, a.l.y}, c);
    return {make_float2(x.hi, y.hi), make_float2(x.lo, y.lo)};
  }
  static __device__ __forceinline__ C neg(C a) {
    return {make_float2(-a.h.x, -a.h.y), make_float2(-a.l.x, -a.l.y)};
  }
  static __device__ __forceinline__ C swap_neg_re(C a) {  // * i
    return {make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)};
  }
  static __device__ __forceinline__ C swap_neg_im(C a) {  // * (-i)
    return {make_float2(a.h.y, -a.h.x), make_float2(a.l.y, -a.l.x)};
  }
  static __device__ __forceinline__ C renorm(C a) {
    const float2 s = add2(a.h, a.l);
    return {s, sub2(a.l, sub2(s, a.h))};
  }
  static __device__ __forceinline__ C tw0(C a) { return a; }
  static __device__ __forceinline__ C from_df(df re, df im) {
    return {make_float2(re.hi, im.hi), make_float2(re.lo, im.lo)};
  }
  static __device__ __forceinline__ df re_df(C v) { return df{v.h.x, v.l.x}; }
  static __device__ __forceinline__ df im_df(C v) { return df{v.h.y, v.l.y}; }
  static __device__ __forceinline__ C ld(const G* p) {
    G v = *p;
    return from_df(df_from_double(v.x), df_from_double(v.y));
  }
  static __device__ __forceinline__ void st(G* p, C v) {
    double re, im;
    df_pair_to_double(re_df(v), im_df(v), re, im);
    *p = make_double2(re, im);
  }
  static __device__ __forceinline__ C lds(const S& s) { return {make_float2(s.x, s.y), make_float2(s.z, s.w)}; }
  static __device__ __forceinline__ S sts(C v) { return make_float4(v.h.x, v.h.y, v.l.x, v.l.y); }
  // entry idx of a table of cnt entries (high parts, then low parts)
  static __device__ __forceinline__ W ldw(const void* base, int idx, int cnt) {
    const float4* t = (const float4*)base;
    return {__ldg(t + idx), __ldg(t + cnt + idx)};
  }
  // twiddle of direction SIGN: the tables are direction-specific already
  template <int SIGN>
  static __device__ __forceinline__ W twd(const W& w) {
    return w;
  }
  static __device__ __forceinline__ C conj(C a) { return {make_float2(a.h.x, -a.h.y), make_float2(a.l.x, -a.l.y)}; }
  static __device__ __forceinline__ DD c8() {
    return {(float)0.70710678118654752440, (float)(0.70710678118654752440 - (double)(float)0.70710678118654752440)};
  }
};

// constants of a policy: a double split at compile time into float hi + lo
template <class P>
struct Kc;
template <>
struct Kc<F32> {
  static __device__ __forceinline__ float k(float h, float) { return h; }
};
template <>
struct Kc<FDD> {
  static __device__ __forceinline__ DD k(float h, float l) { return {h, l}; }
};
// a double constant split at compile time into float hi + lo
#define PG_KC(P, c) Kc<P>::k((float)(c), (float)((c) - (double)(float)(c)))

// multiply by SIGN*i
template <class P, int SIGN>
__device__ __forceinline__ typename P::C msi(typename P::C a) {
  return SIGN < 0 ? P::swap_neg_im(a) : P::swap_neg_re(a);
}

template <class P, int SIGN>
__device__ __forceinline__ void bf4(typename P::C& a0, typename P::C& a1, typename P::C& a2, typename P::C& a3) {
  typedef typename P::C C;
  C t0 = P::add(a0, a2), t1 = P::sub(a0, a2);
  C t2 = P::add(a1, a3), t3 = msi<P, SIGN>(P::sub(a1, a3));
  a0 = P::add(t0, t2);
  a2 = P::sub(t0, t2);
  a1 = P::add(t1, t3);
  a3 = P::sub(t1, t3);
}

// in-place radix-8 DFT, natural order in and out
template <class P, int SIGN>
__device__ __forceinline__ void bf8(typename P::C* v) {
  typedef typename P::C C;
  bf4<P, SIGN>(v[0], v[2], v[4], v[6]);
  bf4<P, SIGN>(v[1], v[3], v[5], v[7]);
  const auto c = P::c8();
  // W8^1 z = c (z + S i z);  W8^3 z = c (S i z - z)
  C o1 = P::scal(P::add(v[3], msi<P, SIGN>(v[3])), c);
  C o3 = P::scal(P::sub(msi<P, SIGN>(v[7]), v[7]), c);
  C o2 = msi<P, SIGN>(v[5]);
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = P::add(e0, o0);
  v[4] = P::sub(e0, o0);
  v[1] = P::add(e1, o1);
  v[5] = P::sub(e1, o1);
  v[2] = P::add(e2, o2);
  v[6] = P::sub(e2, o2);
  v[3] = P::add(e3, o3);
  v[7] = P::sub(e3, o3);
}

// ---- block-quantised float-float radix-8 butterflies -----------------------------
// FQ: float-float values whose high words are rounded, before each radix-8
// butterfly, to a grid common to the butterfly, so that every addition of
// high words inside it is exact and needs no TwoSum (2 packed operations per
// complex addition instead of 8).  With m the largest high word of the
// butterfly's 16 components, m < 2^(T-4), the grid is q = 2^(T-24): every
// partial sum of the butterfly is bounded by (4 + 4 sqrt 2) m < 2^T (the
// sqrt(1/2) products included), so every sum of grid points is a float.
// Rounding h to the grid adds h - round(h) (|.| <= q/2) to the low word, whose
// own rounding is then 2^-24 of a larger low word: the error of a stage is
// about 2^-45 of the butterfly's largest component (relative L2 error about
// 1e-13 per 512-point pass on uniform data, against 1e-14 for the TwoSum
// form).  Loads, stores, twiddle products and the radix-2/4 stage are those
// of FDD.
struct FQ : FDD {};

// h rounded to the grid of c (c = 1.5 * 2^(T-1) or 1.5 * 2^T: ulp(c) = q or
// 2q), the difference moved to the low word
__device__ __forceinline__ FDD::C fq_round(FDD::C a, float2 c) {
  const float2 hq = sub2(add2(a.h, c), c);
  return {hq, add2(a.l, sub2(a.h, hq))};
}
__device__ __forceinline__ FDD::C fq_add(FDD::C a, FDD::C b) { return {add2(a.h, b.h), add2(a.l, b.l)}; }
__device__ __forceinline__ FDD::C fq_sub(FDD::C a, FDD::C b) { return {sub2(a.h, b.h), sub2(a.l, b.l)}; }
// sqrt(1/2) * a (exact product of the high words: value + error), high word
// back on the grid with c2 = 1.5 * 2^T (|product| <= 4 sqrt 2 m < 2^(T-1.5))
__device__ __forceinline__ FDD::C fq_c8(FDD::C a, float2 c2) {
  constexpr double k = 0.70710678118654752440;
  const float2 ch = make_float2((float)k, (float)k);
  const float2 cl = make_float2((float)(k - (double)(float)k), (float)(k - (double)(float)k));
  const float2 p = mul2(a.h, ch);
  float2 e = fma2(a.h, ch, neg2(p));
  e = fma2(a.h, cl, e);
  e = fma2(a.l, ch, e);
  const float2 pq = sub2(add2(p, c2), c2);
  return {pq, add2(e, sub2(p, pq))};
}
template <int SIGN>
__device__ __forceinline__ void fq_bf4(FDD::C& a0, FDD::C& a1, FDD::C& a2, FDD::C& a3) {
  FDD::C t0 = fq_add(a0, a2), t1 = fq_sub(a0, a2);
  FDD::C t2 = fq_add(a1, a3), t3 = msi<FDD, SIGN>(fq_sub(a1, a3));
  a0 = fq_add(t0, t2);
  a2 = fq_sub(t0, t2);
  a1 = fq_add(t1, t3);
  a3 = fq_sub(t1, t3);
}
// in-place radix-8 DFT of unnormalised float-float values (natural order)
template <int SIGN>
__device__ __forceinline__ void bf8q(FDD::C* v) {
  float m = fmaxf(fabsf(v[0].h.x), fabsf(v[0].h.y));
#pragma unroll
  for (int r = 1; r < 8; r++) m = fmaxf(m, fmaxf(fabsf(v[r].h.x), fabsf(v[r].h.y)));
  // m < 2^(e-126) for the biased exponent e of m: T = e - 122; the clamp keeps
  // c2 finite (magnitudes near the float limit overflow the sums anyway)
  const unsigned eb = min(__float_as_uint(m) & 0x7F800000u, 249u << 23);
  const float c1s = __uint_as_float(eb + (4u << 23) + 0x400000u);  // 1.5 * 2^(T-1)
  const float c2s = __uint_as_float(eb + (5u << 23) + 0x400000u);  // 1.5 * 2^T
  const float2 c1 = make_float2(c1s, c1s), c2 = make_float2(c2s, c2s);
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = fq_round(v[r], c1);
  fq_bf4<SIGN>(v[0], v[2], v[4], v[6]);
  fq_bf4<SIGN>(v[1], v[3], v[5], v[7]);
  // W8^1 z = c (z + S i z);  W8^3 z = c (S i z - z)
  const FDD::C o1 = fq_c8(fq_add(v[3], msi<FDD, SIGN>(v[3])), c2);
  const FDD::C o3 = fq_c8(fq_sub(msi<FDD, SIGN>(v[7]), v[7]), c2);
  const FDD::C o2 = msi<FDD, SIGN>(v[5]);
  const FDD::C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = fq_add(e0, o0);
  v[4] = fq_sub(e0, o0);
  v[1] = fq_add(e1, o1);
  v[5] = fq_sub(e1, o1);
  v[2] = fq_add(e2, o2);
  v[6] = fq_sub(e2, o2);
  v[3] = fq_add(e3, o3);
  v[7] = fq_sub(e3, o3);
}
// the radix-8 butterfly of a policy
template <class P, int SIGN>
__device__ __forceinline__ void bf8x(typename P::C* v) {
  if constexpr (std::is_same<P, FQ>::value)
    bf8q<SIGN>(v);
  else
    bf8<P, SIGN>(v);
}

// ---- 64-bit block-fixed-point arithmetic (double API) -------------------------
// FX: the double API's arithmetic of the radix-8 kernel.  A tile's values
// are converted, after loading, to 64-bit integers on one grid common to the
// tile: with E the largest biased exponent of the tile's doubles, a double
// m * 2^(e - 1075) (53-bit mantissa m) becomes X = (m << 5) >> (E - e), so
// x = X * 2^(E - 1080) and |X| < 2^58: 58 significant bits against the
// tile's largest component (a double holds 53 against its own magnitude).
// Additions and subtractions are exact 64-bit integer operations.  Before
// every stage but the first the tile is renormalised (block floating point
// per stage): at the shared-memory exchange each warp ORs the high words of
// its values' magnitudes, the tile's OR gives the bit length of its largest
// component (within one bit), and every value is shifted left or right by
// the same amount so that the largest stays below 2^60 (fx_normalise).  The
// stage's twiddles are scaled by 1/4 (element 0 of a butterfly, whose
// twiddle is 1, is shifted right by 2), so a butterfly's inputs have modulus
// below 2^58.5, its partial sums and outputs below 2^61.5 and the twiddle
// product's sum a.re + a.im below 2^61: nothing overflows whatever the
// data, and data that does not grow (a spike spreading into a flat
// spectrum) keeps its bits instead of paying for the worst-case growth.
// Products are 64 x 64 -> high 64 bits from 32-bit pieces (mh: the
// low-by-low part and the carries of the cross terms are dropped, error
// within 2 units of the result), complex products in Gauss's
// three-multiplication form, the sqrt(1/2) products of the butterflies as
// a - a (1 - sqrt(1/2)).  Every rounding is a few units at 2^-58..2^-56 of
// the tile's current magnitude, below the 2^-53 relative rounding of FP64
// arithmetic.  Results are rounded to nearest double when stored
// (x = Y * 2^(E - 1080 + the stages' shifts)).  A tile holding an infinity
// or NaN stores NaN everywhere; results below 2^-1022 are stored as zero.
// 32x32 -> 64-bit signed products, alone or added to a 64-bit value, as one
// mul.wide / mad.wide each, so that a chain of them accumulates in the
// multiplier's own 64-bit adder
__device__ __forceinline__ long long fx_mulw(int a, int b) {
  long long d;
  asm("mul.wide.s32 %0, %1, %2;" : "=l"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ long long fx_madw(int a, int b, long long c) {
  long long d;
  asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
  return d;
}

struct FX {
  typedef longlong2 S;  // shared memory: (re, im)
  typedef double2 G;
  struct C {
    long long x, y;
  };
  // twiddle w / 4 = c + i s scaled by 2^64, each part stored as (hi, lo),
  // value hi * 2^32 + lo with lo in [-2^31, 2^31): a = (c.hi, c.lo, s.hi,
  // s.lo), n = -s (split on its own, so no negation can overflow)
  struct W {
    int4 a;
    int2 n;
  };
  struct K8 {};  // tag of the sqrt(1/2) constant
  static __device__ __forceinline__ C add(C a, C b) { return {a.x + b.x, a.y + b.y}; }
  static __device__ __forceinline__ C sub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
  static __device__ __forceinline__ C neg(C a) { return {-a.x, -a.y}; }
  static __device__ __forceinline__ C swap_neg_re(C a) { return {-a.y, a.x}; }  // * i
  static __device__ __forceinline__ C swap_neg_im(C a) { return {a.y, -a.x}; }  // * (-i)
  static __device__ __forceinline__ C renorm(C a) { return a; }
  static __device__ __forceinline__ C conj(C a) { return {a.x, -a.y}; }
  static __device__ __forceinline__ C lds(const S& s) { return {s.x, s.y}; }
  static __device__ __forceinline__ S sts(C v) { return make_longlong2(v.x, v.y); }
  // x * w / 2^64 rounded to the nearest unit, within 3/4 of a unit: x = xh
  // 2^32 + xl, w = wh 2^32 + wl with signed low halves; xh * wh plus the two
  // cross terms, summed exactly in 64 bits (|x|, |w| < 2^62.5 keep each
  // below 2^61.5) and rounded once; the low-by-low part (below 1/4 of a
  // unit, of either sign) is dropped.  Without a systematic loss no
  // correction term is needed: 0 maps to 0, and errors do not pile up in
  // one output bin (a floor's steady half unit would, in proportion to
  // sqrt(N) of the result's norm).
  static __device__ __forceinline__ long long mh(long long x, int2 w) {
    const unsigned xu = (unsigned)x;
    const int xl = (int)xu;
    const int xh = (int)(x >> 32) + (int)(xu >> 31);
    const long long s = fx_madw(xl, w.x, fx_mulw(xh, w.y));
    const int c = (int)(s >> 32) + (int)((unsigned)s >> 31);
    return fx_madw(xh, w.x, (long long)c);
  }
  // (x + i y) (c + i s) / 2^64, each part rounded once: with x = xh 2^32 +
  // xl and y, c, s split alike, Re = xh ch - yh sh + round(m / 2^32), m = xh
  // cl + xl ch - yh sl - yl sh (exact in 64 bits: |x|, |y| < 2^60 and |c|,
  // |s| <= 2^62 keep each term below 2^61), Im alike; the low-by-low terms
  // (below 1/2 of a unit together) are dropped.  Twelve 32x32->64-bit
  // multiply-adds and a few integer adds per product, within 1 unit.
  static __device__ __forceinline__ C mul(C a, const W& w) {
    const unsigned xu = (unsigned)a.x, yu = (unsigned)a.y;
    const int xl = (int)xu, yl = (int)yu;
    const int xh = (int)(a.x >> 32) + (int)(xu >> 31), yh = (int)(a.y >> 32) + (int)(yu >> 31);
    const long long rm = fx_madw(yl, w.n.x, fx_madw(yh, w.n.y, fx_madw(xl, w.a.x, fx_mulw(xh, w.a.y))));
    const long long im = fx_madw(yl, w.a.x, fx_madw(yh, w.a.y, fx_madw(xl, w.a.z, fx_mulw(xh, w.a.w))));
    const int rc = (int)(rm >> 32) + (int)((unsigned)rm >> 31);
    const int ic = (int)(im >> 32) + (int)((unsigned)im >> 31);
    return {fx_madw(xh, w.a.x, fx_madw(yh, w.n.x, (long long)rc)), fx_madw(xh, w.a.z, fx_madw(yh, w.a.x, (long long)ic))};
  }
  static __device__ __forceinline__ K8 c8() { return {}; }
  // a * sqrt(1/2) = a - a (1 - sqrt(1/2)), the product rounded
  static __device__ __forceinline__ C scal(C a, K8) {
    const int2 k = make_int2(1257966796, 102865788);  // (1 - sqrt(1/2)) 2^64
    return {a.x - mh(a.x, k), a.y - mh(a.y, k)};
  }
  // element 0 of a twiddled stage (twiddle 1, scaled by 1/4, rounded to nearest)
  static __device__ __forceinline__ C tw0(C a) { return {(a.x + 2) >> 2, (a.y + 2) >> 2}; }
  static __device__ __forceinline__ W ldw(const void* base, int idx, int cnt) {
    const int4* t = (const int4*)base;
    return {__ldg(t + idx), __ldg((const int2*)(t + cnt) + idx)};
  }
  template <int SIGN>
  static __device__ __forceinline__ W twd(const W& w) {
    return w;  // direction-specific tables
  }
};
template <class P>
__host__ __device__ constexpr bool is_fx() {
  return std::is_same<P, FX>::value;
}

// double bits -> X on the tile grid of largest biased exponent E (E >= 1)
__device__ __forceinline__ long long fx_from_bits(long long b, int E) {
  const unsigned long long u = (unsigned long long)b;
  const int e = (int)(u >> 52) & 0x7FF;
  const unsigned long long m = (u & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  const int d = min(E - max(e, 1), 63);
  const long long X = (long long)((m << 5) >> d);
  return b < 0 ? -X : X;
}
// Y * 2^eo rounded to the nearest double (ties away from zero); eo == INT_MIN:
// NaN.  When every value of the tile lands in the normal range (-1022 <= eo
// <= 960 with |Y| < 2^63, the same branch in every thread) the rounding is
// branch-free: |Y| normalised by its leading-zero count, 53 bits kept plus
// the next bit as the rounding increment, whose carry into bit 53 moves into
// the exponent field by itself.
__device__ __forceinline__ double fx_to_double(long long Y, int eo) {
  if (eo >= -1022 && eo <= 960) {
    const long long sg = Y >> 63;
    const unsigned long long a = (unsigned long long)((Y ^ sg) - sg);
    const int lz = __clzll((long long)a);
    const unsigned long long n = a << (lz & 63);
    const unsigned long long m = (n >> 11) + ((n >> 10) & 1ull);  // 2^52 <= m <= 2^53
    const unsigned long long bits = ((unsigned long long)(eo + 1085 - lz) << 52) + m;
    return __longlong_as_double(a ? (long long)(bits | ((unsigned long long)sg & 0x8000000000000000ull)) : 0ll);
  }
  if (eo == INT_MIN) return __longlong_as_double(0x7FF8000000000000ll);
  const unsigned long long sgn = (unsigned long long)Y & 0x8000000000000000ull;
  const unsigned long long a = Y < 0 ? (unsigned long long)(-Y) : (unsigned long long)Y;
  if (a == 0) return 0.0;
  const int lz = __clzll((long long)a);
  const unsigned long long n = a << lz;  // bit 63 set
  unsigned long long mant = (n >> 11) + ((n >> 10) & 1ull);  // ties away, as the fast path
  int eb = eo + 1086 - lz;
  if (mant >> 53) {
    mant >>= 1;
    eb++;
  }
  if (eb <= 0) return __longlong_as_double((long long)sgn);  // below 2^-1022: zero
  if (eb >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)eb << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}
// The tile's entry into FX: v holds the thread's eight values as double bits
// (gload<FX>); every thread of the block takes part (one barrier).  Returns
// the exponent of the stored results (fx_to_double) for a length-N line.
template <int N, int K = 8>
__device__ __forceinline__ int fx_enter(FX::C (&v)[K], int conj_in) {
  __shared__ unsigned red[32];
  unsigned em = 0;
#pragma unroll
  for (int r = 0; r < K; r++) {
    em = max(em, (unsigned)(v[r].x >> 32) & 0x7FF00000u);
    em = max(em, (unsigned)(v[r].y >> 32) & 0x7FF00000u);
  }
  em = __reduce_max_sync(0xffffffffu, em);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = em;
  __syncthreads();
  em = lane < (int)(blockDim.x >> 5) ? red[lane] : 0u;
  em = __reduce_max_sync(0xffffffffu, em);
  const int Eraw = (int)(em >> 20);
  const int E = max(Eraw, 1);
#pragma unroll
  for (int r = 0; r < K; r++) {
    v[r].x = fx_from_bits(v[r].x, E);
    v[r].y = fx_from_bits(v[r].y, E);
    if (conj_in) v[r].y = -v[r].y;
  }
  return Eraw == 0x7FF ? INT_MIN : E - 1080;
}

// The tile's entry when its input holds FX mantissas of the previous pass
// (fx_in): element r's value is v[r] * 2^ex[r], |v[r]| < 2^58 (stored
// normalised, fx_store_normalise).  The new grid is 2^(max ex): the line with
// the largest exponent keeps its mantissas, the others are shifted right to
// it, rounded to nearest; an exponent INT_MAX (a previous tile that held an
// infinity or NaN) makes the tile NaN.  Returns the exponent of the grid.
__device__ __forceinline__ int fx_enter_linked(FX::C (&v)[8], const int (&ex)[8], int conj_in) {
  __shared__ int red[32];
  int em = ex[0];
#pragma unroll
  for (int r = 1; r < 8; r++) em = max(em, ex[r]);
  em = __reduce_max_sync(0xffffffffu, em);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = em;
  __syncthreads();
  em = lane < (int)(blockDim.x >> 5) ? red[lane] : INT_MIN;
  em = __reduce_max_sync(0xffffffffu, em);
  if (em == INT_MAX) return INT_MIN;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int d = min(em - ex[r], 62);
    if (d > 0) {
      const long long h = 1ll << (d - 1);
      v[r].x = (v[r].x + h) >> d;
      v[r].y = (v[r].y + h) >> d;
    }
    if (conj_in) v[r].y = -v[r].y;
  }
  return em;
}

// Block normalisation of a stage (see FX): fx_ormag before the exchange's
// barrier (each warp's OR of |high words| into slot[warp]), fx_normal_shift
// after it (the tile's shift: the largest component below 2^60), fx_shift
// on every value.
template <int K>
__device__ __forceinline__ unsigned fx_ormag(const FX::C (&v)[K]) {
  unsigned acc = 0;
#pragma unroll
  for (int r = 0; r < K; r++) {
    const int hx = (int)(v[r].x >> 32), hy = (int)(v[r].y >> 32);
    acc |= (unsigned)(hx ^ (hx >> 31)) | (unsigned)(hy ^ (hy >> 31));
  }
  return acc;
}
__device__ __forceinline__ void fx_ormag_publish(unsigned m, unsigned* slot) {
  m = __reduce_or_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) slot[threadIdx.x >> 5] = m;
}
// right shift (> 0) or left shift (< 0) bringing the bit length of the
// tile's largest component to at most `bits` (60 before a stage, 58 for
// mantissas stored for the next pass; the OR of the high words gives it
// within one bit: an exact negative power of two reads one bit short)
__device__ __forceinline__ int fx_normal_shift(const unsigned* slot, int bits = 60) {
  const int lane = threadIdx.x & 31;
  unsigned m = lane < (int)(blockDim.x >> 5) ? slot[lane] : 0u;
  m = __reduce_or_sync(0xffffffffu, m);
  const int bl = 32 + (m ? 32 - __clz((int)m) : 0);
  return bl - (bits - 1);
}
// v * 2^-s for every value, -31 < s < 32, rounded to nearest (ties up) for
// s > 0, exact for s <= 0 (no value loses a bit: the tile's largest is below
// 2^32 when s < 0).  s is the same in every thread of the block: one
// uniform branch picks the direction, and each value costs a 64-bit add and
// shift or a shift alone.
template <int K>
__device__ __forceinline__ void fx_shift_all(FX::C (&v)[K], int s) {
  if (s > 0) {
    const long long h = 1ll << (s - 1);
#pragma unroll
    for (int r = 0; r < K; r++) v[r] = {(v[r].x + h) >> s, (v[r].y + h) >> s};
  } else if (s < 0) {
#pragma unroll
    for (int r = 0; r < K; r++) v[r] = {v[r].x << -s, v[r].y << -s};
  }
}
__device__ __forceinline__ unsigned* fx_slots() {
  __shared__ unsigned slots[2][32];  // per-warp ORs of two consecutive stages
  return &slots[0][0];
}
// Results kept for the next pass (fx_out): the tile renormalised so that its
// largest component is below 2^58 (one more barrier); returns the shift to
// add to the results' exponent.  slot: the parity the last exchange did not
// use (every thread has passed its reads).
template <int K>
__device__ __forceinline__ int fx_store_normalise(FX::C (&v)[K], unsigned* slot) {
  unsigned acc = 0;
#pragma unroll
  for (int r = 0; r < K; r++) {
    const int hx = (int)(v[r].x >> 32), hy = (int)(v[r].y >> 32);
    acc |= (unsigned)(hx ^ (hx >> 31)) | (unsigned)(hy ^ (hy >> 31));
  }
  fx_ormag_publish(acc, slot);
  __syncthreads();
  const int sh = fx_normal_shift(slot, 58);
  fx_shift_all(v, sh);
  return sh;
}

// Shared-memory layout of a tile: L lines at stride lsp_of, element p of a
// line at index pad(p).  The layouts below make every stage exchange of the
// kernel free of bank conflicts; they were chosen by simulating the
// exchanges' shared-memory addresses (wavefronts per warp access) for every
// instantiated length, tile height and orientation.
//   FP32 (8-byte elements): an XOR swizzle of the low four bits by bits 3..6
//     (a permutation of [0, N)); column tiles (adjacent lines in one warp)
//     spread the lines' starts with 16/L extra elements, short row tiles hold
//     several lines per warp and need N/8.
//   float-float (16-byte elements): p + p/8 (one instruction: these kernels
//     are bound by instruction issue) and a stride of N + N/8 + 1, with 2 or 4
//     more for column tiles of 4 or 2 lines.
template <class P>
__device__ __forceinline__ int pad(int p) {
  return sizeof(typename P::S) == 8 ? (p ^ ((p >> 3) & 15)) : (p + (p >> 3));
}

template <class P, int N, int L, bool ROW>
__host__ __device__ constexpr int lsp_of() {
  return sizeof(typename P::S) == 8
             ? N + (ROW ? (N >= 128 ? 0 : (N == 64 ? 8 : N / 8)) : (L == 1 ? 0 : (16 / L > 1 ? 16 / L : 1)))
             : N + N / 8 + (ROW ? (N <= 32 ? 0 : 1) : (L >= 8 || L == 1 ? 1 : (L == 4 ? 2 : 4)));
}

__host__ __device__ constexpr int n8_of(int N) { return N >= 4096 ? 4 : (N >= 512 ? 3 : (N >= 64 ? 2 : 1)); }
__host__ __device__ constexpr int pow8(int a) { return a == 4 ? 4096 : (a == 3 ? 512 : (a == 2 ? 64 : 8)); }
// entries of the radix-8 kernel's stage-major twiddle table (fast_tw_count)
__host__ __device__ constexpr int fast_tw_n(int N) {
  return pow8(n8_of(N)) - 8 + (N / pow8(n8_of(N)) - 1) * pow8(n8_of(N));
}

struct FastArgs {
  const void* src;
  void* dst;
  const void* tw;
  long long sIa, sOa;
  int nb;
  long long bext[PG_MAX_BATCH];
  long long bsI[PG_MAX_BATCH];
  long long bsO[PG_MAX_BATCH];
  long long nlines;
  int conj_in, conj_out;
  int in_df, out_df;  // double API: the array holds float-float pairs (an intermediate)
  int fastL;          // requested lines per CTA (0: default): 512 takes 2, 4, 8, 16; 1024 takes 2, 4, 8;
                      // 2048 takes 2, 4; 4096 takes 1, 2
  // logical sequence of a line (pass_tile.cuh semantics): element e of the
  // length-N input is input element e - Zi when 0 <= e - Zi < Ni, else 0
  // (zero-padding); for c2r the position is first folded to the half
  // spectrum (k = e or N - e, the mirrored half conjugated); output element
  // k is logical position Zo + k, k < No (truncation); r2c reads real input,
  // c2r writes the real parts.  plain: c2c with the whole line on both sides.
  // REDFT10 / REDFT01 (real-to-real DCT-II / DCT-III, Makhoul's method on a
  // length-N complex FFT): 10 loads v[m] = x[2m] (m < N/2) or x[2(N-1-m)+1]
  // and stores y_k = 2 Re(W_4N^k V_k); 01 loads (x_k - i x_(N-k)) W_4N^-k
  // (x_N = 0), runs the inverse FFT and stores Re w_m at 2m (m < N/2) or
  // 2(N-1-m)+1.  tw2: the length-4N twiddle table.
  int mode;           // 0 c2c, 1 r2c, 2 c2r, 3 REDFT10, 4 REDFT01
  int Zi, Ni, Zo, No;
  int plain;
  // adjoint weights: 1 = c2r loads halve the interior half-spectrum bins
  // (0 < k < N/2), 2 = r2c stores double them
  int wmode;
  const void* tw2;
  int staged;  // host only: PassParams::staged
  // FX mantissas kept between radix-8 passes (PassParams::fx_in / fx_out)
  int fx_in, fx_out;
  const int* lexp_in;
  int* lexp_out;
  long long lexp_in_n;
  int gin_np[PG_MAX_BATCH];
  long long gin_pext[2 * PG_MAX_BATCH], gin_pcoef[2 * PG_MAX_BATCH];
  long long gin_bofs[PG_MAX_BATCH];
  long long gin_k, gout_off;
  // paired real lines (PassParams::pair): each line of the tile is real
  // line a (at the line's offsets) and real line b (at + pairI on the input
  // side, + pairO on the output side)
  int pair;
  long long pairI, pairO;
};

// IO kinds of the radix-8 kernel: 0 plain c2c lines, 1 general I/O (r2c,
// c2r, windows, adjoint weights), 2 the DCTs; 3 and 4 the same as 1 and 2
// for paired inverse passes (c2r, REDFT01: two real lines combined before
// the transform, FX only), compiled separately so that the other kernels
// carry none of their registers
__host__ __device__ constexpr bool io_dct(int IO) { return IO == 2 || IO == 4; }
__host__ __device__ constexpr bool io_pinv(int IO) { return IO >= 3; }

// global element access: native format, or float-float pairs for the
// intermediate arrays of the double API (same 16 bytes per complex value).
// CG: load through L2 only (data written earlier in the same launch).
template <bool CG, class T>
__device__ __forceinline__ T gld(const T* p) {
  if (CG) return __ldcg(p);
  return *p;
}
template <class P, bool CG>
__device__ __forceinline__ typename P::C gload(const typename P::G* p, int df);
template <>
__device__ __forceinline__ F32::C gload<F32, false>(const F32::G* p, int) { return *p; }
template <>
__device__ __forceinline__ F32::C gload<F32, true>(const F32::G* p, int) { return __ldcg(p); }
template <bool CG>
__device__ __forceinline__ FDD::C gload_fdd(const FDD::G* p, int isdf) {
  if (isdf) {  // (re.hi, re.lo, im.hi, im.lo)
    float4 v = gld<CG>((const float4*)p);
    return {make_float2(v.x, v.z), make_float2(v.y, v.w)};
  }
  double2 v = gld<CG>(p);
  return FDD::from_df(df_from_double(v.x), df_from_double(v.y));
}
template <>
__device__ __forceinline__ FDD::C gload<FDD, false>(const FDD::G* p, int df) { return gload_fdd<false>(p, df); }
template <>
__device__ __forceinline__ FDD::C gload<FDD, true>(const FDD::G* p, int df) { return gload_fdd<true>(p, df); }
template <>
__device__ __forceinline__ FDD::C gload<FQ, false>(const FDD::G* p, int df) { return gload_fdd<false>(p, df); }
template <>
__device__ __forceinline__ FDD::C gload<FQ, true>(const FDD::G* p, int df) { return gload_fdd<true>(p, df); }
// FX: the raw bits of the doubles (converted by fx_enter)
template <>
__device__ __forceinline__ FX::C gload<FX, false>(const FX::G* p, int) {
  const double2 v = *p;
  return {__double_as_longlong(v.x), __double_as_longlong(v.y)};
}
template <>
__device__ __forceinline__ FX::C gload<FX, true>(const FX::G* p, int) {
  const double2 v = __ldcg(p);
  return {__double_as_longlong(v.x), __double_as_longlong(v.y)};
}
template <class P>
__device__ __forceinline__ void gstore(typename P::G* p, typename P::C v, int df);
template <>
__device__ __forceinline__ void gstore<F32>(F32::G* p, F32::C v, int) { *p = v; }
template <>
__device__ __forceinline__ void gstore<FDD>(FDD::G* p, FDD::C v, int df) {
  if (df) {
    FDD::C n = FDD::renorm(v);
    *(float4*)p = make_float4(n.h.x, n.l.x, n.h.y, n.l.y);
  } else {
    FDD::st(p, v);
  }
}
template <>
__device__ __forceinline__ void gstore<FQ>(FDD::G* p, FDD::C v, int df) {
  gstore<FDD>(p, v, df);
}
// FX: `df` carries the exponent of the results (fx_enter)
template <>
__device__ __forceinline__ void gstore<FX>(FX::G* p, FX::C v, int eo) {
  *p = make_double2(fx_to_double(v.x, eo), fx_to_double(v.y, eo));
}

// store of a complex result: FX with fx_out keeps the mantissas for the next
// radix-8 pass (the line's exponent goes to lexp_out)
template <class P>
__device__ __forceinline__ void gput(const FastArgs& a, typename P::G* p, typename P::C v, int df) {
  if constexpr (is_fx<P>()) {
    if (a.fx_out) {
      *(longlong2*)p = make_longlong2(v.x, v.y);
      return;
    }
  }
  gstore<P>(p, v, df);
}

// real-array element access (r2c input, c2r output)
template <class P, bool CG>
__device__ __forceinline__ typename P::C rload(const void* src, long long i);
template <>
__device__ __forceinline__ F32::C rload<F32, false>(const void* src, long long i) {
  return make_float2(((const float*)src)[i], 0.f);
}
template <>
__device__ __forceinline__ F32::C rload<F32, true>(const void* src, long long i) {
  return make_float2(__ldcg((const float*)src + i), 0.f);
}
template <>
__device__ __forceinline__ FDD::C rload<FDD, false>(const void* src, long long i) {
  return FDD::from_df(df_from_double(((const double*)src)[i]), df{0.f, 0.f});
}
template <>
__device__ __forceinline__ FDD::C rload<FDD, true>(const void* src, long long i) {
  return FDD::from_df(df_from_double(__ldcg((const double*)src + i)), df{0.f, 0.f});
}
// FX: the double's raw bits (converted by fx_enter), zero imaginary part
template <>
__device__ __forceinline__ FX::C rload<FX, false>(const void* src, long long i) {
  return {__double_as_longlong(((const double*)src)[i]), 0ll};
}
template <>
__device__ __forceinline__ FX::C rload<FX, true>(const void* src, long long i) {
  return {__double_as_longlong(__ldcg((const double*)src + i)), 0ll};
}
// eo: FX's result exponent (fx_enter), unused by the other policies
template <class P>
__device__ __forceinline__ void rstore(void* dst, long long i, typename P::C v, int eo);
template <>
__device__ __forceinline__ void rstore<F32>(void* dst, long long i, F32::C v, int) {
  ((float*)dst)[i] = v.x;
}
template <>
__device__ __forceinline__ void rstore<FDD>(void* dst, long long i, FDD::C v, int) {
  ((double*)dst)[i] = df_to_double_sel(FDD::re_df(v));
}
template <>
__device__ __forceinline__ void rstore<FX>(void* dst, long long i, FX::C v, int eo) {
  ((double*)dst)[i] = fx_to_double(v.x, eo);
}
template <class P>
__device__ __forceinline__ typename P::C czero();
template <>
__device__ __forceinline__ F32::C czero<F32>() { return make_float2(0.f, 0.f); }
template <>
__device__ __forceinline__ FDD::C czero<FDD>() { return {make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
template <>
__device__ __forceinline__ FX::C czero<FX>() { return {0ll, 0ll}; }
// FX before fx_enter: conjugation and halving of the raw doubles
__device__ __forceinline__ FX::C fx_conj_raw(FX::C v) {
  return {v.x, (long long)((unsigned long long)v.y ^ 0x8000000000000000ull)};
}
__device__ __forceinline__ FX::C fx_half_raw(FX::C v) {
  return {__double_as_longlong(__longlong_as_double(v.x) * 0.5), __double_as_longlong(__longlong_as_double(v.y) * 0.5)};
}

// real input x_j of a real-to-real line (zero outside the embedded range)
template <class P, bool CG>
__device__ __forceinline__ typename P::C rx(const FastArgs& a, long long off, int j) {
  const int q = j - a.Zi;
  if (q < 0 || q >= a.Ni) return czero<P>();
  return rload<P, CG>(a.src, off + (long long)q * a.sIa);
}

// element e (0..N-1) of a line's logical input sequence (FastArgs comment);
// DCT: the kernel runs a REDFT10 / REDFT01 pass (compiled separately, so the
// other kernels carry no DCT code)
template <class P, bool CG, bool DCT = false, bool PINV = false>
__device__ __forceinline__ typename P::C load_elem(const FastArgs& a, long long off, int e, int N) {
  typedef typename P::C C;
  if constexpr (is_fx<P>()) {
    if (a.pair && (a.mode == 1 || a.mode == 3)) {  // r2c / REDFT10: line a's input as the real part, line b's as the imaginary
      const int j = DCT ? (2 * e < N ? 2 * e : 2 * (N - 1 - e) + 1) : e;
      return {rx<P, CG>(a, off, j).x, rx<P, CG>(a, off + a.pairI, j).x};
    }
  }
  if constexpr (DCT) {
    if (a.mode == 3) return rx<P, CG>(a, off, 2 * e < N ? 2 * e : 2 * (N - 1 - e) + 1);
    C xk = rx<P, CG>(a, off, e);
    C xm = e == 0 ? czero<P>() : rx<P, CG>(a, off, N - e);
    if constexpr (is_fx<P>()) {
      // raw x_k - i x_(N-k); the rotation by W_4N^-k follows fx_enter (fast_body)
      return {xk.x, (long long)((unsigned long long)xm.x ^ 0x8000000000000000ull)};
    } else {
      C z = P::sub(xk, P::swap_neg_re(xm));  // x_k - i x_(N-k)
      return P::mul(z, P::template twd<1>(P::ldw(a.tw2, e, 4 * N)));
    }
  }
  bool mirror = false;
  int q, k = e;
  if (a.mode == 2) {
    mirror = 2 * e > N;
    k = mirror ? N - e : e;
  }
  q = k - a.Zi;
  if (q < 0 || q >= a.Ni) return czero<P>();
  C v = a.mode == 1 ? rload<P, CG>(a.src, off + (long long)q * a.sIa)
                    : gload<P, CG>((const typename P::G*)a.src + off + (long long)q * a.sIa, a.in_df);
  if constexpr (is_fx<P>()) {  // raw doubles until fx_enter
    if (a.conj_in) v = fx_conj_raw(v);
    if (a.wmode == 1 && k != 0 && 2 * k != N) v = fx_half_raw(v);
    // paired c2r: the DC and Nyquist bins' imaginary parts (which a c2r
    // ignores) zeroed, so that each line's spectrum is exactly Hermitian and
    // its inverse real: nothing leaks into the partner line
    if constexpr (PINV) {
      if (k == 0 || 2 * k == N) v.y = 0;
    }
    return mirror ? fx_conj_raw(v) : v;
  } else {
    if (a.conj_in) v = P::conj(v);
    if (a.wmode == 1 && k != 0 && 2 * k != N) v = P::scal(v, PG_KC(P, 0.5));
    return mirror ? P::conj(v) : v;
  }
}

// store logical output position e of a line (kept when Zo <= e < Zo + No)
// (eo: FX's result exponent)
template <class P, bool DCT = false, bool PINV = false>
__device__ __forceinline__ void store_elem(const FastArgs& a, long long off, int e, typename P::C v, int N,
                                           int eo = 0) {
  if constexpr (DCT) {
    if (a.mode == 3) {  // y_e = 2 Re(W_4N^e V_e)
      v = P::mul(v, P::template twd<-1>(P::ldw(a.tw2, e, 4 * N)));
      v = P::add(v, v);
      if constexpr (is_fx<P>()) eo = eo == INT_MIN ? eo : eo + 2;  // FX twiddles carry 1/4
    } else {
      e = 2 * e < N ? 2 * e : 2 * (N - 1 - e) + 1;
    }
  }
  const int k = e - a.Zo;
  if (k < 0 || k >= a.No) return;
  if (a.wmode == 2 && e != 0 && 2 * e != N) v = P::add(v, v);
  if (a.conj_out) v = P::conj(v);
  if constexpr (PINV) {  // paired c2r / REDFT01: z = y_a + i y_b
    rstore<P>(a.dst, off + (long long)k * a.sOa, v, eo);
    rstore<P>(a.dst, off + a.pairO + (long long)k * a.sOa, {v.y, v.x}, eo);
    return;
  }
  if (a.mode >= 2)
    rstore<P>(a.dst, off + (long long)k * a.sOa, v, eo);
  else
    gput<P>(a, (typename P::G*)a.dst + off + (long long)k * a.sOa, v, is_fx<P>() ? eo : a.out_df);
}

// Paired real lines (FastArgs::pair): the thread's outputs z[pos[r]] of the
// complex line z = x_a + i x_b (line `l` of the tile) go through shared
// memory; then, with the output side's thread mapping (rows: a line's
// threads along it; columns: consecutive threads on consecutive lines, so
// that both real lines' stores stay coalesced), each thread takes z[k] and
// z[N - k] of eight positions k: X_a[k] = (z[k] + conj z[N - k]) / 2 and
// X_b[k] = -i (z[k] - conj z[N - k]) / 2, each halving rounded half to even
// (the sums stay below 2^62.5, the halves below 2^61.5, so that a REDFT10
// rotation of them cannot overflow), stored as two lines.  Every thread of
// the block takes part (two barriers).
template <class P, bool DCT, bool ROW_OUT, int N, int L, int LSP, int K>
__device__ __forceinline__ void fx_pair_store(const FastArgs& a, const typename P::C (&v)[K], const int (&pos)[K], int l,
                                              typename P::S* buf, const long long* offO, long long g0, int eo) {
  typedef typename P::C C;
  constexpr int TPL = N / 8;
  __syncthreads();  // the last exchange's loads are done
#pragma unroll
  for (int r = 0; r < K; r++) buf[l * LSP + pad<P>(pos[r])] = P::sts(v[r]);
  __syncthreads();
  const int l2 = ROW_OUT ? (int)threadIdx.x / TPL : (int)threadIdx.x % L;
  const int t2 = ROW_OUT ? (int)threadIdx.x % TPL : (int)threadIdx.x / L;
  if (g0 + l2 >= a.nlines) return;
  const typename P::S* line = buf + l2 * LSP;
  const auto half = [](long long x) { return (x + ((x >> 1) & 1)) >> 1; };
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int k = t2 + r * TPL;
    const C z = P::lds(line[pad<P>(k)]), zm = P::lds(line[pad<P>((N - k) & (N - 1))]);
    const C xa = {half(z.x + zm.x), half(z.y - zm.y)};
    const C xb = {half(z.y + zm.y), half(zm.x - z.x)};
    store_elem<P, DCT>(a, offO[l2], k, xa, N, eo);
    store_elem<P, DCT>(a, offO[l2] + a.pairO, k, xb, N, eo);
  }
}

// bytes before the exchange area of a tile: the lines' input and output
// offsets, and for FX the previous pass's line index of each line's element 0
// (fx_in), rounded up to 16 bytes (one-line tiles of 4096 points)
template <class P>
__host__ __device__ constexpr int fast_hdr(int L) {
  return is_fx<P>() ? (24 * L + 15) / 16 * 16 : 16 * L;  // the exchange area is 16-byte aligned
}

// ROW_IN: the axis is contiguous on the input side (thread t walks the line);
// otherwise consecutive threads take consecutive (adjacent) lines.  ROW_OUT
// likewise for the output; when they differ the last stage is re-staged
// through shared memory so that both sides stay coalesced.
// Shared memory: one buffer of L lines at stride lsp_of, index pad(p) within
// a line.
// One tile (L lines) of the pass, run by the L * N/8 threads of a block:
// the body of the stand-alone kernel k_fast, and a task of the batched
// persistent kernel.  `blk` is the tile index, `sm_raw` the block's dynamic
// shared memory (fast_smem_bytes).
template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT, int IO>
__device__ __forceinline__ void fast_body(const FastArgs& a, typename P::C (&v)[8], long long g0, const long long* offO,
                                          typename P::S* buf, const typename P::C* v2 = nullptr);
// IO: 0 plain c2c lines (the hot kernels carry no other load/store code),
// 1 r2c / c2r / windows / adjoint weights (load_elem, store_elem), 2 the DCTs
template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT, bool CG = false, int IO = 0>
__device__ __forceinline__ void fast_tile(const FastArgs& a, long long blk, unsigned char* sm_raw) {
  typedef typename P::C C;
  typedef typename P::S S;
  typedef typename P::G G;
  constexpr int TPL = N / 8;  // threads per line
  long long* offI = (long long*)sm_raw;
  long long* offO = offI + L;
  S* buf = (S*)(sm_raw + fast_hdr<P>(L));

  const int tid = threadIdx.x;
  const long long g0 = blk * L;
  if (tid < L) {
    long long g = g0 + tid;
    if (g >= a.nlines) g = a.nlines - 1;  // tail CTA: clamp (duplicate work, never stored)
    long long oi = 0, oo = 0, gi = 0;
    int pc = 0;
    for (int b = 0; b < a.nb; b++) {
      long long e = a.bext[b];
      long long idx = g % e;
      g /= e;
      oi += idx * a.bsI[b];
      oo += idx * a.bsO[b];
      if constexpr (is_fx<P>()) {
        if (a.fx_in) {  // the previous pass's line index: this dimension's pieces
          long long x = idx + a.gin_bofs[b];
          for (int q = 0; q < a.gin_np[b]; q++, pc++) {
            const long long ep = a.gin_pext[pc];
            gi += (x % ep) * a.gin_pcoef[pc];
            x /= ep;
          }
        }
      }
    }
    offI[tid] = oi;
    offO[tid] = oo;
    if constexpr (is_fx<P>()) offO[L + tid] = gi;  // fx_in: previous pass's line of element 0
  }
  __syncthreads();
  const int l = ROW_IN ? tid / TPL : tid % L;
  const int t = ROW_IN ? tid % TPL : tid / L;

  C v[8];
  if constexpr (IO == 0) {
    const G* src = (const G*)a.src + offI[l] + (long long)t * a.sIa;
    const long long st = (long long)TPL * a.sIa;
#pragma unroll
    for (int r = 0; r < 8; r++) {
      v[r] = gload<P, CG>(src + r * st, a.in_df);
      if (!is_fx<P>() && a.conj_in) v[r] = P::conj(v[r]);  // FX: in fx_enter
    }
  } else {
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = load_elem<P, CG, io_dct(IO), io_pinv(IO)>(a, offI[l], t + r * TPL, N);
  }
  if constexpr (io_pinv(IO)) {  // paired c2r / REDFT01: line b's input beside line a's
    C v2[8];
#pragma unroll
    for (int r = 0; r < 8; r++) v2[r] = load_elem<P, CG, io_dct(IO), true>(a, offI[l] + a.pairI, t + r * TPL, N);
    fast_body<P, SIGN, N, L, ROW_IN, ROW_OUT, IO>(a, v, g0, offO, buf, v2);
  } else {
    fast_body<P, SIGN, N, L, ROW_IN, ROW_OUT, IO>(a, v, g0, offO, buf);
  }
}

// Stages and store of one tile after the load: v holds elements t + r*TPL of
// line l (the input thread mapping); offO the output offsets of the tile's
// lines; buf the exchange area (L lines of lsp_of elements).
template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT, int IO>
__device__ __forceinline__ void fast_body(const FastArgs& a, typename P::C (&v)[8], long long g0, const long long* offO,
                                          typename P::S* buf, const typename P::C* v2) {
  typedef typename P::C C;
  typedef typename P::S S;
  typedef typename P::G G;
  constexpr int TPL = N / 8;  // threads per line
  constexpr int NS8 = n8_of(N);
  constexpr int Q = N / pow8(NS8);  // last radix: 1, 2 or 4
  constexpr int LSP = lsp_of<P, N, L, ROW_IN>();
  const int tid = threadIdx.x;
  const int l = ROW_IN ? tid / TPL : tid % L;
  const int t = ROW_IN ? tid % TPL : tid / L;
  const bool live = (g0 + l) < a.nlines;
  const void* tw = a.tw;  // stage-major table (TW_F32_STG, TW_DFP_*_STG)
  constexpr int TWN = fast_tw_n(N);
  S* line = buf + l * LSP;
  int sdf = a.out_df;  // FX: the results' exponent instead
  int fx_e = 0, fx_sh = 0;  // FX: the tile's grid exponent and the stages' shifts
  if constexpr (is_fx<P>() && io_pinv(IO)) {
    // paired c2r / REDFT01: both lines on one grid, then z = X_a + i X_b
    // (REDFT01: each line's spectrum rotated first), exact integer sums
    C w[16];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      w[r] = v[r];
      w[8 + r] = v2[r];
    }
    fx_e = fx_enter<N, 16>(w, 0);
    if (a.mode == 4) {
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const typename P::W tw4 = P::template twd<1>(P::ldw(a.tw2, t + r * TPL, 4 * N));
        w[r] = P::mul(w[r], tw4);
        w[8 + r] = P::mul(w[8 + r], tw4);
      }
      fx_sh += 2;
    }
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = {w[r].x - w[8 + r].y, w[r].y + w[8 + r].x};
  } else if constexpr (is_fx<P>()) {
    if (IO == 0 && a.fx_in) {  // mantissas of the previous radix-8 pass, each with its line's exponent
      const long long gl = offO[L + l];
      int ex[8];
#pragma unroll
      for (int r = 0; r < 8; r++) ex[r] = __ldg(a.lexp_in + min(gl + (long long)(t + r * TPL) * a.gin_k, a.lexp_in_n - 1));
      fx_e = fx_enter_linked(v, ex, a.conj_in);
    } else {
      fx_e = fx_enter<N>(v, IO == 0 ? a.conj_in : 0);  // IO 1: conjugated in load_elem
    }
    if constexpr (io_dct(IO)) {
      if (a.mode == 4) {  // REDFT01: (x_k - i x_(N-k)) W_4N^-k, twiddles carrying 1/4
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = P::mul(v[r], P::template twd<1>(P::ldw(a.tw2, t + r * TPL, 4 * N)));
        fx_sh += 2;
      }
    }
  }
  bf8x<P, SIGN>(v);  // stage 0 (Ns = 1, no twiddles)
  int Ns = 1;
  // radix-8 stages 1 .. NS8-1 through shared memory
#pragma unroll
  for (int s = 1; s < NS8; s++) {
    if (s > 1) __syncthreads();  // previous stage's loads are done
    if constexpr (is_fx<P>()) fx_ormag_publish(fx_ormag(v), fx_slots() + 32 * (s & 1));
    {
      const int k = t % Ns;
      const int base = (t - k) * 8 + k;
#pragma unroll
      for (int r = 0; r < 8; r++) line[pad<P>(base + r * Ns)] = P::sts(v[r]);
    }
    __syncthreads();
    Ns *= 8;
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = P::lds(line[pad<P>(t + r * TPL)]);
    if constexpr (is_fx<P>()) {
      const int sh = fx_normal_shift(fx_slots() + 32 * (s & 1));
      fx_shift_all(v, sh);
      fx_sh += sh + 2;
    }
    const int k = t % Ns;
    v[0] = P::tw0(v[0]);
#pragma unroll
    for (int r = 1; r < 8; r++) v[r] = P::mul(v[r], P::template twd<SIGN>(P::ldw(tw, Ns - 8 + (r - 1) * Ns + k, TWN)));
    bf8x<P, SIGN>(v);
  }
  if constexpr (is_fx<P>()) {
    if (Q == 1 && a.fx_out) fx_sh += fx_store_normalise(v, fx_slots() + 32 * (NS8 & 1));
    sdf = fx_e == INT_MIN ? INT_MIN : fx_e + fx_sh;
    if (Q == 1 && a.fx_out && tid < L && g0 + tid < a.nlines) a.lexp_out[a.gout_off + g0 + tid] = sdf == INT_MIN ? INT_MAX : sdf;
  }
  if (Q == 1) {
    // v holds the last stage (Ns = N/8, k = t): outputs y[t + r*TPL]
    if constexpr ((IO == 1 || IO == 2) && is_fx<P>()) {
      if (a.pair && (a.mode == 1 || a.mode == 3)) {  // r2c / REDFT10: separate the two spectra
        int pos[8];
#pragma unroll
        for (int r = 0; r < 8; r++) pos[r] = t + r * TPL;
        fx_pair_store<P, io_dct(IO), ROW_OUT, N, L, LSP>(a, v, pos, l, buf, offO, g0, sdf);
        return;
      }
    }
    if (ROW_IN == ROW_OUT) {
      if (live) {
        if constexpr (IO == 0) {
          G* dst = (G*)a.dst + offO[l] + (long long)t * a.sOa;
          const long long st = (long long)TPL * a.sOa;
#pragma unroll
          for (int r = 0; r < 8; r++) gput<P>(a, dst + r * st, a.conj_out ? P::conj(v[r]) : v[r], sdf);
        } else {
#pragma unroll
          for (int r = 0; r < 8; r++) store_elem<P, io_dct(IO), io_pinv(IO)>(a, offO[l], t + r * TPL, v[r], N, sdf);
        }
      }
      return;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 8; r++) line[pad<P>(t + r * TPL)] = P::sts(v[r]);
  } else {
    // radix-Q stage (Q = 2 or 4) with Ns = N/Q: butterflies j = t + b*TPL, k = j
    if (NS8 > 1) __syncthreads();
    if constexpr (is_fx<P>()) fx_ormag_publish(fx_ormag(v), fx_slots() + 32 * (NS8 & 1));
    {
      const int k = t % Ns;
      const int base = (t - k) * 8 + k;
#pragma unroll
      for (int r = 0; r < 8; r++) line[pad<P>(base + r * Ns)] = P::sts(v[r]);
    }
    __syncthreads();
    constexpr int NB = 8 / Q;
    constexpr int NQ = N / Q;
    int qsh = 0;
    if constexpr (is_fx<P>()) {
      qsh = fx_normal_shift(fx_slots() + 32 * (NS8 & 1));
      fx_sh += qsh + 2;
      sdf = fx_e == INT_MIN ? INT_MIN : fx_e + fx_sh;
    }
    C w[8];
#pragma unroll
    for (int b = 0; b < NB; b++)
#pragma unroll
      for (int r = 0; r < Q; r++) w[b * Q + r] = P::lds(line[pad<P>(t + b * TPL + r * NQ)]);
    if constexpr (is_fx<P>()) fx_shift_all(w, qsh);
#pragma unroll
    for (int b = 0; b < NB; b++) {
      const int j = t + b * TPL;
#pragma unroll
      for (int r = 0; r < Q; r++) {
        const C x = w[b * Q + r];
        w[b * Q + r] = r > 0 ? P::mul(x, P::template twd<SIGN>(P::ldw(tw, NQ - 8 + (r - 1) * NQ + j, TWN))) : P::tw0(x);
      }
      if (Q == 2) {
        C x0 = w[b * 2], x1 = w[b * 2 + 1];
        w[b * 2] = P::add(x0, x1);
        w[b * 2 + 1] = P::sub(x0, x1);
      } else {
        bf4<P, SIGN>(w[b * Q], w[b * Q + 1], w[b * Q + 2], w[b * Q + 3]);
      }
    }
    if constexpr (is_fx<P>()) {
      if (a.fx_out) {
        fx_sh += fx_store_normalise(w, fx_slots() + 32 * ((NS8 + 1) & 1));
        sdf = fx_e == INT_MIN ? INT_MIN : fx_e + fx_sh;
        if (tid < L && g0 + tid < a.nlines) a.lexp_out[a.gout_off + g0 + tid] = sdf == INT_MIN ? INT_MAX : sdf;
      }
    }
    if constexpr ((IO == 1 || IO == 2) && is_fx<P>()) {
      if (a.pair && (a.mode == 1 || a.mode == 3)) {  // r2c / REDFT10: separate the two spectra
        int pos[8];
#pragma unroll
        for (int b = 0; b < NB; b++)
#pragma unroll
          for (int r = 0; r < Q; r++) pos[b * Q + r] = t + b * TPL + r * NQ;
        fx_pair_store<P, io_dct(IO), ROW_OUT, N, L, LSP>(a, w, pos, l, buf, offO, g0, sdf);
        return;
      }
    }
    if (ROW_IN == ROW_OUT) {
      if (live) {
        if constexpr (IO == 0) {
          G* dst = (G*)a.dst + offO[l];
#pragma unroll
          for (int b = 0; b < NB; b++)
#pragma unroll
            for (int r = 0; r < Q; r++) {
              C o = a.conj_out ? P::conj(w[b * Q + r]) : w[b * Q + r];
              gput<P>(a, dst + (long long)(t + b * TPL + r * NQ) * a.sOa, o, sdf);
            }
        } else {
#pragma unroll
          for (int b = 0; b < NB; b++)
#pragma unroll
            for (int r = 0; r < Q; r++) store_elem<P, io_dct(IO), io_pinv(IO)>(a, offO[l], t + b * TPL + r * NQ, w[b * Q + r], N, sdf);
        }
      }
      return;
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; b++)
#pragma unroll
      for (int r = 0; r < Q; r++) line[pad<P>(t + b * TPL + r * NQ)] = P::sts(w[b * Q + r]);
  }
  // re-staged store with the output's thread mapping
  __syncthreads();
  {
    const int l2 = ROW_OUT ? tid / TPL : tid % L;
    const int t2 = ROW_OUT ? tid % TPL : tid / L;
    if ((g0 + l2) < a.nlines) {
      G* d2 = (G*)a.dst + offO[l2];
      const S* line2 = buf + l2 * LSP;
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const int k = t2 + r * TPL;
        C o = P::lds(line2[pad<P>(k)]);
        if constexpr (IO == 0) {
          if (a.conj_out) o = P::conj(o);
          gput<P>(a, d2 + (long long)k * a.sOa, o, sdf);
        } else {
          store_elem<P, io_dct(IO), io_pinv(IO)>(a, offO[l2], k, o, N, sdf);
        }
      }
    }
  }
}

// resident CTAs per SM the register budget is fitted to: 1024 threads for
// float-float (64 registers), no bound for FP32
template <class P, int T>
constexpr int fast_min_blocks() {
  return sizeof(typename P::S) == 16 && T <= 1024 ? 1024 / T : 1;
}

template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT, int IO = 0>
__global__ void __launch_bounds__(L*(N / 8), (fast_min_blocks<P, L*(N / 8)>())) k_fast(const FastArgs a) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  fast_tile<P, SIGN, N, L, ROW_IN, ROW_OUT, false, IO>(a, blockIdx.x, sm_raw);
}

template <class P, int N, int L>
constexpr size_t fast_smem_bytes() {
  return fast_hdr<P>(L) + (size_t)L * (sizeof(typename P::S) == 8 ? N + 16 : N + N / 8 + 4) * sizeof(typename P::S);
}

// ---- staged persistent variant (plain c2c passes) ---------------------------
// Each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...  The input
// of its next tile is copied global -> shared memory by the copy engine while
// the current tile is transformed: row tiles as one cp.async.bulk per line,
// column tiles (L adjacent lines) as tensor-map boxes of L lines x up to 256
// elements.  The copies complete on an mbarrier; the threads read their eight
// elements from the staging area, the area is released by a CTA barrier and
// the next tile's copies are issued before the stages run.  So the global
// loads' latency is off the critical path and no registers hold a second
// tile.  Shared memory: up to 128 bytes of alignment, staging (L*N elements in
// the global format), the mbarrier (16 bytes), two sets of output offsets,
// the exchange area.
template <class P, int N, int L>
constexpr size_t staged_smem_bytes() {
  return 128 + (size_t)L * N * sizeof(typename P::G) + 16 + fast_smem_bytes<P, N, L>();
}
// a staged-load wait gives up after this many nanoseconds (error word set)
constexpr unsigned long long STAGED_WAIT_NS = 2000000000ull;

template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT>
__global__ void __launch_bounds__(L*(N / 8))
    k_fast_staged(const __grid_constant__ FastArgs a, const __grid_constant__ CUtensorMap tm, int* err) {
  typedef typename P::C C;
  typedef typename P::G G;
  typedef typename P::S S;
  constexpr int TPL = N / 8;
  constexpr int ESZ = (int)sizeof(G);
  constexpr uint32_t LINE_BYTES = (uint32_t)N * ESZ;
  constexpr int BOX = N < 256 ? N : 256;  // elements per tensor box (column tiles)
  extern __shared__ __align__(16) unsigned char sm_dyn[];
  // staging area on a 128-byte boundary (tensor-map copies)
  unsigned char* sm_raw = sm_dyn + ((128u - (tma::smem_addr(sm_dyn) & 127u)) & 127u);
  const G* stage = (const G*)sm_raw;
  const uint32_t st_addr = tma::smem_addr(sm_raw);
  const uint32_t mb = st_addr + L * LINE_BYTES;
  long long* offO2 = (long long*)(sm_raw + L * LINE_BYTES + 16);
  S* buf = (S*)(sm_raw + L * LINE_BYTES + 16 + 16 * L);
  const int tid = threadIdx.x;
  const long long ntiles = (a.nlines + L - 1) / L;
  if (tid == 0) {
    tma::mbar_init(mb, 1);
    tma::mbar_init_fence();
    if (!ROW_IN) tma::prefetch_tensormap(&tm);
  }
  __syncthreads();
  // copies of tile tl: row tiles one line per lane 0..L-1, column tiles by thread 0
  auto issue = [&](long long tl) {
    const long long g0 = tl * L;
    if constexpr (ROW_IN) {
      if (tid < L) {
        const long long nv = min((long long)L, a.nlines - g0);
        if (tid == 0) tma::mbar_arrive_tx(mb, (uint32_t)nv * LINE_BYTES);
        if (tid < nv) {
          long long g = g0 + tid, oi = 0;
          for (int b = 0; b < a.nb; b++) {
            const long long e = a.bext[b];
            oi += (g % e) * a.bsI[b];
            g /= e;
          }
          tma::bulk_load(st_addr + tid * LINE_BYTES, (const G*)a.src + oi, LINE_BYTES, mb);
        }
      }
    } else {
      if (tid == 0) {
        // the tile's lines are adjacent along batch dimension 0 (extent a
        // multiple of L); tensor dimensions: 4-byte words of dimension 0,
        // elements, batch dimensions 1..3
        long long g = g0;
        const int c0 = (int)(g % a.bext[0]) * (ESZ / 4);
        g /= a.bext[0];
        int c[3] = {0, 0, 0};
        for (int b = 1; b < a.nb; b++) {
          c[b - 1] = (int)(g % a.bext[b]);
          g /= a.bext[b];
        }
        tma::mbar_arrive_tx(mb, L * LINE_BYTES);
#pragma unroll
        for (int e0 = 0; e0 < N; e0 += BOX) tma::tensor_load5(st_addr + e0 * L * ESZ, &tm, c0, e0, c[0], c[1], c[2], mb);
      }
    }
  };
  long long tile = blockIdx.x;
  if (tile < ntiles) issue(tile);
  uint32_t parity = 0;
  int sel = 0;
  for (; tile < ntiles; tile += gridDim.x, parity ^= 1, sel ^= 1) {
    const long long g0 = tile * L;
    long long* offO = offO2 + sel * L;
    if (tid < L) {
      long long g = g0 + tid;
      if (g >= a.nlines) g = a.nlines - 1;  // tail tile: never stored
      long long oo = 0;
      for (int b = 0; b < a.nb; b++) {
        const long long e = a.bext[b];
        oo += (g % e) * a.bsO[b];
        g /= e;
      }
      offO[tid] = oo;
    }
    const bool ok = tma::mbar_wait(mb, parity, STAGED_WAIT_NS);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicExch(err, 1);
        tma::mbar_wait(mb, parity, STAGED_WAIT_NS);  // the copies of this tile, bounded
      }
      return;
    }
    const int l = ROW_IN ? tid / TPL : tid % L;
    const int t = ROW_IN ? tid % TPL : tid / L;
    C v[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
      const int e = t + r * TPL;
      v[r] = gload<P, false>(ROW_IN ? stage + l * N + e : stage + e * L + l, a.in_df);
      if (a.conj_in) v[r] = P::conj(v[r]);
    }
    __syncthreads();  // staging area free; offO visible; the previous tile is done
    if (tile + gridDim.x < ntiles) issue(tile + gridDim.x);
    fast_body<P, SIGN, N, L, ROW_IN, ROW_OUT, 0>(a, v, g0, offO, buf);
  }
}

// Host side of the staged variant (fft_fast.cu): false when the pass cannot
// be staged with L lines per tile (disabled, alignment, a column tile that
// would straddle batch dimension 0, more than 4 batch dimensions); fills the
// tensor map of column tiles.
bool staged_setup(const FastArgs& a, int N, int L, int esz, bool row_in, CUtensorMap* tm);
int* staged_err_word();
int sm_count();

template <class P, int SIGN, int N, int L, bool RI, bool RO>
int launch_staged(const FastArgs& a, const CUtensorMap& tm, cudaStream_t s) {
  constexpr int T = L * (N / 8);
  constexpr size_t smem = staged_smem_bytes<P, N, L>();
  static int per_sm = 0;  // resident CTAs per SM, found once per instantiation
  if (!per_sm) {
    cudaError_t e = cudaFuncSetAttribute(k_fast_staged<P, SIGN, N, L, RI, RO>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_fast_staged<P, SIGN, N, L, RI, RO>, T, smem);
    if (e != cudaSuccess) return (int)e;
    per_sm = nb > 0 ? nb : 1;
  }
  int* err = staged_err_word();
  if (!err) return (int)cudaErrorMemoryAllocation;
  const long long ntiles = (a.nlines + L - 1) / L;
  const long long grid = std::min(ntiles, (long long)per_sm * sm_count());
  k_fast_staged<P, SIGN, N, L, RI, RO><<<(unsigned)grid, T, smem, s>>>(a, tm, err);
  return (int)cudaGetLastError();
}

template <class P, int SIGN, int N, int L, int IO = 0>
int launch4(const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  constexpr int T = L * (N / 8);
  const size_t smem = fast_smem_bytes<P, N, L>();
  if constexpr (IO == 0 && !is_fx<P>() && staged_smem_bytes<P, N, L>() <= 227 * 1024) {
    CUtensorMap tm;
    if (staged_setup(a, N, L, (int)sizeof(typename P::G), row_in, &tm)) {
      if (row_in && row_out) return launch_staged<P, SIGN, N, L, true, true>(a, tm, s);
      if (!row_in && !row_out) return launch_staged<P, SIGN, N, L, false, false>(a, tm, s);
      if (row_in) return launch_staged<P, SIGN, N, L, true, false>(a, tm, s);
      return launch_staged<P, SIGN, N, L, false, true>(a, tm, s);
    }
  }
  long long grid = (a.nlines + L - 1) / L;
  if (grid > 2147483647LL) return (int)cudaErrorInvalidConfiguration;
  cudaError_t e = cudaSuccess;
  // the attribute is set once per kernel instantiation
#define PG_FAST_LAUNCH(RI, RO)                                                                            \
  do {                                                                                                    \
    static bool attr_done = false;                                                                        \
    if (!attr_done) {                                                                                     \
      e = cudaFuncSetAttribute(k_fast<P, SIGN, N, L, RI, RO, IO>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                               (int)smem);                                                                \
      if (e != cudaSuccess) return (int)e;                                                                \
      attr_done = true;                                                                                   \
    }                                                                                                     \
    k_fast<P, SIGN, N, L, RI, RO, IO><<<(unsigned)grid, T, smem, s>>>(a);                                \
  } while (0)
  if (row_in && row_out)
    PG_FAST_LAUNCH(true, true);
  else if (!row_in && !row_out)
    PG_FAST_LAUNCH(false, false);
  else if (row_in)
    PG_FAST_LAUNCH(true, false);
  else
    PG_FAST_LAUNCH(false, true);
#undef PG_FAST_LAUNCH
  return (int)cudaGetLastError();
}

// Arguments of the fast kernel for a pass, or false when the pass is not
// covered (fft_fast.cu).
bool fast_args(const PassParams& p, int arith, FastArgs* a, bool* row_in, bool* row_out);

// Launchers, one explicit instantiation set per translation unit
// (fft_fast_<arith>_<dir>_<range>.cu) so the build compiles them in parallel.
template <class P, int SIGN>
int launch_small(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
template <class P, int SIGN>
int launch_large(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
// r2c / c2r / windowed / weighted passes of 16..4096 points, default tile
// heights (fft_fast_gio_<arith>_<dir>.cu)
template <class P, int SIGN>
int launch_gio(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
// REDFT10 (SIGN -1) / REDFT01 (SIGN +1) passes of 16..512 points with the same
// orientation on both sides, default tile heights (fft_fast_dct_<arith>_<dir>.cu)
template <class P, int SIGN>
int launch_dct(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
// paired inverse passes (IO kinds 3 and 4): c2r (fft_fast_gioinv_fx_<dir>.cu)
// and REDFT01 (fft_fast_dctinv_fx_bwd.cu), 64-bit fixed point
template <class P, int SIGN>
int launch_gio_pinv(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
template <class P, int SIGN>
int launch_dct_pinv(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);

}  // namespace fast
}  // namespace pg

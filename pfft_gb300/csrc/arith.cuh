// Arithmetic policies for the transform kernels.
//
// Three policies share one kernel body:
//   ArF32  - float storage, float arithmetic (the pfftf_ API).
//   ArF64  - double storage, native FP64 arithmetic.  On GB300 the FP64 pipe
//            issues at roughly 1/70 of the FP32 rate, so this policy is kept
//            only as a selectable reference path.
//   ArDF   - double storage, float-float ("df64") arithmetic on the FP32 pipes.
//            A double is split into hi+lo floats with integer bit operations
//            only (no FP64 instruction), the transform runs in float-float with
//            error-free TwoSum / FMA-based TwoProd, and the result is rounded
//            back to double with integer operations.  Unit roundoff is about
//            2^-47, which keeps a 3-D transform well inside 1e-12 relative L2.
//
// All float operations that must not be contracted or reassociated use the
// explicit __fadd_rn / __fmul_rn / __fmaf_rn intrinsics.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

// ---------------------------------------------------------------------------
// float-float scalar
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df df_quick(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = df_two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return df_quick(s.hi, e);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_quick(p, e);
}
// a*b - c*d with a single renormalisation (used by the complex product)
__device__ __forceinline__ df df_mul_sub(df a, df b, df c, df d) {
  float p1 = __fmul_rn(a.hi, b.hi);
  float e1 = __fmaf_rn(a.hi, b.hi, -p1);
  float p2 = __fmul_rn(c.hi, d.hi);
  float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  df s = df_two_sum(p1, -p2);
  float e = __fadd_rn(s.lo, __fsub_rn(e1, e2));
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(-c.hi, d.lo, e);
  e = __fmaf_rn(-c.lo, d.hi, e);
  return df_quick(s.hi, e);
}
// a*b + c*d
__device__ __forceinline__ df df_mul_add(df a, df b, df c, df d) {
  return df_mul_sub(a, b, df_neg(c), d);
}

// Host-side / compile-time split of a double constant into hi+lo floats.
// Used only on compile-time constants so no FP64 instruction is emitted.
#define PG_DF_CONST(c) (::pg::df{(float)(c), (float)((c) - (double)(float)(c))})

// double -> float-float with integer and exact float operations only (no
// FP64 instruction, no leading-zero count, no branch).
// hi is the double with its mantissa truncated to 24 bits: the exponent is
// rebiased by bit arithmetic ((e - 896) mod 256 = low8(e) ^ 0x80).  The 29
// remaining mantissa bits r are turned into floats exactly by subtracting two
// floats of the same exponent, one with part of r in its mantissa field and
// one without (lo1: bits 28..6 of r, lo2: bits 5..0); lo = lo1 + lo2 keeps 24
// significant bits.  Magnitudes outside [2^-126, 2^127] are flushed (to 0 /
// inf, NaN stays NaN when its payload has high bits); below 2^-80 lo2 and
// below 2^-103 lo1 underflow, and the relative precision degrades to 2^-47
// and 2^-24.
__device__ __forceinline__ df df_from_double(double x) {
  const unsigned h32 = (unsigned)__double2hiint(x), l32 = (unsigned)__double2loint(x);
  const unsigned sign = h32 & 0x80000000u;
  const unsigned e = (h32 >> 20) & 0x7FFu;
  const unsigned t = (h32 << 3) | (l32 >> 29);  // low 9 bits of e, then the top 23 mantissa bits
  float hi = __uint_as_float(((t & 0x7FFFFFFFu) ^ 0x40000000u) | sign);
  const unsigned b1 = (((h32 & 0x7FF00000u) << 3) - (919u << 23)) | sign;  // 2^(e-1046), valid for e >= 920
  const unsigned b2 = b1 - (23u << 23);                                      // 2^(e-1069), valid for e >= 943
  const float lo1 = __fsub_rn(__uint_as_float(b1 | ((l32 >> 6) & 0x7FFFFFu)), __uint_as_float(b1));
  const float lo2 = __fsub_rn(__uint_as_float(b2 | ((l32 & 63u) << 17)), __uint_as_float(b2));
  float lo = e >= 943u ? __fadd_rn(lo1, lo2) : (e >= 920u ? lo1 : 0.f);
  if (e - 897u >= 254u) {  // outside the float range: signed zero, inf or NaN
    hi = __uint_as_float(e < 897u ? sign : (sign | 0x7F800000u | (t & 0x7FFFFFu)));
    lo = 0.f;
  }
  return {hi, lo};
}

// float-float -> double without FP64 instructions.  After renormalising
// (|lo| <= ulp(hi)/2), lo is turned into a signed integer count L of the last
// place of hi's double (|L| <= 2^28) by an exact power-of-two scaling and one
// float -> int conversion (round to nearest), and L is added to the bit
// pattern of hi as a double: the sum, correctly rounded.  The sum never leaves
// hi's binade upwards; downwards only when hi is a power of two and lo has
// the opposite sign, where the lower binade's last place is half as large and
// the scale doubles.  Below 2^-74 the scale 2^(52-e) would overflow a float
// and is applied in two steps.  Results below 2^-126 are flushed to zero.
__device__ __forceinline__ double df_to_double(df v) {
  const float hi = __fadd_rn(v.hi, v.lo);
  const float lo = __fsub_rn(v.lo, __fsub_rn(hi, v.hi));
  const unsigned uh = __float_as_uint(hi), ul = __float_as_uint(lo);
  const unsigned ehb = uh & 0x7F800000u;
  const bool opp = ((uh ^ ul) & 0x80000000u) != 0u;
  unsigned sb = (306u << 23) - ehb;                    // 2^(52 - e_hi)
  if (opp && (uh & 0x7FFFFFu) == 0u) sb += 1u << 23;   // lower binade: twice the scale
  float lf;
  if ((sb >> 23) <= 254u) {
    lf = __fmul_rn(lo, __uint_as_float(sb));
  } else {
    lf = __fmul_rn(__fmul_rn(lo, __uint_as_float((127u + 64u) << 23)), __uint_as_float(sb - (64u << 23)));
  }
  int L = __float2int_rn(lf);
  if (uh & 0x80000000u) L = -L;  // count in the direction of hi's magnitude
  const unsigned dh = (uh & 0x80000000u) | (((uh & 0x7FFFFFFFu) >> 3) + (896u << 20));
  unsigned long long P = (((unsigned long long)dh << 32) | (uh << 29)) + (unsigned long long)(long long)L;
  if (ehb == 0u) P = (unsigned long long)(uh & 0x80000000u) << 32;
  if (ehb == 0x7F800000u)
    P = ((unsigned long long)((uh & 0x80000000u) | 0x7FF00000u | ((uh & 0x7FFFFFu) >> 3)) << 32) | (uh << 29);
  return __longlong_as_double((long long)P);
}

// Fast path of float-float -> double, bit-identical to df_to_double where
// `ok` is set and cheaper because it carries none of the range cases: a
// caller converts with it and falls back to the full routine (per complex
// value) where `ok` is false.  The radix-8 and mixed-radix kernels store
// through it (it shortens the ALU-bound store phase of a last pass: 512^3
// complex128, 1.17 -> 1.06 ms); their loads use the branch-free
// df_from_double, which measured faster there than a fast path with a
// fallback.
//
// float-float -> double where the renormalised high word h has a biased
// exponent in 52..254 (|h| >= 2^-75: the scale 2^(52 - e_h) is a float)
// and a non-zero mantissa field (the sum cannot leave h's binade
// downwards), and for zeros.  The sign of h is folded into the scale, so
// that the rounded count L is already directed.
__device__ __forceinline__ double df_to_double_fast(df v, bool& ok) {
  const float hi = __fadd_rn(v.hi, v.lo);
  const float lo = __fsub_rn(v.lo, __fsub_rn(hi, v.hi));
  const unsigned uh = __float_as_uint(hi);
  const unsigned sign = uh & 0x80000000u;
  const unsigned ehb = uh & 0x7F800000u;
  const unsigned sb = (306u << 23) - ehb;  // 2^(52 - e_hi)
  const int L = __float2int_rn(__fmul_rn(lo, __uint_as_float(sb | sign)));
  const unsigned dh = sign | (((uh & 0x7FFFFFFFu) >> 3) + (896u << 20));
  unsigned long long P = (((unsigned long long)dh << 32) | (uh << 29)) + (unsigned long long)(long long)L;
  const bool zero = ehb == 0u;
  if (zero) P = (unsigned long long)sign << 32;
  ok = ((ehb - (52u << 23)) <= (202u << 23) && (uh & 0x7FFFFFu) != 0u) || zero;
  return __longlong_as_double((long long)P);
}

// The store conversion as the kernels use it: the fast path, and the full
// routine for a value (or pair) outside it.
__device__ __forceinline__ double df_to_double_sel(df v) {
  bool ok;
  const double r = df_to_double_fast(v, ok);
  return ok ? r : df_to_double(v);
}
__device__ __forceinline__ void df_pair_to_double(df a, df b, double& ra, double& rb) {
  bool oa, ob;
  ra = df_to_double_fast(a, oa);
  rb = df_to_double_fast(b, ob);
  if (!(oa && ob)) {
    ra = df_to_double(a);
    rb = df_to_double(b);
  }
}

// ---------------------------------------------------------------------------
// Policies
// ---------------------------------------------------------------------------
struct ArF32 {
  typedef float2 sm_t;   // shared memory / twiddle element
  typedef float2 gc_t;   // global complex element
  typedef float gr_t;    // global real element
  typedef float R;       // arithmetic real
  struct C {
    float x, y;
  };
  static constexpr int kId = 0;
  static __device__ __forceinline__ C make(R a, R b) { return {a, b}; }
  static __device__ __forceinline__ R rzero() { return 0.f; }
  static __device__ __forceinline__ C zero() { return {0.f, 0.f}; }
  static __device__ __forceinline__ R rneg(R a) { return -a; }
  static __device__ __forceinline__ R radd(R a, R b) { return a + b; }
  static __device__ __forceinline__ R rsub(R a, R b) { return a - b; }
  static __device__ __forceinline__ R rmul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R rconst(double c) { return (float)c; }
  static __device__ __forceinline__ C add(C a, C b) { return {a.x + b.x, a.y + b.y}; }
  static __device__ __forceinline__ C sub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
  static __device__ __forceinline__ C conj(C a) { return {a.x, -a.y}; }
  static __device__ __forceinline__ C neg(C a) { return {-a.x, -a.y}; }
  static __device__ __forceinline__ C scale(C a, R s) { return {a.x * s, a.y * s}; }
  // a * w
  static __device__ __forceinline__ C mul(C a, C w) {
    return {__fmaf_rn(a.x, w.x, -a.y * w.y), __fmaf_rn(a.x, w.y, a.y * w.x)};
  }
  static __device__ __forceinline__ C lds(sm_t v) { return {v.x, v.y}; }
  static __device__ __forceinline__ sm_t sts(C v) { return make_float2(v.x, v.y); }
  static __device__ __forceinline__ C ldc(const gc_t* p) { gc_t v = *p; return {v.x, v.y}; }
  static __device__ __forceinline__ C cvc(gc_t v) { return {v.x, v.y}; }
  static __device__ __forceinline__ R cvr(gr_t v) { return v; }
  static __device__ __forceinline__ void stc(gc_t* p, C v) { *p = make_float2(v.x, v.y); }
  static __device__ __forceinline__ R ldr(const gr_t* p) { return *p; }
  static __device__ __forceinline__ void str(gr_t* p, R v) { *p = v; }
};

struct ArF64 {
  typedef double2 sm_t;
  typedef double2 gc_t;
  typedef double gr_t;
  typedef double R;
  struct C {
    double x, y;
  };
  static constexpr int kId = 1;
  static __device__ __forceinline__ C make(R a, R b) { return {a, b}; }
  static __device__ __forceinline__ R rzero() { return 0.0; }
  static __device__ __forceinline__ C zero() { return {0.0, 0.0}; }
  static __device__ __forceinline__ R rneg(R a) { return -a; }
  static __device__ __forceinline__ R radd(R a, R b) { return a + b; }
  static __device__ __forceinline__ R rsub(R a, R b) { return a - b; }
  static __device__ __forceinline__ R rmul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R rconst(double c) { return c; }
  static __device__ __forceinline__ C add(C a, C b) { return {a.x + b.x, a.y + b.y}; }
  static __device__ __forceinline__ C sub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
  static __device__ __forceinline__ C conj(C a) { return {a.x, -a.y}; }
  static __device__ __forceinline__ C neg(C a) { return {-a.x, -a.y}; }
  static __device__ __forceinline__ C scale(C a, R s) { return {a.x * s, a.y * s}; }
  static __device__ __forceinline__ C mul(C a, C w) {
    return {__fma_rn(a.x, w.x, -a.y * w.y), __fma_rn(a.x, w.y, a.y * w.x)};
  }
  static __device__ __forceinline__ C lds(sm_t v) { return {v.x, v.y}; }
  static __device__ __forceinline__ sm_t sts(C v) { return make_double2(v.x, v.y); }
  static __device__ __forceinline__ C ldc(const gc_t* p) { gc_t v = *p; return {v.x, v.y}; }
  static __device__ __forceinline__ C cvc(gc_t v) { return {v.x, v.y}; }
  static __device__ __forceinline__ R cvr(gr_t v) { return v; }
  static __device__ __forceinline__ void stc(gc_t* p, C v) { *p = make_double2(v.x, v.y); }
  static __device__ __forceinline__ R ldr(const gr_t* p) { return *p; }
  static __device__ __forceinline__ void str(gr_t* p, R v) { *p = v; }
};

struct ArDF {
  typedef float4 sm_t;  // (re.hi, re.lo, im.hi, im.lo)
  typedef double2 gc_t;
  typedef double gr_t;
  typedef df R;
  struct C {
    df x, y;
  };
  static constexpr int kId = 2;
  static __device__ __forceinline__ C make(R a, R b) { return {a, b}; }
  static __device__ __forceinline__ R rzero() { return {0.f, 0.f}; }
  static __device__ __forceinline__ C zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
  static __device__ __forceinline__ R rneg(R a) { return df_neg(a); }
  static __device__ __forceinline__ R radd(R a, R b) { return df_add(a, b); }
  static __device__ __forceinline__ R rsub(R a, R b) { return df_sub(a, b); }
  static __device__ __forceinline__ R rmul(R a, R b) { return df_mul(a, b); }
  static __device__ __forceinline__ C add(C a, C b) { return {df_add(a.x, b.x), df_add(a.y, b.y)}; }
  static __device__ __forceinline__ C sub(C a, C b) { return {df_sub(a.x, b.x), df_sub(a.y, b.y)}; }
  static __device__ __forceinline__ C conj(C a) { return {a.x, df_neg(a.y)}; }
  static __device__ __forceinline__ C neg(C a) { return {df_neg(a.x), df_neg(a.y)}; }
  static __device__ __forceinline__ C scale(C a, R s) { return {df_mul(a.x, s), df_mul(a.y, s)}; }
  static __device__ __forceinline__ C mul(C a, C w) {
    return {df_mul_sub(a.x, w.x, a.y, w.y), df_mul_add(a.x, w.y, a.y, w.x)};
  }
  static __device__ __forceinline__ C lds(sm_t v) { return {{v.x, v.y}, {v.z, v.w}}; }
  static __device__ __forceinline__ sm_t sts(C v) { return make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo); }
  static __device__ __forceinline__ C ldc(const gc_t* p) {
    gc_t v = *p;
    return {df_from_double(v.x), df_from_double(v.y)};
  }
  static __device__ __forceinline__ C cvc(gc_t v) { return {df_from_double(v.x), df_from_double(v.y)}; }
  static __device__ __forceinline__ R cvr(gr_t v) { return df_from_double(v); }
  static __device__ __forceinline__ void stc(gc_t* p, C v) {
    *p = make_double2(df_to_double(v.x), df_to_double(v.y));
  }
  static __device__ __forceinline__ R ldr(const gr_t* p) { return df_from_double(*p); }
  static __device__ __forceinline__ void str(gr_t* p, R v) { *p = df_to_double(v); }
};

// global load, optionally bypassing L1 (data written by other CTAs of the
// same launch, published through a fence + counter)
template <bool CG, class T>
__device__ __forceinline__ T ldraw(const T* p) {
  if constexpr (CG)
    return __ldcg(p);
  else
    return *p;
}

// compile-time constant of the policy's real type
template <class A>
__device__ __forceinline__ typename A::R rconst(double c);
template <>
__device__ __forceinline__ float rconst<ArF32>(double c) { return (float)c; }
template <>
__device__ __forceinline__ double rconst<ArF64>(double c) { return c; }
template <>
__device__ __forceinline__ df rconst<ArDF>(double c) { return PG_DF_CONST(c); }

}  // namespace pg

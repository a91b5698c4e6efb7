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

// double -> float-float using integer operations only.
// hi is the double with its mantissa truncated to 24 bits; lo is the rounded
// remainder.  Magnitudes outside [2^-126, 2^127] are flushed (to 0 / inf);
// below 2^-74 the lo part underflows and the relative precision degrades to
// single precision.
__device__ __forceinline__ df df_from_double(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  unsigned sign = (unsigned)(b >> 63) << 31;
  int e = (int)((b >> 52) & 0x7FF);
  unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  int ef = e - 896;  // float biased exponent
  if (ef <= 0) return {__uint_as_float(sign), 0.f};
  if (ef >= 255) return {__uint_as_float(sign | 0x7F800000u), 0.f};
  float hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29));
  unsigned r = (unsigned)(m & 0x1FFFFFFFull);  // 29 low bits
  // exact conversion of the two parts of r (6 + 23 bits) via the 2^23 trick
  float rh = __fsub_rn(__uint_as_float(0x4B000000u | (r >> 23)), 8388608.f);
  float rl = __fsub_rn(__uint_as_float(0x4B000000u | (r & 0x7FFFFFu)), 8388608.f);
  float rf = __fmaf_rn(rh, 8388608.f, rl);  // one rounding
  int es = e - 1075 + 127;                   // scale 2^(e-1075)
  float lo = 0.f;
  if (es > 0) lo = __fmul_rn(rf, __uint_as_float((unsigned)es << 23));
  return {hi, sign ? -lo : lo};
}

// float -> double bit pattern, exact, integer operations only (normal floats
// and zero; subnormal floats are flushed to zero).
__device__ __forceinline__ unsigned long long f2d_bits(float f) {
  unsigned u = __float_as_uint(f);
  unsigned long long s = (unsigned long long)(u >> 31) << 63;
  unsigned ef = (u >> 23) & 0xFF;
  if (ef == 0) return s;
  if (ef == 255) return s | 0x7FF0000000000000ull | ((unsigned long long)(u & 0x7FFFFF) << 29);
  return s | ((unsigned long long)(ef + 896) << 52) | ((unsigned long long)(u & 0x7FFFFF) << 29);
}

// float-float -> double (round toward zero on the last bits), integer ops only.
// hi and lo are first merged into one 64-bit two's complement fixed-point
// number in units of 2^(ehi-23-29), then normalised.
__device__ __forceinline__ double df_to_double(df v) {
  unsigned uh = __float_as_uint(v.hi);
  unsigned eh = (uh >> 23) & 0xFF;
  if (eh == 0) {
    // hi is zero (or subnormal): fall back to lo alone
    return __longlong_as_double((long long)f2d_bits(v.lo));
  }
  if (eh == 255) return __longlong_as_double((long long)f2d_bits(v.hi));
  long long mh = (long long)((uh & 0x7FFFFF) | 0x800000) << 29;  // 53-bit magnitude
  if (uh >> 31) mh = -mh;
  unsigned ul = __float_as_uint(v.lo);
  unsigned el = (ul >> 23) & 0xFF;
  long long acc = mh;
  if (el != 0) {
    long long ml = (long long)((ul & 0x7FFFFF) | 0x800000);
    int sh = (int)el - (int)eh + 29;  // lo mantissa weight relative to acc units
    long long t;
    if (sh >= 0) {
      t = sh < 34 ? (ml << sh) : 0;  // |lo| cannot exceed |hi| much; guard anyway
    } else {
      t = sh > -25 ? (ml >> (-sh)) : 0;
    }
    acc += (ul >> 31) ? -t : t;
  }
  if (acc == 0) return 0.0;
  unsigned long long s = 0;
  unsigned long long a = (unsigned long long)acc;
  if (acc < 0) {
    s = 1ull << 63;
    a = (unsigned long long)(-acc);
  }
  int lz = __clzll((long long)a);  // a < 2^55
  int shift = 11 - lz;             // bring leading 1 to bit 52
  int e = (int)eh + 896 + shift;   // double biased exponent
  unsigned long long mant = shift >= 0 ? (a >> shift) : (a << (-shift));
  return __longlong_as_double((long long)(s | ((unsigned long long)e << 52) | (mant & 0xFFFFFFFFFFFFFull)));
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
  static __device__ __forceinline__ void stc(gc_t* p, C v) {
    *p = make_double2(df_to_double(v.x), df_to_double(v.y));
  }
  static __device__ __forceinline__ R ldr(const gr_t* p) { return df_from_double(*p); }
  static __device__ __forceinline__ void str(gr_t* p, R v) { *p = df_to_double(v); }
};

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

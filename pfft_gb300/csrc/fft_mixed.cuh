// Register-resident mixed-radix pass for c2c lines of 3 * 2^a and 5 * 2^a
// points (the companion of the radix-8 kernel in fft_fast.cuh).
//
// Every thread owns E values of its line (E = 12 for 3 * 2^a lengths, radices
// 3, 4 and 2; E = 20 for 5 * 2^a with FP32, E = 10 with float-float, radices
// 5, 4 / 2), N/E threads per line.  The radix schedule is fixed at compile
// time, so every index of every stage is a constant expression: a stage of
// radix R runs E/R butterflies per thread, b = t + i * N/E, with inputs
// x[b + r N/R], twiddles W_{Ns R}^{(b mod Ns) r} and outputs at
// (b - b mod Ns) R + b mod Ns + r Ns (Stockham autosort).  The first stage
// loads from global memory, the last stores to global memory (both
// coalesced as in the radix-8 kernel), the stages in between exchange
// through one shared-memory buffer.  Same arithmetic policies (F32, FDD), the
// same tile layout rules (pad, lsp_of) and the same FastArgs.
#pragma once
#include "fft_fast.cuh"

namespace pg {
namespace fast {

// compile-time radix schedule of a length
template <int N>
struct MixedSched {
  static constexpr bool three = N % 3 == 0;
  static constexpr int E_f32 = three ? 12 : 20;
  static constexpr int E_dd = three ? 12 : 10;
  // radix of stage s (0-based): the odd factor first, then 4s, then a 2
  static constexpr int m2 = three ? N / 3 : N / 5;  // the power of two
  static constexpr int odd = three ? 3 : 5;
  static constexpr int log2m = m2 >= 512 ? 9 : m2 >= 256 ? 8 : m2 >= 128 ? 7 : m2 >= 64 ? 6 : m2 >= 32 ? 5
                               : m2 >= 16 ? 4 : m2 >= 8 ? 3 : m2 >= 4 ? 2 : m2 >= 2 ? 1 : 0;
  template <int E>
  __host__ __device__ static constexpr int stages() {
    // with E = 10 only radix 2 divides E besides 5
    return E == 10 ? 1 + log2m : 1 + log2m / 2 + (log2m & 1);
  }
  template <int E>
  __host__ __device__ static constexpr int radix(int s) {
    return s == 0 ? odd : (E == 10 ? 2 : ((log2m & 1) && s == stages<E>() - 1 ? 2 : 4));
  }
};



template <class P, int SIGN>
__device__ __forceinline__ void bf2(typename P::C* v) {
  typename P::C a = v[0], b = v[1];
  v[0] = P::add(a, b);
  v[1] = P::sub(a, b);
}

template <class P, int SIGN>
__device__ __forceinline__ void bf3(typename P::C* v) {
  typedef typename P::C C;
  constexpr double S3 = 0.86602540378443864676372317075294;
  C t = P::add(v[1], v[2]);
  C u = P::sub(v[1], v[2]);
  C a0 = v[0];
  v[0] = P::add(a0, t);
  C m = P::sub(a0, P::scal(t, PG_KC(P, 0.5)));
  C su = msi<P, SIGN>(P::scal(u, PG_KC(P, S3)));
  v[1] = P::add(m, su);
  v[2] = P::sub(m, su);
}

template <class P, int SIGN>
__device__ __forceinline__ void bf5(typename P::C* v) {
  typedef typename P::C C;
  constexpr double C1 = 0.30901699437494742410229341718282;   // cos(2 pi / 5)
  constexpr double C2 = -0.80901699437494742410229341718282;  // cos(4 pi / 5)
  constexpr double S1 = 0.95105651629515357211643933337938;   // sin(2 pi / 5)
  constexpr double S2 = 0.58778525229247312916870595463907;   // sin(4 pi / 5)
  C a0 = v[0];
  C t1 = P::add(v[1], v[4]), t2 = P::add(v[2], v[3]);
  C u1 = P::sub(v[1], v[4]), u2 = P::sub(v[2], v[3]);
  v[0] = P::add(a0, P::add(t1, t2));
  C m1 = P::add(a0, P::add(P::scal(t1, PG_KC(P, C1)), P::scal(t2, PG_KC(P, C2))));
  C m2 = P::add(a0, P::add(P::scal(t1, PG_KC(P, C2)), P::scal(t2, PG_KC(P, C1))));
  C n1 = msi<P, SIGN>(P::add(P::scal(u1, PG_KC(P, S1)), P::scal(u2, PG_KC(P, S2))));
  C n2 = msi<P, SIGN>(P::sub(P::scal(u1, PG_KC(P, S2)), P::scal(u2, PG_KC(P, S1))));
  v[1] = P::add(m1, n1);
  v[4] = P::sub(m1, n1);
  v[2] = P::add(m2, n2);
  v[3] = P::sub(m2, n2);
}

// ---- block-quantised butterflies (FQ, fft_fast.cuh) ---------------------------------
// The R inputs of a butterfly are rounded to a grid q = 2^(T-24) common to the
// butterfly, T = e - 126 + H for the biased exponent e of the largest high
// word m (m < 2^(e-126)), with 2^H above the radix's bound on every partial
// sum: 2m (radix 2), 4m (radix 4), (2 + sqrt 3) m (radix 3),
// (1 + 2|C1| + 2|C2|) m + 2 (S1 + S2) m = 6.3 m (radix 5, with C, S the
// cosines and sines of 2 pi / 5 and 4 pi / 5), and H >= 2 in any case: the
// rounding x + c1 - c1 (c1 = 0.75 * 2^T) stays in c1's binade, so on the grid,
// only for |x| < 2^(T-2).  H = 2 for radices 2, 3 and 4, 3 for radix 5.  Sums of grid points
// below 2^T are exact; the products with the radix's constants (at most
// sqrt 3 m for radix 3, 1.9 m for radix 5: below 2^(T-1)) are put back on the
// grid one binade up (ulp 2q), their remainders moved to the low words.
template <int R>
__host__ __device__ constexpr int fq_head() {
  return R == 5 ? 3 : 2;
}
template <int R>
__device__ __forceinline__ void fq_grid(const FDD::C* v, float2& c1, float2& c2) {
  constexpr unsigned H = (unsigned)fq_head<R>();
  float m = fmaxf(fabsf(v[0].h.x), fabsf(v[0].h.y));
#pragma unroll
  for (int r = 1; r < R; r++) m = fmaxf(m, fmaxf(fabsf(v[r].h.x), fabsf(v[r].h.y)));
  const unsigned eb = min(__float_as_uint(m) & 0x7F800000u, (253u - H) << 23);  // c2 stays finite
  const float a = __uint_as_float(eb + (H << 23) + 0x400000u);         // 1.5 * 2^(T-1): ulp q
  const float b = __uint_as_float(eb + ((H + 1u) << 23) + 0x400000u);  // 1.5 * 2^T: ulp 2q
  c1 = make_float2(a, a);
  c2 = make_float2(b, b);
}
// k * a for a float-float constant k (exact product of the high words plus
// its error terms), the high word back on the grid of c
__device__ __forceinline__ FDD::C fq_mulc(FDD::C a, DD k, float2 c) {
  const float2 kh = make_float2(k.hi, k.hi), kl = make_float2(k.lo, k.lo);
  const float2 p = mul2(a.h, kh);
  float2 e = fma2(a.h, kh, neg2(p));
  e = fma2(a.h, kl, e);
  e = fma2(a.l, kh, e);
  const float2 pq = sub2(add2(p, c), c);
  return {pq, add2(e, sub2(p, pq))};
}
template <int SIGN>
__device__ __forceinline__ void fq_bf3(FDD::C* v) {
  constexpr double S3 = 0.86602540378443864676372317075294;
  float2 c1, c2;
  fq_grid<3>(v, c1, c2);
#pragma unroll
  for (int r = 0; r < 3; r++) v[r] = fq_round(v[r], c1);
  const FDD::C t = fq_add(v[1], v[2]), u = fq_sub(v[1], v[2]), a0 = v[0];
  v[0] = fq_add(a0, t);
  const FDD::C m = fq_sub(a0, fq_mulc(t, PG_KC(FDD, 0.5), c2));
  const FDD::C su = msi<FDD, SIGN>(fq_mulc(u, PG_KC(FDD, S3), c2));
  v[1] = fq_add(m, su);
  v[2] = fq_sub(m, su);
}
template <int SIGN>
__device__ __forceinline__ void fq_bf5(FDD::C* v) {
  constexpr double C1 = 0.30901699437494742410229341718282;
  constexpr double C2 = -0.80901699437494742410229341718282;
  constexpr double S1 = 0.95105651629515357211643933337938;
  constexpr double S2 = 0.58778525229247312916870595463907;
  float2 c1, c2;
  fq_grid<5>(v, c1, c2);
#pragma unroll
  for (int r = 0; r < 5; r++) v[r] = fq_round(v[r], c1);
  const FDD::C a0 = v[0];
  const FDD::C t1 = fq_add(v[1], v[4]), t2 = fq_add(v[2], v[3]);
  const FDD::C u1 = fq_sub(v[1], v[4]), u2 = fq_sub(v[2], v[3]);
  v[0] = fq_add(a0, fq_add(t1, t2));
  const FDD::C m1 = fq_add(a0, fq_add(fq_mulc(t1, PG_KC(FDD, C1), c2), fq_mulc(t2, PG_KC(FDD, C2), c2)));
  const FDD::C m2 = fq_add(a0, fq_add(fq_mulc(t1, PG_KC(FDD, C2), c2), fq_mulc(t2, PG_KC(FDD, C1), c2)));
  const FDD::C n1 =
      msi<FDD, SIGN>(fq_add(fq_mulc(u1, PG_KC(FDD, S1), c2), fq_mulc(u2, PG_KC(FDD, S2), c2)));
  const FDD::C n2 =
      msi<FDD, SIGN>(fq_sub(fq_mulc(u1, PG_KC(FDD, S2), c2), fq_mulc(u2, PG_KC(FDD, S1), c2)));
  v[1] = fq_add(m1, n1);
  v[4] = fq_sub(m1, n1);
  v[2] = fq_add(m2, n2);
  v[3] = fq_sub(m2, n2);
}

// ---- 64-bit fixed-point butterflies (FX, fft_fast.cuh) ------------------------------
// The radices' constants c as rounded 64-bit fractions (hi, lo) of c 2^64,
// or of 1 - c or 1 + c where c itself does not fit below 2^63; a product
// is then x - x (1 - c) or x (1 + c) - x, each high product rounded once
// (FX::mh).  x / 2 rounds half to even (no steady bias on the exact ties).
__device__ __forceinline__ long long fx_half(long long x) { return (x + ((x >> 1) & 1)) >> 1; }
__device__ __forceinline__ FX::C fx_half(FX::C a) { return {fx_half(a.x), fx_half(a.y)}; }
__device__ __forceinline__ FX::C fx_kmul(FX::C a, int2 k) { return {FX::mh(a.x, k), FX::mh(a.y, k)}; }
__device__ __forceinline__ FX::C fx_kmul_1m(FX::C a, int2 k) {  // a (1 - k)
  return {a.x - FX::mh(a.x, k), a.y - FX::mh(a.y, k)};
}
__device__ __forceinline__ FX::C fx_kmul_m1(FX::C a, int2 k) {  // a (k - 1)
  return {FX::mh(a.x, k) - a.x, FX::mh(a.y, k) - a.y};
}
template <int SIGN>
__device__ __forceinline__ void fx_bf3(FX::C* v) {
  const int2 k1mS3 = make_int2(575416509, 1033546850);  // (1 - sqrt(3)/2) 2^64
  const FX::C t = FX::add(v[1], v[2]), u = FX::sub(v[1], v[2]), a0 = v[0];
  v[0] = FX::add(a0, t);
  const FX::C m = FX::sub(a0, fx_half(t));
  const FX::C su = msi<FX, SIGN>(fx_kmul_1m(u, k1mS3));
  v[1] = FX::add(m, su);
  v[2] = FX::sub(m, su);
}
template <int SIGN>
__device__ __forceinline__ void fx_bf5(FX::C* v) {
  const int2 kC1 = make_int2(1327217885, -1079689717);   // cos(2 pi / 5) 2^64
  const int2 k1pC2 = make_int2(820265763, 1079689717);   // (1 + cos(4 pi / 5)) 2^64
  const int2 k1mS1 = make_int2(210210662, -581434099);   // (1 - sin(2 pi / 5)) 2^64
  const int2 k1mS2 = make_int2(1770448860, 1429016722);  // (1 - sin(4 pi / 5)) 2^64
  const FX::C a0 = v[0];
  const FX::C t1 = FX::add(v[1], v[4]), t2 = FX::add(v[2], v[3]);
  const FX::C u1 = FX::sub(v[1], v[4]), u2 = FX::sub(v[2], v[3]);
  v[0] = FX::add(a0, FX::add(t1, t2));
  const FX::C m1 = FX::add(a0, FX::add(fx_kmul(t1, kC1), fx_kmul_m1(t2, k1pC2)));
  const FX::C m2 = FX::add(a0, FX::add(fx_kmul_m1(t1, k1pC2), fx_kmul(t2, kC1)));
  const FX::C n1 = msi<FX, SIGN>(FX::add(fx_kmul_1m(u1, k1mS1), fx_kmul_1m(u2, k1mS2)));
  const FX::C n2 = msi<FX, SIGN>(FX::sub(fx_kmul_1m(u1, k1mS2), fx_kmul_1m(u2, k1mS1)));
  v[1] = FX::add(m1, n1);
  v[4] = FX::sub(m1, n1);
  v[2] = FX::add(m2, n2);
  v[3] = FX::sub(m2, n2);
}

template <class P, int SIGN, int R>
__device__ __forceinline__ void bfR(typename P::C* v) {
  if constexpr (is_fx<P>() && (R == 3 || R == 5)) {
    if constexpr (R == 3) fx_bf3<SIGN>(v);
    if constexpr (R == 5) fx_bf5<SIGN>(v);
  } else if constexpr (std::is_same<P, FQ>::value) {
    if constexpr (R == 2 || R == 4) {
      float2 c1, c2;
      fq_grid<R>(v, c1, c2);
#pragma unroll
      for (int r = 0; r < R; r++) v[r] = fq_round(v[r], c1);
      if constexpr (R == 2) {
        const FDD::C a = v[0], b = v[1];
        v[0] = fq_add(a, b);
        v[1] = fq_sub(a, b);
      } else {
        fq_bf4<SIGN>(v[0], v[1], v[2], v[3]);
      }
    }
    if constexpr (R == 3) fq_bf3<SIGN>(v);
    if constexpr (R == 5) fq_bf5<SIGN>(v);
  } else {
    if constexpr (R == 2) bf2<P, SIGN>(v);
    if constexpr (R == 3) bf3<P, SIGN>(v);
    if constexpr (R == 4) bf4<P, SIGN>(v[0], v[1], v[2], v[3]);
    if constexpr (R == 5) bf5<P, SIGN>(v);
  }
}

template <class P>
__host__ __device__ constexpr int mixed_E(int N) {
  return sizeof(typename P::S) == 8 ? (N % 3 == 0 ? 12 : 20) : (N % 3 == 0 ? 12 : 10);
}

// stage s: v holds this stage's inputs (E/R butterflies of R values); run
// the butterflies, then either store to global (last stage) or exchange
// through shared memory into the next stage's inputs
template <class P, int SIGN, int N, int E, int s>
struct MixedStage {
  typedef typename P::C C;
  typedef typename P::S S;
  static constexpr int NS = MixedSched<N>::template stages<E>();
  static constexpr int R = MixedSched<N>::template radix<E>(s);
  static constexpr int TPL = N / E;

  __host__ __device__ static constexpr int ns() {  // product of the radices before stage s
    int p = 1;
    for (int q = 0; q < s; q++) p *= MixedSched<N>::template radix<E>(q);
    return p;
  }

  // twiddles and butterflies of this stage (inputs in v, outputs in place;
  // FX twiddles carry 1/4, element 0 of a twiddled stage takes it alone)
  static __device__ __forceinline__ void compute(C* v, int t, const void* tw) {
    constexpr int Ns = ns();
#pragma unroll
    for (int i = 0; i < E / R; i++) {
      const int b = t + i * TPL;
      if (Ns > 1) {
        const int k = b % Ns;
        constexpr int step = N / (Ns * R);
        if constexpr (is_fx<P>()) v[i * R] = P::tw0(v[i * R]);
#pragma unroll
        for (int r = 1; r < R; r++) v[i * R + r] = P::mul(v[i * R + r], P::template twd<SIGN>(P::ldw(tw, k * r * step, N)));
      }
      bfR<P, SIGN, R>(v + i * R);
    }
  }

  // shared-memory index of output r of butterfly i (natural position)
  static __device__ __forceinline__ int out_pos(int t, int i, int r) {
    constexpr int Ns = ns();
    const int b = t + i * TPL;
    const int k = b % Ns;
    return (b - k) * R + k + r * Ns;
  }
};

// fxsh (FX): the shifts and twiddle scalings so far, added to the results'
// exponent; each exchange brings the tile's largest component to 59 bits
// (every thread of the block takes part: the exchanges are block-wide)
template <class P, int SIGN, int N, int E, int s>
__device__ __forceinline__ void mixed_stages(typename P::C (&v)[E], int t, const void* tw, typename P::S* line, int& fxsh) {
  typedef MixedStage<P, SIGN, N, E, s> St;
  St::compute(v, t, tw);
  if constexpr (s + 1 < St::NS) {
    // exchange: outputs to shared memory, next stage's inputs back
    __syncthreads();  // the previous exchange's loads are done
    if constexpr (is_fx<P>()) fx_ormag_publish(fx_ormag(v), fx_slots() + 32 * (s & 1));
#pragma unroll
    for (int i = 0; i < E / St::R; i++)
#pragma unroll
      for (int r = 0; r < St::R; r++) line[pad<P>(St::out_pos(t, i, r))] = P::sts(v[i * St::R + r]);
    __syncthreads();
    constexpr int R2 = MixedSched<N>::template radix<E>(s + 1);
#pragma unroll
    for (int i = 0; i < E / R2; i++)
#pragma unroll
      for (int r = 0; r < R2; r++) v[i * R2 + r] = P::lds(line[pad<P>(t + i * (N / E) + r * (N / R2))]);
    if constexpr (is_fx<P>()) {
      const int sh = fx_normal_shift(fx_slots() + 32 * (s & 1));
      fx_shift_all(v, sh);
      fxsh += sh + 2;  // the next stage is twiddled
    }
    mixed_stages<P, SIGN, N, E, s + 1>(v, t, tw, line, fxsh);
  }
}

// One tile (L lines) of a mixed-radix pass: L * N/E threads.
template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT, bool CG = false>
__device__ __forceinline__ void mixed_tile(const FastArgs& a, long long blk, unsigned char* sm_raw) {
  typedef typename P::C C;
  typedef typename P::S S;
  typedef typename P::G G;
  constexpr int E = mixed_E<P>(N);
  constexpr int TPL = N / E;
  constexpr int NS = MixedSched<N>::template stages<E>();
  constexpr int RL = MixedSched<N>::template radix<E>(NS - 1);  // last radix
  constexpr int R0 = MixedSched<N>::template radix<E>(0);
  constexpr int LSP = lsp_of<P, N, L, ROW_IN>();
  long long* offI = (long long*)sm_raw;
  long long* offO = offI + L;
  S* buf = (S*)(sm_raw + 16 * L);

  const int tid = threadIdx.x;
  const long long g0 = blk * L;
  if (tid < L) {
    long long g = g0 + tid;
    if (g >= a.nlines) g = a.nlines - 1;  // tail tile: clamp (duplicate work, never stored)
    long long oi = 0, oo = 0;
    for (int b = 0; b < a.nb; b++) {
      long long e = a.bext[b];
      long long idx = g % e;
      g /= e;
      oi += idx * a.bsI[b];
      oo += idx * a.bsO[b];
    }
    offI[tid] = oi;
    offO[tid] = oo;
  }
  __syncthreads();
  const int l = ROW_IN ? tid / TPL : tid % L;
  const int t = ROW_IN ? tid % TPL : tid / L;
  const bool live = (g0 + l) < a.nlines;
  const void* tw = a.tw;  // natural-order table of N entries
  S* line = buf + l * LSP;

  // plain c2c lines only (fast_args sends no other mode here)
  C v[E];
  {
    const G* src = (const G*)a.src + offI[l];
#pragma unroll
    for (int i = 0; i < E / R0; i++)
#pragma unroll
      for (int r = 0; r < R0; r++) {
        const long long e = t + i * TPL + r * (N / R0);
        C x = gload<P, CG>(src + e * a.sIa, a.in_df);
        if constexpr (is_fx<P>())
          v[i * R0 + r] = x;  // double bits; fx_enter conjugates
        else
          v[i * R0 + r] = a.conj_in ? P::conj(x) : x;
      }
  }
  // FX: the tile onto its grid; sdf the results' exponent
  int fxsh = 0, sdf = a.out_df;
  int fx_e = 0;
  if constexpr (is_fx<P>()) fx_e = fx_enter<N, E>(v, a.conj_in);
  mixed_stages<P, SIGN, N, E, 0>(v, t, tw, line, fxsh);
  if constexpr (is_fx<P>()) sdf = fx_e == INT_MIN ? INT_MIN : fx_e + fxsh;
  // last stage: output r of butterfly i is element t + i * TPL + r * N/RL
  if (ROW_IN == ROW_OUT) {
    if (live) {
      G* dst = (G*)a.dst + offO[l];
#pragma unroll
      for (int i = 0; i < E / RL; i++)
#pragma unroll
        for (int r = 0; r < RL; r++) {
          const int e = t + i * TPL + r * (N / RL);
          C o = v[i * RL + r];
          gstore<P>(dst + (long long)e * a.sOa, a.conj_out ? P::conj(o) : o, sdf);
        }
    }
    return;
  }
  // transposing pass: restage with the output's thread mapping
  __syncthreads();
#pragma unroll
  for (int i = 0; i < E / RL; i++)
#pragma unroll
    for (int r = 0; r < RL; r++) line[pad<P>(t + i * TPL + r * (N / RL))] = P::sts(v[i * RL + r]);
  __syncthreads();
  const int l2 = ROW_OUT ? tid / TPL : tid % L;
  const int t2 = ROW_OUT ? tid % TPL : tid / L;
  if ((g0 + l2) < a.nlines) {
    G* d2 = (G*)a.dst + offO[l2];
    const S* line2 = buf + l2 * LSP;
#pragma unroll
    for (int q = 0; q < E; q++) {
      const int k = t2 + q * TPL;
      C o = P::lds(line2[pad<P>(k)]);
      gstore<P>(d2 + (long long)k * a.sOa, a.conj_out ? P::conj(o) : o, sdf);
    }
  }
}

template <class P, int SIGN, int N, int L, bool ROW_IN, bool ROW_OUT>
__global__ void __launch_bounds__(L*(N / mixed_E<P>(N))) k_mixed(const FastArgs a) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  mixed_tile<P, SIGN, N, L, ROW_IN, ROW_OUT>(a, blockIdx.x, sm_raw);
}

template <class P, int N, int L>
constexpr size_t mixed_smem_bytes() {
  return 16 * L + (size_t)L * (sizeof(typename P::S) == 8 ? N + 16 : N + N / 8 + 4) * sizeof(typename P::S);
}

// lines per CTA: about 256 threads
template <class P>
__host__ __device__ constexpr int mixed_L(int N) {
  return 256 / (N / mixed_E<P>(N)) > 0 ? 256 / (N / mixed_E<P>(N)) : 1;
}

template <class P, int SIGN, int N>
int launch_mixed_n(const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  constexpr int L = mixed_L<P>(N);
  constexpr int T = L * (N / mixed_E<P>(N));
  const size_t smem = mixed_smem_bytes<P, N, L>();
  long long grid = (a.nlines + L - 1) / L;
  if (grid > 2147483647LL) return (int)cudaErrorInvalidConfiguration;
  cudaError_t e = cudaSuccess;
#define PG_MIXED_LAUNCH(RI, RO)                                                                            \
  do {                                                                                                     \
    static bool attr_done = false;                                                                         \
    if (!attr_done) {                                                                                      \
      e = cudaFuncSetAttribute(k_mixed<P, SIGN, N, L, RI, RO>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                               (int)smem);                                                                 \
      if (e != cudaSuccess) return (int)e;                                                                 \
      attr_done = true;                                                                                    \
    }                                                                                                      \
    k_mixed<P, SIGN, N, L, RI, RO><<<(unsigned)grid, T, smem, s>>>(a);                                     \
  } while (0)
  if (row_in && row_out)
    PG_MIXED_LAUNCH(true, true);
  else if (!row_in && !row_out)
    PG_MIXED_LAUNCH(false, false);
  else if (row_in)
    PG_MIXED_LAUNCH(true, false);
  else
    PG_MIXED_LAUNCH(false, true);
#undef PG_MIXED_LAUNCH
  return (int)cudaGetLastError();
}

// lengths with a mixed-radix kernel
__host__ __device__ constexpr bool mixed_supported(int N) {
  return N == 24 || N == 40 || N == 48 || N == 80 || N == 96 || N == 160 || N == 192 || N == 320 || N == 384 ||
         N == 640 || N == 768;
}

// launchers, one instantiation set per unit (fft_mixed_<arith>_<dir>_<family>.cu)
template <class P, int SIGN>
int launch_mixed_three(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);
template <class P, int SIGN>
int launch_mixed_five(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s);

}  // namespace fast
}  // namespace pg

// Generic pass: butterflies, gather/scatter of every mode, and the tile
// routine shared by the per-pass kernel (fft_pass.cu) and the batched
// persistent kernel (batch.cu).
//
// Shared-memory Stockham autosort FFT, mixed radix.  A stage of radix R with
// Ns = product of the earlier radices maps, for j < M/R and k = j mod Ns,
//   x[j + r*M/R] * W_{Ns*R}^{k*r}  --DFT_R-->  y[(j-k)*R + k + r*Ns]
// so after the last stage the line is in natural order.  Radices 2,3,4,5,8,16
// have dedicated butterflies, small odd primes (7, 11, 13) use a register DFT
// with table twiddles, and any other prime uses a shared-memory ping-pong stage.
#pragma once
#include "arith.cuh"
#include "pass.h"

namespace pg {

// Complex values a thread holds in registers in one register stage: 16 for
// FP32, 8 for float-float and FP64 (whose values are twice as wide), so that
// the stage fits the register file without spilling.
template <class A>
__host__ __device__ constexpr int max_elems() {
  return A::kId == ARITH_F32 ? 16 : 8;
}

template <class A, bool CG = false>
struct K {
  typedef typename A::C C;
  typedef typename A::R R;
  typedef typename A::sm_t S;

  // multiply by SIGN*i
  template <int SIGN>
  static __device__ __forceinline__ C mul_si(C a) {
    if (SIGN < 0) return A::make(a.y, A::rneg(a.x));
    return A::make(A::rneg(a.y), a.x);
  }
  // multiply by a constant (cr + i*ci)
  static __device__ __forceinline__ C cmul(C a, R cr, R ci) {
    return A::make(A::rsub(A::rmul(a.x, cr), A::rmul(a.y, ci)), A::radd(A::rmul(a.x, ci), A::rmul(a.y, cr)));
  }
  template <int SIGN>
  static __device__ __forceinline__ C tw(const S* t, int idx) {
    C w = A::lds(t[idx]);
    return SIGN < 0 ? w : A::conj(w);
  }

  template <int SIGN>
  static __device__ __forceinline__ void dft4(C& a0, C& a1, C& a2, C& a3) {
    C t0 = A::add(a0, a2), t1 = A::sub(a0, a2);
    C t2 = A::add(a1, a3), t3 = mul_si<SIGN>(A::sub(a1, a3));
    a0 = A::add(t0, t2);
    a2 = A::sub(t0, t2);
    a1 = A::add(t1, t3);
    a3 = A::sub(t1, t3);
  }

  // multiply by W8^e (e = 1, 3) of direction SIGN
  template <int SIGN, int E>
  static __device__ __forceinline__ C w8(C z) {
    const R c = rconst<A>(0.70710678118654752440084436210485);
    if (E == 1) {
      // c*((x - S*y) + i(y + S*x))
      C t = SIGN < 0 ? A::make(A::radd(z.x, z.y), A::rsub(z.y, z.x)) : A::make(A::rsub(z.x, z.y), A::radd(z.y, z.x));
      return A::make(A::rmul(t.x, c), A::rmul(t.y, c));
    } else {
      // c*((-x - S*y) + i(-y + S*x))
      C t = SIGN < 0 ? A::make(A::rsub(z.y, z.x), A::rneg(A::radd(z.x, z.y))) : A::make(A::rneg(A::radd(z.x, z.y)), A::rsub(z.x, z.y));
      return A::make(A::rmul(t.x, c), A::rmul(t.y, c));
    }
  }

  template <int SIGN, int R_>
  static __device__ __forceinline__ void dft(C* v, const S* t, int M) {
    if constexpr (R_ == 2) {
      C a = v[0], b = v[1];
      v[0] = A::add(a, b);
      v[1] = A::sub(a, b);
    } else if constexpr (R_ == 4) {
      dft4<SIGN>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R_ == 8) {
      dft4<SIGN>(v[0], v[2], v[4], v[6]);
      dft4<SIGN>(v[1], v[3], v[5], v[7]);
      C o1 = w8<SIGN, 1>(v[3]);
      C o2 = mul_si<SIGN>(v[5]);
      C o3 = w8<SIGN, 3>(v[7]);
      C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
      C o0 = v[1];
      v[0] = A::add(e0, o0);
      v[4] = A::sub(e0, o0);
      v[1] = A::add(e1, o1);
      v[5] = A::sub(e1, o1);
      v[2] = A::add(e2, o2);
      v[6] = A::sub(e2, o2);
      v[3] = A::add(e3, o3);
      v[7] = A::sub(e3, o3);
    } else if constexpr (R_ == 16) {
      // 4 x 4: columns q, rows m (n = 4m + q)
#pragma unroll
      for (int q = 0; q < 4; q++) dft4<SIGN>(v[q], v[q + 4], v[q + 8], v[q + 12]);
      // after dft4 on (q, q+4, q+8, q+12): v[q + 4*k1] = Y_q[k1]
      const R c1 = rconst<A>(0.92387953251128675612818318939679);  // cos(pi/8)
      const R s1 = rconst<A>(0.38268343236508977172845998403040);  // sin(pi/8)
      const R sg1 = SIGN < 0 ? A::rneg(s1) : s1;
      const R sg3 = SIGN < 0 ? A::rneg(c1) : c1;
      // W16^{q*k1}: q=1: k1=1 -> W^1, k1=2 -> W^2, k1=3 -> W^3
      v[1 + 4] = cmul(v[1 + 4], c1, sg1);
      v[1 + 8] = w8<SIGN, 1>(v[1 + 8]);
      v[1 + 12] = cmul(v[1 + 12], s1, sg3);
      // q=2: W^2, W^4, W^6
      v[2 + 4] = w8<SIGN, 1>(v[2 + 4]);
      v[2 + 8] = mul_si<SIGN>(v[2 + 8]);
      v[2 + 12] = w8<SIGN, 3>(v[2 + 12]);
      // q=3: W^3, W^6, W^9 = -W^1
      v[3 + 4] = cmul(v[3 + 4], s1, sg3);
      v[3 + 8] = w8<SIGN, 3>(v[3 + 8]);
      v[3 + 12] = A::neg(cmul(v[3 + 12], c1, sg1));
      // rows: for each k1, DFT4 over q -> X[k1 + 4*k2]
      C o[16];
#pragma unroll
      for (int k1 = 0; k1 < 4; k1++) {
        C a0 = v[0 + 4 * k1], a1 = v[1 + 4 * k1], a2 = v[2 + 4 * k1], a3 = v[3 + 4 * k1];
        dft4<SIGN>(a0, a1, a2, a3);
        o[k1] = a0;
        o[k1 + 4] = a1;
        o[k1 + 8] = a2;
        o[k1 + 12] = a3;
      }
#pragma unroll
      for (int i = 0; i < 16; i++) v[i] = o[i];
    } else if constexpr (R_ == 3) {
      const R h = rconst<A>(0.5);
      const R s3 = rconst<A>(0.86602540378443864676372317075294);
      C t = A::add(v[1], v[2]);
      C u = A::sub(v[1], v[2]);
      C a0 = v[0];
      v[0] = A::add(a0, t);
      C m = A::sub(a0, A::make(A::rmul(t.x, h), A::rmul(t.y, h)));
      C su = mul_si<SIGN>(A::make(A::rmul(u.x, s3), A::rmul(u.y, s3)));
      v[1] = A::add(m, su);
      v[2] = A::sub(m, su);
    } else if constexpr (R_ == 5) {
      const R c1 = rconst<A>(0.30901699437494742410229341718282);   // cos(2pi/5)
      const R c2 = rconst<A>(-0.80901699437494742410229341718282);  // cos(4pi/5)
      const R s1 = rconst<A>(0.95105651629515357211643933337938);   // sin(2pi/5)
      const R s2 = rconst<A>(0.58778525229247312916870595463907);   // sin(4pi/5)
      C a0 = v[0];
      C t1 = A::add(v[1], v[4]), t2 = A::add(v[2], v[3]);
      C u1 = A::sub(v[1], v[4]), u2 = A::sub(v[2], v[3]);
      v[0] = A::add(a0, A::add(t1, t2));
      C m1 = A::add(a0, A::add(A::make(A::rmul(t1.x, c1), A::rmul(t1.y, c1)), A::make(A::rmul(t2.x, c2), A::rmul(t2.y, c2))));
      C m2 = A::add(a0, A::add(A::make(A::rmul(t1.x, c2), A::rmul(t1.y, c2)), A::make(A::rmul(t2.x, c1), A::rmul(t2.y, c1))));
      C n1 = A::add(A::make(A::rmul(u1.x, s1), A::rmul(u1.y, s1)), A::make(A::rmul(u2.x, s2), A::rmul(u2.y, s2)));
      C n2 = A::sub(A::make(A::rmul(u1.x, s2), A::rmul(u1.y, s2)), A::make(A::rmul(u2.x, s1), A::rmul(u2.y, s1)));
      n1 = mul_si<SIGN>(n1);
      n2 = mul_si<SIGN>(n2);
      v[1] = A::add(m1, n1);
      v[4] = A::sub(m1, n1);
      v[2] = A::add(m2, n2);
      v[3] = A::sub(m2, n2);
    } else {
      // generic small odd radix with table twiddles W_M^{(n*k mod R)*M/R}
      C o[R_];
      const int step = M / R_;
#pragma unroll
      for (int k = 0; k < R_; k++) {
        C acc = v[0];
#pragma unroll
        for (int n = 1; n < R_; n++) {
          int e = (n * k) % R_;
          acc = A::add(acc, e == 0 ? v[n] : A::mul(v[n], tw<SIGN>(t, e * step)));
        }
        o[k] = acc;
      }
#pragma unroll
      for (int k = 0; k < R_; k++) v[k] = o[k];
    }
  }

  // One register-staged Stockham stage of radix R_ over L lines.
  template <int SIGN, int R_>
  static __device__ __forceinline__ void reg_stage(S* buf, int L, int M, int LS, int Ns, const S* t) {
    constexpr int NB = max_elems<A>() / R_ > 0 ? max_elems<A>() / R_ : 1;
    C v[NB][R_];
    int jj[NB], ll[NB];
    const int MR = M / R_;
    const int total = L * MR;
#pragma unroll
    for (int i = 0; i < NB; i++) {
      int b = threadIdx.x + i * blockDim.x;
      ll[i] = -1;
      jj[i] = 0;
      if (b < total) {
        int l = b / MR;
        int j = b - l * MR;
        ll[i] = l;
        jj[i] = j;
        const S* src = buf + l * LS + j;
#pragma unroll
        for (int r = 0; r < R_; r++) v[i][r] = A::lds(src[r * MR]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NB; i++) {
      if (ll[i] >= 0) {
        int j = jj[i];
        int k = j % Ns;
        if (Ns > 1) {
          int step = M / (Ns * R_);
#pragma unroll
          for (int r = 1; r < R_; r++) v[i][r] = A::mul(v[i][r], tw<SIGN>(t, k * r * step));
        }
        dft<SIGN, R_>(v[i], t, M);
        S* dst = buf + ll[i] * LS + (j - k) * R_ + k;
#pragma unroll
        for (int r = 0; r < R_; r++) dst[r * Ns] = A::sts(v[i][r]);
      }
    }
    __syncthreads();
  }

  // Generic radix stage (any R), shared-memory ping-pong: reads a, writes b.
  template <int SIGN>
  static __device__ void generic_stage(const S* a, S* b, int L, int M, int LS, int Ns, int R_, const S* t) {
    const int MR = M / R_;
    const int total = L * M;
    const int step = M / (Ns * R_);
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      int l = e / M;
      int rem = e - l * M;
      int j = rem % MR;
      int kk = rem / MR;  // output digit 0..R-1
      int k = j % Ns;
      const S* src = a + l * LS + j;
      C acc = A::lds(src[0]);
      long long base = (long long)k + (long long)kk * Ns;
      for (int r = 1; r < R_; r++) {
        int idx = (int)(((long long)step * r * base) % M);
        acc = A::add(acc, A::mul(A::lds(src[r * MR]), tw<SIGN>(t, idx)));
      }
      b[l * LS + (j - k) * R_ + k + kk * Ns] = A::sts(acc);
    }
    __syncthreads();
  }

  static __device__ __forceinline__ int shsign(const ShiftSign& s, long long i) {
    if (!s.en) return 1;
    long long tt = i + s.start;
    if (tt < s.thresh) return (tt & 1) ? -s.extra : s.extra;
    return 1;
  }

  static __device__ __forceinline__ C apply_sign(C v, int sg) { return sg < 0 ? A::neg(v) : v; }
  static __device__ __forceinline__ R rsign(R v, int sg) { return sg < 0 ? A::rneg(v) : v; }

  // logical input (complex) element q of line l, with conj and shift sign
  static __device__ __forceinline__ C load_c(const PassParams& p, long long off, int q, int lsg) {
    const typename A::gc_t* src = (const typename A::gc_t*)p.src;
    const typename A::gc_t* ptr = src + off + (long long)q * p.sIa;
    C v;
    if constexpr (A::kId == ARITH_DF) {
      if (p.in_df)
        v = A::lds(ldraw<CG>((const float4*)ptr));
      else
        v = A::cvc(ldraw<CG>(ptr));
    } else {
      v = A::cvc(ldraw<CG>(ptr));
    }
    if (p.conj_in) v = A::conj(v);
    return apply_sign(v, lsg * shsign(p.ashI, q));
  }
  static __device__ __forceinline__ R load_r(const PassParams& p, long long off, int q, int lsg) {
    const typename A::gr_t* src = (const typename A::gr_t*)p.src;
    R v = A::cvr(ldraw<CG>(src + off + (long long)q * p.sIa));
    return rsign(v, lsg * shsign(p.ashI, q));
  }
  // logical real input x~_i (embedded), zero outside the data range
  static __device__ __forceinline__ R xr(const PassParams& p, long long off, int i, int lsg) {
    int q = i - p.Zi;
    if (q < 0 || q >= p.Ni) return A::rzero();
    return load_r(p, off, q, lsg);
  }
  static __device__ __forceinline__ C xc(const PassParams& p, long long off, int i, int lsg) {
    int q = i - p.Zi;
    if (q < 0 || q >= p.Ni) return A::zero();
    return load_c(p, off, q, lsg);
  }

  // value of the length-M sequence at position pos for line l
  template <bool C2C_ONLY = false>
  static __device__ __forceinline__ C gather(const PassParams& p, long long off, int pos, int lsg) {
    if (C2C_ONLY) return xc(p, off, pos, lsg);
    const int N = p.N, M = p.M;
    switch (p.mode) {
      case MODE_C2C:
        return xc(p, off, pos, lsg);
      case MODE_R2C:
      case MODE_R2HC:
      case MODE_DHT:
      case MODE_COPYR:
        return A::make(xr(p, off, pos, lsg), A::rzero());
      case MODE_C2R: {
        int k = (2 * pos <= M) ? pos : M - pos;
        C v = xc(p, off, k, lsg);
        if (p.wmode == 1 && k != 0 && 2 * k != M) v = A::scale(v, rconst<A>(0.5));
        return (2 * pos <= M) ? v : A::conj(v);
      }
      case MODE_HC2R: {
        if (pos == 0) return A::make(xr(p, off, 0, lsg), A::rzero());
        if (2 * pos == M) return A::make(xr(p, off, pos, lsg), A::rzero());
        if (2 * pos < M) return A::make(xr(p, off, pos, lsg), xr(p, off, M - pos, lsg));
        return A::make(xr(p, off, M - pos, lsg), A::rneg(xr(p, off, pos, lsg)));
      }
      case MODE_RE00: {
        int i = pos < N ? pos : M - pos;
        return A::make(xr(p, off, i, lsg), A::rzero());
      }
      case MODE_RO00: {
        if (pos == 0 || pos == N + 1) return A::zero();
        if (pos <= N) return A::make(xr(p, off, pos - 1, lsg), A::rzero());
        return A::make(A::rneg(xr(p, off, M - pos - 1, lsg)), A::rzero());
      }
      case MODE_RE10:
      case MODE_RO10: {
        if (!(pos & 1)) return A::zero();
        if (pos < 2 * N) return A::make(xr(p, off, (pos - 1) >> 1, lsg), A::rzero());
        R v = xr(p, off, (M - pos - 1) >> 1, lsg);
        return A::make(p.mode == MODE_RO10 ? A::rneg(v) : v, A::rzero());
      }
      case MODE_RE11:
      case MODE_RO11: {
        if (!(pos & 1)) return A::zero();
        if (pos < 2 * N) return A::make(xr(p, off, (pos - 1) >> 1, lsg), A::rzero());
        if (pos > 6 * N) {
          R v = xr(p, off, (M - pos - 1) >> 1, lsg);
          return A::make(p.mode == MODE_RO11 ? A::rneg(v) : v, A::rzero());
        }
        return A::zero();
      }
      case MODE_RE01: {
        if (pos < N) return A::make(xr(p, off, pos, lsg), A::rzero());
        if (pos > 3 * N) return A::make(xr(p, off, M - pos, lsg), A::rzero());
        return A::zero();
      }
      case MODE_RO01: {
        if (pos >= 1 && pos <= N) return A::make(xr(p, off, pos - 1, lsg), A::rzero());
        if (pos > 3 * N) return A::make(A::rneg(xr(p, off, M - pos - 1, lsg)), A::rzero());
        return A::zero();
      }
    }
    return A::zero();
  }

  // output element k (logical index o = Zo + k) of line l
  template <bool C2C_ONLY = false>
  static __device__ __forceinline__ void scatter(const PassParams& p, const S* line, long long off, int k, int lsg) {
    const int o = p.Zo + k;
    const int sg = lsg * shsign(p.ashO, k);
    switch (C2C_ONLY ? (int)MODE_C2C : p.mode) {
      case MODE_C2C:
      case MODE_R2C: {
        C v = A::lds(line[o]);
        if (p.wmode == 2 && o != 0 && 2 * o != p.M) v = A::scale(v, rconst<A>(2.0));
        if (p.conj_out) v = A::conj(v);
        typename A::gc_t* dst = (typename A::gc_t*)p.dst;
        if constexpr (A::kId == ARITH_DF) {
          if (p.out_df) {
            *(float4*)(dst + off + (long long)k * p.sOa) = A::sts(apply_sign(v, sg));
            return;
          }
        }
        A::stc(dst + off + (long long)k * p.sOa, apply_sign(v, sg));
        return;
      }
      default:
        break;
    }
    R r;
    switch (p.mode) {
      case MODE_C2R:
      case MODE_COPYR:
      case MODE_RE00:
      case MODE_RE10:
      case MODE_HC2R:
        r = A::lds(line[o]).x;
        break;
      case MODE_RO00:
      case MODE_RO10:
        r = A::rneg(A::lds(line[o + 1]).y);
        break;
      case MODE_RE01:
      case MODE_RE11:
        r = A::lds(line[2 * o + 1]).x;
        break;
      case MODE_RO01:
      case MODE_RO11:
        r = A::rneg(A::lds(line[2 * o + 1]).y);
        break;
      case MODE_R2HC:
        r = (2 * o <= p.N) ? A::lds(line[o]).x : A::lds(line[p.N - o]).y;
        break;
      case MODE_DHT: {
        C v = A::lds(line[o]);
        r = A::rsub(v.x, v.y);
        break;
      }
      default:
        r = A::rzero();
    }
    typename A::gr_t* dst = (typename A::gr_t*)p.dst;
    A::str(dst + off + (long long)k * p.sOa, rsign(r, sg));
  }
};

// One tile (L lines) of a pass.  smraw: dynamic shared memory of at least
// p.smem_bytes.  CG: read global memory through L2 only (batched launches,
// where the input was written by other CTAs of the same launch).
// SMALL: a c2c pass with radices 2, 3, 4, 5, 7 and 8 only (no 11, 13, 16 or
// generic-prime stage, no real-data modes); the kernel then needs far fewer
// registers.
template <class A, int SIGN, bool CG, bool SMALL = false>
__device__ __forceinline__ void pass_tile(const PassParams& p, long long tile, unsigned char* smraw) {
  typedef K<A, CG> KK;
  typedef typename A::sm_t S;
  // per-line metadata first, then the data buffer(s)
  long long* offI = (long long*)smraw;
  long long* offO = offI + p.L;
  int* sgI = (int*)(offO + p.L);
  int* sgO = sgI + p.L;
  int meta = (int)(((2 * sizeof(long long) + 2 * sizeof(int)) * p.L + 15) & ~15);
  S* buf = (S*)(smraw + meta);
  S* buf2 = buf + (size_t)p.L * p.LS;

  const long long g0 = tile * p.L;
  int L = p.L;
  if (g0 + L > p.nlines) L = (int)(p.nlines - g0);

  for (int l = threadIdx.x; l < L; l += blockDim.x) {
    long long g = g0 + l;
    long long oi = 0, oo = 0;
    int si = 1, so = 1;
    for (int b = 0; b < p.nb; b++) {
      long long e = p.bext[b];
      long long idx = g % e;
      g /= e;
      oi += idx * p.bsI[b];
      oo += idx * p.bsO[b];
      si *= KK::shsign(p.bshI[b], idx);
      so *= KK::shsign(p.bshO[b], idx);
    }
    offI[l] = oi;
    offO[l] = oo;
    sgI[l] = si;
    sgO[l] = so;
  }
  __syncthreads();

  // gather
  const int M = p.M;
  const int tot = L * M;
  if (p.in_contig) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      int l = e / M;
      int pos = e - l * M;
      buf[l * p.LS + pos] = A::sts(KK::template gather<SMALL>(p, offI[l], pos, sgI[l]));
    }
  } else {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      int pos = e / L;
      int l = e - pos * L;
      buf[l * p.LS + pos] = A::sts(KK::template gather<SMALL>(p, offI[l], pos, sgI[l]));
    }
  }
  __syncthreads();

  // FFT stages
  const S* t = (const S*)p.tw;
  int Ns = 1;
  S* cur = buf;
  S* alt = buf2;
  for (int s = 0; s < p.nst; s++) {
    int R_ = p.radix[s];
    switch (R_) {
      case 2: KK::template reg_stage<SIGN, 2>(cur, L, M, p.LS, Ns, t); break;
      case 3: KK::template reg_stage<SIGN, 3>(cur, L, M, p.LS, Ns, t); break;
      case 4: KK::template reg_stage<SIGN, 4>(cur, L, M, p.LS, Ns, t); break;
      case 5: KK::template reg_stage<SIGN, 5>(cur, L, M, p.LS, Ns, t); break;
      case 7: KK::template reg_stage<SIGN, 7>(cur, L, M, p.LS, Ns, t); break;
      case 8: KK::template reg_stage<SIGN, 8>(cur, L, M, p.LS, Ns, t); break;
      case 11: if (!SMALL) KK::template reg_stage<SIGN, 11>(cur, L, M, p.LS, Ns, t); break;
      case 13: if (!SMALL) KK::template reg_stage<SIGN, 13>(cur, L, M, p.LS, Ns, t); break;
      case 16: if (!SMALL) KK::template reg_stage<SIGN, 16>(cur, L, M, p.LS, Ns, t); break;
      default: if (!SMALL) {
        KK::template generic_stage<SIGN>(cur, alt, L, M, p.LS, Ns, R_, t);
        S* tmp = cur;
        cur = alt;
        alt = tmp;
      }
    }
    Ns *= R_;
  }

  // scatter
  const int No = p.No;
  const int toto = L * No;
  if (p.out_contig) {
    for (int e = threadIdx.x; e < toto; e += blockDim.x) {
      int l = e / No;
      int k = e - l * No;
      KK::template scatter<SMALL>(p, cur + l * p.LS, offO[l], k, sgO[l]);
    }
  } else {
    for (int e = threadIdx.x; e < toto; e += blockDim.x) {
      int k = e / L;
      int l = e - k * L;
      KK::template scatter<SMALL>(p, cur + l * p.LS, offO[l], k, sgO[l]);
    }
  }
}


template <class A, int SIGN>
__global__ void __launch_bounds__(512) k_pass(const PassParams p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  pass_tile<A, SIGN, false>(p, blockIdx.x, smraw);
}

// The same for passes of radices 2..8 only, at two CTAs of up to 512
// threads per SM (at most 64 registers).
template <class A, int SIGN>
__global__ void __launch_bounds__(512, 2) k_pass_small(const PassParams p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  pass_tile<A, SIGN, false, true>(p, blockIdx.x, smraw);
}

// true for a c2c pass whose every stage has radix 2, 3, 4, 5, 7 or 8
inline bool pass_is_small(const PassParams& p) {
  if (p.pingpong || p.mode != MODE_C2C) return false;
  for (int s = 0; s < p.nst; s++) {
    const int r = p.radix[s];
    if (r != 2 && r != 3 && r != 4 && r != 5 && r != 7 && r != 8) return false;
  }
  return true;
}

}  // namespace pg

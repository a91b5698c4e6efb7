/* CPU oracle for the GB300 PFFT library.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is compiled into
 * oracle/_build/liboracle.so and called from tests/, from the smoke check and
 * from the benchmark's CPU-baseline leg.  The product (libpfft_gb300.so) never
 * links, loads or calls it.
 *
 * It restates, in plain C and FP64, what the reference PFFT computes for one
 * process (np = 1), as a sequence of whole-array steps in natural axis order:
 *
 *   read the input layout (TRANSPOSED_IN permutation, r2c padding)
 *   conjugate the input of FORWARD c2r            kernel/partrafo.c:428-443,
 *                                                 api/api-basic.c:279-292
 *   (-1)^k input signs for SHIFTED_OUT            api/api-basic.c:1186-1238
 *   per axis: embed (zero-pad) -> 1-D transform -> truncate
 *                                                 kernel/outrafo.c:118-168,
 *                                                 kernel/ousample.c:208-339
 *   (-1)^k output signs for SHIFTED_IN            api/api-basic.c:1242-1285
 *   conjugate the output of BACKWARD r2c
 *   write the output layout (TRANSPOSED_OUT permutation, c2r padding)
 *
 * The 1-D transforms are FFTW's (FFTW 3.3.4, the version the reference's CI
 * pins in conf/travis-install-fftw.sh; not vendored, not installed here), by
 * their published definitions: unnormalised DFT with exponent sign `sign`,
 * r2c = first n/2+1 bins of the forward DFT of real data, c2r = backward DFT
 * of the Hermitian extension (imaginary parts of DC / Nyquist ignored), and
 * the eleven r2r kinds R2HC..RODFT11.  c2c/r2c/c2r use a recursive
 * mixed-radix FFT (Bluestein for large prime lengths); r2r is evaluated
 * directly from its definition, accumulated in double.  Twiddles and the r2r
 * trigonometric tables come from long double sin/cos.
 *
 * Pinning: the oracle is checked (tests/test_oracle.py) against the
 * reference's own checks - the round trips of tests/simple_check_*.c on the
 * reference's sizes with the reference's golden generator and its 1e-12
 * tolerance, and the c2r-versus-c2c comparison of
 * tests/simple_check_c2r_c2c.c - and against numpy / scipy as independent
 * implementations of the FFTW definitions.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  double re, im;
} cpx;

/* ------------------------------------------------------------------------ */
/* 1-D complex FFT engine                                                    */
/* ------------------------------------------------------------------------ */
typedef struct fplan {
  long n;
  int nf;
  long fac[64];
  cpx *tw; /* W_n^k = exp(-2 pi i k / n), k < n */
  /* Bluestein for prime n > 64 */
  int blue;
  long m;
  cpx *chirp;  /* exp(-i pi k^2 / n), k < n */
  cpx *bfft;   /* FFT_m of the conjugate chirp filter */
  struct fplan *sub;
} fplan;

static void cis(long k, long n, double *c, double *s) {
  long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)(k % n) / (long double)n;
  *c = (double)cosl(a);
  *s = (double)sinl(a);
}

static fplan *fplan_make(long n);

static fplan *fplan_make(long n) {
  fplan *p = (fplan *)calloc(1, sizeof(fplan));
  p->n = n;
  p->tw = (cpx *)malloc(sizeof(cpx) * (size_t)(n > 0 ? n : 1));
  for (long k = 0; k < n; k++) {
    double c, s;
    cis(k, n, &c, &s);
    p->tw[k].re = c;
    p->tw[k].im = -s;
  }
  long m = n;
  int is_prime = n > 1;
  for (long f = 2; f * f <= n; f++)
    if (n % f == 0) is_prime = 0;
  if (is_prime && n > 64) {
    p->blue = 1;
    long mm = 1;
    while (mm < 2 * n - 1) mm <<= 1;
    p->m = mm;
    p->sub = fplan_make(mm);
    p->chirp = (cpx *)malloc(sizeof(cpx) * (size_t)n);
    for (long k = 0; k < n; k++) {
      /* exp(-i pi k^2/n) = W_{2n}^{k^2 mod 2n} */
      long e = (long)(((__int128)k * k) % (2 * n));
      double c, s;
      cis(e, 2 * n, &c, &s);
      p->chirp[k].re = c;
      p->chirp[k].im = -s;
    }
    return p;
  }
  while (m > 1) {
    long f;
    if (m % 4 == 0)
      f = 4;
    else if (m % 2 == 0)
      f = 2;
    else {
      for (f = 3; f * f <= m; f += 2)
        if (m % f == 0) break;
      if (f * f > m) f = m;
    }
    p->fac[p->nf++] = f;
    m /= f;
  }
  return p;
}

static void fplan_free(fplan *p) {
  if (!p) return;
  free(p->tw);
  free(p->chirp);
  free(p->bfft);
  fplan_free(p->sub);
  free(p);
}

/* y[0..n) = DFT of x[0], x[s], x[2s], ...; forward kernel, conj trick for +1 */
static void fft_rec(const cpx *x, long s, cpx *y, long n, const fplan *P, long twstep, int lev, cpx *tmp) {
  if (n == 1) {
    y[0] = x[0];
    return;
  }
  long p = P->fac[lev], m = n / p;
  for (long q = 0; q < p; q++) fft_rec(x + q * s, s * p, y + q * m, m, P, twstep * p, lev + 1, tmp);
  /* combine: Y[k + j m] = sum_q W_n^{q(k + j m)} Y_q[k] */
  for (long k = 0; k < m; k++) {
    for (long q = 0; q < p; q++) {
      cpx a = y[q * m + k];
      cpx w = P->tw[(twstep * q * k) % P->n];
      tmp[q].re = a.re * w.re - a.im * w.im;
      tmp[q].im = a.re * w.im + a.im * w.re;
    }
    if (p == 2) {
      y[k].re = tmp[0].re + tmp[1].re;
      y[k].im = tmp[0].im + tmp[1].im;
      y[k + m].re = tmp[0].re - tmp[1].re;
      y[k + m].im = tmp[0].im - tmp[1].im;
    } else if (p == 4) {
      cpx a0 = tmp[0], a1 = tmp[1], a2 = tmp[2], a3 = tmp[3];
      cpx t0 = {a0.re + a2.re, a0.im + a2.im}, t1 = {a0.re - a2.re, a0.im - a2.im};
      cpx t2 = {a1.re + a3.re, a1.im + a3.im}, t3 = {a1.re - a3.re, a1.im - a3.im};
      /* forward: multiply t3 by -i */
      cpx t3m = {t3.im, -t3.re};
      y[k].re = t0.re + t2.re;
      y[k].im = t0.im + t2.im;
      y[k + 2 * m].re = t0.re - t2.re;
      y[k + 2 * m].im = t0.im - t2.im;
      y[k + m].re = t1.re + t3m.re;
      y[k + m].im = t1.im + t3m.im;
      y[k + 3 * m].re = t1.re - t3m.re;
      y[k + 3 * m].im = t1.im - t3m.im;
    } else {
      long step = P->n / p; /* W_p^e = W_n^{e n/p} */
      for (long j = 0; j < p; j++) {
        double re = 0, im = 0;
        for (long q = 0; q < p; q++) {
          cpx w = P->tw[((q * j) % p) * step];
          re += tmp[q].re * w.re - tmp[q].im * w.im;
          im += tmp[q].re * w.im + tmp[q].im * w.re;
        }
        y[k + j * m].re = re;
        y[k + j * m].im = im;
      }
    }
  }
}

/* in-place DFT of a contiguous line with exponent sign `sign`;
 * work must hold 2*n + max factor (or 3*m for Bluestein) entries */
static void fft_line(cpx *a, const fplan *P, int sign, cpx *work) {
  long n = P->n;
  if (n <= 1) return;
  if (sign > 0)
    for (long k = 0; k < n; k++) a[k].im = -a[k].im;
  if (P->blue) {
    long m = P->m;
    cpx *u = work, *v = work + m, *w2 = work + 2 * m;
    memset(u, 0, sizeof(cpx) * (size_t)m);
    for (long k = 0; k < n; k++) {
      cpx c = P->chirp[k];
      u[k].re = a[k].re * c.re - a[k].im * c.im;
      u[k].im = a[k].re * c.im + a[k].im * c.re;
    }
    /* filter b_k = conj(chirp_k) for |k| < n, circular */
    memset(v, 0, sizeof(cpx) * (size_t)m);
    for (long k = 0; k < n; k++) {
      v[k].re = P->chirp[k].re;
      v[k].im = -P->chirp[k].im;
      if (k) v[m - k] = v[k];
    }
    fft_line(u, P->sub, -1, w2);
    fft_line(v, P->sub, -1, w2);
    for (long k = 0; k < m; k++) {
      cpx x = u[k], y = v[k];
      u[k].re = x.re * y.re - x.im * y.im;
      u[k].im = x.re * y.im + x.im * y.re;
    }
    fft_line(u, P->sub, +1, w2);
    for (long k = 0; k < n; k++) {
      cpx x = {u[k].re / (double)m, u[k].im / (double)m}, c = P->chirp[k];
      a[k].re = x.re * c.re - x.im * c.im;
      a[k].im = x.re * c.im + x.im * c.re;
    }
  } else {
    cpx *y = work, *tmp = work + n;
    fft_rec(a, 1, y, n, P, 1, 0, tmp);
    memcpy(a, y, sizeof(cpx) * (size_t)n);
  }
  if (sign > 0)
    for (long k = 0; k < n; k++) a[k].im = -a[k].im;
}

static long work_len(const fplan *P) {
  if (P->blue) return 3 * P->m + work_len(P->sub);
  long mx = 1;
  for (int i = 0; i < P->nf; i++)
    if (P->fac[i] > mx) mx = P->fac[i];
  return 2 * P->n + mx + 8;
}

/* ------------------------------------------------------------------------ */
/* r2r kinds by definition (FFTW manual, "1d Real-even/odd DFTs", "DHT")     */
/* ------------------------------------------------------------------------ */
enum { K_R2HC = 0, K_HC2R, K_DHT, K_RE00, K_RE01, K_RE10, K_RE11, K_RO00, K_RO01, K_RO10, K_RO11 };

/* cos / sin of pi * m / den for m < 2 den, from long double sin/cos once per
 * transformed axis (the r2r definitions need angles pi * num / den only) */
typedef struct {
  long den;
  double *c, *s;
} trig_tab;

static long r2r_den(long n, int kind) {
  switch (kind) {
    case K_RE00: return n - 1 > 0 ? n - 1 : 1;
    case K_RO00: return n + 1;
    case K_RE01: case K_RE10: case K_RO01: case K_RO10: return 2 * n;
    case K_RE11: case K_RO11: return 4 * n;
    default: return n; /* R2HC, HC2R, DHT: angles 2 pi j k / n */
  }
}

static void trig_make(trig_tab *t, long den) {
  t->den = den;
  t->c = (double *)malloc(sizeof(double) * 2 * (size_t)den);
  t->s = (double *)malloc(sizeof(double) * 2 * (size_t)den);
  for (long m = 0; m < 2 * den; m++) {
    long double a = 3.141592653589793238462643383279502884L * (long double)m / (long double)den;
    t->c[m] = (double)cosl(a);
    t->s[m] = (double)sinl(a);
  }
}

static void trig_free(trig_tab *t) {
  free(t->c);
  free(t->s);
}

static double cospi_frac(const trig_tab *t, long num) {
  long two = 2 * t->den;
  long r = num % two;
  if (r < 0) r += two;
  return t->c[r];
}
static double sinpi_frac(const trig_tab *t, long num) {
  long two = 2 * t->den;
  long r = num % two;
  if (r < 0) r += two;
  return t->s[r];
}

/* One line of a real-to-real transform, by direct evaluation of FFTW's
 * definitions (doc of FFTW 3.3, "What FFTW Really Computes"), accumulated in
 * double.  t: the table of trig_make(r2r_den(n, kind)). */
static void r2r_line(const double *x, double *y, long n, int kind, const trig_tab *t) {
  for (long k = 0; k < n; k++) {
    double acc = 0;
    switch (kind) {
      case K_RE00:
        acc = x[0] + ((k & 1) ? -x[n - 1] : x[n - 1]);
        for (long j = 1; j < n - 1; j++) acc += 2.0 * x[j] * cospi_frac(t, j * k);
        break;
      case K_RE01:
        acc = x[0];
        for (long j = 1; j < n; j++) acc += 2.0 * x[j] * cospi_frac(t, j * (2 * k + 1));
        break;
      case K_RE10:
        for (long j = 0; j < n; j++) acc += 2.0 * x[j] * cospi_frac(t, (2 * j + 1) * k);
        break;
      case K_RE11:
        for (long j = 0; j < n; j++) acc += 2.0 * x[j] * cospi_frac(t, (2 * j + 1) * (2 * k + 1));
        break;
      case K_RO00:
        for (long j = 0; j < n; j++) acc += 2.0 * x[j] * sinpi_frac(t, (j + 1) * (k + 1));
        break;
      case K_RO01:
        acc = (k & 1) ? -x[n - 1] : x[n - 1];
        for (long j = 0; j < n - 1; j++) acc += 2.0 * x[j] * sinpi_frac(t, (j + 1) * (2 * k + 1));
        break;
      case K_RO10:
        for (long j = 0; j < n; j++) acc += 2.0 * x[j] * sinpi_frac(t, (2 * j + 1) * (k + 1));
        break;
      case K_RO11:
        for (long j = 0; j < n; j++) acc += 2.0 * x[j] * sinpi_frac(t, (2 * j + 1) * (2 * k + 1));
        break;
      case K_R2HC:
        if (2 * k <= n) {
          for (long j = 0; j < n; j++) acc += x[j] * cospi_frac(t, 2 * j * k);
        } else {
          long kk = n - k;
          for (long j = 0; j < n; j++) acc -= x[j] * sinpi_frac(t, 2 * j * kk);
        }
        break;
      case K_HC2R:
        acc = x[0];
        for (long j = 1; 2 * j < n; j++)
          acc += 2.0 * (x[j] * cospi_frac(t, 2 * j * k) - x[n - j] * sinpi_frac(t, 2 * j * k));
        if (n % 2 == 0) acc += x[n / 2] * ((k & 1) ? -1.0 : 1.0);
        break;
      case K_DHT:
        for (long j = 0; j < n; j++) acc += x[j] * (cospi_frac(t, 2 * j * k) + sinpi_frac(t, 2 * j * k));
        break;
    }
    y[k] = (double)acc;
  }
}

/* ------------------------------------------------------------------------ */
/* whole-array axis transforms                                               */
/* ------------------------------------------------------------------------ */
#define MAXD 8
typedef struct {
  int d;
  long ext[MAXD]; /* natural extents, howmany is the innermost extra dim */
  long hm;
  int cplx;
  double *data;   /* natural order, interleaved if complex */
} arr;

static long arr_count(const arr *a) {
  long c = a->hm;
  for (int t = 0; t < a->d; t++) c *= a->ext[t];
  return c;
}

typedef struct {
  int axis, kind; /* 0 c2c, 1 r2c, 2 c2r, 3+ r2r kind (offset by 3) */
  int sign;
  long N, Ni, Zi, No, Zo;
  int skip;
  const fplan *P;
  const trig_tab *T; /* r2r kinds */
  const arr *src;
  arr *dst;
  long nlines;
  long lo, hi; /* line range for this worker */
} axjob;

static void *axis_worker(void *arg) {
  axjob *J = (axjob *)arg;
  const arr *A = J->src;
  arr *B = J->dst;
  int a = J->axis;
  long inner_s = A->hm, outer;
  for (int t = A->d - 1; t > a; t--) inner_s *= A->ext[t];
  long inner_d = B->hm;
  for (int t = B->d - 1; t > a; t--) inner_d *= B->ext[t];
  (void)outer;
  long N = J->N;
  long wl = J->P ? work_len(J->P) : 8;
  cpx *line = (cpx *)calloc((size_t)(N + 2), sizeof(cpx));
  cpx *work = (cpx *)calloc((size_t)wl + 2, sizeof(cpx));
  double *rl = (double *)calloc((size_t)(N + 2), sizeof(double));
  double *ro = (double *)calloc((size_t)(N + 2), sizeof(double));
  for (long g = J->lo; g < J->hi; g++) {
    long o = g / inner_s, in = g % inner_s; /* inner_s == inner_d (other axes unchanged) */
    const double *sp = A->data;
    double *dp = B->data;
    long ofs_s = (o * A->ext[a]) * inner_s + in, ofs_d = (o * B->ext[a]) * inner_d + in;
    int kind = J->kind;
    if (kind == 0 || kind == 1) {
      for (long k = 0; k < N; k++) line[k].re = line[k].im = 0;
      for (long q = 0; q < J->Ni; q++) {
        long e = ofs_s + q * inner_s;
        cpx v;
        if (A->cplx) {
          v.re = sp[2 * e];
          v.im = sp[2 * e + 1];
        } else {
          v.re = sp[e];
          v.im = 0;
        }
        line[J->Zi + q] = v;
      }
      if (!J->skip) fft_line(line, J->P, kind == 1 ? -1 : J->sign, work);
      for (long q = 0; q < J->No; q++) {
        long e = ofs_d + q * inner_d;
        dp[2 * e] = line[J->Zo + q].re;
        dp[2 * e + 1] = line[J->Zo + q].im;
      }
    } else if (kind == 2) { /* c2r: half spectrum embedded at Zi of N/2+1 */
      long h = N / 2 + 1;
      for (long k = 0; k < N; k++) line[k].re = line[k].im = 0;
      for (long q = 0; q < J->Ni; q++) {
        long e = ofs_s + q * inner_s;
        line[J->Zi + q].re = sp[2 * e];
        line[J->Zi + q].im = sp[2 * e + 1];
      }
      for (long k = 1; k < h; k++)
        if (N - k > k) {
          line[N - k].re = line[k].re;
          line[N - k].im = -line[k].im;
        }
      /* FFTW ignores the imaginary parts of DC and (even n) Nyquist */
      line[0].im = 0;
      if (N % 2 == 0) line[N / 2].im = 0;
      fft_line(line, J->P, +1, work);
      for (long q = 0; q < J->No; q++) dp[ofs_d + q * inner_d] = line[J->Zo + q].re;
    } else { /* r2r */
      for (long k = 0; k < N; k++) rl[k] = 0;
      for (long q = 0; q < J->Ni; q++) rl[J->Zi + q] = sp[ofs_s + q * inner_s];
      if (J->skip)
        memcpy(ro, rl, sizeof(double) * (size_t)N);
      else
        r2r_line(rl, ro, N, kind - 3, J->T);
      for (long q = 0; q < J->No; q++) dp[ofs_d + q * inner_d] = ro[J->Zo + q];
    }
  }
  free(line);
  free(work);
  free(rl);
  free(ro);
  return NULL;
}

static void axis_transform(const arr *A, arr *B, int axis, int kind, int sign, long N, long Ni, long Zi, long No,
                           long Zo, int skip, int nthreads) {
  long nlines = arr_count(A) / A->ext[axis];
  fplan *P = (kind <= 2) ? fplan_make(N) : NULL;
  trig_tab T = {0, NULL, NULL};
  if (kind > 2 && !skip) trig_make(&T, r2r_den(N, kind - 3));
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  if (nlines < nthreads) nthreads = (int)(nlines > 0 ? nlines : 1);
  pthread_t th[256];
  axjob jobs[256];
  for (int i = 0; i < nthreads; i++) {
    axjob J = {axis, kind, sign, N, Ni, Zi, No, Zo, skip, P, &T, A, B, nlines, nlines * i / nthreads,
               nlines * (i + 1) / nthreads};
    jobs[i] = J;
  }
  if (nthreads == 1)
    axis_worker(&jobs[0]);
  else {
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, axis_worker, &jobs[i]);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
  }
  fplan_free(P);
  if (T.c) trig_free(&T);
}

/* ------------------------------------------------------------------------ */
/* layouts                                                                   */
/* ------------------------------------------------------------------------ */
/* memory order of the natural axes (transposed: axes 1..r, then 0, then rest) */
static void axis_order(int d, int r, int transposed, int *ord) {
  if (!transposed) {
    for (int t = 0; t < d; t++) ord[t] = t;
    return;
  }
  for (int t = 0; t < r; t++) ord[t] = t + 1;
  ord[r] = 0;
  for (int t = r + 1; t < d; t++) ord[t] = t;
}

/* copy between a natural-order array (logical extents) and a memory layout with
 * stored extents `st` (>= logical) in axis order `ord`; dir 0: mem -> nat */
static void relayout(arr *nat, double *mem, const long *st, const int *ord, int dir) {
  int d = nat->d;
  long strides[MAXD];
  long s = nat->hm;
  for (int i = d - 1; i >= 0; i--) {
    strides[ord[i]] = s;
    s *= st[ord[i]];
  }
  long cnt = arr_count(nat);
  int w = nat->cplx ? 2 : 1;
  for (long e = 0; e < cnt; e++) {
    long r = e, h = r % nat->hm, off = h;
    r /= nat->hm;
    for (int t = d - 1; t >= 0; t--) {
      long i = r % nat->ext[t];
      r /= nat->ext[t];
      off += i * strides[t];
    }
    for (int c = 0; c < w; c++) {
      if (dir == 0)
        nat->data[w * e + c] = mem[w * off + c];
      else
        mem[w * off + c] = nat->data[w * e + c];
    }
  }
}

/* (-1)^k sign of one axis index as PFFT's twiddle loops compute it */
static int shift_sign(long i, long start, long thresh, int extra) {
  long t = i + start;
  if (t < thresh) return (t % 2) ? -extra : extra;
  return 1;
}

static void apply_signs(arr *A, const long *start, const long *thresh, const int *extra, const int *skip) {
  long cnt = arr_count(A);
  int w = A->cplx ? 2 : 1;
  for (long e = 0; e < cnt; e++) {
    long r = e / A->hm;
    int f = 1;
    for (int t = A->d - 1; t >= 0; t--) {
      long i = r % A->ext[t];
      r /= A->ext[t];
      if (!(skip && skip[t])) f *= shift_sign(i, start[t], thresh[t], extra[t]);
    }
    if (f < 0)
      for (int c = 0; c < w; c++) A->data[w * e + c] = -A->data[w * e + c];
  }
}

/* ------------------------------------------------------------------------ */
/* the oracle entry point                                                    */
/* ------------------------------------------------------------------------ */
#define F_TIN (1u << 0)
#define F_TOUT (1u << 1)
#define F_SIN (1u << 2)
#define F_SOUT (1u << 3)

/* kind: 0 c2c, 1 r2c, 2 c2r, 3 r2r.  in/out: double arrays in the user
 * layouts (complex interleaved).  padded: real rows padded to 2(n/2+1).
 * mesh_rank: rank of the process mesh that defines the transposed layouts.
 * Returns 0, or -1 for an unsupported request. */
int oracle_execute(int d, const long long *n_, const long long *ni_, const long long *no_, long long howmany,
                   int kind, int padded, int sign, const int *kinds, const int *skip, unsigned flags, int mesh_rank,
                   const double *in, double *out, int nthreads) {
  long n[MAXD], ni[MAXD], no[MAXD];
  if (d < 1 || d > MAXD) return -1;
  for (int t = 0; t < d; t++) {
    n[t] = (long)n_[t];
    ni[t] = (long)ni_[t];
    no[t] = (long)no_[t];
    if (ni[t] > n[t] || no[t] > n[t]) return -1;
  }
  int ord_in[MAXD], ord_out[MAXD];
  axis_order(d, mesh_rank, (flags & F_TIN) != 0, ord_in);
  axis_order(d, mesh_rank, (flags & F_TOUT) != 0, ord_out);

  /* input: logical and stored extents */
  arr A;
  A.d = d;
  A.hm = (long)howmany;
  long st_in[MAXD];
  for (int t = 0; t < d; t++) A.ext[t] = st_in[t] = ni[t];
  A.cplx = (kind == 0 || kind == 2);
  if (kind == 1 && padded) st_in[d - 1] = 2 * (ni[d - 1] / 2 + 1);
  if (kind == 2) A.ext[d - 1] = st_in[d - 1] = ni[d - 1] / 2 + 1;
  A.data = (double *)calloc((size_t)arr_count(&A) * (A.cplx ? 2 : 1), sizeof(double));
  relayout(&A, (double *)in, st_in, ord_in, 0);

  int csign = sign;
  if (kind == 2 && sign == -1) { /* FORWARD c2r: conjugate, compute BACKWARD */
    long c = arr_count(&A);
    for (long e = 0; e < c; e++) A.data[2 * e + 1] = -A.data[2 * e + 1];
    csign = +1;
  }
  if (kind == 1 && sign == +1) csign = -1;
  if (kind == 3) csign = -1;

  if (flags & F_SOUT) { /* input twiddles */
    long start[MAXD], thresh[MAXD];
    int extra[MAXD];
    for (int t = 0; t < d; t++) {
      start[t] = (flags & F_SIN) ? -ni[t] / 2 : 0;
      thresh[t] = ni[t] / 2;
      extra[t] = ((flags & F_SIN) && ((n[t] / 2) % 2)) ? -1 : 1;
    }
    apply_signs(&A, start, thresh, extra, skip);
  }

  /* axis order: last dims first; c2r transforms the last axis last */
  int axes[MAXD], na = 0;
  if (kind == 2) {
    for (int t = 0; t < d - 1; t++) axes[na++] = t;
    axes[na++] = d - 1;
  } else {
    for (int t = d - 1; t >= 0; t--) axes[na++] = t;
  }
  for (int i = 0; i < na; i++) {
    int a = axes[i];
    arr B = A;
    long N = n[a], Ni = ni[a], No = no[a];
    long Zi = (flags & F_SIN) ? (N - Ni) / 2 : 0, Zo = (flags & F_SOUT) ? (N - No) / 2 : 0;
    int k = 0, sk = skip ? skip[a] : 0;
    if (a == d - 1 && kind == 1) {
      k = 1;
      long pni = N / 2 + 1, pno = No / 2 + 1;
      B.ext[a] = pno;
      B.cplx = 1;
      No = pno;
      Zo = pni - pno; /* kernel/ousample.c:288-297 */
    } else if (a == d - 1 && kind == 2) {
      k = 2;
      long pni = Ni / 2 + 1, pno = N / 2 + 1;
      Ni = pni;
      Zi = pno - pni; /* kernel/ousample.c:310-318 */
      B.ext[a] = No;
      B.cplx = 0;
    } else if (kind == 3) {
      k = 3 + (kinds ? kinds[a] : K_RE00);
      B.ext[a] = No;
    } else {
      k = 0;
      B.ext[a] = No;
    }
    B.data = (double *)calloc((size_t)arr_count(&B) * (B.cplx ? 2 : 1), sizeof(double));
    axis_transform(&A, &B, a, k, csign, N, Ni, Zi, No, Zo, sk, nthreads);
    free(A.data);
    A = B;
  }

  if (flags & F_SIN) { /* output twiddles */
    long start[MAXD], thresh[MAXD];
    int extra[MAXD];
    for (int t = 0; t < d; t++) {
      start[t] = (flags & F_SOUT) ? -no[t] / 2 : 0;
      thresh[t] = no[t] / 2;
      extra[t] = 1;
    }
    apply_signs(&A, start, thresh, extra, skip);
  }
  if (kind == 1 && sign == +1) { /* BACKWARD r2c: conjugate the output */
    long c = arr_count(&A);
    for (long e = 0; e < c; e++) A.data[2 * e + 1] = -A.data[2 * e + 1];
  }
  long st_out[MAXD];
  for (int t = 0; t < d; t++) st_out[t] = A.ext[t];
  if (kind == 2 && padded) st_out[d - 1] = 2 * (no[d - 1] / 2 + 1);
  relayout(&A, out, st_out, ord_out, 1);
  free(A.data);
  return 0;
}

/* plain complex DFT of contiguous lines (used by the tests to pin the engine) */
int oracle_fft_lines(long n, long nlines, int sign, double *data) {
  fplan *P = fplan_make(n);
  cpx *work = (cpx *)calloc((size_t)work_len(P) + 2, sizeof(cpx));
  for (long l = 0; l < nlines; l++) fft_line((cpx *)(data + 2 * l * n), P, sign, work);
  free(work);
  fplan_free(P);
  return 0;
}

int oracle_r2r_line(long n, int kind, const double *x, double *y) {
  trig_tab t;
  trig_make(&t, r2r_den(n, kind));
  r2r_line(x, y, n, kind, &t);
  trig_free(&t);
  return 0;
}

/* Round-trip acceptance checks of the PFFT test suite, as a plain C program
 * against the drop-in header and library, on a 1x1 process mesh.
 *
 * Each case follows the reference's check programs (tests/simple_check_*.c,
 * tests/minimal_check_*.c, listed in tests/run_checks.sh:7-72): plan a
 * forward and a backward transform, fill the input with the golden generator
 * (pfft_init_input_*), run forward, clear the input (pfft_clear_input_*), run
 * backward, divide by the logical transform size and report the maximum
 * absolute error against the generator (pfft_check_output_*).  The suite
 * accepts a case when that error is below 1e-12 (tests/run_checks.sh:75).
 *
 * Usage: roundtrip_checks [case ...]   (no argument: every case)
 * Prints one line per case: "<name> maxerror = <err>;".
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include <pfft.h>

enum { C2C, R2C, R2R, C2R };

typedef struct {
  const char *name;
  int kind;          /* forward kind; the backward is its inverse (C2C, C2R<->R2C, R2R) */
  int rnk;
  ptrdiff_t n[4];    /* logical transform size */
  ptrdiff_t ni[4];   /* forward input size (oversampled cases), 0: = n */
  unsigned flags_f;  /* forward flags (besides MEASURE | DESTROY_INPUT) */
  unsigned flags_b;  /* backward flags */
  int inplace;       /* forward and backward on one array */
  int newarray;      /* plan on one pair of arrays, execute on another */
  int kinds_f[4], kinds_b[4];
  int check_with_n;  /* generator indexed with n instead of ni (4-d oversampled r2c) */
} rt_case;

#define TO PFFT_TRANSPOSED_OUT
#define TI PFFT_TRANSPOSED_IN
#define PAD PFFT_PADDED_R2C
#define K3F {PFFT_REDFT00, PFFT_REDFT01, PFFT_RODFT00, 0}
#define K3B {PFFT_REDFT00, PFFT_REDFT10, PFFT_RODFT00, 0}
#define K4F {PFFT_REDFT00, PFFT_REDFT01, PFFT_RODFT00, PFFT_RODFT10}
#define K4B {PFFT_REDFT00, PFFT_REDFT10, PFFT_RODFT00, PFFT_RODFT01}

static const rt_case CASES[] = {
    {"minimal_check_c2c", C2C, 3, {2, 2, 4}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"minimal_check_c2c_transposed", C2C, 3, {2, 2, 4}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_c2c", C2C, 3, {29, 27, 31}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_c2c_transposed", C2C, 3, {29, 27, 31}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_c2c_4d", C2C, 4, {13, 14, 19, 17}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_c2c_4d_transposed", C2C, 4, {13, 14, 19, 17}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_c2c_inplace", C2C, 3, {29, 27, 31}, {0}, 0, 0, 1, 0, {0}, {0}, 0},
    {"simple_check_c2c_transposed_inplace", C2C, 3, {29, 27, 31}, {0}, TO, TI, 1, 0, {0}, {0}, 0},
    {"simple_check_c2c_newarray", C2C, 3, {29, 27, 31}, {0}, 0, 0, 0, 1, {0}, {0}, 0},
    {"simple_check_c2c_transposed_newarray", C2C, 3, {29, 27, 31}, {0}, TO, TI, 0, 1, {0}, {0}, 0},
    {"simple_check_r2c", R2C, 3, {29, 27, 32}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_r2c_transposed", R2C, 3, {29, 27, 32}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_r2c_4d", R2C, 4, {13, 14, 19, 17}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_r2c_4d_transposed", R2C, 4, {13, 14, 19, 17}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_r2c_newarray", R2C, 3, {29, 27, 31}, {0}, 0, 0, 0, 1, {0}, {0}, 0},
    {"simple_check_r2c_transposed_newarray", R2C, 3, {29, 27, 31}, {0}, TO, TI, 0, 1, {0}, {0}, 0},
    {"simple_check_r2c_padded_newarray", R2C, 3, {29, 27, 31}, {0}, PAD, PAD, 0, 1, {0}, {0}, 0},
    {"simple_check_r2c_padded_transposed_newarray", R2C, 3, {29, 27, 31}, {0}, PAD | TO, PAD | TI, 0, 1, {0}, {0},
     0},
    {"simple_check_r2r", R2R, 3, {29, 27, 31}, {0}, 0, 0, 0, 0, K3F, K3B, 0},
    {"simple_check_r2r_transposed", R2R, 3, {29, 27, 31}, {0}, TO, TI, 0, 0, K3F, K3B, 0},
    {"simple_check_r2r_4d", R2R, 4, {13, 14, 19, 17}, {0}, 0, 0, 0, 0, K4F, K4B, 0},
    {"simple_check_r2r_4d_transposed", R2R, 4, {13, 14, 19, 17}, {0}, TO, TI, 0, 0, K4F, K4B, 0},
    {"simple_check_ousam_c2c", C2C, 3, {29, 27, 31}, {16, 16, 16}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_c2c_transposed", C2C, 3, {29, 27, 31}, {16, 16, 16}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_c2c_4d", C2C, 4, {13, 14, 19, 17}, {8, 8, 8, 8}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_c2c_4d_transposed", C2C, 4, {13, 14, 19, 17}, {8, 8, 8, 8}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_r2c", R2C, 3, {29, 27, 31}, {16, 16, 16}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_r2c_transposed", R2C, 3, {29, 27, 31}, {16, 16, 16}, TO, TI, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_r2c_padded", R2C, 3, {29, 27, 31}, {16, 16, 16}, PAD, PAD, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_r2c_4d", R2C, 4, {13, 14, 15, 17}, {8, 8, 8, 8}, 0, 0, 0, 0, {0}, {0}, 1},
    {"simple_check_ousam_r2c_4d_transposed", R2C, 4, {13, 14, 15, 17}, {8, 8, 8, 8}, TO, TI, 0, 0, {0}, {0}, 1},
    {"simple_check_ousam_c2r", C2R, 3, {29, 27, 31}, {16, 16, 16}, 0, 0, 0, 0, {0}, {0}, 0},
    {"simple_check_ousam_r2r", R2R, 3, {29, 27, 31}, {16, 16, 16}, 0, 0, 0, 0, K3F, K3B, 0},
    {"simple_check_ousam_r2r_transposed", R2R, 3, {29, 27, 31}, {16, 16, 16}, TO, TI, 0, 0, K3F, K3B, 0},
    /* the same checks (golden data, 1e-12 bound) at sizes beyond the
     * reference's suite, where the double API's default arithmetic runs the
     * radix-8 kernel's 64-bit fixed point on every power-of-two axis */
    {"large_check_c2c_128", C2C, 3, {128, 128, 128}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"large_check_c2c_256_transposed", C2C, 3, {256, 256, 256}, {0}, TO, TI, 0, 0, {0}, {0}, 0},
    {"large_check_c2c_512x256x128", C2C, 3, {512, 256, 128}, {0}, 0, 0, 0, 0, {0}, {0}, 0},
    {"large_check_r2c_256_padded_transposed", R2C, 3, {256, 256, 256}, {0}, PAD | TO, PAD | TI, 0, 0, {0}, {0}, 0},
};

/* logical length of a real-to-real transform (the normalisation factor) */
static ptrdiff_t r2r_len(int kind, ptrdiff_t n) {
  if (kind == PFFT_REDFT00) return 2 * (n - 1);
  if (kind == PFFT_RODFT00) return 2 * (n + 1);
  return 2 * n;
}

static ptrdiff_t local_size(int kind, const rt_case *c, const ptrdiff_t *ni, const ptrdiff_t *no, unsigned flags,
                            MPI_Comm comm, ptrdiff_t *lni, ptrdiff_t *lis, ptrdiff_t *lno, ptrdiff_t *los) {
  switch (kind) {
    case C2C:
      return pfft_local_size_many_dft(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, comm, flags,
                                      lni, lis, lno, los);
    case R2C:
      return pfft_local_size_many_dft_r2c(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, comm,
                                          flags, lni, lis, lno, los);
    case C2R:
      return pfft_local_size_many_dft_c2r(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, comm,
                                          flags, lni, lis, lno, los);
    default:
      return pfft_local_size_many_r2r(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, comm, flags,
                                      lni, lis, lno, los);
  }
}

static pfft_plan plan(int kind, const rt_case *c, const ptrdiff_t *ni, const ptrdiff_t *no, void *in, void *out,
                      MPI_Comm comm, int sign, const int *kinds, unsigned flags) {
  flags |= PFFT_MEASURE | PFFT_DESTROY_INPUT;
  switch (kind) {
    case C2C:
      return pfft_plan_many_dft(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, in, out, comm,
                                sign, flags);
    case R2C:
      return pfft_plan_many_dft_r2c(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, in, out, comm,
                                    sign, flags);
    case C2R:
      return pfft_plan_many_dft_c2r(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, in, out, comm,
                                    sign, flags);
    default: {
      pfft_r2r_kind k[4];
      for (int t = 0; t < c->rnk; t++) k[t] = (pfft_r2r_kind)kinds[t];
      return pfft_plan_many_r2r(c->rnk, c->n, ni, no, 1, PFFT_DEFAULT_BLOCKS, PFFT_DEFAULT_BLOCKS, in, out, comm, k,
                                flags);
    }
  }
}

static void execute(pfft_plan p, int kind, void *in, void *out, int newarray) {
  if (!newarray) {
    pfft_execute(p);
    return;
  }
  switch (kind) {
    case C2C: pfft_execute_dft(p, in, out); break;
    case R2C: pfft_execute_dft_r2c(p, in, out); break;
    case C2R: pfft_execute_dft_c2r(p, in, out); break;
    default: pfft_execute_r2r(p, in, out);
  }
}

static ptrdiff_t prod(int rnk, const ptrdiff_t *v) {
  ptrdiff_t p = 1;
  for (int t = 0; t < rnk; t++) p *= v[t];
  return p;
}

/* returns the maximum error, or a negative value when planning failed */
static double run_case(const rt_case *c, MPI_Comm comm) {
  const int rnk = c->rnk;
  ptrdiff_t ni[4], no[4], lni[4], lis[4], ln[4], ls[4], lno[4], los[4];
  for (int t = 0; t < rnk; t++) {
    ni[t] = c->ni[t] ? c->ni[t] : c->n[t];
    no[t] = ni[t];
  }
  const int kind_b = c->kind == R2C ? C2R : (c->kind == C2R ? R2C : c->kind);
  ptrdiff_t af = local_size(c->kind, c, ni, c->n, c->flags_f, comm, lni, lis, ln, ls);
  ptrdiff_t ab = local_size(kind_b, c, c->n, no, c->flags_b, comm, ln, ls, lno, los);
  ptrdiff_t alloc = af > ab ? af : ab;
  /* the input side is real for r2c / r2r, the output side for c2r / r2r */
  const int real_in = c->kind == R2C || c->kind == R2R;
  void *in = real_in ? (void *)pfft_alloc_real(2 * alloc) : (void *)pfft_alloc_complex(alloc);
  void *out = c->inplace ? in
              : (c->kind == C2R || c->kind == R2R) ? (void *)pfft_alloc_real(2 * alloc)
                                                   : (void *)pfft_alloc_complex(alloc);
  void *pin = in, *pout = out;
  if (c->newarray) { /* plan on scratch arrays, execute on in / out */
    pin = real_in ? (void *)pfft_alloc_real(2 * alloc) : (void *)pfft_alloc_complex(alloc);
    pout = (c->kind == C2R || c->kind == R2R) ? (void *)pfft_alloc_real(2 * alloc) : (void *)pfft_alloc_complex(alloc);
  }
  pfft_plan pf = plan(c->kind, c, ni, c->n, pin, pout, comm, PFFT_FORWARD, c->kinds_f, c->flags_f);
  pfft_plan pb = plan(kind_b, c, c->n, no, pout, pin, comm, PFFT_BACKWARD, c->kinds_b, c->flags_b);
  double err = -1.0;
  if (pf && pb) {
    const ptrdiff_t *gi = c->check_with_n ? c->n : ni;
    switch (c->kind) {
      case C2C: pfft_init_input_complex(rnk, gi, lni, lis, (pfft_complex *)in); break;
      case C2R: pfft_init_input_complex_hermitian(rnk, gi, lni, lis, (pfft_complex *)in); break;
      default: pfft_init_input_real(rnk, gi, lni, lis, (double *)in);
    }
    execute(pf, c->kind, in, out, c->newarray);
    if (!c->inplace) {
      switch (c->kind) {
        case C2C: pfft_clear_input_complex(rnk, gi, lni, lis, (pfft_complex *)in); break;
        case C2R: pfft_clear_input_complex_hermitian(rnk, gi, lni, lis, (pfft_complex *)in); break;
        default: pfft_clear_input_real(rnk, gi, lni, lis, (double *)in);
      }
    }
    execute(pb, kind_b, out, in, c->newarray);
    double scale = 1.0;
    for (int t = 0; t < rnk; t++) scale *= (double)(c->kind == R2R ? r2r_len(c->kinds_f[t], c->n[t]) : c->n[t]);
    const ptrdiff_t cnt = prod(rnk, lno);
    if (c->kind == C2C || c->kind == C2R) {
      pfft_complex *a = (pfft_complex *)in;
      for (ptrdiff_t l = 0; l < cnt; l++) {
        a[l][0] /= scale;
        a[l][1] /= scale;
      }
    } else {
      double *a = (double *)in;
      for (ptrdiff_t l = 0; l < cnt; l++) a[l] /= scale;
    }
    switch (c->kind) {
      case C2C: err = pfft_check_output_complex(rnk, gi, lno, los, (const pfft_complex *)in, comm); break;
      case C2R: err = pfft_check_output_complex_hermitian(rnk, gi, lno, los, (const pfft_complex *)in, comm); break;
      default: err = pfft_check_output_real(rnk, gi, lno, los, (const double *)in, comm);
    }
  }
  if (pf) pfft_destroy_plan(pf);
  if (pb) pfft_destroy_plan(pb);
  if (c->newarray) {
    pfft_free(pin);
    pfft_free(pout);
  }
  if (!c->inplace) pfft_free(out);
  pfft_free(in);
  return err;
}

int main(int argc, char **argv) {
  MPI_Comm comm;
  MPI_Init(&argc, &argv);
  pfft_init();
  if (pfft_create_procmesh_2d(MPI_COMM_WORLD, 1, 1, &comm)) {
    fprintf(stderr, "cannot create a 1x1 process mesh\n");
    return 2;
  }
  int rc = 0;
  const int ncases = (int)(sizeof(CASES) / sizeof(CASES[0]));
  for (int i = 0; i < ncases; i++) {
    int want = argc < 2;
    for (int a = 1; a < argc; a++) want |= strcmp(argv[a], CASES[i].name) == 0;
    if (!want) continue;
    double err = run_case(&CASES[i], comm);
    if (err < 0) {
      printf("%s planning failed\n", CASES[i].name);
      rc = 1;
    } else {
      printf("%s maxerror = %6.2e;\n", CASES[i].name, err);
    }
    fflush(stdout);
  }
  MPI_Comm_free(&comm);
  pfft_cleanup();
  MPI_Finalize();
  return rc;
}

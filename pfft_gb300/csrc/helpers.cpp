// Host-side parts of the PFFT API that touch no transform: set-up, memory,
// process meshes, golden-data generators, vector helpers, printing, command
// line parsing and plan timers.  Behaviour follows the reference:
//   api/api-basic.c:41-189   golden generator init_scalar / init_array / check_array
//   api/api-basic.c:254-292  plain_index (not row-major; reproduced as written)
//   api/api-basic.c:596-710  array printing
//   kernel/malloc.c:28-54    allocation (here: CUDA managed memory)
//   kernel/procmesh.c:36-89  process meshes
//   kernel/timer.c:53-373    plan timers and their vector layout
//   util/getargs.c:35-126    command line parsing
//   util/util.c:114-204      vector helpers and rank-0 printing
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <complex>
#include <vector>
#include "../../include/pfft.h"
#include "../../include/pfft_gb300.h"
#include "core.h"

using namespace pg;

struct pfft_plan_s {
  Plan* p;
};
struct pfftf_plan_s {
  Plan* p;
};

struct pfft_timer_s {
  int rnk_pm, rnk_trafo, rnk_remap, iter;
  double whole;
  double* trafo;
  double* remap;
  double remap_3dto2d[2];
  double itwiddle, otwiddle;
};
struct pfftf_timer_s : pfft_timer_s {};

namespace {

int g_nthreads = 1;

enum { AT_REAL = 1, AT_COMPLEX = 2, AT_HERM = 3 };

INT plain_index(int rnk, const INT* n, const INT* kv) {
  INT k = 0;
  for (int t = 0; t < rnk; t++) k += k * n[t] + kv[t];
  return k;
}

template <class R>
std::complex<R> init_scalar(int rnk, const INT* n, const INT* i) {
  R m = (R)plain_index(rnk, n, i);
  if (m == 0) return std::complex<R>((R)1500.0, (R)1250.0);
  R two_m = 2 * m, two_m1 = 2 * m + 1;
  return std::complex<R>((R)(1000.0 / two_m), (R)(1000.0 / two_m1));
}

template <class R>
std::complex<R> init_scalar_periodic(int rnk, const INT* n, const INT* ind) {
  INT p[PG_MAX_DIMS + 1];
  for (int t = 0; t < rnk; t++) p[t] = ind[t] % n[t];
  return init_scalar<R>(rnk, n, p);
}

void vector_index(int rnk, const INT* n, INT k, INT* kv) {
  for (int t = rnk - 1; t >= 0; t--) {
    kv[t] = k % n[t];
    k = (k - kv[t]) / n[t];
  }
}

INT prod(int d, const INT* v) {
  INT p = 1;
  for (int t = 0; t < d; t++) p *= v[t];
  return p;
}

bool is_device_only(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice;
}

template <class R>
void init_array(int rnk, const INT* n, const INT* ln, const INT* ls, int type, void* data) {
  INT tot = prod(rnk, ln);
  size_t esz = (type == AT_REAL) ? sizeof(R) : 2 * sizeof(R);
  bool dev = is_device_only(data);
  std::vector<unsigned char> tmp;
  unsigned char* h = (unsigned char*)data;
  if (dev) {
    tmp.resize((size_t)tot * esz);
    h = tmp.data();
  }
  INT kl[PG_MAX_DIMS + 1], kg[PG_MAX_DIMS + 1], km[PG_MAX_DIMS + 1];
  for (INT k = 0; k < tot; k++) {
    vector_index(rnk, ln, k, kl);
    for (int t = 0; t < rnk; t++) {
      kg[t] = kl[t] + ls[t];
      km[t] = n[t] - kg[t];
    }
    std::complex<R> d1 = init_scalar_periodic<R>(rnk, n, kg);
    if (type == AT_REAL) {
      ((R*)h)[k] = (kg[rnk - 1] < n[rnk - 1]) ? d1.real() : (R)0;
    } else if (type == AT_COMPLEX) {
      ((R*)h)[2 * k] = d1.real();
      ((R*)h)[2 * k + 1] = d1.imag();
    } else {
      std::complex<R> d2 = init_scalar_periodic<R>(rnk, n, km);
      // the reference combines in double complex (conj promotes) and rounds once
      std::complex<double> v = 0.5 * (std::complex<double>(d1) + std::conj(std::complex<double>(d2)));
      ((R*)h)[2 * k] = (R)v.real();
      ((R*)h)[2 * k + 1] = (R)v.imag();
    }
  }
  if (dev) cudaMemcpy(data, h, tmp.size(), cudaMemcpyHostToDevice);
}

template <class R>
void clear_array(int rnk, const INT* ln, int type, void* data) {
  INT tot = prod(rnk, ln);
  size_t esz = (type == AT_REAL) ? sizeof(R) : 2 * sizeof(R);
  if (is_device_only(data))
    cudaMemset(data, 0, (size_t)tot * esz);
  else
    memset(data, 0, (size_t)tot * esz);
}

template <class R>
R check_array(int rnk, const INT* n, const INT* ln, const INT* ls, int type, const void* data) {
  INT tot = prod(rnk, ln);
  size_t esz = (type == AT_REAL) ? sizeof(R) : 2 * sizeof(R);
  std::vector<unsigned char> tmp;
  const unsigned char* h = (const unsigned char*)data;
  if (is_device_only(data)) {
    tmp.resize((size_t)tot * esz);
    cudaMemcpy(tmp.data(), data, tmp.size(), cudaMemcpyDeviceToHost);
    h = tmp.data();
  }
  INT kl[PG_MAX_DIMS + 1], kg[PG_MAX_DIMS + 1], km[PG_MAX_DIMS + 1];
  R maxerr = 0;
  for (INT k = 0; k < tot; k++) {
    vector_index(rnk, ln, k, kl);
    for (int t = 0; t < rnk; t++) {
      kg[t] = kl[t] + ls[t];
      km[t] = n[t] - kg[t];
    }
    std::complex<R> d1 = init_scalar_periodic<R>(rnk, n, kg);
    R err;
    if (type == AT_REAL) {
      err = (kg[rnk - 1] < n[rnk - 1]) ? (R)fabs((double)(((const R*)h)[k] - d1.real())) : (R)0;
    } else {
      std::complex<R> v(((const R*)h)[2 * k], ((const R*)h)[2 * k + 1]);
      if (type == AT_HERM) {
        std::complex<double> ref =
            0.5 * (std::complex<double>(d1) + std::conj(std::complex<double>(init_scalar_periodic<R>(rnk, n, km))));
        err = (R)std::abs(std::complex<double>(v) - ref);
      } else {
        err = (R)std::abs(std::complex<double>(v - d1));
      }
    }
    if (err > maxerr) maxerr = err;
  }
  return maxerr;
}

void print_array(const double* dd, const float* df, const INT* n, const INT* start, const char* name, int cplx) {
  INT l = 0;
  if (n[0] * n[1] * n[2] < 1) return;
  for (INT k0 = 0; k0 < n[0]; k0++) {
    printf("%s(%td,%td:%td,%td:%td):\n", name, start[0] + k0, start[1], start[1] + n[1] - 1, start[2],
           start[2] + n[2] - 1);
    for (INT k1 = 0; k1 < n[1]; k1++) {
      printf("  ");
      for (INT k2 = 0; k2 < n[2]; k2++, l++) {
        double re = dd ? dd[cplx ? 2 * l : l] : df[cplx ? 2 * l : l];
        if (cplx) {
          double im = dd ? dd[2 * l + 1] : df[2 * l + 1];
          printf("  %.2e + %.2ei,", re, im);
        } else {
          printf("  %.2e,", re);
        }
      }
      printf("\n");
    }
  }
  printf("\n");
}

// ---- timers (kernel/timer.c) ------------------------------------------------------
pfft_timer_s* mktimer(int rnk_pm) {
  pfft_timer_s* t = (pfft_timer_s*)malloc(sizeof(pfft_timer_s));
  t->rnk_pm = rnk_pm;
  t->rnk_trafo = 2 * rnk_pm + 2;
  t->rnk_remap = 2 * rnk_pm;
  t->trafo = (double*)calloc((size_t)t->rnk_trafo, sizeof(double));
  t->remap = (double*)calloc((size_t)t->rnk_remap, sizeof(double));
  t->iter = 0;
  t->whole = 0;
  t->remap_3dto2d[0] = t->remap_3dto2d[1] = 0;
  t->itwiddle = t->otwiddle = 0;
  return t;
}
pfft_timer_s* timer_from_plan(const Plan* p) {
  pfft_timer_s* t = mktimer(p->timer.rnk_pm);
  t->iter = p->timer.iter;
  t->whole = p->timer.whole;
  for (int k = 0; k < t->rnk_trafo && k < (int)p->timer.trafo.size(); k++) t->trafo[k] = p->timer.trafo[k];
  for (int k = 0; k < t->rnk_remap && k < (int)p->timer.remap.size(); k++) t->remap[k] = p->timer.remap[k];
  return t;
}
pfft_timer_s* copy_timer(const pfft_timer_s* o) {
  pfft_timer_s* c = mktimer(o->rnk_pm);
  c->iter = o->iter;
  c->whole = o->whole;
  for (int k = 0; k < o->rnk_trafo; k++) c->trafo[k] = o->trafo[k];
  for (int k = 0; k < o->rnk_remap; k++) c->remap[k] = o->remap[k];
  c->remap_3dto2d[0] = o->remap_3dto2d[0];
  c->remap_3dto2d[1] = o->remap_3dto2d[1];
  c->itwiddle = o->itwiddle;
  c->otwiddle = o->otwiddle;
  return c;
}
size_t timer_len(const pfft_timer_s* t) { return (size_t)(t->rnk_trafo + t->rnk_remap + 9); }
double* timer2vec(const pfft_timer_s* t) {
  double* v = (double*)malloc(sizeof(double) * timer_len(t));
  int m = 0;
  v[m++] = t->rnk_pm;
  v[m++] = t->rnk_trafo;
  v[m++] = t->rnk_remap;
  v[m++] = t->iter;
  v[m++] = t->whole;
  for (int k = 0; k < t->rnk_trafo; k++) v[m++] = t->trafo[k];
  for (int k = 0; k < t->rnk_remap; k++) v[m++] = t->remap[k];
  v[m++] = t->remap_3dto2d[0];
  v[m++] = t->remap_3dto2d[1];
  v[m++] = t->itwiddle;
  v[m++] = t->otwiddle;
  return v;
}
pfft_timer_s* vec2timer(const double* v) {
  pfft_timer_s* t = mktimer((int)v[0]);
  int m = 3;
  t->iter = (int)v[m++];
  t->whole = v[m++];
  for (int k = 0; k < t->rnk_trafo; k++) t->trafo[k] = v[m++];
  for (int k = 0; k < t->rnk_remap; k++) t->remap[k] = v[m++];
  t->remap_3dto2d[0] = v[m++];
  t->remap_3dto2d[1] = v[m++];
  t->itwiddle = v[m++];
  t->otwiddle = v[m++];
  return t;
}
void fprint_timer(FILE* f, const Plan* p, const pfft_timer_s* t0, int adv) {
  pfft_timer_s* t = copy_timer(t0);
  if (t->iter > 0) {
    t->whole /= t->iter;
    for (int k = 0; k < t->rnk_trafo; k++) t->trafo[k] /= t->iter;
    for (int k = 0; k < t->rnk_remap; k++) t->remap[k] /= t->iter;
  }
  const char* pre = (p->d.sign == -1) ? "pfft_forw" : "pfft_back";
  fprintf(f, "%s(%d) = %.6e;  %% whole trafo\n", pre, 1, t->whole);
  if (adv) {
    for (int k = 0; k < t->rnk_trafo; k++) fprintf(f, "%s_trafo%d(%d) = %.6e;\n", pre, k + 1, 1, t->trafo[k]);
    for (int k = 0; k < t->rnk_remap; k++) fprintf(f, "%s_remap%d(%d) = %.6e;\n", pre, k + 1, 1, t->remap[k]);
  }
  free(t->trafo);
  free(t->remap);
  free(t);
}
void write_info(FILE* f, const Plan* p) {
  fprintf(f, "\n%% n - FFT size\n%% np - process grid\n%% procs - number of processes\n%% pfft - PFFT runtime\n");
  fprintf(f, "%% index(i) = log(procs(i)) + 1\n");
  fprintf(f, "index(1) = 1;  procs(1) = 1;  np_pfft(1, 1:%d) = [", p->d.mesh_rank);
  for (int t = 0; t < p->d.mesh_rank; t++) fprintf(f, "1 ");
  fprintf(f, "];\nn_pfft(1, 1:%d) = [", p->d.rnk_n);
  for (int t = 0; t < p->d.rnk_n; t++) fprintf(f, "%td ", p->d.n[t]);
  fprintf(f, "];\n");
}

}  // namespace

#define PG_HELPERS(PX, R, C)                                                                              \
  extern "C" {                                                                                            \
  void PX##init(void) { cudaFree(0); }                                                                    \
  void PX##cleanup(void) {                                                                              \
    twiddle_release_all();                                                                                \
    noalloc_forget();                                                                                     \
  }                                                                                                       \
  void PX##plan_with_nthreads(int n) { g_nthreads = n > 0 ? n : 1; }                                      \
  int PX##get_nthreads(void) { return g_nthreads; }                                                       \
  void* PX##malloc(size_t n) {                                                                            \
    void* p = nullptr;                                                                                    \
    if (cudaMallocManaged(&p, n ? n : 1) != cudaSuccess) {                                                \
      cudaGetLastError();                                                                                 \
      fprintf(stderr, "PFFT ERROR: out of memory (%zu bytes)\n", n);                                      \
      return nullptr;                                                                                     \
    }                                                                                                     \
    return p;                                                                                             \
  }                                                                                                       \
  R* PX##alloc_real(size_t n) { return (R*)PX##malloc(sizeof(R) * n); }                                   \
  C* PX##alloc_complex(size_t n) { return (C*)PX##malloc(sizeof(C) * n); }                                \
  void PX##free(void* p) {                                                                                \
    if (p) cudaFree(p);                                                                                   \
  }                                                                                                       \
  void PX##init_input_complex(int rnk, const INT* n, const INT* ln, const INT* ls, C* d) {                \
    init_array<R>(rnk, n, ln, ls, AT_COMPLEX, d);                                                         \
  }                                                                                                       \
  void PX##init_input_complex_3d(const INT* n, const INT* ln, const INT* ls, C* d) {                      \
    init_array<R>(3, n, ln, ls, AT_COMPLEX, d);                                                           \
  }                                                                                                       \
  void PX##init_input_complex_hermitian(int rnk, const INT* n, const INT* ln, const INT* ls, C* d) {      \
    init_array<R>(rnk, n, ln, ls, AT_HERM, d);                                                            \
  }                                                                                                       \
  void PX##init_input_complex_hermitian_3d(const INT* n, const INT* ln, const INT* ls, C* d) {            \
    init_array<R>(3, n, ln, ls, AT_HERM, d);                                                              \
  }                                                                                                       \
  void PX##init_input_real(int rnk, const INT* n, const INT* ln, const INT* ls, R* d) {                   \
    init_array<R>(rnk, n, ln, ls, AT_REAL, d);                                                            \
  }                                                                                                       \
  void PX##init_input_real_3d(const INT* n, const INT* ln, const INT* ls, R* d) {                         \
    init_array<R>(3, n, ln, ls, AT_REAL, d);                                                              \
  }                                                                                                       \
  void PX##clear_input_complex(int rnk, const INT*, const INT* ln, const INT*, C* d) {                    \
    clear_array<R>(rnk, ln, AT_COMPLEX, d);                                                               \
  }                                                                                                       \
  void PX##clear_input_complex_3d(const INT*, const INT* ln, const INT*, C* d) {                          \
    clear_array<R>(3, ln, AT_COMPLEX, d);                                                                 \
  }                                                                                                       \
  void PX##clear_input_complex_hermitian(int rnk, const INT*, const INT* ln, const INT*, C* d) {          \
    clear_array<R>(rnk, ln, AT_HERM, d);                                                                  \
  }                                                                                                       \
  void PX##clear_input_complex_hermitian_3d(const INT*, const INT* ln, const INT*, C* d) {                \
    clear_array<R>(3, ln, AT_HERM, d);                                                                    \
  }                                                                                                       \
  void PX##clear_input_real(int rnk, const INT*, const INT* ln, const INT*, R* d) {                       \
    clear_array<R>(rnk, ln, AT_REAL, d);                                                                  \
  }                                                                                                       \
  void PX##clear_input_real_3d(const INT*, const INT* ln, const INT*, R* d) {                             \
    clear_array<R>(3, ln, AT_REAL, d);                                                                    \
  }                                                                                                       \
  R PX##check_output_complex(int rnk, const INT* n, const INT* ln, const INT* ls, const C* d, MPI_Comm) { \
    return check_array<R>(rnk, n, ln, ls, AT_COMPLEX, d);                                                 \
  }                                                                                                       \
  R PX##check_output_complex_3d(const INT* n, const INT* ln, const INT* ls, const C* d, MPI_Comm) {       \
    return check_array<R>(3, n, ln, ls, AT_COMPLEX, d);                                                   \
  }                                                                                                       \
  R PX##check_output_complex_hermitian(int rnk, const INT* n, const INT* ln, const INT* ls, const C* d,   \
                                       MPI_Comm) {                                                       \
    return check_array<R>(rnk, n, ln, ls, AT_HERM, d);                                                    \
  }                                                                                                       \
  R PX##check_output_complex_hermitian_3d(const INT* n, const INT* ln, const INT* ls, const C* d,        \
                                          MPI_Comm) {                                                    \
    return check_array<R>(3, n, ln, ls, AT_HERM, d);                                                      \
  }                                                                                                       \
  R PX##check_output_real(int rnk, const INT* n, const INT* ln, const INT* ls, const R* d, MPI_Comm) {    \
    return check_array<R>(rnk, n, ln, ls, AT_REAL, d);                                                    \
  }                                                                                                       \
  R PX##check_output_real_3d(const INT* n, const INT* ln, const INT* ls, const R* d, MPI_Comm) {          \
    return check_array<R>(3, n, ln, ls, AT_REAL, d);                                                      \
  }                                                                                                       \
  INT PX##prod_INT(int d, const INT* v) { return prod(d, v); }                                            \
  INT PX##sum_INT(int d, const INT* v) {                                                                  \
    INT s = 0;                                                                                            \
    for (int t = 0; t < d; t++) s += v[t];                                                                \
    return s;                                                                                             \
  }                                                                                                       \
  int PX##equal_INT(int d, const INT* a, const INT* b) {                                                  \
    int e = 1;                                                                                            \
    for (int t = 0; t < d; t++) e *= (a[t] == b[t]);                                                      \
    return e;                                                                                             \
  }                                                                                                       \
  void PX##vcopy_INT(int d, const INT* a, INT* b) {                                                       \
    for (int t = 0; t < d; t++) b[t] = a[t];                                                              \
  }                                                                                                       \
  void PX##vadd_INT(int d, const INT* a, const INT* b, INT* s) {                                          \
    for (int t = 0; t < d; t++) s[t] = a[t] + b[t];                                                       \
  }                                                                                                       \
  void PX##vsub_INT(int d, const INT* a, const INT* b, INT* s) {                                          \
    for (int t = 0; t < d; t++) s[t] = a[t] - b[t];                                                       \
  }                                                                                                       \
  void PX##apr_complex_3d(const C* data, const INT* ln, const INT* ls, const char* name, MPI_Comm) {      \
    fflush(stdout);                                                                                       \
    printf("Rank %d:\n", 0);                                                                              \
    print_array(sizeof(R) == 8 ? (const double*)data : nullptr,                                           \
                sizeof(R) == 4 ? (const float*)data : nullptr, ln, ls, name, 1);                          \
    fflush(stdout);                                                                                       \
  }                                                                                                       \
  void PX##apr_real_3d(const R* data, const INT* ln, const INT* ls, const char* name, MPI_Comm) {         \
    fflush(stdout);                                                                                       \
    printf("Rank %d:\n", 0);                                                                              \
    print_array(sizeof(R) == 8 ? (const double*)data : nullptr,                                           \
                sizeof(R) == 4 ? (const float*)data : nullptr, ln, ls, name, 0);                          \
    fflush(stdout);                                                                                       \
  }                                                                                                       \
  void PX##apr_complex_permuted_3d(const C* data, const INT* ln, const INT* ls, int p0, int p1, int p2,   \
                                   const char* name, MPI_Comm comm) {                                    \
    int pm[3] = {p0, p1, p2};                                                                             \
    INT a[3], b[3];                                                                                       \
    for (int t = 0; t < 3; t++) {                                                                         \
      a[t] = ln[pm[t]];                                                                                   \
      b[t] = ls[pm[t]];                                                                                   \
    }                                                                                                     \
    PX##apr_complex_3d(data, a, b, name, comm);                                                           \
  }                                                                                                       \
  void PX##apr_real_permuted_3d(const R* data, const INT* ln, const INT* ls, int p0, int p1, int p2,      \
                                const char* name, MPI_Comm comm) {                                       \
    int pm[3] = {p0, p1, p2};                                                                             \
    INT a[3], b[3];                                                                                       \
    for (int t = 0; t < 3; t++) {                                                                         \
      a[t] = ln[pm[t]];                                                                                   \
      b[t] = ls[pm[t]];                                                                                   \
    }                                                                                                     \
    PX##apr_real_3d(data, a, b, name, comm);                                                              \
  }                                                                                                       \
  void PX##vfprintf(MPI_Comm, FILE* stream, const char* format, va_list ap) { vfprintf(stream, format, ap); } \
  void PX##fprintf(MPI_Comm comm, FILE* stream, const char* format, ...) {                                \
    va_list ap;                                                                                           \
    va_start(ap, format);                                                                                 \
    PX##vfprintf(comm, stream, format, ap);                                                               \
    va_end(ap);                                                                                           \
  }                                                                                                       \
  void PX##printf(MPI_Comm comm, const char* format, ...) {                                               \
    va_list ap;                                                                                           \
    va_start(ap, format);                                                                                 \
    PX##vfprintf(comm, stdout, format, ap);                                                               \
    va_end(ap);                                                                                           \
  }                                                                                                       \
  void PX##get_args(int argc, char** argv, const char* name, int need, unsigned type, void* par) {        \
    for (int it = 0; it < argc; it++) {                                                                   \
      if (strcmp(argv[it], name) != 0) continue;                                                          \
      if (type == PFFT_SWITCH) {                                                                          \
        *(int*)par = 1;                                                                                   \
        return;                                                                                           \
      }                                                                                                   \
      int given = 0;                                                                                      \
      while (it + given + 1 < argc && argv[it + given + 1] && argv[it + given + 1][0] != '-') given++;    \
      if (given < need) {                                                                                 \
        PX##printf(MPI_COMM_WORLD, "!!! Warning: Not enough command line arguments for %s !!!\n", name);  \
        return;                                                                                           \
      }                                                                                                   \
      for (int t = 0; t < need; t++) {                                                                    \
        const char* a = argv[it + 1 + t];                                                                 \
        switch (type) {                                                                                   \
          case PFFT_INT: ((int*)par)[t] = (int)strtol(a, NULL, 0); break;                                 \
          case PFFT_PTRDIFF_T: ((ptrdiff_t*)par)[t] = (ptrdiff_t)strtol(a, NULL, 0); break;               \
          case PFFT_FLOAT: ((float*)par)[t] = strtof(a, NULL); break;                                     \
          case PFFT_DOUBLE: ((double*)par)[t] = strtod(a, NULL); break;                                   \
          case PFFT_LDOUBLE: ((long double*)par)[t] = strtold(a, NULL); break;                            \
          case PFFT_UNSIGNED: ((unsigned*)par)[t] = (unsigned)strtoul(a, NULL, 0); break;                 \
          default:                                                                                        \
            PX##fprintf(MPI_COMM_WORLD, stderr, "!!! Error: PFFT_DATATYPE of %s not supported. !!!\n",    \
                        name);                                                                            \
            return;                                                                                       \
        }                                                                                                 \
      }                                                                                                   \
      return;                                                                                             \
    }                                                                                                     \
  }                                                                                                       \
  int PX##create_procmesh(int rnk, MPI_Comm comm, const int* np, MPI_Comm* cart) {                        \
    int size = 0, num = 1;                                                                                \
    MPI_Comm_size(comm, &size);                                                                           \
    for (int t = 0; t < rnk; t++) num *= np[t];                                                           \
    if (num != size) return 1;                                                                            \
    std::vector<int> per(rnk, 1), dims(np, np + rnk);                                                     \
    return MPI_Cart_create(comm, rnk, dims.data(), per.data(), 1, cart);                                  \
  }                                                                                                       \
  int PX##create_procmesh_1d(MPI_Comm comm, int np0, MPI_Comm* cart) {                                    \
    return PX##create_procmesh(1, comm, &np0, cart);                                                      \
  }                                                                                                       \
  int PX##create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm* cart) {                           \
    int np[2] = {np0, np1};                                                                               \
    return PX##create_procmesh(2, comm, np, cart);                                                        \
  }                                                                                                       \
  void PX##reset_timer(PX##plan ths) {                                                                    \
    if (!ths) return;                                                                                     \
    TimerData& t = ths->p->timer;                                                                         \
    t.iter = 0;                                                                                           \
    t.whole = 0;                                                                                          \
    for (auto& v : t.trafo) v = 0;                                                                        \
    for (auto& v : t.remap) v = 0;                                                                        \
  }                                                                                                       \
  PX##timer PX##get_timer(const PX##plan ths) { return ths ? (PX##timer)timer_from_plan(ths->p) : nullptr; } \
  void PX##print_average_timer(const PX##plan ths, MPI_Comm) {                                            \
    if (!ths) return;                                                                                     \
    write_info(stdout, ths->p);                                                                           \
    pfft_timer_s* t = timer_from_plan(ths->p);                                                            \
    fprint_timer(stdout, ths->p, t, 0);                                                                   \
    PX##destroy_timer((PX##timer)t);                                                                      \
  }                                                                                                       \
  void PX##print_average_timer_adv(const PX##plan ths, MPI_Comm) {                                        \
    if (!ths) return;                                                                                     \
    write_info(stdout, ths->p);                                                                           \
    pfft_timer_s* t = timer_from_plan(ths->p);                                                            \
    fprint_timer(stdout, ths->p, t, 1);                                                                   \
    PX##destroy_timer((PX##timer)t);                                                                      \
  }                                                                                                       \
  void PX##write_average_timer(const PX##plan ths, const char* name, MPI_Comm) {                          \
    if (!ths) return;                                                                                     \
    FILE* f = fopen(name, "a");                                                                           \
    if (!f) return;                                                                                       \
    write_info(f, ths->p);                                                                                \
    pfft_timer_s* t = timer_from_plan(ths->p);                                                            \
    fprint_timer(f, ths->p, t, 0);                                                                        \
    PX##destroy_timer((PX##timer)t);                                                                      \
    fclose(f);                                                                                            \
  }                                                                                                       \
  void PX##write_average_timer_adv(const PX##plan ths, const char* name, MPI_Comm) {                      \
    if (!ths) return;                                                                                     \
    FILE* f = fopen(name, "a");                                                                           \
    if (!f) return;                                                                                       \
    write_info(f, ths->p);                                                                                \
    pfft_timer_s* t = timer_from_plan(ths->p);                                                            \
    fprint_timer(f, ths->p, t, 1);                                                                        \
    PX##destroy_timer((PX##timer)t);                                                                      \
    fclose(f);                                                                                            \
  }                                                                                                       \
  PX##timer PX##copy_timer(const PX##timer o) { return o ? (PX##timer)copy_timer(o) : nullptr; }          \
  void PX##average_timer(PX##timer t) {                                                                   \
    if (!t || t->iter <= 0) return;                                                                       \
    t->whole /= t->iter;                                                                                  \
    for (int k = 0; k < t->rnk_trafo; k++) t->trafo[k] /= t->iter;                                        \
    for (int k = 0; k < t->rnk_remap; k++) t->remap[k] /= t->iter;                                        \
    for (int k = 0; k < 2; k++) t->remap_3dto2d[k] /= t->iter;                                            \
    t->itwiddle /= t->iter;                                                                               \
    t->otwiddle /= t->iter;                                                                               \
    t->iter = 1;                                                                                          \
  }                                                                                                       \
  PX##timer PX##add_timers(const PX##timer a, const PX##timer b) {                                        \
    pfft_timer_s* r = copy_timer(a);                                                                      \
    r->iter += b->iter;                                                                                   \
    r->whole += b->whole;                                                                                 \
    for (int k = 0; k < r->rnk_trafo; k++) r->trafo[k] += b->trafo[k];                                    \
    for (int k = 0; k < r->rnk_remap; k++) r->remap[k] += b->remap[k];                                    \
    for (int k = 0; k < 2; k++) r->remap_3dto2d[k] += b->remap_3dto2d[k];                                 \
    r->itwiddle += b->itwiddle;                                                                           \
    r->otwiddle += b->otwiddle;                                                                           \
    return (PX##timer)r;                                                                                  \
  }                                                                                                       \
  PX##timer PX##reduce_max_timer(const PX##timer t, MPI_Comm) { return (PX##timer)copy_timer(t); }        \
  double* PX##convert_timer2vec(const PX##timer t) { return timer2vec(t); }                               \
  PX##timer PX##convert_vec2timer(const double* v) { return (PX##timer)vec2timer(v); }                    \
  void PX##destroy_timer(PX##timer t) {                                                                   \
    if (!t) return;                                                                                       \
    free(t->trafo);                                                                                       \
    free(t->remap);                                                                                       \
    free(t);                                                                                              \
  }                                                                                                       \
  }

PG_HELPERS(pfft_, double, pfft_complex)
PG_HELPERS(pfftf_, float, pfftf_complex)

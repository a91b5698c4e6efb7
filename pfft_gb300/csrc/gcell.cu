// Ghost-cell exchange and reduce on one GPU.
//
// Reference: gcell/gcells_plan.c (plan_rgc_internal :80-199, local_size_gc
// :51-76, exchange_gc :379-398, reduce_gc :401-420, zero padding :424-455,
// truncation :458-486) and gcell/gcells_sendrecv.c.  With a single rank every
// neighbour is the rank itself, so the exchange is a periodic wrap of the
// compact block into the (gc_below + n + gc_above) box,
//     box[k] = block[(k - gc_below) mod n]   (per axis),
// and the reduce is its adjoint: every block cell receives the sum of all box
// cells that are its periodic images, then the box is truncated back to the
// compact block and the rest of the buffer is zeroed.
//
// Both operations are in place on the user's buffer.  The box overlaps the
// block it is built from, so the block (exchange) or the box (reduce) is first
// copied into plan-owned scratch memory and one gather / scatter-add kernel
// writes the result.
#include <stdio.h>
#include <string.h>
#include <chrono>
#include "../../include/pfft.h"
#include "../../include/pfft_gb300.h"
#include "core.h"

using namespace pg;

namespace {

struct GcDims {
  long long n[3], gb[3], ng[3];
  long long tuple;  // reals per cell
};

// box <- periodic wrap of the compact block held in src
template <class T>
__global__ void k_gc_gather(const T* __restrict__ src, T* __restrict__ box, GcDims g, long long ncell) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
    long long r = c;
    long long k2 = r % g.ng[2];
    r /= g.ng[2];
    long long k1 = r % g.ng[1];
    long long k0 = r / g.ng[1];
    long long j0 = (k0 - g.gb[0]) % g.n[0];
    long long j1 = (k1 - g.gb[1]) % g.n[1];
    long long j2 = (k2 - g.gb[2]) % g.n[2];
    if (j0 < 0) j0 += g.n[0];
    if (j1 < 0) j1 += g.n[1];
    if (j2 < 0) j2 += g.n[2];
    const T* s = src + ((j0 * g.n[1] + j1) * g.n[2] + j2) * g.tuple;
    T* d = box + c * g.tuple;
    for (long long h = 0; h < g.tuple; h++) d[h] = s[h];
  }
}

// block cell j <- sum of its periodic images in the box held in src
template <class T>
__global__ void k_gc_reduce(const T* __restrict__ src, T* __restrict__ blk, GcDims g, long long ncell) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
    long long r = c;
    long long j2 = r % g.n[2];
    r /= g.n[2];
    long long j1 = r % g.n[1];
    long long j0 = r / g.n[1];
    // first image along each axis
    long long s0 = j0 + g.gb[0], s1 = j1 + g.gb[1], s2 = j2 + g.gb[2];
    s0 -= (s0 / g.n[0]) * g.n[0];
    s1 -= (s1 / g.n[1]) * g.n[1];
    s2 -= (s2 / g.n[2]) * g.n[2];
    for (long long h = 0; h < g.tuple; h++) {
      T acc = 0;
      for (long long k0 = s0; k0 < g.ng[0]; k0 += g.n[0])
        for (long long k1 = s1; k1 < g.ng[1]; k1 += g.n[1])
          for (long long k2 = s2; k2 < g.ng[2]; k2 += g.n[2])
            acc += src[((k0 * g.ng[1] + k1) * g.ng[2] + k2) * g.tuple + h];
      blk[c * g.tuple + h] = acc;
    }
  }
}

struct GcPlan {
  int prec;  // 0 float, 1 double
  void* data;
  GcDims g;
  long long ncomp, nbox;  // cells
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  cudaStream_t stream = 0;
  // timers (gcell/gctimer.c layout: iter, whole, pad_zeros, exchange)
  double texg[4] = {0, 0, 0, 0};
  double tred[4] = {0, 0, 0, 0};
};

size_t esz(const GcPlan* p) { return p->prec ? sizeof(double) : sizeof(float); }

int launch_grid(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

bool dev_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

GcPlan* make_gc(int prec, int rnk, const INT* n_user, INT howmany, const INT* gcb_user, const INT* gca_user,
                void* data, MPI_Comm comm, unsigned flags, bool complex_data) {
  INT n[8], gcb[8], gca[8];
  for (int t = 0; t < rnk; t++) {
    n[t] = n_user[t];
    gcb[t] = gcb_user ? gcb_user[t] : 0;
    gca[t] = gca_user ? gca_user[t] : 0;
  }
  INT tuple = howmany;
  if (complex_data) {  // api/api-adv.c:295-324
    flags &= ~GC_PADDED;
    if (flags & GC_R2C) {
      n[rnk - 1] = n[rnk - 1] / 2 + 1;
      flags &= ~GC_R2C;
    }
    tuple = 2 * howmany;
  }
  if (flags & GC_PADDED) n[rnk - 1] = 2 * (n[rnk - 1] / 2 + 1);  // api/api-adv.c:250-252
  bool nothing = true;
  for (int t = 0; t < rnk; t++)
    if (gcb[t] != 0 || gca[t] != 0) nothing = false;
  if (nothing) return nullptr;
  if (rnk != 3) {
    fprintf(stderr, "Error: Gcell send only available for three dimensions.\n");
    return nullptr;
  }
  if (!comm_valid(comm)) return nullptr;
  int cd = comm_cart_dims(comm);
  int rnk_pm = cd > 0 ? cd : 1;
  // gcell/gcells_plan.c:222-234: cyclic shift of the distributed dims
  INT pn[3], pgb[3], pga[3];
  for (int t = 0; t < 3; t++) {
    int s = (t < rnk_pm && (flags & GC_TRANSPOSED)) ? (t + 1) % rnk_pm : t;
    pn[t] = n[s];
    pgb[t] = gcb[s];
    pga[t] = gca[s];
  }
  GcPlan* p = new GcPlan();
  p->prec = prec;
  p->data = data;
  p->ncomp = 1;
  p->nbox = 1;
  for (int t = 0; t < 3; t++) {
    if (pn[t] <= 0 || pgb[t] < 0 || pga[t] < 0) {
      delete p;
      return nullptr;
    }
    p->g.n[t] = pn[t];
    p->g.gb[t] = pgb[t];
    p->g.ng[t] = pgb[t] + pn[t] + pga[t];
    p->ncomp *= pn[t];
    p->nbox *= p->g.ng[t];
  }
  p->g.tuple = tuple;
  p->scratch_bytes = (size_t)p->nbox * tuple * esz(p);
  if (cuda_check(cudaMalloc(&p->scratch, p->scratch_bytes), "ghost-cell scratch")) {
    delete p;
    return nullptr;
  }
  return p;
}

template <class T>
int gc_exchange_t(GcPlan* p, void* data) {
  size_t cb = (size_t)p->ncomp * p->g.tuple * sizeof(T);
  cudaError_t e = cudaMemcpyAsync(p->scratch, data, cb, cudaMemcpyDeviceToDevice, p->stream);
  if (e != cudaSuccess) return (int)e;
  k_gc_gather<T><<<launch_grid(p->nbox), 256, 0, p->stream>>>((const T*)p->scratch, (T*)data, p->g, p->nbox);
  return (int)cudaGetLastError();
}

template <class T>
int gc_reduce_t(GcPlan* p, void* data) {
  size_t bb = (size_t)p->nbox * p->g.tuple * sizeof(T);
  size_t cb = (size_t)p->ncomp * p->g.tuple * sizeof(T);
  cudaError_t e = cudaMemcpyAsync(p->scratch, data, bb, cudaMemcpyDeviceToDevice, p->stream);
  if (e != cudaSuccess) return (int)e;
  k_gc_reduce<T><<<launch_grid(p->ncomp), 256, 0, p->stream>>>((const T*)p->scratch, (T*)data, p->g, p->ncomp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (bb > cb) e = cudaMemsetAsync((char*)data + cb, 0, bb - cb, p->stream);
  return (int)e;
}

void gc_run(GcPlan* p, bool reduce) {
  if (!p) return;
  auto t0 = std::chrono::steady_clock::now();
  size_t bb = (size_t)p->nbox * p->g.tuple * esz(p);
  void* d = p->data;
  void* tmp = nullptr;
  if (!dev_ptr(d)) {  // host buffer: stage through a device copy
    if (cuda_check(cudaMalloc(&tmp, bb), "ghost-cell staging")) return;
    size_t in_b = reduce ? bb : (size_t)p->ncomp * p->g.tuple * esz(p);
    if (cuda_check(cudaMemcpyAsync(tmp, d, in_b, cudaMemcpyHostToDevice, p->stream), "ghost-cell upload")) {
      cudaFree(tmp);
      return;
    }
    d = tmp;
  }
  int rc;
  if (reduce)
    rc = p->prec ? gc_reduce_t<double>(p, d) : gc_reduce_t<float>(p, d);
  else
    rc = p->prec ? gc_exchange_t<double>(p, d) : gc_exchange_t<float>(p, d);
  if (!rc && tmp) rc = (int)cudaMemcpyAsync(p->data, tmp, bb, cudaMemcpyDeviceToHost, p->stream);
  if (!rc) rc = (int)cudaStreamSynchronize(p->stream);
  if (tmp) cudaFree(tmp);
  if (rc) {
    cuda_check((cudaError_t)rc, reduce ? "reduce" : "exchange");
    return;
  }
  double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  double* tm = reduce ? p->tred : p->texg;
  tm[0] += 1;
  tm[1] += dt;
  tm[3] += dt;
}

struct GcTimer {
  double v[4];
};

}  // namespace

struct pfft_gcplan_s {
  GcPlan* p;
};
struct pfftf_gcplan_s {
  GcPlan* p;
};
struct pfft_gctimer_s {
  GcTimer t;
};
struct pfftf_gctimer_s {
  GcTimer t;
};

#define PG_GC_API(PX, PREC, R, C)                                                                          \
  extern "C" {                                                                                             \
  INT PX##local_size_many_gc(int rnk, const INT* ln, const INT* ls, INT howmany, const INT* gcb,          \
                             const INT* gca, INT* lngc, INT* lgcs) {                                      \
    INT mem = howmany;                                                                                     \
    for (int t = 0; t < rnk; t++) {                                                                        \
      INT b = gcb ? gcb[t] : 0, a = gca ? gca[t] : 0;                                                      \
      lngc[t] = b + ln[t] + a;                                                                             \
      lgcs[t] = ls[t] - b;                                                                                 \
      mem *= lngc[t];                                                                                      \
    }                                                                                                      \
    return mem;                                                                                            \
  }                                                                                                        \
  INT PX##local_size_gc(int rnk, const INT* ln, const INT* ls, const INT* gcb, const INT* gca, INT* lngc,  \
                        INT* lgcs) {                                                                       \
    return PX##local_size_many_gc(rnk, ln, ls, 1, gcb, gca, lngc, lgcs);                                   \
  }                                                                                                        \
  INT PX##local_size_gc_3d(const INT* ln, const INT* ls, const INT* gcb, const INT* gca, INT* lngc,        \
                           INT* lgcs) {                                                                    \
    return PX##local_size_many_gc(3, ln, ls, 1, gcb, gca, lngc, lgcs);                                     \
  }                                                                                                        \
  static PX##gcplan PX##gcwrap(GcPlan* p) {                                                                \
    if (!p) return nullptr;                                                                                \
    PX##gcplan w = new PX##gcplan_s;                                                                       \
    w->p = p;                                                                                              \
    return w;                                                                                              \
  }                                                                                                        \
  PX##gcplan PX##plan_many_rgc(int rnk, const INT* n, INT hm, const INT*, const INT* gcb, const INT* gca,  \
                               R* data, MPI_Comm comm, unsigned fl) {                                     \
    return PX##gcwrap(make_gc(PREC, rnk, n, hm, gcb, gca, data, comm, fl, false));                         \
  }                                                                                                        \
  PX##gcplan PX##plan_many_cgc(int rnk, const INT* n, INT hm, const INT*, const INT* gcb, const INT* gca,  \
                               C* data, MPI_Comm comm, unsigned fl) {                                     \
    return PX##gcwrap(make_gc(PREC, rnk, n, hm, gcb, gca, data, comm, fl, true));                          \
  }                                                                                                        \
  PX##gcplan PX##plan_rgc(int rnk, const INT* n, const INT* gcb, const INT* gca, R* data, MPI_Comm comm,   \
                          unsigned fl) {                                                                  \
    return PX##plan_many_rgc(rnk, n, 1, nullptr, gcb, gca, data, comm, fl);                                \
  }                                                                                                        \
  PX##gcplan PX##plan_cgc(int rnk, const INT* n, const INT* gcb, const INT* gca, C* data, MPI_Comm comm,   \
                          unsigned fl) {                                                                  \
    return PX##plan_many_cgc(rnk, n, 1, nullptr, gcb, gca, data, comm, fl);                                \
  }                                                                                                        \
  PX##gcplan PX##plan_rgc_3d(const INT* n, const INT* gcb, const INT* gca, R* data, MPI_Comm comm,         \
                             unsigned fl) {                                                               \
    return PX##plan_rgc(3, n, gcb, gca, data, comm, fl);                                                   \
  }                                                                                                        \
  PX##gcplan PX##plan_cgc_3d(const INT* n, const INT* gcb, const INT* gca, C* data, MPI_Comm comm,         \
                             unsigned fl) {                                                               \
    return PX##plan_cgc(3, n, gcb, gca, data, comm, fl);                                                   \
  }                                                                                                        \
  void PX##exchange(PX##gcplan ths) {                                                                      \
    if (ths) gc_run(ths->p, false);                                                                        \
  }                                                                                                        \
  void PX##reduce(PX##gcplan ths) {                                                                        \
    if (ths) gc_run(ths->p, true);                                                                         \
  }                                                                                                        \
  void PX##destroy_gcplan(PX##gcplan ths) {                                                                \
    if (!ths) return;                                                                                      \
    if (ths->p->scratch) cudaFree(ths->p->scratch);                                                        \
    delete ths->p;                                                                                         \
    delete ths;                                                                                            \
  }                                                                                                        \
  int PX##gb300_gc_set_stream(PX##gcplan ths, void* stream) {                                              \
    if (!ths) return -1;                                                                                   \
    ths->p->stream = (cudaStream_t)stream;                                                                 \
    return 0;                                                                                              \
  }                                                                                                        \
  void PX##reset_gctimers(PX##gcplan ths) {                                                                \
    if (!ths) return;                                                                                      \
    memset(ths->p->texg, 0, sizeof(ths->p->texg));                                                         \
    memset(ths->p->tred, 0, sizeof(ths->p->tred));                                                         \
  }                                                                                                        \
  PX##gctimer PX##get_gctimer_exg(const PX##gcplan ths) {                                                  \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, ths->p->texg, sizeof(t->t.v));                                                          \
    return t;                                                                                              \
  }                                                                                                        \
  PX##gctimer PX##get_gctimer_red(const PX##gcplan ths) {                                                  \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, ths->p->tred, sizeof(t->t.v));                                                          \
    return t;                                                                                              \
  }                                                                                                        \
  static void PX##fprint_gct(FILE* f, const char* pre, const double* v) {                                  \
    double it = v[0] > 0 ? v[0] : 1;                                                                       \
    fprintf(f, "%s(1) = %.6e;  %% whole\n", pre, v[1] / it);                                               \
    fprintf(f, "%s_pad_zeros(1) = %.6e;\n%s_exchange(1) = %.6e;\n", pre, v[2] / it, pre, v[3] / it);       \
  }                                                                                                        \
  void PX##print_average_gctimer(const PX##gcplan ths, MPI_Comm) {                                         \
    PX##fprint_gct(stdout, "pfft_gc_exg", ths->p->texg);                                                   \
    PX##fprint_gct(stdout, "pfft_gc_red", ths->p->tred);                                                   \
  }                                                                                                        \
  void PX##print_average_gctimer_adv(const PX##gcplan ths, MPI_Comm c) { PX##print_average_gctimer(ths, c); } \
  void PX##write_average_gctimer(const PX##gcplan ths, const char* name, MPI_Comm) {                       \
    FILE* f = fopen(name, "a");                                                                            \
    if (!f) return;                                                                                        \
    PX##fprint_gct(f, "pfft_gc_exg", ths->p->texg);                                                        \
    PX##fprint_gct(f, "pfft_gc_red", ths->p->tred);                                                        \
    fclose(f);                                                                                             \
  }                                                                                                        \
  void PX##write_average_gctimer_adv(const PX##gcplan ths, const char* name, MPI_Comm c) {                 \
    PX##write_average_gctimer(ths, name, c);                                                               \
  }                                                                                                        \
  PX##gctimer PX##copy_gctimer(const PX##gctimer o) {                                                      \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    t->t = o->t;                                                                                           \
    return t;                                                                                              \
  }                                                                                                        \
  void PX##average_gctimer(PX##gctimer t) {                                                                \
    if (t->t.v[0] <= 0) return;                                                                            \
    for (int k = 1; k < 4; k++) t->t.v[k] /= t->t.v[0];                                                    \
    t->t.v[0] = 1;                                                                                         \
  }                                                                                                        \
  PX##gctimer PX##add_gctimers(const PX##gctimer a, const PX##gctimer b) {                                 \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    for (int k = 0; k < 4; k++) t->t.v[k] = a->t.v[k] + b->t.v[k];                                         \
    return t;                                                                                              \
  }                                                                                                        \
  PX##gctimer PX##reduce_max_gctimer(const PX##gctimer t, MPI_Comm) { return PX##copy_gctimer(t); }        \
  void PX##convert_gctimer2vec(const PX##gctimer t, double* v) { memcpy(v, t->t.v, sizeof(t->t.v)); }      \
  PX##gctimer PX##convert_vec2gctimer(const double* v) {                                                   \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, v, sizeof(t->t.v));                                                                     \
    return t;                                                                                              \
  }                                                                                                        \
  void PX##destroy_gctimer(PX##gctimer t) { delete t; }                                                    \
  }

PG_GC_API(pfft_, 1, double, pfft_complex)
PG_GC_API(pfftf_, 0, float, pfftf_complex)

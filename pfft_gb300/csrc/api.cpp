// extern "C" entry points of the PFFT API (transform part) for pfft_ (double)
// and pfftf_ (float).  Each entry point keeps the reference's name, argument
// meaning and error behaviour:
//   api/api-basic.c:215-253   init / cleanup / destroy
//   api/api-basic.c:736-1040  *_3d and plain wrappers -> many
//   api/api-adv.c:30-217      local_size_many_*, plan_many_*, *_skipped
//   kernel/partrafo.c:337-373 plan rejection rules (planner returns NULL)
//   api/api-basic.c:1044-1147 execute / execute_dft / execute_dft_r2c / ...
#include <stdio.h>
#include <string.h>
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

namespace {

unsigned trafo_of(unsigned base, unsigned flags) {
  if ((base & (TR_R2C | TR_C2R)) && (flags & F_PADDED_R2C)) return base | TR_PADDED;
  return base;
}

INT do_local_size(int rnk, const INT* n, const INT* ni, const INT* no, INT howmany, MPI_Comm comm,
                  unsigned base, unsigned flags, INT* lni, INT* lis, INT* lno, INT* los) {
  if (!comm_valid(comm) || rnk < 1 || rnk > PG_MAX_DIMS) {
    report("local_size: invalid communicator or rank");
    for (int t = 0; t < rnk && t < PG_MAX_DIMS; t++) lni[t] = lis[t] = lno[t] = los[t] = 0;
    return 0;
  }
  SizeQuery q;
  q.rnk_n = rnk;
  q.n = n;
  q.ni = ni;
  q.no = no;
  q.howmany = howmany;
  q.trafo = trafo_of(base, flags);
  q.pfft_flags = flags;
  q.cart_dims = comm_cart_dims(comm);
  if (flags & F_SHIFTED_IN)
    for (int t = 0; t < rnk; t++)
      if (ni[t] % 2) fprintf(stderr, "PFFT ERROR: flag PFFT_SHIFTED_IN requires ni to be an even number\n");
  if (flags & F_SHIFTED_OUT)
    for (int t = 0; t < rnk; t++)
      if (no[t] % 2) fprintf(stderr, "PFFT ERROR: flag PFFT_SHIFTED_OUT requires no to be an even number\n");
  return local_size(q, lni, lis, lno, los);
}

void do_local_block(int rnk, const INT* ni, const INT* no, MPI_Comm comm, int pid, unsigned base, unsigned flags,
                    INT* lni, INT* lis, INT* lno, INT* los) {
  if (pid != 0) {
    report("local_block: process id %d does not exist on a single-rank mesh", pid);
    for (int t = 0; t < rnk; t++) lni[t] = lis[t] = lno[t] = los[t] = 0;
    return;
  }
  do_local_size(rnk, ni, ni, no, 1, comm, base, flags, lni, lis, lno, los);
}

Plan* do_plan(int prec, int rnk, const INT* n, const INT* ni, const INT* no, INT howmany, void* in, void* out,
              MPI_Comm comm, int sign, const int* kinds, const int* skip, unsigned base, unsigned flags) {
  // kernel/partrafo.c:337-373
  if (flags & (F_SHIFTED_IN | F_SHIFTED_OUT))
    for (int t = 0; t < rnk; t++)
      if (n[t] % 2) return nullptr;
  if ((flags & F_TRANSPOSED_OUT) && (flags & F_TRANSPOSED_IN)) return nullptr;
  if ((base & TR_R2C) && (flags & F_TRANSPOSED_IN)) return nullptr;
  if ((base & TR_C2R) && (flags & F_TRANSPOSED_OUT)) return nullptr;
  if (!comm_valid(comm)) return nullptr;
  int cd = comm_cart_dims(comm);
  int rnk_pm = cd > 0 ? cd : 1;
  if (rnk < rnk_pm) return nullptr;
  if (rnk == rnk_pm && rnk != 3) return nullptr;
  if (rnk > PG_MAX_DIMS || howmany < 1) {
    report("plan: unsupported rank or howmany");
    return nullptr;
  }
  PlanDesc d;
  d.prec = prec;
  d.rnk_n = rnk;
  d.n.assign(n, n + rnk);
  d.ni.assign(ni, ni + rnk);
  d.no.assign(no, no + rnk);
  d.howmany = howmany;
  d.trafo = trafo_of(base, flags);
  d.sign = (base & TR_R2R) ? -1 : sign;
  if (kinds) d.kinds.assign(kinds, kinds + rnk);
  if (skip) d.skip.assign(skip, skip + rnk);
  d.pfft_flags = flags;
  d.cart_dims = cd;
  d.mesh_rank = effective_mesh_rank(rnk, cd);
  d.mesh3d = (rnk == 3 && cd == 3);
  d.local_ni.resize(rnk);
  d.local_i_start.resize(rnk);
  d.local_no.resize(rnk);
  d.local_o_start.resize(rnk);
  SizeQuery q;
  q.rnk_n = rnk;
  q.n = n;
  q.ni = ni;
  q.no = no;
  q.howmany = howmany;
  q.trafo = d.trafo;
  q.pfft_flags = flags;
  q.cart_dims = cd;
  d.alloc_local = local_size(q, d.local_ni.data(), d.local_i_start.data(), d.local_no.data(), d.local_o_start.data());
  Plan* pl = make_plan(d, in, out);
  if (!pl) {
    fprintf(stderr, "PFFT ERROR: plan creation failed\n");
  }
  return pl;
}

void do_execute(Plan* pl, void* in, void* out) {
  if (!pl) {
    fprintf(stderr, "!!! Error: Can not execute PFFT Plan == NULL !!!\n");
    return;
  }
  execute_plan(pl, in, out, false);
}

}  // namespace

#define PG_API(PX, PREC, R, C)                                                                            \
  extern "C" {                                                                                            \
  INT PX##local_size_many_dft(int rnk, const INT* n, const INT* ni, const INT* no, INT hm, const INT*,   \
                              const INT*, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c, INT* e) {  \
    return do_local_size(rnk, n, ni, no, hm, comm, TR_C2C, fl, a, b, c, e);                              \
  }                                                                                                       \
  INT PX##local_size_many_dft_r2c(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,           \
                                  const INT*, const INT*, MPI_Comm comm, unsigned fl, INT* a, INT* b,    \
                                  INT* c, INT* e) {                                                      \
    return do_local_size(rnk, n, ni, no, hm, comm, TR_R2C, fl, a, b, c, e);                              \
  }                                                                                                       \
  INT PX##local_size_many_dft_c2r(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,           \
                                  const INT*, const INT*, MPI_Comm comm, unsigned fl, INT* a, INT* b,    \
                                  INT* c, INT* e) {                                                      \
    return do_local_size(rnk, n, ni, no, hm, comm, TR_C2R, fl, a, b, c, e);                              \
  }                                                                                                       \
  INT PX##local_size_many_r2r(int rnk, const INT* n, const INT* ni, const INT* no, INT hm, const INT*,   \
                              const INT*, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c, INT* e) {  \
    return do_local_size(rnk, n, ni, no, hm, comm, TR_R2R, fl, a, b, c, e);                              \
  }                                                                                                       \
  INT PX##local_size_dft(int rnk, const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,      \
                         INT* e) {                                                                       \
    return do_local_size(rnk, n, n, n, 1, comm, TR_C2C, fl, a, b, c, e);                                 \
  }                                                                                                       \
  INT PX##local_size_dft_r2c(int rnk, const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,  \
                             INT* e) {                                                                   \
    return do_local_size(rnk, n, n, n, 1, comm, TR_R2C, fl, a, b, c, e);                                 \
  }                                                                                                       \
  INT PX##local_size_dft_c2r(int rnk, const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,  \
                             INT* e) {                                                                   \
    return do_local_size(rnk, n, n, n, 1, comm, TR_C2R, fl, a, b, c, e);                                 \
  }                                                                                                       \
  INT PX##local_size_r2r(int rnk, const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,      \
                         INT* e) {                                                                       \
    return do_local_size(rnk, n, n, n, 1, comm, TR_R2R, fl, a, b, c, e);                                 \
  }                                                                                                       \
  INT PX##local_size_dft_3d(const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c, INT* e) {  \
    return do_local_size(3, n, n, n, 1, comm, TR_C2C, fl, a, b, c, e);                                   \
  }                                                                                                       \
  INT PX##local_size_dft_r2c_3d(const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,        \
                                INT* e) {                                                                \
    return do_local_size(3, n, n, n, 1, comm, TR_R2C, fl, a, b, c, e);                                   \
  }                                                                                                       \
  INT PX##local_size_dft_c2r_3d(const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c,        \
                                INT* e) {                                                                \
    return do_local_size(3, n, n, n, 1, comm, TR_C2R, fl, a, b, c, e);                                   \
  }                                                                                                       \
  INT PX##local_size_r2r_3d(const INT* n, MPI_Comm comm, unsigned fl, INT* a, INT* b, INT* c, INT* e) {  \
    return do_local_size(3, n, n, n, 1, comm, TR_R2R, fl, a, b, c, e);                                   \
  }                                                                                                       \
  void PX##local_block_many_dft(int rnk, const INT* ni, const INT* no, const INT*, const INT*,           \
                                MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c, INT* e) {   \
    do_local_block(rnk, ni, no, comm, pid, TR_C2C, fl, a, b, c, e);                                      \
  }                                                                                                       \
  void PX##local_block_many_dft_r2c(int rnk, const INT* ni, const INT* no, const INT*, const INT*,       \
                                    MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c,         \
                                    INT* e) {                                                            \
    do_local_block(rnk, ni, no, comm, pid, TR_R2C, fl, a, b, c, e);                                      \
  }                                                                                                       \
  void PX##local_block_many_dft_c2r(int rnk, const INT* ni, const INT* no, const INT*, const INT*,       \
                                    MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c,         \
                                    INT* e) {                                                            \
    do_local_block(rnk, ni, no, comm, pid, TR_C2R, fl, a, b, c, e);                                      \
  }                                                                                                       \
  void PX##local_block_many_r2r(int rnk, const INT* ni, const INT* no, const INT*, const INT*,           \
                                MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c, INT* e) {   \
    do_local_block(rnk, ni, no, comm, pid, TR_R2R, fl, a, b, c, e);                                      \
  }                                                                                                       \
  void PX##local_block_dft(int rnk, const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b,   \
                           INT* c, INT* e) {                                                             \
    do_local_block(rnk, n, n, comm, pid, TR_C2C, fl, a, b, c, e);                                        \
  }                                                                                                       \
  void PX##local_block_dft_r2c(int rnk, const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a,       \
                               INT* b, INT* c, INT* e) {                                                 \
    do_local_block(rnk, n, n, comm, pid, TR_R2C, fl, a, b, c, e);                                        \
  }                                                                                                       \
  void PX##local_block_dft_c2r(int rnk, const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a,       \
                               INT* b, INT* c, INT* e) {                                                 \
    do_local_block(rnk, n, n, comm, pid, TR_C2R, fl, a, b, c, e);                                        \
  }                                                                                                       \
  void PX##local_block_r2r(int rnk, const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b,   \
                           INT* c, INT* e) {                                                             \
    do_local_block(rnk, n, n, comm, pid, TR_R2R, fl, a, b, c, e);                                        \
  }                                                                                                       \
  void PX##local_block_dft_3d(const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c, \
                              INT* e) {                                                                  \
    do_local_block(3, n, n, comm, pid, TR_C2C, fl, a, b, c, e);                                          \
  }                                                                                                       \
  void PX##local_block_dft_r2c_3d(const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b,     \
                                  INT* c, INT* e) {                                                      \
    do_local_block(3, n, n, comm, pid, TR_R2C, fl, a, b, c, e);                                          \
  }                                                                                                       \
  void PX##local_block_dft_c2r_3d(const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b,     \
                                  INT* c, INT* e) {                                                      \
    do_local_block(3, n, n, comm, pid, TR_C2R, fl, a, b, c, e);                                          \
  }                                                                                                       \
  void PX##local_block_r2r_3d(const INT* n, MPI_Comm comm, int pid, unsigned fl, INT* a, INT* b, INT* c, \
                              INT* e) {                                                                  \
    do_local_block(3, n, n, comm, pid, TR_R2R, fl, a, b, c, e);                                          \
  }                                                                                                       \
  static PX##plan PX##wrap(Plan* p) {                                                                     \
    if (!p) return nullptr;                                                                               \
    PX##plan w = new PX##plan_s;                                                                          \
    w->p = p;                                                                                             \
    return w;                                                                                             \
  }                                                                                                       \
  PX##plan PX##plan_many_dft_skipped(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,        \
                                     const INT*, const INT*, const int* skip, C* in, C* out,             \
                                     MPI_Comm comm, int sign, unsigned fl) {                             \
    return PX##wrap(do_plan(PREC, rnk, n, ni, no, hm, in, out, comm, sign, nullptr, skip, TR_C2C, fl));  \
  }                                                                                                       \
  PX##plan PX##plan_many_dft_r2c_skipped(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,    \
                                         const INT*, const INT*, const int* skip, R* in, C* out,         \
                                         MPI_Comm comm, int sign, unsigned fl) {                         \
    return PX##wrap(do_plan(PREC, rnk, n, ni, no, hm, in, out, comm, sign, nullptr, skip, TR_R2C, fl));  \
  }                                                                                                       \
  PX##plan PX##plan_many_dft_c2r_skipped(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,    \
                                         const INT*, const INT*, const int* skip, C* in, R* out,         \
                                         MPI_Comm comm, int sign, unsigned fl) {                         \
    return PX##wrap(do_plan(PREC, rnk, n, ni, no, hm, in, out, comm, sign, nullptr, skip, TR_C2R, fl));  \
  }                                                                                                       \
  PX##plan PX##plan_many_r2r_skipped(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,        \
                                     const INT*, const INT*, const int* skip, R* in, R* out,             \
                                     MPI_Comm comm, const PX##r2r_kind* kinds, unsigned fl) {            \
    return PX##wrap(do_plan(PREC, rnk, n, ni, no, hm, in, out, comm, -1, (const int*)kinds, skip,        \
                            TR_R2R, fl));                                                                 \
  }                                                                                                       \
  PX##plan PX##plan_many_dft(int rnk, const INT* n, const INT* ni, const INT* no, INT hm, const INT* ib, \
                             const INT* ob, C* in, C* out, MPI_Comm comm, int sign, unsigned fl) {        \
    return PX##plan_many_dft_skipped(rnk, n, ni, no, hm, ib, ob, nullptr, in, out, comm, sign, fl);       \
  }                                                                                                       \
  PX##plan PX##plan_many_dft_r2c(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,            \
                                 const INT* ib, const INT* ob, R* in, C* out, MPI_Comm comm, int sign,   \
                                 unsigned fl) {                                                          \
    return PX##plan_many_dft_r2c_skipped(rnk, n, ni, no, hm, ib, ob, nullptr, in, out, comm, sign, fl);   \
  }                                                                                                       \
  PX##plan PX##plan_many_dft_c2r(int rnk, const INT* n, const INT* ni, const INT* no, INT hm,            \
                                 const INT* ib, const INT* ob, C* in, R* out, MPI_Comm comm, int sign,   \
                                 unsigned fl) {                                                          \
    return PX##plan_many_dft_c2r_skipped(rnk, n, ni, no, hm, ib, ob, nullptr, in, out, comm, sign, fl);   \
  }                                                                                                       \
  PX##plan PX##plan_many_r2r(int rnk, const INT* n, const INT* ni, const INT* no, INT hm, const INT* ib, \
                             const INT* ob, R* in, R* out, MPI_Comm comm, const PX##r2r_kind* kinds,     \
                             unsigned fl) {                                                              \
    return PX##plan_many_r2r_skipped(rnk, n, ni, no, hm, ib, ob, nullptr, in, out, comm, kinds, fl);      \
  }                                                                                                       \
  PX##plan PX##plan_dft(int rnk, const INT* n, C* in, C* out, MPI_Comm comm, int sign, unsigned fl) {     \
    return PX##plan_many_dft(rnk, n, n, n, 1, nullptr, nullptr, in, out, comm, sign, fl);                 \
  }                                                                                                       \
  PX##plan PX##plan_dft_r2c(int rnk, const INT* n, R* in, C* out, MPI_Comm comm, int sign, unsigned fl) { \
    return PX##plan_many_dft_r2c(rnk, n, n, n, 1, nullptr, nullptr, in, out, comm, sign, fl);             \
  }                                                                                                       \
  PX##plan PX##plan_dft_c2r(int rnk, const INT* n, C* in, R* out, MPI_Comm comm, int sign, unsigned fl) { \
    return PX##plan_many_dft_c2r(rnk, n, n, n, 1, nullptr, nullptr, in, out, comm, sign, fl);             \
  }                                                                                                       \
  PX##plan PX##plan_r2r(int rnk, const INT* n, R* in, R* out, MPI_Comm comm, const PX##r2r_kind* kinds,   \
                        unsigned fl) {                                                                   \
    return PX##plan_many_r2r(rnk, n, n, n, 1, nullptr, nullptr, in, out, comm, kinds, fl);                \
  }                                                                                                       \
  PX##plan PX##plan_dft_3d(const INT* n, C* in, C* out, MPI_Comm comm, int sign, unsigned fl) {           \
    return PX##plan_dft(3, n, in, out, comm, sign, fl);                                                   \
  }                                                                                                       \
  PX##plan PX##plan_dft_r2c_3d(const INT* n, R* in, C* out, MPI_Comm comm, int sign, unsigned fl) {       \
    return PX##plan_dft_r2c(3, n, in, out, comm, sign, fl);                                               \
  }                                                                                                       \
  PX##plan PX##plan_dft_c2r_3d(const INT* n, C* in, R* out, MPI_Comm comm, int sign, unsigned fl) {       \
    return PX##plan_dft_c2r(3, n, in, out, comm, sign, fl);                                               \
  }                                                                                                       \
  PX##plan PX##plan_r2r_3d(const INT* n, R* in, R* out, MPI_Comm comm, const PX##r2r_kind* kinds,         \
                           unsigned fl) {                                                                \
    return PX##plan_r2r(3, n, in, out, comm, kinds, fl);                                                  \
  }                                                                                                       \
  void PX##execute(const PX##plan plan) {                                                                 \
    if (!plan) {                                                                                          \
      do_execute(nullptr, nullptr, nullptr);                                                              \
      return;                                                                                             \
    }                                                                                                     \
    do_execute(plan->p, plan->p->in, plan->p->out);                                                       \
  }                                                                                                       \
  void PX##execute_dft(const PX##plan plan, C* in, C* out) {                                              \
    do_execute(plan ? plan->p : nullptr, in, out);                                                        \
  }                                                                                                       \
  void PX##execute_dft_r2c(const PX##plan plan, R* in, C* out) {                                          \
    do_execute(plan ? plan->p : nullptr, in, out);                                                        \
  }                                                                                                       \
  void PX##execute_dft_c2r(const PX##plan plan, C* in, R* out) {                                          \
    do_execute(plan ? plan->p : nullptr, in, out);                                                        \
  }                                                                                                       \
  void PX##execute_r2r(const PX##plan plan, R* in, R* out) {                                              \
    do_execute(plan ? plan->p : nullptr, in, out);                                                        \
  }                                                                                                       \
  void PX##execute_adjoint(const PX##plan plan) {                                                         \
    if (!plan) {                                                                                          \
      do_execute(nullptr, nullptr, nullptr);                                                              \
      return;                                                                                             \
    }                                                                                                     \
    execute_plan(plan->p, plan->p->out, plan->p->in, true);                                               \
  }                                                                                                       \
  void PX##execute_adjoint_arrays(const PX##plan plan, void* gout, void* gin) {                           \
    if (!plan) {                                                                                          \
      do_execute(nullptr, nullptr, nullptr);                                                              \
      return;                                                                                             \
    }                                                                                                     \
    execute_plan(plan->p, gout, gin, true);                                                               \
  }                                                                                                       \
  void PX##destroy_plan(PX##plan plan) {                                                                  \
    if (!plan) {                                                                                          \
      fprintf(stderr, "!!! Error: Can not finalize PFFT Plan == NULL !!!\n");                             \
      return;                                                                                             \
    }                                                                                                     \
    destroy_plan(plan->p);                                                                                \
    delete plan;                                                                                          \
  }                                                                                                       \
  int PX##gb300_set_stream(PX##plan plan, void* stream) {                                                 \
    if (!plan) return -1;                                                                                 \
    plan->p->stream = (cudaStream_t)stream;                                                               \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_set_sync(PX##plan plan, int sync) {                                                       \
    if (!plan) return -1;                                                                                 \
    plan->p->sync = sync != 0;                                                                            \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_set_graph(PX##plan plan, int on) {                                                        \
    if (!plan) return -1;                                                                                 \
    plan->p->use_graph = on != 0;                                                                         \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_set_pipeline(PX##plan plan, int on) {                                                     \
    if (!plan) return -1;                                                                                 \
    plan->p->pipeline = on != 0;                                                                          \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_plan_info(const PX##plan plan, int* npasses, double* bytes, size_t* ws_bytes) {           \
    if (!plan) return -1;                                                                                 \
    if (npasses) *npasses = (int)plan->p->fwd.passes.size();                                              \
    if (bytes) {                                                                                          \
      double b = 0;                                                                                       \
      for (const auto& ps : plan->p->fwd.passes) b += ps.bytes;                                           \
      *bytes = b;                                                                                         \
    }                                                                                                     \
    if (ws_bytes) *ws_bytes = plan->p->ws_cap[0] + plan->p->ws_cap[1];                                    \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_pass_kernel(const PX##plan plan, int i) {                                                \
    if (!plan || i < 0 || i >= (int)plan->p->fwd.passes.size()) return -1;                                \
    return fast_pass_eligible(plan->p->fwd.passes[i].p, plan->p->arith) ? 1 : 0;                         \
  }                                                                                                       \
  int PX##gb300_pass_fx_link(const PX##plan plan, int i) {                                              \
    if (!plan || i < 0 || i >= (int)plan->p->fwd.passes.size()) return -1;                                \
    const PassParams& q = plan->p->fwd.passes[i].p;                                                       \
    return (q.fx_in ? 1 : 0) | (q.fx_out ? 2 : 0) | (q.pair ? 4 : 0);                                     \
  }                                                                                                       \
  int PX##gb300_plan_arith(const PX##plan plan) {                                                        \
    if (!plan) return -1;                                                                                 \
    return plan->p->arith;                                                                                \
  }                                                                                                       \
  int PX##gb300_pass_info(const PX##plan plan, int i, int* axis, int* M, int* L, int* threads,            \
                          int* smem, double* bytes) {                                                    \
    if (!plan || i < 0 || i >= (int)plan->p->fwd.passes.size()) return -1;                                \
    const Pass& ps = plan->p->fwd.passes[i];                                                              \
    if (axis) *axis = ps.axis;                                                                            \
    if (M) *M = ps.p.M;                                                                                   \
    if (L) *L = ps.p.L;                                                                                   \
    if (threads) *threads = ps.p.threads;                                                                 \
    if (smem) *smem = ps.p.smem_bytes;                                                                    \
    if (bytes) *bytes = ps.bytes;                                                                         \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_set_pass_timing(PX##plan plan, int on) {                                                 \
    if (!plan) return -1;                                                                                 \
    plan->p->time_passes = on != 0;                                                                       \
    plan->p->pass_ms.assign(plan->p->fwd.passes.size(), 0.0);                                             \
    plan->p->timed_runs = 0;                                                                              \
    return 0;                                                                                             \
  }                                                                                                       \
  int PX##gb300_pass_time(const PX##plan plan, int i, double* ms_total, int* runs) {                      \
    if (!plan || i < 0 || i >= (int)plan->p->pass_ms.size()) return -1;                                   \
    if (ms_total) *ms_total = plan->p->pass_ms[i];                                                        \
    if (runs) *runs = plan->p->timed_runs;                                                                \
    return 0;                                                                                             \
  }                                                                                                       \
  }

PG_API(pfft_, 1, double, pfft_complex)
PG_API(pfftf_, 0, float, pfftf_complex)

extern "C" {
int pfft_gb300_last_error(void) { return last_error_code(); }
const char* pfft_gb300_last_error_string(void) { return last_error_string(); }
void pfft_gb300_clear_error(void) { clear_error(); }
long long pfft_gb300_pipelined_executes(void) { return pipelined_executes(); }
void pfft_gb300_set_kernel_path(int path) { set_kernel_path(path ? 1 : 0); }
int pfft_gb300_get_kernel_path(void) { return kernel_path(); }
void pfft_gb300_set_staged(int mode) { set_staged_mode(mode); }
int pfft_gb300_get_staged(void) { return staged_mode(); }
long long pfft_gb300_staged_launches(void) { return staged_launches(); }
int pfft_gb300_staged_status(void) {
  int* w = staged_err_word_if_any();
  if (!w) return 0;
  int h = 0;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, w, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(w, 0, sizeof(int));
  return e == cudaSuccess ? (h ? 1 : 0) : -(int)e;
}
int pfft_gb300_set_double_arith(int mode) {
  if (mode != DARITH_DF && mode != DARITH_NATIVE && mode != DARITH_AUTO && mode != DARITH_DFQ) return -1;
  set_double_arith(mode);
  return 0;
}
int pfft_gb300_get_double_arith(void) { return double_arith(); }
int pfft_gb300_set_fx_link(int on) {
  const int old = fx_link();
  set_fx_link(on);
  return old;
}
}

/* PFFT C API, GB300 build.
 *
 * Drop-in header for the transform-execution path of PFFT (mpip/pfft): the
 * same function names, argument lists, integer type (ptrdiff_t), complex
 * types and flag values as the reference's api/pfft.h, for the double
 * (pfft_) and float (pfftf_) precisions.  Every transform executes on one
 * GB300 GPU; the process mesh collapses to a single rank (see mpi.h).
 *
 * Reference interface replaced, by group (file:line in the PFFT tree):
 *   prototypes          api/pfft.h:69-502   (PFFT_DEFINE_API)
 *   instantiation        api/pfft.h:522-523  (pfft_, pfftf_; pfftl_ omitted:
 *                                             the GPU has no long double)
 *   r2r kinds            api/pfft.h:45-58
 *   flags                api/pfft.h:528-572
 *   complex / kind types api/pfft.h:515-520  (FFTW-compatible layouts)
 *
 * Arrays passed to the planners and executors may be device memory, managed
 * memory (pfft_alloc_* returns managed memory) or plain host memory; host
 * arrays are staged through device buffers inside pfft_execute.  Device
 * resident arrays give full HBM bandwidth.
 *
 * Project extensions (adjoint, batching, streams, wisdom, errors) are in
 * pfft_gb300.h.
 */
#ifndef PFFT_H
#define PFFT_H 1

#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include "mpi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- FFTW-compatible scalar types (api/pfft.h:515-520) ------------------ */
#ifndef FFTW3_H
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef enum fftw_r2r_kind_do_not_use_me {
  FFTW_R2HC = 0, FFTW_HC2R = 1, FFTW_DHT = 2,
  FFTW_REDFT00 = 3, FFTW_REDFT01 = 4, FFTW_REDFT10 = 5, FFTW_REDFT11 = 6,
  FFTW_RODFT00 = 7, FFTW_RODFT01 = 8, FFTW_RODFT10 = 9, FFTW_RODFT11 = 10
} fftw_r2r_kind;
typedef fftw_r2r_kind fftwf_r2r_kind;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#endif
#ifndef FFTW_MPI_DEFAULT_BLOCK
#define FFTW_MPI_DEFAULT_BLOCK (0)
#endif

typedef fftw_complex pfft_complex;
typedef fftwf_complex pfftf_complex;
typedef fftw_r2r_kind pfft_r2r_kind;
typedef fftwf_r2r_kind pfftf_r2r_kind;

/* ---- r2r kinds and directions (api/pfft.h:45-61) ------------------------ */
#define PFFT_R2HC FFTW_R2HC
#define PFFT_HC2R FFTW_HC2R
#define PFFT_DHT FFTW_DHT
#define PFFT_REDFT00 FFTW_REDFT00
#define PFFT_REDFT01 FFTW_REDFT01
#define PFFT_REDFT10 FFTW_REDFT10
#define PFFT_REDFT11 FFTW_REDFT11
#define PFFT_RODFT00 FFTW_RODFT00
#define PFFT_RODFT01 FFTW_RODFT01
#define PFFT_RODFT10 FFTW_RODFT10
#define PFFT_RODFT11 FFTW_RODFT11
#define PFFT_FORWARD FFTW_FORWARD
#define PFFT_BACKWARD FFTW_BACKWARD

/* ---- prototypes (api/pfft.h:69-502), one expansion per precision -------- */
#define PFFT_GB300_DECLARE(PX, R, C, INT)                                                          \
  typedef struct PX##plan_s *PX##plan;                                                             \
  typedef struct PX##gcplan_s *PX##gcplan;                                                         \
  typedef struct PX##timer_s *PX##timer;                                                           \
  typedef struct PX##gctimer_s *PX##gctimer;                                                       \
  /* set-up, threads, memory, execution: api/pfft.h:77-92 */                                       \
  void PX##init(void);                                                                             \
  void PX##cleanup(void);                                                                          \
  void PX##plan_with_nthreads(int nthreads);                                                       \
  int PX##get_nthreads(void);                                                                      \
  void *PX##malloc(size_t n);                                                                      \
  R *PX##alloc_real(size_t n);                                                                     \
  C *PX##alloc_complex(size_t n);                                                                  \
  void PX##free(void *p);                                                                          \
  void PX##execute(const PX##plan plan);                                                           \
  void PX##execute_dft(const PX##plan plan, C *in, C *out);                                        \
  void PX##execute_dft_r2c(const PX##plan plan, R *in, C *out);                                    \
  void PX##execute_dft_c2r(const PX##plan plan, C *in, R *out);                                    \
  void PX##execute_r2r(const PX##plan plan, R *in, R *out);                                        \
  void PX##destroy_plan(PX##plan plan);                                                            \
  /* golden-data helpers: api/pfft.h:94-149 */                                                     \
  void PX##init_input_complex_3d(const INT *n, const INT *ln, const INT *ls, C *data);             \
  void PX##init_input_complex(int rnk, const INT *n, const INT *ln, const INT *ls, C *data);       \
  void PX##init_input_complex_hermitian_3d(const INT *n, const INT *ln, const INT *ls, C *data);   \
  void PX##init_input_complex_hermitian(int rnk, const INT *n, const INT *ln, const INT *ls,       \
                                        C *data);                                                  \
  void PX##init_input_real_3d(const INT *n, const INT *ln, const INT *ls, R *data);                \
  void PX##init_input_real(int rnk, const INT *n, const INT *ln, const INT *ls, R *data);          \
  void PX##clear_input_complex_3d(const INT *n, const INT *ln, const INT *ls, C *data);            \
  void PX##clear_input_complex(int rnk, const INT *n, const INT *ln, const INT *ls, C *data);      \
  void PX##clear_input_complex_hermitian_3d(const INT *n, const INT *ln, const INT *ls, C *data);  \
  void PX##clear_input_complex_hermitian(int rnk, const INT *n, const INT *ln, const INT *ls,      \
                                         C *data);                                                 \
  void PX##clear_input_real_3d(const INT *n, const INT *ln, const INT *ls, R *data);               \
  void PX##clear_input_real(int rnk, const INT *n, const INT *ln, const INT *ls, R *data);         \
  R PX##check_output_complex_3d(const INT *n, const INT *ln, const INT *ls, const C *data,         \
                                MPI_Comm comm);                                                    \
  R PX##check_output_complex(int rnk, const INT *n, const INT *ln, const INT *ls, const C *data,   \
                             MPI_Comm comm);                                                       \
  R PX##check_output_complex_hermitian_3d(const INT *n, const INT *ln, const INT *ls,              \
                                          const C *data, MPI_Comm comm);                           \
  R PX##check_output_complex_hermitian(int rnk, const INT *n, const INT *ln, const INT *ls,        \
                                       const C *data, MPI_Comm comm);                              \
  R PX##check_output_real_3d(const INT *n, const INT *ln, const INT *ls, const R *data,            \
                             MPI_Comm comm);                                                       \
  R PX##check_output_real(int rnk, const INT *n, const INT *ln, const INT *ls, const R *data,      \
                          MPI_Comm comm);                                                          \
  /* data distribution: api/pfft.h:151-278 */                                                      \
  INT PX##local_size_dft_3d(const INT *n, MPI_Comm comm, unsigned flags, INT *lni, INT *lis,       \
                            INT *lno, INT *los);                                                   \
  INT PX##local_size_dft_r2c_3d(const INT *n, MPI_Comm comm, unsigned flags, INT *lni, INT *lis,   \
                                INT *lno, INT *los);                                               \
  INT PX##local_size_dft_c2r_3d(const INT *n, MPI_Comm comm, unsigned flags, INT *lni, INT *lis,   \
                                INT *lno, INT *los);                                               \
  INT PX##local_size_r2r_3d(const INT *n, MPI_Comm comm, unsigned flags, INT *lni, INT *lis,       \
                            INT *lno, INT *los);                                                   \
  INT PX##local_size_dft(int rnk, const INT *n, MPI_Comm comm, unsigned flags, INT *lni,           \
                         INT *lis, INT *lno, INT *los);                                            \
  INT PX##local_size_dft_r2c(int rnk, const INT *n, MPI_Comm comm, unsigned flags, INT *lni,       \
                             INT *lis, INT *lno, INT *los);                                        \
  INT PX##local_size_dft_c2r(int rnk, const INT *n, MPI_Comm comm, unsigned flags, INT *lni,       \
                             INT *lis, INT *lno, INT *los);                                        \
  INT PX##local_size_r2r(int rnk, const INT *n, MPI_Comm comm, unsigned flags, INT *lni,           \
                         INT *lis, INT *lno, INT *los);                                            \
  INT PX##local_size_many_dft(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany,    \
                              const INT *iblock, const INT *oblock, MPI_Comm comm, unsigned flags, \
                              INT *lni, INT *lis, INT *lno, INT *los);                             \
  INT PX##local_size_many_dft_r2c(int rnk, const INT *n, const INT *ni, const INT *no,             \
                                  INT howmany, const INT *iblock, const INT *oblock,               \
                                  MPI_Comm comm, unsigned flags, INT *lni, INT *lis, INT *lno,     \
                                  INT *los);                                                       \
  INT PX##local_size_many_dft_c2r(int rnk, const INT *n, const INT *ni, const INT *no,             \
                                  INT howmany, const INT *iblock, const INT *oblock,               \
                                  MPI_Comm comm, unsigned flags, INT *lni, INT *lis, INT *lno,     \
                                  INT *los);                                                       \
  INT PX##local_size_many_r2r(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany,    \
                              const INT *iblock, const INT *oblock, MPI_Comm comm, unsigned flags, \
                              INT *lni, INT *lis, INT *lno, INT *los);                             \
  void PX##local_block_dft_3d(const INT *n, MPI_Comm comm, int pid, unsigned flags, INT *lni,      \
                              INT *lis, INT *lno, INT *los);                                       \
  void PX##local_block_dft_r2c_3d(const INT *n, MPI_Comm comm, int pid, unsigned flags, INT *lni,  \
                                  INT *lis, INT *lno, INT *los);                                   \
  void PX##local_block_dft_c2r_3d(const INT *n, MPI_Comm comm, int pid, unsigned flags, INT *lni,  \
                                  INT *lis, INT *lno, INT *los);                                   \
  void PX##local_block_r2r_3d(const INT *n, MPI_Comm comm, int pid, unsigned flags, INT *lni,      \
                              INT *lis, INT *lno, INT *los);                                       \
  void PX##local_block_dft(int rnk, const INT *n, MPI_Comm comm, int pid, unsigned flags,          \
                           INT *lni, INT *lis, INT *lno, INT *los);                                \
  void PX##local_block_dft_r2c(int rnk, const INT *n, MPI_Comm comm, int pid, unsigned flags,      \
                               INT *lni, INT *lis, INT *lno, INT *los);                            \
  void PX##local_block_dft_c2r(int rnk, const INT *n, MPI_Comm comm, int pid, unsigned flags,      \
                               INT *lni, INT *lis, INT *lno, INT *los);                            \
  void PX##local_block_r2r(int rnk, const INT *n, MPI_Comm comm, int pid, unsigned flags,          \
                           INT *lni, INT *lis, INT *lno, INT *los);                                \
  void PX##local_block_many_dft(int rnk, const INT *ni, const INT *no, const INT *iblock,          \
                                const INT *oblock, MPI_Comm comm, int pid, unsigned flags,         \
                                INT *lni, INT *lis, INT *lno, INT *los);                           \
  void PX##local_block_many_dft_r2c(int rnk, const INT *ni, const INT *no, const INT *iblock,      \
                                    const INT *oblock, MPI_Comm comm, int pid, unsigned flags,     \
                                    INT *lni, INT *lis, INT *lno, INT *los);                       \
  void PX##local_block_many_dft_c2r(int rnk, const INT *ni, const INT *no, const INT *iblock,      \
                                    const INT *oblock, MPI_Comm comm, int pid, unsigned flags,     \
                                    INT *lni, INT *lis, INT *lno, INT *los);                       \
  void PX##local_block_many_r2r(int rnk, const INT *ni, const INT *no, const INT *iblock,          \
                                const INT *oblock, MPI_Comm comm, int pid, unsigned flags,         \
                                INT *lni, INT *lis, INT *lno, INT *los);                           \
  /* planners: api/pfft.h:280-343 */                                                               \
  PX##plan PX##plan_dft_3d(const INT *n, C *in, C *out, MPI_Comm comm, int sign, unsigned flags);  \
  PX##plan PX##plan_dft_r2c_3d(const INT *n, R *in, C *out, MPI_Comm comm, int sign,               \
                               unsigned flags);                                                    \
  PX##plan PX##plan_dft_c2r_3d(const INT *n, C *in, R *out, MPI_Comm comm, int sign,               \
                               unsigned flags);                                                    \
  PX##plan PX##plan_r2r_3d(const INT *n, R *in, R *out, MPI_Comm comm, const PX##r2r_kind *kinds,  \
                           unsigned flags);                                                        \
  PX##plan PX##plan_dft(int rnk, const INT *n, C *in, C *out, MPI_Comm comm, int sign,             \
                        unsigned flags);                                                           \
  PX##plan PX##plan_dft_r2c(int rnk, const INT *n, R *in, C *out, MPI_Comm comm, int sign,         \
                            unsigned flags);                                                       \
  PX##plan PX##plan_dft_c2r(int rnk, const INT *n, C *in, R *out, MPI_Comm comm, int sign,         \
                            unsigned flags);                                                       \
  PX##plan PX##plan_r2r(int rnk, const INT *n, R *in, R *out, MPI_Comm comm,                       \
                        const PX##r2r_kind *kinds, unsigned flags);                                \
  PX##plan PX##plan_many_dft(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany,     \
                             const INT *iblock, const INT *oblock, C *in, C *out, MPI_Comm comm,   \
                             int sign, unsigned flags);                                            \
  PX##plan PX##plan_many_dft_r2c(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany, \
                                 const INT *iblock, const INT *oblock, R *in, C *out,              \
                                 MPI_Comm comm, int sign, unsigned flags);                         \
  PX##plan PX##plan_many_dft_c2r(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany, \
                                 const INT *iblock, const INT *oblock, C *in, R *out,              \
                                 MPI_Comm comm, int sign, unsigned flags);                         \
  PX##plan PX##plan_many_r2r(int rnk, const INT *n, const INT *ni, const INT *no, INT howmany,     \
                             const INT *iblock, const INT *oblock, R *in, R *out, MPI_Comm comm,   \
                             const PX##r2r_kind *kinds, unsigned flags);                           \
  PX##plan PX##plan_many_dft_skipped(int rnk, const INT *n, const INT *ni, const INT *no,          \
                                     INT howmany, const INT *iblock, const INT *oblock,            \
                                     const int *skip, C *in, C *out, MPI_Comm comm, int sign,      \
                                     unsigned flags);                                              \
  PX##plan PX##plan_many_dft_r2c_skipped(int rnk, const INT *n, const INT *ni, const INT *no,      \
                                         INT howmany, const INT *iblock, const INT *oblock,        \
                                         const int *skip, R *in, C *out, MPI_Comm comm, int sign,  \
                                         unsigned flags);                                          \
  PX##plan PX##plan_many_dft_c2r_skipped(int rnk, const INT *n, const INT *ni, const INT *no,      \
                                         INT howmany, const INT *iblock, const INT *oblock,        \
                                         const int *skip, C *in, R *out, MPI_Comm comm, int sign,  \
                                         unsigned flags);                                          \
  PX##plan PX##plan_many_r2r_skipped(int rnk, const INT *n, const INT *ni, const INT *no,          \
                                     INT howmany, const INT *iblock, const INT *oblock,            \
                                     const int *skip, R *in, R *out, MPI_Comm comm,                \
                                     const PX##r2r_kind *kinds, unsigned flags);                   \
  /* integer vector helpers: api/pfft.h:345-359 */                                                 \
  INT PX##prod_INT(int d, const INT *vec);                                                         \
  INT PX##sum_INT(int d, const INT *vec);                                                          \
  int PX##equal_INT(int d, const INT *vec1, const INT *vec2);                                      \
  void PX##vcopy_INT(int d, const INT *vec1, INT *vec2);                                           \
  void PX##vadd_INT(int d, const INT *vec1, const INT *vec2, INT *sum);                            \
  void PX##vsub_INT(int d, const INT *vec1, const INT *vec2, INT *sum);                            \
  /* array printing: api/pfft.h:361-380 */                                                         \
  void PX##apr_complex_3d(const C *data, const INT *ln, const INT *ls, const char *name,           \
                          MPI_Comm comm);                                                          \
  void PX##apr_complex_permuted_3d(const C *data, const INT *ln, const INT *ls, int perm0,         \
                                   int perm1, int perm2, const char *name, MPI_Comm comm);         \
  void PX##apr_real_3d(const R *data, const INT *ln, const INT *ls, const char *name,              \
                       MPI_Comm comm);                                                             \
  void PX##apr_real_permuted_3d(const R *data, const INT *ln, const INT *ls, int perm0, int perm1, \
                                int perm2, const char *name, MPI_Comm comm);                       \
  /* command line helper: api/pfft.h:382-384 */                                                    \
  void PX##get_args(int argc, char **argv, const char *name, int neededArgs, unsigned type,        \
                    void *parameter);                                                              \
  /* plan timers: api/pfft.h:386-412 */                                                            \
  void PX##reset_timer(PX##plan ths);                                                              \
  PX##timer PX##get_timer(const PX##plan ths);                                                     \
  void PX##print_average_timer(const PX##plan ths, MPI_Comm comm);                                 \
  void PX##print_average_timer_adv(const PX##plan ths, MPI_Comm comm);                             \
  void PX##write_average_timer(const PX##plan ths, const char *name, MPI_Comm comm);               \
  void PX##write_average_timer_adv(const PX##plan ths, const char *name, MPI_Comm comm);           \
  PX##timer PX##copy_timer(const PX##timer orig);                                                  \
  void PX##average_timer(PX##timer ths);                                                           \
  PX##timer PX##add_timers(const PX##timer sum1, const PX##timer sum2);                            \
  PX##timer PX##reduce_max_timer(const PX##timer ths, MPI_Comm comm);                              \
  double *PX##convert_timer2vec(const PX##timer ths);                                              \
  PX##timer PX##convert_vec2timer(const double *times);                                            \
  void PX##destroy_timer(PX##timer ths);                                                           \
  /* rank-0 printing: api/pfft.h:416-421 */                                                        \
  void PX##vfprintf(MPI_Comm comm, FILE *stream, const char *format, va_list ap);                  \
  void PX##fprintf(MPI_Comm comm, FILE *stream, const char *format, ...);                          \
  void PX##printf(MPI_Comm comm, const char *format, ...);                                         \
  /* process meshes: api/pfft.h:423-431 */                                                         \
  int PX##create_procmesh(int rnk, MPI_Comm comm, const int *np, MPI_Comm *comm_cart);             \
  int PX##create_procmesh_1d(MPI_Comm comm, int np0, MPI_Comm *comm_cart_1d);                      \
  int PX##create_procmesh_2d(MPI_Comm comm, int np0, int np1, MPI_Comm *comm_cart_2d);             \
  /* ghost cells: api/pfft.h:433-471 */                                                            \
  INT PX##local_size_gc_3d(const INT *ln, const INT *ls, const INT *gc_below, const INT *gc_above, \
                           INT *lngc, INT *lgcs);                                                  \
  INT PX##local_size_gc(int rnk, const INT *ln, const INT *ls, const INT *gc_below,                \
                        const INT *gc_above, INT *lngc, INT *lgcs);                                \
  INT PX##local_size_many_gc(int rnk, const INT *ln, const INT *ls, INT howmany,                   \
                             const INT *gc_below, const INT *gc_above, INT *lngc, INT *lgcs);      \
  PX##gcplan PX##plan_rgc_3d(const INT *n, const INT *gc_below, const INT *gc_above, R *data,      \
                             MPI_Comm comm, unsigned gc_flags);                                    \
  PX##gcplan PX##plan_cgc_3d(const INT *n, const INT *gc_below, const INT *gc_above, C *data,      \
                             MPI_Comm comm, unsigned gc_flags);                                    \
  PX##gcplan PX##plan_rgc(int rnk, const INT *n, const INT *gc_below, const INT *gc_above,         \
                          R *data, MPI_Comm comm, unsigned gc_flags);                              \
  PX##gcplan PX##plan_cgc(int rnk, const INT *n, const INT *gc_below, const INT *gc_above,         \
                          C *data, MPI_Comm comm, unsigned gc_flags);                              \
  PX##gcplan PX##plan_many_rgc(int rnk, const INT *n, INT howmany, const INT *block,               \
                               const INT *gc_below, const INT *gc_above, R *data, MPI_Comm comm,   \
                               unsigned gc_flags);                                                 \
  PX##gcplan PX##plan_many_cgc(int rnk, const INT *n, INT howmany, const INT *block,               \
                               const INT *gc_below, const INT *gc_above, C *data, MPI_Comm comm,   \
                               unsigned gc_flags);                                                 \
  void PX##exchange(PX##gcplan ths);                                                               \
  void PX##reduce(PX##gcplan ths);                                                                 \
  void PX##destroy_gcplan(PX##gcplan ths);                                                         \
  /* ghost-cell timers: api/pfft.h:473-502 */                                                      \
  void PX##reset_gctimers(PX##gcplan ths);                                                         \
  PX##gctimer PX##get_gctimer_exg(const PX##gcplan ths);                                           \
  PX##gctimer PX##get_gctimer_red(const PX##gcplan ths);                                           \
  void PX##print_average_gctimer(const PX##gcplan ths, MPI_Comm comm);                             \
  void PX##print_average_gctimer_adv(const PX##gcplan ths, MPI_Comm comm);                         \
  void PX##write_average_gctimer(const PX##gcplan ths, const char *name, MPI_Comm comm);           \
  void PX##write_average_gctimer_adv(const PX##gcplan ths, const char *name, MPI_Comm comm);       \
  PX##gctimer PX##copy_gctimer(const PX##gctimer orig);                                            \
  void PX##average_gctimer(PX##gctimer ths);                                                       \
  PX##gctimer PX##add_gctimers(const PX##gctimer sum1, const PX##gctimer sum2);                    \
  PX##gctimer PX##reduce_max_gctimer(const PX##gctimer ths, MPI_Comm comm);                        \
  void PX##convert_gctimer2vec(const PX##gctimer ths, double *times);                              \
  PX##gctimer PX##convert_vec2gctimer(const double *times);                                        \
  void PX##destroy_gctimer(PX##gctimer ths);

PFFT_GB300_DECLARE(pfft_, double, pfft_complex, ptrdiff_t)
PFFT_GB300_DECLARE(pfftf_, float, pfftf_complex, ptrdiff_t)

/* ---- flags (api/pfft.h:528-572), identical bit values ------------------- */
#define PFFT_TRANSPOSED_NONE (0U)
#define PFFT_TRANSPOSED_IN (1U << 0)
#define PFFT_TRANSPOSED_OUT (1U << 1)
#define PFFT_SHIFTED_NONE (0U)
#define PFFT_SHIFTED_IN (1U << 2)
#define PFFT_SHIFTED_OUT (1U << 3)
#define PFFT_MEASURE (0U)
#define PFFT_ESTIMATE (1U << 4)
#define PFFT_PATIENT (1U << 5)
#define PFFT_EXHAUSTIVE (1U << 6)
#define PFFT_NO_TUNE (0U)
#define PFFT_TUNE (1U << 7)
#define PFFT_PRESERVE_INPUT (1U << 8)
#define PFFT_DESTROY_INPUT (1U << 9)
#define PFFT_BUFFERED_INPLACE (1U << 10)
#define PFFT_PADDED_R2C (1U << 11)
#define PFFT_PADDED_C2R (PFFT_PADDED_R2C)

#define PFFT_DEFAULT_BLOCK FFTW_MPI_DEFAULT_BLOCK
#define PFFT_DEFAULT_BLOCKS NULL
#define PFFT_NO_GCELLS NULL
#define FPFFT_DEFAULT_BLOCKS (-1)
#define FPFFT_NO_GCELLS (-1)

#define PFFT_INT (1U)
#define PFFT_PTRDIFF_T (2U)
#define PFFT_FLOAT (3U)
#define PFFT_DOUBLE (4U)
#define PFFT_LDOUBLE (5U)
#define PFFT_UNSIGNED (6U)
#define PFFT_SWITCH (7U)

#define PFFT_GC_TRANSPOSED_NONE (0U)
#define PFFT_GC_TRANSPOSED (1U << 0)
#define PFFT_GC_SENDRECV (1U << 1)
#define PFFT_GC_RMA (1U << 2)
#define PFFT_GC_R2C (1U << 3)
#define PFFT_GC_PADDED (1U << 4)
#define PFFT_GC_C2R (PFFT_GC_R2C)
#define PFFT_GC_PADDED_R2C (PFFT_GC_R2C | PFFT_GC_PADDED)
#define PFFT_GC_PADDED_C2R (PFFT_GC_C2R | PFFT_GC_PADDED)

#ifdef __cplusplus
}
#endif

#endif /* PFFT_H */

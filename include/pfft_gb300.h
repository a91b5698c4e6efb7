/* GB300 extensions to the PFFT C API.
 *
 * None of these entry points exists in the reference PFFT; they cover what a
 * single-GPU build adds around the unchanged pfft_/pfftf_ API of pfft.h:
 * adjoint execution (for differentiation), stream / graph control, batched
 * execution of many plans, plan introspection, arithmetic selection, wisdom
 * for the autotuner and error reporting.
 */
#ifndef PFFT_GB300_H
#define PFFT_GB300_H 1

#include <stddef.h>
#include "pfft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Adjoint of the plan's linear map, from the plan's `out` array into its `in`
 * array (both keep the plan's layouts).  c2c: the unnormalised transform of
 * the opposite sign; r2c: c2r of the half spectrum with the interior bins
 * halved (adjoint for the real inner product); c2r: r2c with the interior
 * bins doubled; zero-padding and truncation swap roles. */
void pfft_execute_adjoint(const pfft_plan plan);
void pfftf_execute_adjoint(const pfftf_plan plan);
/* Same with explicit arrays: gout has the plan's output layout, gin receives
 * the input layout. */
void pfft_execute_adjoint_arrays(const pfft_plan plan, void *gout, void *gin);
void pfftf_execute_adjoint_arrays(const pfftf_plan plan, void *gout, void *gin);

/* Execution control.  stream is a cudaStream_t (default: the legacy default
 * stream).  sync=1 (default) makes pfft_execute return after the work is done,
 * like the reference; sync=0 leaves it queued on the stream.  graph=1 replays
 * the pass launches from a captured CUDA graph (re-captured when the arrays
 * change). All return 0 on success, -1 for a NULL plan. */
int pfft_gb300_set_stream(pfft_plan plan, void *stream);
int pfftf_gb300_set_stream(pfftf_plan plan, void *stream);
int pfft_gb300_set_sync(pfft_plan plan, int sync);
int pfftf_gb300_set_sync(pfftf_plan plan, int sync);
int pfft_gb300_set_graph(pfft_plan plan, int graph);
int pfftf_gb300_set_graph(pfftf_plan plan, int graph);

/* Introspection: number of passes, algorithmic bytes of one execute (sum over
 * passes of elements read + written), and plan-owned workspace bytes. */
int pfft_gb300_plan_info(const pfft_plan plan, int *npasses, double *bytes, size_t *ws_bytes);
int pfftf_gb300_plan_info(const pfftf_plan plan, int *npasses, double *bytes, size_t *ws_bytes);
int pfft_gb300_pass_info(const pfft_plan plan, int i, int *axis, int *M, int *L, int *threads, int *smem,
                         double *bytes);
int pfftf_gb300_pass_info(const pfftf_plan plan, int i, int *axis, int *M, int *L, int *threads, int *smem,
                          double *bytes);

/* Per-pass timing with CUDA events recorded on the plan's stream around every
 * pass launch of pfft_execute (also feeds the plan timer's stage slots).
 * pass_time returns the accumulated milliseconds of pass i and the number of
 * timed executions. */
int pfft_gb300_set_pass_timing(pfft_plan plan, int on);
int pfftf_gb300_set_pass_timing(pfftf_plan plan, int on);
int pfft_gb300_pass_time(const pfft_plan plan, int i, double *ms_total, int *runs);
int pfftf_gb300_pass_time(const pfftf_plan plan, int i, double *ms_total, int *runs);

/* Arithmetic of the double API: 0 = float-float on the FP32 pipes (default),
 * 1 = native FP64.  Applies to plans created afterwards. */
void pfft_gb300_set_double_arith(int mode);
int pfft_gb300_get_double_arith(void);

/* Kernel selection: 1 (default) runs power-of-two c2c passes on the
 * register-resident radix-8 kernel, 0 uses the general pass kernel everywhere
 * (also set by the environment variable PFFT_GB300_KERNEL=generic). */
void pfft_gb300_set_kernel_path(int path);
int pfft_gb300_get_kernel_path(void);

/* Last error (CUDA error code or library error) and its message. */
int pfft_gb300_last_error(void);
const char *pfft_gb300_last_error_string(void);
void pfft_gb300_clear_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PFFT_GB300_H */

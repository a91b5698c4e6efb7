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
 * change).  pipeline=1 (default) overlaps, for out-of-place executes on host
 * arrays, the host-to-device copy of the input with the leading passes and
 * the device-to-host copy of the output with the last pass, where the pass
 * layout allows it; pipeline=0 stages whole arrays.  All return 0 on
 * success, -1 for a NULL plan. */
int pfft_gb300_set_stream(pfft_plan plan, void *stream);
int pfftf_gb300_set_stream(pfftf_plan plan, void *stream);
int pfft_gb300_set_sync(pfft_plan plan, int sync);
int pfftf_gb300_set_sync(pfftf_plan plan, int sync);
int pfft_gb300_set_graph(pfft_plan plan, int graph);
int pfftf_gb300_set_graph(pfftf_plan plan, int graph);
int pfft_gb300_set_pipeline(pfft_plan plan, int pipeline);
int pfftf_gb300_set_pipeline(pfftf_plan plan, int pipeline);

/* The CUDA stream (cudaStream_t) of a ghost-cell plan's exchange and reduce
 * (default: the legacy default stream).  Both stay synchronous: they return
 * once their work on that stream is done.  Returns 0, or -1 for a NULL plan. */
int pfft_gb300_gc_set_stream(pfft_gcplan plan, void *stream);
int pfftf_gb300_gc_set_stream(pfftf_gcplan plan, void *stream);
/* Executes (both precisions) that went through the host-array pipeline so far
 * in this process. */
long long pfft_gb300_pipelined_executes(void);

/* Introspection: number of passes, algorithmic bytes of one execute (sum over
 * passes of elements read + written), and plan-owned workspace bytes. */
int pfft_gb300_plan_info(const pfft_plan plan, int *npasses, double *bytes, size_t *ws_bytes);
int pfftf_gb300_plan_info(const pfftf_plan plan, int *npasses, double *bytes, size_t *ws_bytes);
/* Kernel of pass i: 1 = register-resident radix-8 kernel, 0 = general pass
 * kernel, -1 = no such pass. */
int pfft_gb300_pass_kernel(const pfft_plan plan, int i);
int pfftf_gb300_pass_kernel(const pfftf_plan plan, int i);
/* Fixed-point mantissas kept across pass i's boundaries (double plans, mode
 * 2): bit 0 = its input holds the previous pass's mantissas, bit 1 = its
 * output keeps them for the next pass; bit 2 = the pass (r2c or REDFT10)
 * transforms two real lines per complex line; -1 = no such pass. */
int pfft_gb300_pass_fx_link(const pfft_plan plan, int i);
int pfftf_gb300_pass_fx_link(const pfftf_plan plan, int i);
/* Arithmetic a plan runs in: 0 FP32 (float API), 1 FP64 class (modes 1 and 2
 * of pfft_gb300_set_double_arith), 2 float-float. */
int pfft_gb300_plan_arith(const pfft_plan plan);
int pfftf_gb300_plan_arith(const pfftf_plan plan);
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

/* Batched execution: many plans (uneven sizes, one precision) run as
 * persistent launches - work queues of (plan, pass, tile) entries with
 * per-plan pass dependencies - replayed from one CUDA graph: plans whose
 * passes all run on the radix-8 tile in one queue (a kernel with four CTAs
 * per SM), the others in a second (three CTAs per SM), the two launches on
 * forked streams.  Each plan runs on the arrays it was planned with.
 * batch_execute returns 0, a CUDA error, or -2 if a dependency wait timed out
 * (the kernels bound every wait).  batch_info: tasks of both queues, CTAs of
 * both launches. */
typedef struct pfft_gb300_batch_s *pfft_gb300_batch;
pfft_gb300_batch pfft_gb300_batch_create(int nplans, const pfft_plan *plans);
pfft_gb300_batch pfftf_gb300_batch_create(int nplans, const pfftf_plan *plans);
int pfft_gb300_batch_execute(pfft_gb300_batch batch);
int pfft_gb300_batch_set_stream(pfft_gb300_batch batch, void *stream);
int pfft_gb300_batch_set_graph(pfft_gb300_batch batch, int graph);
int pfft_gb300_batch_info(pfft_gb300_batch batch, int *ntasks, int *grid, int *threads, double *bytes);
void pfft_gb300_batch_destroy(pfft_gb300_batch batch);
/* Test hook: runs the batch kernel on a queue whose dependency is never met,
 * with the given wait limit; returns -2 when the bounded wait expired. */
int pfft_gb300_batch_wait_selftest(long long spin_limit);

/* Test hook: the double -> float-float -> double conversion of the double
 * API's kernels, element by element (device arrays, queued on `stream`). */
int pfft_gb300_selftest_df_roundtrip(const double *in, double *out, long long n, void *stream);

/* Test hook: the fast path of the float-float -> double conversion against
 * the full routine on n device float pairs (hi, lo).  counts: two zeroed
 * device words that receive the number of values the fast path took and how
 * many of its results differ from the full routine's. */
int pfft_gb300_selftest_df_fast(const float *pairs, long long n, unsigned long long *counts, void *stream);

/* Arithmetic of the double API, for plans created afterwards:
 *   0  float-float on the FP32 pipes with TwoSum additions (48-49
 *      significant bits; relative L2 error of a transform about 1e-14);
 *      opt-in: narrower than FFTW double
 *   1  native FP64 on every pass (general kernel; FP64 issues at about 1/70
 *      of the FP32 rate on GB300)
 *   2  default: FP64-class.  Power-of-two c2c, r2c, c2r, REDFT10 and REDFT01
 *      passes run the radix-8 kernel in 64-bit block fixed point (int64
 *      mantissas on a per-tile grid renormalised at every stage, exact
 *      additions, 64-bit twiddles; measured as accurate as native FP64),
 *      every other pass native FP64.
 *   3  float-float whose c2c passes on the radix-8 and mixed-radix kernels
 *      (2^a, 3 * 2^a, 5 * 2^a points) round the high words of each butterfly
 *      to a common grid, so that the butterfly's additions are exact without
 *      TwoSum: fewer FP32 operations, relative L2 error about 2e-13 per
 *      pass; other passes as in mode 0; opt-in: narrower than FFTW double.
 * The environment variable PFFT_GB300_F64_ARITH=df|native|auto|dfq sets the
 * initial mode.  Returns 0, or -1 for an unknown mode. */
int pfft_gb300_set_double_arith(int mode);
int pfft_gb300_get_double_arith(void);

/* Mode 2 keeps the int64 mantissas (and one exponent per line) between two
 * consecutive radix-8 passes instead of rounding them to double in between
 * (on by default; the environment variable PFFT_GB300_FX_LINK=0 sets it off).
 * Applies to plans created afterwards.  Returns the previous setting.
 * Mode 2 also transforms two real lines per complex line in r2c, c2r,
 * REDFT10 and REDFT01 passes whose first batch dimension has an even extent
 * (pfft_gb300_pass_fx_link reports it); the environment variable
 * PFFT_GB300_PAIR=0 turns that off for the process. */
int pfft_gb300_set_fx_link(int on);

/* Autotuning and wisdom.  Plans created with PFFT_PATIENT, PFFT_EXHAUSTIVE
 * or PFFT_TUNE time the candidate configurations of every pass (radix-8
 * kernel tile height; general kernel radix order and lines per CTA) on the
 * planned arrays - overwriting the output array (and an in-place array), as
 * FFTW's measuring planners do - and keep the fastest.  The choices are kept
 * as wisdom, keyed by a complete description of the pass, and reused by any
 * later plan with the same pass.  No counterpart in the reference's API (PFFT
 * leaves wisdom to FFTW).  Import/export return 1 on success, 0 on failure;
 * the exported string is released with free(). */
char *pfft_gb300_export_wisdom_to_string(void);
int pfft_gb300_import_wisdom_from_string(const char *wisdom);
int pfft_gb300_export_wisdom_to_filename(const char *filename);
int pfft_gb300_import_wisdom_from_filename(const char *filename);
void pfft_gb300_forget_wisdom(void);
int pfft_gb300_wisdom_entries(void);

/* Kernel selection: 1 (default) runs power-of-two c2c passes on the
 * register-resident radix-8 kernel, 0 uses the general pass kernel everywhere
 * (also set by the environment variable PFFT_GB300_KERNEL=generic). */
void pfft_gb300_set_kernel_path(int path);
int pfft_gb300_get_kernel_path(void);

/* Staged variant of the radix-8 kernel for plain c2c passes: persistent CTAs
 * whose next tile is copied global -> shared memory by the copy engine
 * (bulk / tensor-map copies on an mbarrier) while the current tile is
 * transformed.  1 (default): per pass, as the autotuner or wisdom chose, else
 * on for float column passes; 2: wherever the pass layout allows; 0: off
 * (also PFFT_GB300_STAGED=0/1/2).  staged_launches counts its launches in
 * this process.  staged_status waits for the device, returns 1 if a staged
 * load wait expired since the last call (the results of that execute are
 * wrong), 0 if not, or a negative cudaError_t value, and clears the flag.
 * No counterpart in the reference's API. */
void pfft_gb300_set_staged(int mode);
int pfft_gb300_get_staged(void);
long long pfft_gb300_staged_launches(void);
int pfft_gb300_staged_status(void);

/* Ghost-cell exchange that allocates nothing.  No counterpart in the
 * reference PFFT.  For callers that cannot allocate device memory when they
 * need the halo (solver loops that pre-size every buffer, memory-pool budgets,
 * code that must not let cudaMalloc/cudaFree synchronise the device):
 * the same periodic-wrap exchange as a ghost-cell plan's pfft_exchange, for a
 * 3-D block of n[0] x n[1] x n[2] cells with `tuple` reals per cell (1 for
 * real data, 2 for complex, times howmany) stored at the start of `data`,
 * expanded in place into the (gc_below + n + gc_above) box.  precision: 1 =
 * double, 0 = float.  `data` must be managed memory or device memory of the
 * current device (another GPU's pointer: cudaErrorInvalidDevice, host
 * memory: cudaErrorInvalidValue); `stream` is a cudaStream_t (NULL: the
 * legacy default stream); the call only queues work.
 * Scratch: a fixed 32 MiB array in the library's device image (every GPU that
 * loads this code holds it until exit); blocks larger than 32 MiB are refused
 * (cudaErrorMemoryAllocation returned, nothing queued), and so are sizes
 * whose products overflow.  The first call on a device looks up the array's
 * device address and the SM count; make that first call before any stream
 * capture.  After cudaDeviceReset, call pfft_cleanup() so that the next call
 * looks them up again.  All calls share the array: calls whose GPU work
 * overlaps (different streams, no ordering) race.  Returns 0 or a
 * cudaError_t value. */
int pfft_gb300_exchange_noalloc(int precision, const ptrdiff_t *n, const ptrdiff_t *gc_below,
                                const ptrdiff_t *gc_above, ptrdiff_t tuple, void *data, void *stream);

/* Last error (CUDA error code or library error) and its message. */
int pfft_gb300_last_error(void);
const char *pfft_gb300_last_error_string(void);
void pfft_gb300_clear_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PFFT_GB300_H */

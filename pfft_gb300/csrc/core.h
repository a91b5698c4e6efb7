// Internal declarations shared by the host-side translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "pass.h"

typedef ptrdiff_t INT;

namespace pg {

// ---- internal transform-type flags --------------------------------------
// Same meaning as the reference's PFFTI_TRAFO_* set (kernel/ipfft.h:138-165),
// own encoding: R2R is a single bit here; SKIP/PHANTOM/PADDED are modifiers.
enum : unsigned {
  TR_C2C = 1u << 0,
  TR_R2C = 1u << 1,
  TR_C2R = 1u << 2,
  TR_R2R = 1u << 3,
  TR_SKIP = 1u << 4,
  TR_PHANTOM = 1u << 5,
  TR_PADDED = 1u << 6,
  TR_RDFT = TR_R2C | TR_C2R,
};

// public flag bits (identical values to pfft.h)
enum : unsigned {
  F_TRANSPOSED_IN = 1u << 0,
  F_TRANSPOSED_OUT = 1u << 1,
  F_SHIFTED_IN = 1u << 2,
  F_SHIFTED_OUT = 1u << 3,
  F_ESTIMATE = 1u << 4,
  F_PATIENT = 1u << 5,
  F_EXHAUSTIVE = 1u << 6,
  F_TUNE = 1u << 7,
  F_PRESERVE_INPUT = 1u << 8,
  F_DESTROY_INPUT = 1u << 9,
  F_BUFFERED_INPLACE = 1u << 10,
  F_PADDED_R2C = 1u << 11,
};

enum : unsigned {
  GC_TRANSPOSED = 1u << 0,
  GC_SENDRECV = 1u << 1,
  GC_RMA = 1u << 2,
  GC_R2C = 1u << 3,
  GC_PADDED = 1u << 4,
};

// ---- errors ---------------------------------------------------------------
void set_error(int code, const std::string& msg);
void report(const char* fmt, ...);  // "PFFT ERROR: ..." to stderr + last error
int cuda_check(cudaError_t e, const char* what);
int last_error_code();
const char* last_error_string();
void clear_error();

// ---- single-rank communicator registry (mpi_shim.cpp) ----------------------
int comm_cart_dims(int comm);  // 0 = not Cartesian
bool comm_valid(int comm);

// ---- layout engine (layout.cpp) -------------------------------------------
struct SizeQuery {
  int rnk_n;
  const INT* n;
  const INT* ni;
  const INT* no;
  INT howmany;
  unsigned trafo;       // TR_* of the whole plan (R2C/C2R may carry TR_PADDED)
  unsigned pfft_flags;
  int cart_dims;        // dimension of the (Cartesian) communicator
};
// Local sizes and the number of elements to allocate, single rank.
INT local_size(const SizeQuery& q, INT* lni, INT* lis, INT* lno, INT* los);
// Effective mesh rank used for the transposed layouts (3-D on a 3-D mesh is
// remapped to a 2-D mesh first).
int effective_mesh_rank(int rnk_n, int cart_dims);

// ---- twiddle tables (twiddle.cpp) ----------------------------------------
const void* twiddle_table(int M, int arith, cudaError_t* err);
void twiddle_release_all();
// forget the allocation-free exchange's per-device set-up (gcell_noalloc.cu)
void noalloc_forget();

// ---- array layouts ------------------------------------------------------------
#define PG_MAX_DIMS 7
struct Layout {
  int d = 0;
  bool cplx = true;
  INT ext[PG_MAX_DIMS] = {0};     // stored extent per natural axis
  INT stride[PG_MAX_DIMS] = {0};  // element stride per natural axis
  INT hm = 1, hm_stride = 1;
  INT span = 0;                   // elements covered (max offset + 1)
};
// compact layout with axes in the given memory order (outermost first)
Layout compact_layout(int d, const INT* ext, const int* order, INT hm, bool cplx);

// ---- plans ---------------------------------------------------------------------
enum BufId { BUF_IN = 0, BUF_OUT = 1, BUF_WSA = 2, BUF_WSB = 3 };

struct Pass {
  PassParams p;
  int src = BUF_IN, dst = BUF_OUT;
  int axis = 0;
  double bytes = 0;  // algorithmic bytes moved (read + write)
};

struct PassProgram {
  std::vector<Pass> passes;
  size_t ws_bytes[2] = {0, 0};
  Layout in_layout, out_layout;
};

struct PlanDesc {
  int prec = 1;  // 0 float, 1 double
  int rnk_n = 0;
  std::vector<INT> n, ni, no;
  INT howmany = 1;
  unsigned trafo = TR_C2C;  // TR_C2C / TR_R2C / TR_C2R / TR_R2R (+TR_PADDED)
  int sign = -1;
  std::vector<int> kinds;
  std::vector<int> skip;
  unsigned pfft_flags = 0;
  int cart_dims = 2;
  int mesh_rank = 2;       // effective
  bool mesh3d = false;     // 3-D data on a 3-D mesh (real rows unpadded)
  std::vector<INT> local_ni, local_i_start, local_no, local_o_start;
  INT alloc_local = 0;
};

struct TimerData {
  int rnk_pm = 2;
  int iter = 0;
  double whole = 0;
  std::vector<double> trafo, remap;
  double remap_3dto2d[2] = {0, 0};
  double itwiddle = 0, otwiddle = 0;
};

constexpr int PIPE_CHUNKS = 8;  // slabs of the host-array pipeline

struct Plan {
  PlanDesc d;
  int arith = ARITH_DF;
  int quant = 0;        // float-float: block-quantised radix-8 stages (PassParams::quant)
  void* in = nullptr;   // planned arrays
  void* out = nullptr;
  bool inplace = false;
  // PFFT_BUFFERED_INPLACE on an out-of-place plan: the transform runs as an
  // in-place program on the input array (results end up in it); the output
  // array is never written (plan.cpp, make_plan)
  bool buffered = false;
  PassProgram fwd;      // the transform
  PassProgram adj;      // its adjoint (built on demand)
  bool adj_built = false;
  void* ws[2] = {nullptr, nullptr};
  size_t ws_cap[2] = {0, 0};
  void* stage[2] = {nullptr, nullptr};  // device staging for host arrays
  size_t stage_cap[2] = {0, 0};
  cudaStream_t stream = 0;
  bool sync = true;
  bool use_graph = false;
  cudaGraphExec_t graph = nullptr;
  void* graph_in = nullptr;
  void* graph_out = nullptr;
  int graph_dir = 0;
  TimerData timer;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // host-array pipeline (plan.cpp): copy streams and chunk events, made on first use
  cudaStream_t pipe_s[2] = {nullptr, nullptr};
  cudaEvent_t pipe_ev[2][PIPE_CHUNKS] = {};
  cudaEvent_t pipe_done = nullptr;
  bool pipeline = true;  // pipelined staging of host arrays where the program allows it
  // per-line exponent arrays of the FX links of the forward and adjoint
  // programs (plan.cpp, link_fx; one per linked pass boundary)
  std::vector<int*> lexp[2];
  // optional per-pass timing with CUDA events on the plan stream
  bool time_passes = false;
  std::vector<cudaEvent_t> pev;
  std::vector<double> pass_ms;
  int timed_runs = 0;
};

// Build the pass program of a plan (planner.cpp).  Returns false on failure
// (message recorded with set_error).
bool build_program(const PlanDesc& d, int arith, bool inplace, bool adjoint, PassProgram* prog);
// Wisdom and autotuning (tune.cpp): apply recorded choices to a program;
// time the candidates of every pass on the plan's arrays and record the best.
void apply_wisdom(PassProgram* prog, int arith);
bool tune_program(Plan* pl, PassProgram* prog);
// Re-plan the general kernel of a pass (radix order, lines per CTA).
bool refit_pass(PassParams* p, int arith, int pref, int L);
// Re-fit a general pass to at most max_threads threads and max_smem bytes of
// shared memory, halving its lines per CTA from p->L (batched launches).
bool fit_pass_threads(PassParams* p, int arith, int max_threads, int max_smem);
// Run a program with resolved buffers.  Returns a cudaError_t value.
int run_program(Plan* pl, const PassProgram& prog, void* in, void* out, cudaStream_t s);
// Ensure workspace capacity for a program.
bool ensure_workspace(Plan* pl, const PassProgram& prog);

// planner entry used by the C API (plan.cpp)
Plan* make_plan(const PlanDesc& base, void* in, void* out);
void execute_plan(Plan* pl, void* in, void* out, bool adjoint);
void destroy_plan(Plan* pl);

// arithmetic policy of the double API (plan.cpp, plan_double_arith): the
// default keeps FFTW-class answers (64-bit fixed point on the radix-8 passes,
// FP64 elsewhere); native FP64 everywhere; or the opt-in float-float forms
enum { DARITH_DF = 0, DARITH_NATIVE = 1, DARITH_AUTO = 2, DARITH_DFQ = 3 };
int double_arith();
void set_double_arith(int a);
int plan_double_arith(const PlanDesc& d);
long long pipelined_executes();  // executes through the host-array pipeline (plan.cpp)
// FX mantissas kept between radix-8 passes of new double plans (plan.cpp):
// on by default, PFFT_GB300_FX_LINK=0 or set_fx_link(0) turns it off
int fx_link();
void set_fx_link(int v);
void unlink_fx(PassProgram* prog, std::vector<int*>* lexp);

}  // namespace pg

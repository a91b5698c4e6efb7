// Plan objects: creation, execution (device or host arrays), destruction.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <mutex>
#include <string>
#include "core.h"

namespace pg {

// ---- errors ------------------------------------------------------------------
static std::mutex g_err_mu;
static int g_err_code = 0;
static std::string g_err_msg;

void set_error(int code, const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err_code = code;
  g_err_msg = msg;
}

void report(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  fprintf(stderr, "PFFT ERROR: %s\n", buf);
  set_error(-1, buf);
}

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  fprintf(stderr, "PFFT ERROR: %s\n", buf);
  set_error((int)e, buf);
  return (int)e;
}

int last_error_code() {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_err_code;
}
const char* last_error_string() {
  std::lock_guard<std::mutex> lk(g_err_mu);
  static thread_local std::string copy;
  copy = g_err_msg;
  return copy.c_str();
}
void clear_error() {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err_code = 0;
  g_err_msg.clear();
}

static int g_double_arith = -1;
int double_arith() {
  if (g_double_arith < 0) {
    const char* e = getenv("PFFT_GB300_F64_ARITH");
    g_double_arith = (e && strcmp(e, "native") == 0) ? DARITH_NATIVE
                     : (e && strcmp(e, "df") == 0)   ? DARITH_DF
                     : (e && strcmp(e, "dfq") == 0)  ? DARITH_DFQ
                                                     : DARITH_AUTO;
  }
  return g_double_arith;
}
void set_double_arith(int a) { g_double_arith = a; }

// Arithmetic of one double-precision plan.  Native FP64 issues at about 1/64
// of the FP32 rate on this part, so large transforms run in float-float; a
// transform of at most DARITH_AUTO_POINTS points costs no more than a launch
// latency in FP64 and keeps full double rounding.  (Whether the float-float
// radix-8 stages are block-quantised is Plan::quant, set with the arithmetic.)
int plan_double_arith(const PlanDesc& d) {
  const int m = double_arith();
  if (m == DARITH_NATIVE) return ARITH_F64;
  if (m == DARITH_DF || m == DARITH_DFQ) return ARITH_DF;
  double pts = (double)d.howmany;
  for (int t = 0; t < d.rnk_n; t++) pts *= (double)d.n[t];
  return pts <= (double)DARITH_AUTO_POINTS ? ARITH_F64 : ARITH_DF;
}

// Block-quantised float-float butterflies (fft_fast.cuh / fft_mixed.cuh, FQ)
// for the plain c2c passes of a float-float plan: the double-arithmetic
// modes DARITH_DFQ and DARITH_AUTO (above DARITH_AUTO_POINTS); DARITH_DF
// keeps TwoSum additions everywhere.
static void mark_quant(const Plan* pl, PassProgram* prog) {
  for (Pass& ps : prog->passes) ps.p.quant = pl->quant;
}

// ---- plans -------------------------------------------------------------------
bool ensure_workspace(Plan* pl, const PassProgram& prog) {
  for (int k = 0; k < 2; k++) {
    if (prog.ws_bytes[k] > pl->ws_cap[k]) {
      if (pl->ws[k]) cudaFree(pl->ws[k]);
      pl->ws[k] = nullptr;
      pl->ws_cap[k] = 0;
      if (cuda_check(cudaMalloc(&pl->ws[k], prog.ws_bytes[k]), "workspace allocation")) return false;
      pl->ws_cap[k] = prog.ws_bytes[k];
    }
  }
  return true;
}

int run_program(Plan* pl, const PassProgram& prog, void* in, void* out, cudaStream_t s) {
  void* bufs[4] = {in, out, pl->ws[0], pl->ws[1]};
  const bool timing = pl->time_passes && &prog == &pl->fwd;
  const size_t np = prog.passes.size();
  if (timing && pl->pev.size() < np + 1) {
    for (auto e : pl->pev) cudaEventDestroy(e);
    pl->pev.assign(np + 1, nullptr);
    for (auto& e : pl->pev)
      if (cudaEventCreate(&e) != cudaSuccess) return (int)cudaGetLastError();
    pl->pass_ms.assign(np, 0.0);
  }
  if (timing) cudaEventRecord(pl->pev[0], s);
  for (size_t i = 0; i < np; i++) {
    const Pass& ps = prog.passes[i];
    PassParams p = ps.p;
    p.src = bufs[ps.src];
    p.dst = bufs[ps.dst];
    cudaError_t e;
    p.tw = twiddle_table(p.M, pl->arith, &e);
    if (!p.tw) return (int)e;
    int rc = launch_pass(p, pl->arith, s);
    if (rc) return rc;
    if (timing) cudaEventRecord(pl->pev[i + 1], s);
  }
  return 0;
}

// accumulate the per-pass event times of the last run (after a synchronize)
static void collect_pass_times(Plan* pl) {
  if (!pl->time_passes || pl->pev.empty()) return;
  for (size_t i = 0; i + 1 < pl->pev.size() && i < pl->pass_ms.size(); i++) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, pl->pev[i], pl->pev[i + 1]) == cudaSuccess) {
      pl->pass_ms[i] += ms;
      if (i < pl->timer.trafo.size()) pl->timer.trafo[i] += 1e-3 * ms;
    }
  }
  pl->timed_runs++;
}

Plan* make_plan(const PlanDesc& base, void* in, void* out) {
  Plan* pl = new Plan();
  pl->d = base;
  pl->arith = base.prec == 0 ? ARITH_F32 : plan_double_arith(base);
  pl->quant = (pl->arith == ARITH_DF && (double_arith() == DARITH_DFQ || double_arith() == DARITH_AUTO)) ? 1 : 0;
  pl->in = in;
  pl->out = out;
  pl->inplace = (in == out) && in != nullptr;
  if (!build_program(pl->d, pl->arith, pl->inplace, false, &pl->fwd)) {
    delete pl;
    return nullptr;
  }
  mark_quant(pl, &pl->fwd);
  if (!ensure_workspace(pl, pl->fwd)) {
    destroy_plan(pl);
    return nullptr;
  }
  apply_wisdom(&pl->fwd, pl->arith);
  if ((base.pfft_flags & (F_PATIENT | F_EXHAUSTIVE | F_TUNE)) && !tune_program(pl, &pl->fwd)) {
    destroy_plan(pl);
    return nullptr;
  }
  // pre-build twiddle tables so that execution allocates nothing
  for (const Pass& ps : pl->fwd.passes) {
    cudaError_t e;
    bool ok = twiddle_table(ps.p.M, pl->arith, &e) && twiddle_table(ps.p.N, pl->arith, &e);
    if (ok && pl->arith != ARITH_F64) fast_pass_tables(ps.p, pl->arith);  // radix-8 / mixed-radix tables
    if (!ok) {
      cuda_check(e, "twiddle table");
      destroy_plan(pl);
      return nullptr;
    }
  }
  pl->timer.rnk_pm = base.mesh_rank;
  pl->timer.trafo.assign(2 * base.mesh_rank + 2, 0.0);
  pl->timer.remap.assign(2 * base.mesh_rank, 0.0);
  return pl;
}

void destroy_plan(Plan* pl) {
  if (!pl) return;
  for (int k = 0; k < 2; k++) {
    if (pl->ws[k]) cudaFree(pl->ws[k]);
    if (pl->stage[k]) cudaFree(pl->stage[k]);
  }
  if (pl->graph) cudaGraphExecDestroy(pl->graph);
  for (int k = 0; k < 2; k++)
    if (pl->ev[k]) cudaEventDestroy(pl->ev[k]);
  for (auto e : pl->pev) cudaEventDestroy(e);
  delete pl;
}

// true if the GPU can dereference p directly
static bool device_accessible(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static bool ensure_stage(Plan* pl, int k, size_t bytes) {
  if (bytes <= pl->stage_cap[k]) return true;
  if (pl->stage[k]) cudaFree(pl->stage[k]);
  pl->stage[k] = nullptr;
  pl->stage_cap[k] = 0;
  if (cuda_check(cudaMalloc(&pl->stage[k], bytes), "staging allocation")) return false;
  pl->stage_cap[k] = bytes;
  return true;
}

static size_t layout_bytes(const Layout& L, int arith) {
  int e = L.cplx ? (arith == ARITH_F32 ? 8 : 16) : (arith == ARITH_F32 ? 4 : 8);
  return (size_t)L.span * e;
}

void execute_plan(Plan* pl, void* in, void* out, bool adjoint) {
  auto t0 = std::chrono::steady_clock::now();
  if (adjoint && !pl->adj_built) {
    if (!build_program(pl->d, pl->arith, pl->inplace, true, &pl->adj)) {
      report("adjoint not available for this plan");
      return;
    }
    mark_quant(pl, &pl->adj);
    if (!ensure_workspace(pl, pl->adj)) return;
    apply_wisdom(&pl->adj, pl->arith);
    if ((pl->d.pfft_flags & (F_PATIENT | F_EXHAUSTIVE | F_TUNE)) && !tune_program(pl, &pl->adj)) return;
    pl->adj_built = true;
  }
  const PassProgram& prog = adjoint ? pl->adj : pl->fwd;
  if ((in == out) != pl->inplace) {
    report("execute: in-place / out-of-place mismatch with the planned arrays");
    return;
  }
  cudaStream_t s = pl->stream;
  size_t bin = layout_bytes(prog.in_layout, pl->arith);
  size_t bout = layout_bytes(prog.out_layout, pl->arith);
  bool din = device_accessible(in), dout = device_accessible(out);
  void* xin = in;
  void* xout = out;
  if (!din || !dout) {
    // host arrays: stage through device buffers (copies are stream ordered)
    if (!din) {
      // an in-place host array also receives the output (and may hold
      // intermediates up to the larger of the two layouts)
      if (!ensure_stage(pl, 0, (pl->inplace && !dout) ? std::max(bin, bout) : bin)) return;
      xin = pl->stage[0];
      if (cuda_check(cudaMemcpyAsync(xin, in, bin, cudaMemcpyHostToDevice, s), "host-to-device copy")) return;
    }
    if (!dout) {
      if (pl->inplace && !din) {
        xout = xin;
      } else {
        if (!ensure_stage(pl, 1, bout)) return;
        xout = pl->stage[1];
      }
    }
  }
  int rc = 0;
  if (pl->use_graph && din && dout) {
    int dir = adjoint ? 2 : 1;
    if (!pl->graph || pl->graph_in != xin || pl->graph_out != xout || pl->graph_dir != dir) {
      if (pl->graph) cudaGraphExecDestroy(pl->graph);
      pl->graph = nullptr;
      cudaGraph_t g;
      cudaStream_t cs;
      if (cuda_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "graph stream")) return;
      cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      rc = run_program(pl, prog, xin, xout, cs);
      cudaError_t ce = cudaStreamEndCapture(cs, &g);
      cudaStreamDestroy(cs);
      if (rc || ce != cudaSuccess) {
        cuda_check(rc ? (cudaError_t)rc : ce, "graph capture");
        return;
      }
      ce = cudaGraphInstantiate(&pl->graph, g, 0);
      cudaGraphDestroy(g);
      if (cuda_check(ce, "graph instantiate")) return;
      pl->graph_in = xin;
      pl->graph_out = xout;
      pl->graph_dir = dir;
    }
    rc = (int)cudaGraphLaunch(pl->graph, s);
  } else {
    rc = run_program(pl, prog, xin, xout, s);
  }
  if (rc) {
    cuda_check((cudaError_t)rc, "pass launch");
    return;
  }
  if (xout != out) {
    if (cuda_check(cudaMemcpyAsync(out, xout, bout, cudaMemcpyDeviceToHost, s), "device-to-host copy")) return;
  }
  if (pl->sync || xout != out || xin != in) {
    if (cuda_check(cudaStreamSynchronize(s), "execute")) return;
    auto t1 = std::chrono::steady_clock::now();
    pl->timer.whole += std::chrono::duration<double>(t1 - t0).count();
    if (!adjoint && !(pl->use_graph && din && dout)) collect_pass_times(pl);
  }
  pl->timer.iter++;
}

}  // namespace pg

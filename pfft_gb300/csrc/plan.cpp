// Plan objects: creation, execution (device or host arrays), destruction.
#include <atomic>
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

// Arithmetic of one double-precision plan.  The default (DARITH_AUTO) keeps
// FFTW-class double answers: FP64 storage, the radix-8 kernel's 64-bit
// fixed-point arithmetic on the power-of-two c2c passes (58 bits against the
// tile's largest value, PassParams::quant = 2) and native FP64 on every other
// pass.  DARITH_NATIVE runs every pass in FP64 on the general kernel.  The
// float-float arithmetics (DARITH_DF TwoSum, DARITH_DFQ block-quantised
// radix-8 butterflies) carry 48-49 bits and are opt-in: faster on this part,
// whose FP64 pipe issues at about 1/70 of the FP32 rate, but narrower than
// the reference's FFTW double.
int plan_double_arith(const PlanDesc&) {
  const int m = double_arith();
  return (m == DARITH_DF || m == DARITH_DFQ) ? ARITH_DF : ARITH_F64;
}

// PassParams::quant of every pass of a plan: 2 = 64-bit fixed point on the
// radix-8 passes of a default double plan, 1 = block-quantised float-float
// butterflies (DARITH_DFQ), 0 otherwise.
static int plan_quant(const Plan* pl) {
  if (pl->arith == ARITH_F64) return double_arith() == DARITH_AUTO ? 2 : 0;
  if (pl->arith == ARITH_DF) return double_arith() == DARITH_DFQ ? 1 : 0;
  return 0;
}
static void mark_quant(const Plan* pl, PassProgram* prog) {
  for (Pass& ps : prog->passes) ps.p.quant = pl->quant;
}

// Default double plans: r2c, c2r, REDFT10 and REDFT01 passes on the radix-8
// kernel whose batch dimension 0 has an even extent transform two real lines
// per complex line (PassParams::pair; fast_args applies it).  A paired pass
// keeps double output (no FX link out of it).
static int g_pair = -1;  // PFFT_GB300_PAIR=0 turns the pairing off (comparisons)
static void mark_pair(const Plan* pl, PassProgram* prog) {
  if (g_pair < 0) {
    const char* e = getenv("PFFT_GB300_PAIR");
    g_pair = (e && strcmp(e, "0") == 0) ? 0 : 1;
  }
  for (Pass& ps : prog->passes) {
    PassParams& p = ps.p;
    p.pair = 0;
    if (!g_pair || pl->arith != ARITH_F64 || p.quant != 2) continue;
    if (p.mode != MODE_R2C && p.mode != MODE_C2R && p.mode != MODE_RE10 && p.mode != MODE_RE01) continue;
    if (p.nb < 1 || p.bext[0] % 2) continue;
    if (!fast_pass_eligible(p, pl->arith)) continue;
    p.pair = 1;
  }
}

// FX mantissas kept between two consecutive radix-8 passes of a default
// double plan (PassParams::fx_out / fx_in): the first pass stores its int64
// mantissas and one exponent per line, the second reads them and aligns each
// element to its tile's grid, so neither converts to or from double.  The
// second pass must be a plain c2c pass, the first any radix-8 pass with a
// complex output; the second pass's input dimensions are matched to the first
// pass's output dimensions by stride and extent, which gives the previous
// pass's line index of each element (PassParams::gin_np, gin_pext, gin_pcoef, gin_k).
static int g_fx_link = -1;
int fx_link() {
  if (g_fx_link < 0) {
    const char* e = getenv("PFFT_GB300_FX_LINK");
    g_fx_link = (e && strcmp(e, "0") == 0) ? 0 : 1;
  }
  return g_fx_link;
}
void set_fx_link(int v) { g_fx_link = v ? 1 : 0; }

void unlink_fx(PassProgram* prog, std::vector<int*>* lexp) {
  for (int* q : *lexp)
    if (q) cudaFree(q);
  lexp->clear();
  for (Pass& ps : prog->passes) {
    PassParams& p = ps.p;
    p.fx_in = p.fx_out = 0;
    p.lexp_in = nullptr;
    p.lexp_out = nullptr;
    p.lexp_in_n = 0;
    for (int b = 0; b < PG_MAX_BATCH; b++) p.gin_np[b] = 0, p.gin_bofs[b] = 0;
    for (int q = 0; q < 2 * PG_MAX_BATCH; q++) p.gin_pext[q] = 1, p.gin_pcoef[q] = 0;
    p.gin_k = p.gout_off = 0;
  }
}

static bool link_fx(Plan* pl, PassProgram* prog, std::vector<int*>* lexp) {
  unlink_fx(prog, lexp);
  const int P = (int)prog->passes.size();
  if (pl->arith != ARITH_F64 || pl->quant != 2 || !fx_link() || P < 2) return true;
  lexp->assign(P, nullptr);
  for (int i = 0; i + 1 < P; i++) {
    PassParams& a = prog->passes[i].p;
    PassParams& b = prog->passes[i + 1].p;
    const bool b_plain = b.mode == MODE_C2C && b.Zi == 0 && b.Ni == b.N && b.Zo == 0 && b.No == b.N && !b.wmode;
    if (!b_plain || (a.mode != MODE_C2C && a.mode != MODE_R2C) || a.pair) continue;
    if ((a.N & (a.N - 1)) || (b.N & (b.N - 1))) continue;  // the radix-8 kernel on both sides
    if (!fast_pass_eligible(a, pl->arith) || !fast_pass_eligible(b, pl->arith)) continue;
    // b's input dimensions onto a's output dimensions.  Both passes' planner
    // merged dimensions contiguous on both of their sides, so one of b's
    // dimensions may cross several of a's, or lie inside one: it is cut into
    // pieces at a's dimension boundaries (walking its strides upward), each
    // piece contributing its coordinate times a's line-index weight for it
    // (0 inside a's axis).
    struct ADim {
      long long s, e, w;  // stride, extent, line-index weight per unit of coordinate
    };
    std::vector<ADim> ad;
    long long Mj = 1;
    for (int j = 0; j < a.nb; j++) {
      ad.push_back({a.bsO[j], a.bext[j], Mj});
      Mj *= a.bext[j];
    }
    ad.push_back({a.sOa, a.No, 0});
    bool ok = true;
    std::vector<long long> pe, pc;  // pieces of the current dimension
    auto pieces = [&](long long ext, long long stride) {
      pe.clear();
      pc.clear();
      long long cur = stride, rem = ext;
      while (rem > 1 && ok) {
        const ADim* hit = nullptr;
        for (const ADim& x : ad)
          if (x.s > 0 && x.e > 1 && cur % x.s == 0 && cur / x.s < x.e) hit = &x;
        if (!hit) {
          ok = false;
          break;
        }
        const long long m = cur / hit->s;            // position inside a's dimension
        if (hit->e % m) ok = false;
        const long long room = hit->e / m;           // extent left in a's dimension
        const long long p = std::min(rem, room);
        if (rem % p || (p < rem && p != room)) ok = false;
        pe.push_back(p);
        pc.push_back(hit->w * m);
        cur *= p;
        rem /= p;
      }
    };
    int np[PG_MAX_BATCH] = {0};
    long long pext[2 * PG_MAX_BATCH], pcoef[2 * PG_MAX_BATCH];
    int npc = 0;
    for (int d = 0; d < b.nb && ok; d++) {
      pieces(b.bext[d], b.bsI[d]);
      if (npc + (int)pe.size() > 2 * PG_MAX_BATCH) ok = false;
      for (size_t q = 0; ok && q < pe.size(); q++, npc++) {
        pext[npc] = pe[q];
        pcoef[npc] = pc[q];
      }
      np[d] = (int)pe.size();
    }
    long long gk = 0;
    if (ok) {
      pieces(b.N, b.sIa);  // the axis: one piece (a per-element coefficient)
      if (pe.size() > 1) ok = false;
      if (pe.size() == 1) gk = pc[0];
    }
    if (!ok) continue;
    int* q = nullptr;
    if (cuda_check(cudaMalloc(&q, sizeof(int) * (size_t)a.nlines), "line exponents")) return false;
    (*lexp)[i] = q;
    a.fx_out = 1;
    a.lexp_out = q;
    b.fx_in = 1;
    b.lexp_in = q;
    b.lexp_in_n = a.nlines;
    for (int d = 0; d < PG_MAX_BATCH; d++) b.gin_np[d] = d < b.nb ? np[d] : 0;
    for (int x = 0; x < npc; x++) {
      b.gin_pext[x] = pext[x];
      b.gin_pcoef[x] = pcoef[x];
    }
    b.gin_k = gk;
  }
  return true;
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
  pl->quant = plan_quant(pl);
  // PFFT_BUFFERED_INPLACE (api/pfft.h:542; doc/tutorial.tex, "Preserving
  // input data"): an out-of-place plan whose inputs and outputs are both
  // stored in the input array, the output array being scratch.  Here the
  // program is planned in place on the input array (plan-owned workspaces
  // where a pass cannot run in place), so the output array is not touched.
  // PFFT_PRESERVE_INPUT is what every out-of-place plan does anyway (no pass
  // writes the input array), and PFFT_DESTROY_INPUT only permits
  // overwriting it, which no program needs.
  pl->buffered = (base.pfft_flags & F_BUFFERED_INPLACE) && in != out && in != nullptr;
  pl->in = in;
  pl->out = pl->buffered ? in : out;
  pl->inplace = (pl->in == pl->out) && in != nullptr;
  if (!build_program(pl->d, pl->arith, pl->inplace, false, &pl->fwd)) {
    delete pl;
    return nullptr;
  }
  mark_quant(pl, &pl->fwd);
  mark_pair(pl, &pl->fwd);
  if (!ensure_workspace(pl, pl->fwd)) {
    destroy_plan(pl);
    return nullptr;
  }
  apply_wisdom(&pl->fwd, pl->arith);
  if ((base.pfft_flags & (F_PATIENT | F_EXHAUSTIVE | F_TUNE)) && !tune_program(pl, &pl->fwd)) {
    destroy_plan(pl);
    return nullptr;
  }
  if (!link_fx(pl, &pl->fwd, &pl->lexp[0])) {
    destroy_plan(pl);
    return nullptr;
  }
  // pre-build twiddle tables so that execution allocates nothing
  for (const Pass& ps : pl->fwd.passes) {
    cudaError_t e;
    bool ok = twiddle_table(ps.p.M, pl->arith, &e) && twiddle_table(ps.p.N, pl->arith, &e);
    if (ok && (pl->arith != ARITH_F64 || pl->quant == 2)) fast_pass_tables(ps.p, pl->arith);  // radix-8 / mixed-radix tables
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
  for (int k = 0; k < 2; k++) {
    if (pl->pipe_s[k]) cudaStreamDestroy(pl->pipe_s[k]);
    for (int c = 0; c < PIPE_CHUNKS; c++)
      if (pl->pipe_ev[k][c]) cudaEventDestroy(pl->pipe_ev[k][c]);
  }
  if (pl->pipe_done) cudaEventDestroy(pl->pipe_done);
  unlink_fx(&pl->fwd, &pl->lexp[0]);
  unlink_fx(&pl->adj, &pl->lexp[1]);
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

// ---- host-array pipeline ------------------------------------------------------
// Out-of-place executes on host arrays stage both arrays through device
// buffers.  When the leading passes are c2c passes whose slowest batch
// dimension cuts the data into PIPE_CHUNKS slabs that no line crosses (and
// consecutive passes agree on the slab size), the input is copied slab by
// slab on a copy stream and those passes run on each slab as it arrives; when
// the last pass is a c2c pass with one dense batch dimension (lines at a
// stride of at least the batch extent), it runs in PIPE_CHUNKS column chunks,
// each copied back to the host as a pitched 2-D copy on a second copy stream
// while the next chunk is computed.  Other programs stage whole arrays.

static int pass_esz(const PassParams& p, int arith, bool in) {
  const bool c = in ? (p.mode == MODE_C2C || p.mode == MODE_C2R) : (p.mode == MODE_C2C || p.mode == MODE_R2C);
  return c ? (arith == ARITH_F32 ? 8 : 16) : (arith == ARITH_F32 ? 4 : 8);
}

// Bytes of one of C slabs of a c2c pass's input (side 0) or output (side 1)
// along its slowest batch dimension, or 0 when that does not cut the array
// into slabs (the lines of one slab would reach into the next).
static long long slab_bytes(const PassParams& p, int arith, int side, int C) {
  if (p.mode != MODE_C2C || p.nb < 1 || p.nst == 0) return 0;
  const int b = p.nb - 1;
  if (p.bext[b] % C) return 0;
  const long long* bs = side ? p.bsO : p.bsI;
  const long long sa = side ? p.sOa : p.sIa;
  const long long n = side ? p.No : p.Ni;
  if (sa <= 0 || bs[b] <= 0) return 0;
  long long inner = (n - 1) * sa + 1;
  for (int q = 0; q < b; q++) {
    if (bs[q] <= 0) return 0;
    inner += (p.bext[q] - 1) * bs[q];
  }
  if (inner > bs[b]) return 0;
  return (p.bext[b] / C) * bs[b] * pass_esz(p, arith, side == 0);
}

// the lines of chunk k of C along the slowest batch dimension
static PassParams chunk_of(const PassParams& p, int arith, int k, int C) {
  PassParams q = p;
  const int b = p.nb - 1;
  const long long w = p.bext[b] / C, a = (long long)k * w;
  q.bext[b] = w;
  q.nlines = p.nlines / C;
  q.src = (const char*)p.src + a * p.bsI[b] * pass_esz(p, arith, true);
  q.dst = (char*)p.dst + a * p.bsO[b] * pass_esz(p, arith, false);
  q.bshI[b].start += (int)a;
  q.bshO[b].start += (int)a;
  // FX line indices of the slab: its coordinates along b start at a, its
  // lines are global lines k * nlines/C on
  q.gin_bofs[b] = p.gin_bofs[b] + a;
  q.gout_off = p.gout_off + (long long)k * q.nlines;
  return q;
}

static int launch_prog_pass(Plan* pl, const Pass& ps, PassParams p, cudaStream_t s) {
  cudaError_t e;
  p.tw = twiddle_table(p.M, pl->arith, &e);
  if (!p.tw) return (int)e;
  return launch_pass(p, pl->arith, s);
}

static std::atomic<long long> g_pipelined{0};
long long pipelined_executes() { return g_pipelined.load(); }

// 1: executed through the pipeline, 0: not applicable (nothing done), -1: error (reported)
static int run_pipelined(Plan* pl, const PassProgram& prog, void* in, void* out, cudaStream_t s, size_t bin,
                         size_t bout) {
  const int C = PIPE_CHUNKS;
  const int P = (int)prog.passes.size();
  if (P < 2 || pl->inplace) return 0;
  // leading slab passes
  const long long s0 = slab_bytes(prog.passes[0].p, pl->arith, 0, C);
  if (s0 < (8LL << 20) || prog.passes[0].src != BUF_IN) return 0;
  int lead = 0;
  while (lead < P - 1) {
    const PassParams& p = prog.passes[lead].p;
    const long long so = slab_bytes(p, pl->arith, 1, C);
    if (!so) break;
    if (lead > 0 && slab_bytes(p, pl->arith, 0, C) != slab_bytes(prog.passes[lead - 1].p, pl->arith, 1, C)) break;
    lead++;
  }
  if (lead == 0) return 0;
  // last pass in column chunks
  const PassParams& pz = prog.passes[P - 1].p;
  const bool tail = pz.mode == MODE_C2C && pz.nb == 1 && pz.bsO[0] == 1 && pz.sOa >= pz.bext[0] &&
                    pz.bext[0] % C == 0 && pz.nst > 0 && prog.passes[P - 1].dst == BUF_OUT && lead < P - 1;
  if (!ensure_stage(pl, 0, bin) || !ensure_stage(pl, 1, bout)) return -1;
  for (int k = 0; k < 2; k++) {
    if (!pl->pipe_s[k] && cuda_check(cudaStreamCreateWithFlags(&pl->pipe_s[k], cudaStreamNonBlocking), "copy stream"))
      return -1;
    for (int c = 0; c < C; c++)
      if (!pl->pipe_ev[k][c] &&
          cuda_check(cudaEventCreateWithFlags(&pl->pipe_ev[k][c], cudaEventDisableTiming), "pipeline event"))
        return -1;
  }
  if (!pl->pipe_done && cuda_check(cudaEventCreateWithFlags(&pl->pipe_done, cudaEventDisableTiming), "pipeline event"))
    return -1;
  void* bufs[4] = {pl->stage[0], pl->stage[1], pl->ws[0], pl->ws[1]};
  cudaStream_t ci = pl->pipe_s[0], co = pl->pipe_s[1];
  // the copy streams start after the work already queued on the plan stream
  if (cuda_check(cudaEventRecord(pl->pipe_done, s), "pipeline event") ||
      cuda_check(cudaStreamWaitEvent(ci, pl->pipe_done, 0), "pipeline wait"))
    return -1;
  for (int k = 0; k < C; k++) {
    const size_t off = (size_t)k * (size_t)s0;
    if (off < bin) {
      const size_t n = std::min((size_t)s0, bin - off);
      if (cuda_check(cudaMemcpyAsync((char*)bufs[0] + off, (const char*)in + off, n, cudaMemcpyHostToDevice, ci),
                     "host-to-device copy"))
        return -1;
    }
    if (cuda_check(cudaEventRecord(pl->pipe_ev[0][k], ci), "pipeline event")) return -1;
  }
  int rc = 0;
  for (int k = 0; k < C && !rc; k++) {
    if (cuda_check(cudaStreamWaitEvent(s, pl->pipe_ev[0][k], 0), "pipeline wait")) return -1;
    for (int i = 0; i < lead && !rc; i++) {
      const Pass& ps = prog.passes[i];
      PassParams p = ps.p;
      p.src = bufs[ps.src];
      p.dst = bufs[ps.dst];
      rc = launch_prog_pass(pl, ps, chunk_of(p, pl->arith, k, C), s);
    }
  }
  for (int i = lead; i < (tail ? P - 1 : P) && !rc; i++) {
    const Pass& ps = prog.passes[i];
    PassParams p = ps.p;
    p.src = bufs[ps.src];
    p.dst = bufs[ps.dst];
    rc = launch_prog_pass(pl, ps, p, s);
  }
  if (rc) {
    cuda_check((cudaError_t)rc, "pass launch");
    return -1;
  }
  if (tail) {
    const Pass& ps = prog.passes[P - 1];
    PassParams p = ps.p;
    p.src = bufs[ps.src];
    p.dst = bufs[ps.dst];
    const size_t esz = (size_t)pass_esz(p, pl->arith, false);
    const size_t w = (size_t)(p.bext[0] / C) * esz, pitch = (size_t)p.sOa * esz;
    for (int j = 0; j < C; j++) {
      PassParams q = p;
      q.bext[0] = p.bext[0] / C;
      q.nlines = p.nlines / C;
      q.dst = (char*)p.dst + (size_t)j * w;
      q.src = (const char*)p.src + (size_t)j * (size_t)(p.bext[0] / C) * (size_t)p.bsI[0] * pass_esz(p, pl->arith, true);
      q.bshI[0].start += (int)(j * (p.bext[0] / C));
      q.bshO[0].start += (int)(j * (p.bext[0] / C));
      q.gin_bofs[0] = p.gin_bofs[0] + (long long)j * (p.bext[0] / C);  // (the last pass stores doubles)
      rc = launch_prog_pass(pl, ps, q, s);
      if (rc) {
        cuda_check((cudaError_t)rc, "pass launch");
        return -1;
      }
      if (cuda_check(cudaEventRecord(pl->pipe_ev[1][j], s), "pipeline event") ||
          cuda_check(cudaStreamWaitEvent(co, pl->pipe_ev[1][j], 0), "pipeline wait") ||
          cuda_check(cudaMemcpy2DAsync((char*)out + (size_t)j * w, pitch, (const char*)bufs[1] + (size_t)j * w, pitch,
                                       w, (size_t)p.No, cudaMemcpyDeviceToHost, co),
                     "device-to-host copy"))
        return -1;
    }
    if (cuda_check(cudaEventRecord(pl->pipe_done, co), "pipeline event") ||
        cuda_check(cudaStreamWaitEvent(s, pl->pipe_done, 0), "pipeline wait"))
      return -1;
  } else {
    if (cuda_check(cudaMemcpyAsync(out, bufs[1], bout, cudaMemcpyDeviceToHost, s), "device-to-host copy")) return -1;
  }
  if (cuda_check(cudaStreamSynchronize(s), "execute")) return -1;
  g_pipelined++;
  return 1;
}

void execute_plan(Plan* pl, void* in, void* out, bool adjoint) {
  auto t0 = std::chrono::steady_clock::now();
  if (pl->buffered) out = in;  // PFFT_BUFFERED_INPLACE: results go back to the array read
  if (adjoint && !pl->adj_built) {
    if (!build_program(pl->d, pl->arith, pl->inplace, true, &pl->adj)) {
      report("adjoint not available for this plan");
      return;
    }
    mark_quant(pl, &pl->adj);
    mark_pair(pl, &pl->adj);
    if (!ensure_workspace(pl, pl->adj)) return;
    apply_wisdom(&pl->adj, pl->arith);
    if ((pl->d.pfft_flags & (F_PATIENT | F_EXHAUSTIVE | F_TUNE)) && !tune_program(pl, &pl->adj)) return;
    if (!link_fx(pl, &pl->adj, &pl->lexp[1])) return;
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
  if (!din && !dout && pl->pipeline) {
    const int r = run_pipelined(pl, prog, in, out, s, bin, bout);
    if (r < 0) return;
    if (r > 0) {
      auto t1 = std::chrono::steady_clock::now();
      pl->timer.whole += std::chrono::duration<double>(t1 - t0).count();
      pl->timer.iter++;
      return;
    }
  }
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

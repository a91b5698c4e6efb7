// Autotuner and wisdom.
//
// A pass can run with several equivalent configurations: the register-resident
// radix-8 kernel (2, 4, 8 or 16 lines per CTA at 512 points, 2, 4 or 8 at 1024,
// 2 or 4 at 2048, 1 or 2 at 4096) or
// the general kernel with radix order 16-first / 8-first / 4-first and half,
// the planned or twice the planned lines per CTA.  Plans created with
// PFFT_PATIENT, PFFT_EXHAUSTIVE or PFFT_TUNE time every candidate of every
// pass on the planned arrays (as FFTW's measuring planners do, this
// overwrites the output array, and an in-place array) and keep the fastest;
// the choice is recorded as wisdom under a key that describes the pass
// completely (arithmetic, mode, lengths, strides, batch shape, flags), so any
// later plan with the same pass - created with any flags - uses it without
// timing (a tuning planner also skips passes already in wisdom).  Plain c2c
// passes on the radix-8 kernel are also timed with and without its staged
// variant.  Wisdom is exported and imported as text:
//   pfft_gb300-wisdom 2
//   <key> <kpath> <fastL> <pref> <L> <staged>
// (files with the header "pfft_gb300-wisdom 1" and no staged field are read
// with staged = 0, the default).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/pfft_gb300.h"
#include "core.h"

namespace pg {

namespace {

struct Choice {
  int kpath = 0;  // 0 radix-8 kernel where it applies, 1 general kernel
  int fastL = 0;
  int pref = 0;   // radix order of the general kernel
  int L = 0;      // lines per CTA of the general kernel
  int staged = 0; // staged variant of the radix-8 kernel: 0 default, 1 on, 2 off
};

std::mutex g_mu;
std::map<std::string, Choice>& store() {
  static std::map<std::string, Choice> m;
  return m;
}

const char* kHeader = "pfft_gb300-wisdom 2";
const char* kHeader1 = "pfft_gb300-wisdom 1";  // without the staged field (read as 0)

std::string key_of(const PassParams& p, int arith) {
  std::ostringstream k;
  k << "a" << arith << ".m" << p.mode << ".s" << p.sign << ".N" << p.N << ".M" << p.M << ".i" << p.Ni << ":" << p.Zi
    << ".o" << p.No << ":" << p.Zo << ".sa" << p.sIa << ":" << p.sOa << ".n" << p.nlines << ".b";
  for (int b = 0; b < p.nb; b++) k << p.bext[b] << ":" << p.bsI[b] << ":" << p.bsO[b] << ",";
  k << ".f" << p.conj_in << p.conj_out << p.wmode << p.in_df << p.out_df << p.ashI.en << p.ashO.en;
  for (int b = 0; b < p.nb; b++) k << p.bshI[b].en << p.bshO[b].en;
  if (p.quant) k << ".q" << p.quant;
  return k.str();
}

bool apply_choice(PassParams* p, int arith, const Choice& c) {
  PassParams q = *p;
  q.kpath = c.kpath;
  q.fastL = c.fastL;
  q.staged = c.staged;
  if (c.kpath == 1 || !fast_pass_eligible(q, arith)) {
    if (!refit_pass(&q, arith, c.pref, c.L)) return false;
  }
  *p = q;
  return true;
}

// candidate configurations of one pass
std::vector<Choice> candidates(const PassParams& p, int arith) {
  std::vector<Choice> v;
  PassParams q = p;
  q.kpath = 0;
  if (fast_pass_eligible(q, arith)) {
    Choice c;
    v.push_back(c);
    // the other tile heights instantiated for this length (fft_fast_*_[sl].cu)
    std::vector<int> alt;
    const bool plain = p.mode == MODE_C2C && p.Zi == 0 && p.Ni == p.N && p.Zo == 0 && p.No == p.N && !p.wmode;
    // (the r2c / c2r / windowed instantiations have their default heights only)
    if (plain && p.N == 512) alt = {2, 4, 8, 16};
    if (plain && p.N == 1024) alt = {2, 4, 8};
    if (plain && p.N == 2048) alt = {2, 4};
    if (plain && p.N == 4096) alt = {1, 2};
    for (int Lf : alt) {
      c.fastL = Lf;
      v.push_back(c);
    }
    // plain c2c passes: each tile height with and without the staged variant
    if (plain && staged_mode() == 1) {
      const size_t n = v.size();
      for (size_t i = 0; i < n; i++) {
        v[i].staged = 2;
        Choice d = v[i];
        d.staged = 1;
        v.push_back(d);
      }
    }
  }
  const int L0 = p.L;
  for (int pref = 0; pref < 3; pref++) {
    for (int Lm : {L0 / 2, L0, L0 * 2}) {
      if (Lm < 1) continue;
      Choice c;
      c.kpath = 1;
      c.pref = pref;
      c.L = Lm;
      PassParams t = p;
      t.kpath = 1;
      if (!refit_pass(&t, arith, pref, Lm)) continue;
      // skip a radix order identical to one already listed
      bool dup = false;
      for (const Choice& d : v) {
        if (d.kpath != 1 || d.L != Lm) continue;
        PassParams u = p;
        u.kpath = 1;
        refit_pass(&u, arith, d.pref, d.L);
        if (u.nst == t.nst && memcmp(u.radix, t.radix, sizeof(int) * t.nst) == 0) dup = true;
      }
      if (!dup) v.push_back(c);
    }
  }
  return v;
}

float time_pass(const PassParams& p, int arith, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, int* err) {
  const int reps = 3;
  int rc = launch_pass(p, arith, s);  // warm-up (and attribute setup)
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps && !rc; r++) rc = launch_pass(p, arith, s);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  if (rc || e != cudaSuccess) {
    *err = rc ? rc : (int)e;
    return 1e30f;
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms / reps;
}

}  // namespace

void apply_wisdom(PassProgram* prog, int arith) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (Pass& ps : prog->passes) {
    auto it = store().find(key_of(ps.p, arith));
    if (it != store().end()) apply_choice(&ps.p, arith, it->second);
  }
}

bool tune_program(Plan* pl, PassProgram* prog) {
  // the planned arrays must be device memory; otherwise tune on scratch
  void* bufs[4] = {pl->in, pl->out, pl->ws[0], pl->ws[1]};
  void* scratch[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; k++) {
    cudaPointerAttributes a;
    bool dev = bufs[k] && cudaPointerGetAttributes(&a, bufs[k]) == cudaSuccess &&
               (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    if (!dev) {
      const Layout& L = k == 0 ? prog->in_layout : prog->out_layout;
      size_t bytes = (size_t)L.span * (L.cplx ? 16 : 8) + 256;
      if (k == 1 && pl->inplace) {
        bufs[1] = bufs[0];
        continue;
      }
      if (cuda_check(cudaMalloc(&scratch[k], bytes), "tuning scratch")) {
        if (scratch[0]) cudaFree(scratch[0]);
        return false;
      }
      bufs[k] = scratch[k];
    }
  }
  if (pl->inplace) bufs[1] = bufs[0];
  cudaStream_t s;
  cudaEvent_t e0, e1;
  if (cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "tuning stream")) return false;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  bool ok = true;
  for (Pass& ps : prog->passes) {
    PassParams base = ps.p;
    base.src = bufs[ps.src];
    base.dst = bufs[ps.dst];
    cudaError_t te;
    base.tw = twiddle_table(base.M, pl->arith, &te);
    if (!base.tw) {
      ok = false;
      break;
    }
    {  // a pass already in wisdom is not timed again (as FFTW reuses wisdom)
      std::lock_guard<std::mutex> lk(g_mu);
      auto it = store().find(key_of(base, pl->arith));
      if (it != store().end()) {
        apply_choice(&ps.p, pl->arith, it->second);
        continue;
      }
    }
    Choice best;
    float best_ms = 1e30f;
    for (const Choice& c : candidates(base, pl->arith)) {
      PassParams t = base;
      if (!apply_choice(&t, pl->arith, c)) continue;
      int err = 0;
      float ms = time_pass(t, pl->arith, s, e0, e1, &err);
      if (err) {
        cuda_check((cudaError_t)err, "tuning launch");
        ok = false;
        break;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (!ok) break;
    if (best_ms < 1e30f) {
      apply_choice(&ps.p, pl->arith, best);
      std::lock_guard<std::mutex> lk(g_mu);
      store()[key_of(base, pl->arith)] = best;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  for (void* p : scratch)
    if (p) cudaFree(p);
  return ok;
}

}  // namespace pg

using namespace pg;

extern "C" {

char* pfft_gb300_export_wisdom_to_string(void) {
  std::ostringstream o;
  o << kHeader << "\n";
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (const auto& kv : store())
      o << kv.first << " " << kv.second.kpath << " " << kv.second.fastL << " " << kv.second.pref << " "
        << kv.second.L << " " << kv.second.staged << "\n";
  }
  std::string s = o.str();
  char* r = (char*)malloc(s.size() + 1);
  if (r) memcpy(r, s.c_str(), s.size() + 1);
  return r;
}

int pfft_gb300_import_wisdom_from_string(const char* text) {
  if (!text) return 0;
  std::istringstream in(text);
  std::string line;
  if (!std::getline(in, line) || (line != kHeader && line != kHeader1)) return 0;
  const bool v2 = line == kHeader;
  std::map<std::string, Choice> add;
  while (std::getline(in, line)) {
    if (line.empty()) continue;
    std::istringstream ls(line);
    std::string key;
    Choice c;
    if (!(ls >> key >> c.kpath >> c.fastL >> c.pref >> c.L)) return 0;
    if (v2 && !(ls >> c.staged)) return 0;
    if (c.kpath < 0 || c.kpath > 1 || c.pref < 0 || c.pref > 2 || c.L < 0 || c.fastL < 0 || c.staged < 0 ||
        c.staged > 2)
      return 0;
    add[key] = c;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  for (const auto& kv : add) store()[kv.first] = kv.second;
  return 1;
}

int pfft_gb300_export_wisdom_to_filename(const char* filename) {
  FILE* f = fopen(filename, "w");
  if (!f) return 0;
  char* s = pfft_gb300_export_wisdom_to_string();
  int ok = s && fputs(s, f) >= 0;
  free(s);
  return fclose(f) == 0 && ok ? 1 : 0;
}

int pfft_gb300_import_wisdom_from_filename(const char* filename) {
  FILE* f = fopen(filename, "r");
  if (!f) return 0;
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  fclose(f);
  return pfft_gb300_import_wisdom_from_string(text.c_str());
}

void pfft_gb300_forget_wisdom(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  store().clear();
}

int pfft_gb300_wisdom_entries(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return (int)store().size();
}

}  // extern "C"

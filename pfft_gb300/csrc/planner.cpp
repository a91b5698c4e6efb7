// Planner: turns a PFFT plan description into a short program of passes.
//
// The reference executes a plan as r+1 serial stages interleaved with r global
// transposes per half, each stage being embed -> FFTW -> local transpose ->
// truncate (kernel/partrafo-transposed.c:185-291, kernel/outrafo.c:118-168,
// kernel/sertrafo.c:200-295, api/api-basic.c:1044-1107).  On one GPU the
// global transposes are index permutations, so this planner emits exactly one
// pass per transformed axis.  Each pass reads the previous layout and writes
// the next one, so the TRANSPOSED_IN/OUT permutations, zero-padding, truncation,
// r2c/c2r, conjugation and SHIFTED signs are folded into the first or last
// pass instead of being separate sweeps.
#include <algorithm>
#include <cstring>
#include "core.h"

namespace pg {

namespace {

struct Step {
  int axis = 0;
  int mode = MODE_C2C;
  int N = 1, M = 1;
  int Ni = 1, Zi = 0, No = 1, Zo = 0;
  int sign = -1;
  bool identity = false;  // skipped transform
  bool conj_in = false, conj_out = false;
  int wmode = 0;
};

int r2r_mode(int kind) {
  switch (kind) {
    case 0: return MODE_R2HC;
    case 1: return MODE_HC2R;
    case 2: return MODE_DHT;
    case 3: return MODE_RE00;
    case 4: return MODE_RE01;
    case 5: return MODE_RE10;
    case 6: return MODE_RE11;
    case 7: return MODE_RO00;
    case 8: return MODE_RO01;
    case 9: return MODE_RO10;
    case 10: return MODE_RO11;
  }
  return -1;
}

long long complex_len(int mode, long long N) {
  switch (mode) {
    case MODE_RE00: return 2 * (N - 1);
    case MODE_RO00: return 2 * (N + 1);
    case MODE_RE01:
    case MODE_RE10:
    case MODE_RO01:
    case MODE_RO10: return 4 * N;
    case MODE_RE11:
    case MODE_RO11: return 8 * N;
  }
  return N;
}

// Radix schedule of a length-M line.  pref 0: radix 16 first (then one 8, 4
// or 2), 1: radix 8 first, 2: radix 4 first; then 3, 5, 7, 11, 13 and any
// larger prime (generic stage).
bool factorize(int M, int* radix, int* nst, bool* generic, int pref) {
  *nst = 0;
  *generic = false;
  int m = M;
  const int big = pref == 1 ? 8 : (pref == 2 ? 4 : 16);
  while (m % big == 0 && m > big / 2) {
    radix[(*nst)++] = big;
    m /= big;
    if (*nst >= PG_MAX_STAGES) return false;
  }
  if (m % 8 == 0) {
    radix[(*nst)++] = 8;
    m /= 8;
  } else if (m % 4 == 0) {
    radix[(*nst)++] = 4;
    m /= 4;
  } else if (m % 2 == 0) {
    radix[(*nst)++] = 2;
    m /= 2;
  }
  static const int small[] = {3, 5, 7, 11, 13};
  for (int p : small)
    while (m % p == 0) {
      radix[(*nst)++] = p;
      m /= p;
      if (*nst >= PG_MAX_STAGES) return false;
    }
  for (int p = 17; m > 1; p += 2) {
    while (m % p == 0) {
      radix[(*nst)++] = p;
      m /= p;
      *generic = true;
      if (*nst >= PG_MAX_STAGES) return false;
    }
    if ((long long)p * p > m && m > 1) {
      radix[(*nst)++] = m;
      *generic = true;
      m = 1;
    }
  }
  return *nst < PG_MAX_STAGES;
}

// Threads a register stage of radix R needs over `work` = L*M points: each
// thread holds max_elems/R butterflies (at least one); max_elems is 16
// complex values for FP32 and 8 for float-float / FP64 (pass_tile.cuh).
int stage_threads(int R, long long work /* L*M */, int arith) {
  const int maxe = arith == ARITH_F32 ? 16 : 8;
  int nb;
  switch (R) {
    case 2: case 3: case 4: case 5: case 7: case 8: case 11: case 13: case 16: nb = std::max(1, maxe / R); break;
    default: return 0;  // generic stage: any thread count
  }
  long long bfly = work / R;
  return (int)((bfly + nb - 1) / nb);
}

ShiftSign no_sign() {
  ShiftSign s;
  s.en = 0;
  s.start = 0;
  s.thresh = 0;
  s.extra = 1;
  return s;
}

// memory order of the natural axes: transposed layouts move axis 0 behind
// the first r axes (api/api-basic.c:1149-1180)
void axis_order(int d, int r, bool transposed, int* order) {
  if (!transposed) {
    for (int t = 0; t < d; t++) order[t] = t;
    return;
  }
  for (int t = 0; t < r; t++) order[t] = t + 1;
  order[r] = 0;
  for (int t = r + 1; t < d; t++) order[t] = t;
}

bool inplace_safe(const PassParams& p, int esz_in, int esz_out) {
  for (int b = 0; b < p.nb; b++)
    if (p.bsI[b] * esz_in != p.bsO[b] * esz_out) return false;
  long long spanI = (long long)p.Ni * p.sIa * esz_in, spanO = (long long)p.No * p.sOa * esz_out;
  if (p.sIa * esz_in == p.sOa * esz_out && spanI == spanO) return true;
  if (p.sIa == 1 && p.sOa == 1) {
    long long fp = std::max((long long)p.Ni * esz_in, (long long)p.No * esz_out);
    for (int b = 0; b < p.nb; b++)
      if (p.bext[b] > 1 && p.bsI[b] * esz_in < fp) return false;
    return true;
  }
  return false;
}

bool mode_cplx_in(int mode) { return mode == MODE_C2C || mode == MODE_C2R; }
bool mode_cplx_out(int mode) { return mode == MODE_C2C || mode == MODE_R2C; }

}  // namespace

// Re-plan the general kernel of a pass with radix order `pref` and `L`
// lines per CTA (0: keep).  Returns false when the shape does not fit one CTA
// (512 threads, 200 KB of shared memory); the pass is then unchanged.
bool refit_pass(PassParams* p, int arith, int pref, int L) {
  if (p->nst == 0) return L <= 0 || L == p->L;
  PassParams q = *p;
  bool generic = false;
  if (!factorize(q.M, q.radix, &q.nst, &generic, pref)) return false;
  q.pingpong = generic ? 1 : 0;
  if (L > 0) q.L = (int)std::min<long long>(L, std::max(1LL, q.nlines));
  int T = 64;
  for (int st = 0; st < q.nst; st++) T = std::max(T, stage_threads(q.radix[st], (long long)q.L * q.M, arith));
  T = (T + 31) / 32 * 32;
  if (T > 512) return false;
  long long meta = ((2 * 8 + 2 * 4) * (long long)q.L + 15) & ~15LL;
  long long smem = meta + (long long)q.L * q.LS * arith_sm_bytes(arith) * (q.pingpong ? 2 : 1);
  if (smem > 200 * 1024) return false;
  q.threads = T;
  q.smem_bytes = (int)smem;
  *p = q;
  return true;
}

// Re-fit a general pass to at most max_threads threads per CTA (the
// batched persistent launch runs every tile with one block size): halve the
// lines per tile until every register stage's butterflies are covered.
bool fit_pass_threads(PassParams* p, int arith, int max_threads, int max_smem) {
  long long L = p->L;
  for (;;) {
    int T = 32;
    for (int st = 0; st < p->nst; st++) T = std::max(T, stage_threads(p->radix[st], L * p->M, arith));
    T = (T + 31) / 32 * 32;
    long long meta = ((2 * 8 + 2 * 4) * L + 15) & ~15LL;
    long long smem = meta + L * p->LS * (long long)arith_sm_bytes(arith) * (p->pingpong ? 2 : 1);
    if (T <= max_threads && (smem <= max_smem || L == 1)) {
      p->L = (int)L;
      p->threads = T;
      p->smem_bytes = (int)smem;
      return true;
    }
    if (L == 1) return false;
    L = std::max(1LL, L / 2);
  }
}

bool build_program(const PlanDesc& d, int arith, bool inplace, bool adjoint, PassProgram* prog) {
  const int D = d.rnk_n;
  const unsigned kind = d.trafo & (TR_C2C | TR_R2C | TR_C2R | TR_R2R);
  const bool padded = (d.trafo & TR_PADDED) && !d.mesh3d;
  const unsigned fl = d.pfft_flags;
  const int r = d.mesh_rank;
  if (D > PG_MAX_DIMS || D < 1) {
    set_error(1, "rank of the transform not supported");
    return false;
  }

  // ---- stored extents of the user arrays ----------------------------------
  INT ein[PG_MAX_DIMS], eout[PG_MAX_DIMS];
  for (int t = 0; t < D; t++) {
    ein[t] = d.ni[t];
    eout[t] = d.no[t];
  }
  bool cin = true, cout_ = true;
  if (kind == TR_R2C) {
    cin = false;
    ein[D - 1] = padded ? 2 * (d.ni[D - 1] / 2 + 1) : d.ni[D - 1];
    eout[D - 1] = d.no[D - 1] / 2 + 1;
  } else if (kind == TR_C2R) {
    cout_ = false;
    ein[D - 1] = d.ni[D - 1] / 2 + 1;
    eout[D - 1] = padded ? 2 * (d.no[D - 1] / 2 + 1) : d.no[D - 1];
  } else if (kind == TR_R2R) {
    cin = cout_ = false;
  }
  int ord_in[PG_MAX_DIMS], ord_out[PG_MAX_DIMS];
  axis_order(D, r, (fl & F_TRANSPOSED_IN) != 0, ord_in);
  axis_order(D, r, (fl & F_TRANSPOSED_OUT) != 0, ord_out);
  Layout Lin = compact_layout(D, ein, ord_in, d.howmany, cin);
  Layout Lout = compact_layout(D, eout, ord_out, d.howmany, cout_);

  // ---- per-axis steps in forward order ----------------------------------------
  int csign = d.sign;
  bool conj_first = false, conj_last = false;
  if (kind == TR_C2R && d.sign == -1) {  // kernel/partrafo.c:428-443
    conj_first = true;
    csign = +1;
  }
  if (kind == TR_R2C && d.sign == +1) {
    conj_last = true;
    csign = -1;
  }
  std::vector<int> axes;
  if (kind == TR_C2R) {
    for (int t = 0; t < D - 1; t++) axes.push_back(t);
    axes.push_back(D - 1);
  } else {
    for (int t = D - 1; t >= 0; t--) axes.push_back(t);
  }
  std::vector<Step> steps;
  for (int a : axes) {
    Step s;
    s.axis = a;
    const long long N = d.n[a], ni = d.ni[a], no = d.no[a];
    const bool skip = d.skip.size() > (size_t)a && d.skip[a];
    s.N = (int)N;
    s.Ni = (int)ni;
    s.No = (int)no;
    s.Zi = (fl & F_SHIFTED_IN) ? (int)((N - ni) / 2) : 0;
    s.Zo = (fl & F_SHIFTED_OUT) ? (int)((N - no) / 2) : 0;
    s.sign = csign;
    if (ni > N || no > N) {
      set_error(2, "oversampling requires ni <= n and no <= n");
      return false;
    }
    if (a == D - 1 && kind == TR_R2C) {
      if (skip) {
        set_error(3, "skipping the r2c axis is not supported");
        return false;
      }
      s.mode = MODE_R2C;
      s.sign = -1;
      long long pni = N / 2 + 1, pno = no / 2 + 1;
      s.No = (int)pno;
      s.Zo = (int)(pni - pno);  // kernel/ousample.c:288-297
    } else if (a == D - 1 && kind == TR_C2R) {
      if (skip) {
        set_error(3, "skipping the c2r axis is not supported");
        return false;
      }
      s.mode = MODE_C2R;
      s.sign = +1;
      long long pni = ni / 2 + 1, pno = N / 2 + 1;
      s.Ni = (int)pni;
      s.Zi = (int)(pno - pni);  // kernel/ousample.c:310-318
    } else if (kind == TR_R2R) {
      int k = d.kinds.size() > (size_t)a ? d.kinds[a] : 3;
      s.mode = skip ? MODE_COPYR : r2r_mode(k);
      if (s.mode < 0) {
        set_error(4, "unknown r2r kind");
        return false;
      }
      if (s.mode == MODE_RE00 && N < 2) {
        set_error(4, "REDFT00 needs n >= 2");
        return false;
      }
      s.sign = (s.mode == MODE_HC2R) ? +1 : -1;
    } else {
      s.mode = MODE_C2C;
    }
    s.identity = skip;
    s.M = (int)complex_len(s.mode, N);
    if (skip && ni == N && no == N && s.Zi == 0 && s.Zo == 0 &&
        !((fl & F_TRANSPOSED_IN) || (fl & F_TRANSPOSED_OUT)))
      continue;  // nothing to do on this axis
    steps.push_back(s);
  }
  if (steps.empty()) {
    Step s;
    s.axis = D - 1;
    s.mode = cin ? MODE_C2C : MODE_COPYR;
    s.N = s.M = s.Ni = s.No = (int)d.n[D - 1];
    s.identity = true;
    steps.push_back(s);
  }
  const int P = (int)steps.size();
  steps.front().conj_in = conj_first;
  steps.back().conj_out = conj_last;

  // ---- layouts between passes (forward order) ---------------------------------
  std::vector<Layout> lay(P + 1);
  lay[0] = Lin;
  lay[P] = Lout;
  {
    INT ext[PG_MAX_DIMS];
    for (int t = 0; t < D; t++) ext[t] = Lin.ext[t];
    bool c = cin;
    for (int i = 0; i < P - 1; i++) {
      const Step& s = steps[i];
      ext[s.axis] = Lout.ext[s.axis];
      if (s.mode == MODE_R2C) c = true;
      if (s.mode == MODE_C2R) c = false;
      if (kind == TR_C2R && s.axis != D - 1) {
        // complex intermediate of a c2r plan: last axis is still the half spectrum
      }
      bool same = (c == cout_);
      for (int t = 0; t < D; t++) same = same && ext[t] == Lout.ext[t];
      lay[i + 1] = same ? Lout : compact_layout(D, ext, ord_out, d.howmany, c);
    }
  }

  // ---- shift signs of the first / last pass -------------------------------------
  std::vector<ShiftSign> sh_in(D, no_sign()), sh_out(D, no_sign());
  if (fl & F_SHIFTED_OUT) {  // api/api-basic.c:1186-1238
    for (int t = 0; t < D; t++) {
      const bool skip = d.skip.size() > (size_t)t && d.skip[t];
      sh_in[t].en = !skip;
      sh_in[t].start = (int)d.local_i_start[t];
      sh_in[t].thresh = (int)(d.ni[t] / 2);
      sh_in[t].extra = ((fl & F_SHIFTED_IN) && ((d.n[t] / 2) % 2)) ? -1 : 1;
    }
  }
  if (fl & F_SHIFTED_IN) {  // api/api-basic.c:1242-1285
    for (int t = 0; t < D; t++) {
      const bool skip = d.skip.size() > (size_t)t && d.skip[t];
      sh_out[t].en = !skip;
      sh_out[t].start = (int)d.local_o_start[t];
      sh_out[t].thresh = (int)(d.no[t] / 2);
      sh_out[t].extra = 1;
    }
  }

  // ---- adjoint: reverse the chain ------------------------------------------------
  if (adjoint) {
    for (auto& s : steps) {
      if (s.mode != MODE_C2C && s.mode != MODE_R2C && s.mode != MODE_C2R) {
        set_error(5, "the adjoint is implemented for c2c, r2c and c2r plans");
        return false;
      }
      std::swap(s.Ni, s.No);
      std::swap(s.Zi, s.Zo);
      std::swap(s.conj_in, s.conj_out);
      s.sign = -s.sign;
      if (s.mode == MODE_R2C) {
        s.mode = MODE_C2R;
        s.wmode = 1;
      } else if (s.mode == MODE_C2R) {
        s.mode = MODE_R2C;
        s.wmode = 2;
      }
    }
    std::reverse(steps.begin(), steps.end());
    std::reverse(lay.begin(), lay.end());
    std::swap(sh_in, sh_out);
  }

  // ---- pass parameters ------------------------------------------------------------
  const int esz_c = (arith == ARITH_F32) ? 8 : 16;
  const int esz_r = (arith == ARITH_F32) ? 4 : 8;
  const int smesz = arith_sm_bytes(arith);
  prog->passes.clear();
  prog->in_layout = lay[0];
  prog->out_layout = lay[P];
  for (int i = 0; i < P; i++) {
    const Step& s = steps[i];
    const Layout& A = lay[i];
    const Layout& B = lay[i + 1];
    Pass ps;
    PassParams& p = ps.p;
    memset(&p, 0, sizeof(p));
    ps.axis = s.axis;
    p.mode = s.mode;
    p.sign = s.sign;
    p.N = s.N;
    p.M = s.M;
    p.Ni = s.Ni;
    p.Zi = s.Zi;
    p.No = s.No;
    p.Zo = s.Zo;
    p.conj_in = s.conj_in;
    p.conj_out = s.conj_out;
    p.wmode = s.wmode;
    p.sIa = A.stride[s.axis];
    p.sOa = B.stride[s.axis];
    p.ashI = (i == 0) ? sh_in[s.axis] : no_sign();
    p.ashO = (i == P - 1) ? sh_out[s.axis] : no_sign();
    // batch dims: every other axis plus howmany
    struct BD {
      long long ext, si, so;
      ShiftSign shi, sho;
    };
    std::vector<BD> bd;
    for (int t = 0; t < D; t++) {
      if (t == s.axis) continue;
      BD b;
      b.ext = A.ext[t];
      b.si = A.stride[t];
      b.so = B.stride[t];
      b.shi = (i == 0) ? sh_in[t] : no_sign();
      b.sho = (i == P - 1) ? sh_out[t] : no_sign();
      if (b.ext > 1) bd.push_back(b);
    }
    if (d.howmany > 1) {
      BD b;
      b.ext = d.howmany;
      b.si = A.hm_stride;
      b.so = B.hm_stride;
      b.shi = b.sho = no_sign();
      bd.push_back(b);
    }
    std::stable_sort(bd.begin(), bd.end(), [](const BD& x, const BD& y) {
      return std::min(x.si, x.so) < std::min(y.si, y.so);
    });
    // merge dims that are contiguous on both sides (and carry no signs)
    std::vector<BD> mg;
    for (auto& b : bd) {
      if (!mg.empty()) {
        BD& pv = mg.back();
        if (!pv.shi.en && !pv.sho.en && !b.shi.en && !b.sho.en && b.si == pv.si * pv.ext &&
            b.so == pv.so * pv.ext) {
          pv.ext *= b.ext;
          continue;
        }
      }
      mg.push_back(b);
    }
    if ((int)mg.size() > PG_MAX_BATCH) {
      set_error(6, "too many batch dimensions");
      return false;
    }
    p.nb = (int)mg.size();
    p.nlines = 1;
    for (int b = 0; b < p.nb; b++) {
      p.bext[b] = mg[b].ext;
      p.bsI[b] = mg[b].si;
      p.bsO[b] = mg[b].so;
      p.bshI[b] = mg[b].shi;
      p.bshO[b] = mg[b].sho;
      p.nlines *= mg[b].ext;
    }
    p.in_contig = (p.sIa == 1);
    p.out_contig = (p.sOa == 1);
    // stages
    bool generic = false;
    if (s.identity) {
      p.nst = 0;
    } else if (!factorize(s.M, p.radix, &p.nst, &generic, arith == ARITH_F32 ? 0 : 1)) {
      set_error(7, "transform length has too many factors");
      return false;
    }
    p.pingpong = generic ? 1 : 0;
    // lines per CTA and threads
    long long line_bytes = (long long)s.M * smesz;
    long long L = std::max(1LL, 65536 / line_bytes);
    if (!(p.in_contig && p.out_contig)) L = std::max(L, std::min(8LL, 163840 / line_bytes));
    L = std::min(L, 64LL);
    // small problems: keep at least two CTAs per SM (152 SMs) so that a pass
    // is not one latency-bound wave of a few CTAs
    L = std::min(L, std::max(1LL, (p.nlines + 303) / 304));
    L = std::max(1LL, std::min(L, p.nlines));
    int T = 0;
    for (;;) {
      T = 64;
      for (int st = 0; st < p.nst; st++) T = std::max(T, stage_threads(p.radix[st], L * s.M, arith));
      T = (T + 31) / 32 * 32;
      if (T <= 512 || L == 1) break;
      L = std::max(1LL, L / 2);
    }
    if (T > 512) {
      set_error(8, "transform length too large for one pass");
      return false;
    }
    p.L = (int)L;
    p.LS = s.M;
    p.threads = T;
    long long meta = ((2 * 8 + 2 * 4) * L + 15) & ~15LL;
    long long smem = meta + L * p.LS * (long long)smesz * (p.pingpong ? 2 : 1);
    if (smem > 200 * 1024) {
      set_error(8, "transform length too large for one pass (shared memory)");
      return false;
    }
    p.smem_bytes = (int)smem;
    const int ei = mode_cplx_in(s.mode) ? esz_c : esz_r;
    const int eo = mode_cplx_out(s.mode) ? esz_c : esz_r;
    ps.bytes = (double)p.nlines * ((double)p.Ni * ei + (double)p.No * eo);
    prog->passes.push_back(ps);
  }

  // ---- buffers: backwards from the output ---------------------------------------------
  // Constraints: the last pass writes OUT; the input is never written; a pass
  // whose source and destination are the same buffer must be in-place safe;
  // an intermediate may live in OUT only if its layout fits in the output
  // array (the caller's array may be exactly the output layout's size);
  // everything else goes to the plan-owned workspaces (sized to fit).
  std::vector<int> dst(P);
  auto esz_in = [&](int i) { return mode_cplx_in(prog->passes[i].p.mode) ? esz_c : esz_r; };
  auto esz_out = [&](int i) { return mode_cplx_out(prog->passes[i].p.mode) ? esz_c : esz_r; };
  auto lbytes = [&](const Layout& Lx) { return (size_t)Lx.span * (Lx.cplx ? esz_c : esz_r); };
  const size_t cap_out = inplace ? std::max(lbytes(lay[0]), lbytes(lay[P])) : lbytes(lay[P]);
  auto safe = [&](int i) { return inplace_safe(prog->passes[i].p, esz_in(i), esz_out(i)); };
  dst[P - 1] = BUF_OUT;
  for (int i = P - 2; i >= 0; i--) {
    const int cand[4] = {dst[i + 1], BUF_OUT, BUF_WSA, BUF_WSB};
    dst[i] = -1;
    for (int c : cand) {
      if (c == dst[i + 1] && !safe(i + 1)) continue;
      if (c == BUF_OUT && lbytes(lay[i + 1]) > cap_out) continue;
      dst[i] = c;
      break;
    }
  }
  if (inplace && dst[0] == BUF_OUT && !safe(0)) {
    if (P == 1) {
      set_error(9, "this in-place transform needs an out-of-place array");
      return false;
    }
    dst[0] = (dst[1] == BUF_WSA) ? BUF_WSB : BUF_WSA;
  }
  // self-check of the assignment
  for (int i = 0; i < P; i++) {
    int src = (i == 0) ? (inplace ? BUF_OUT : BUF_IN) : dst[i - 1];
    bool ok = dst[i] >= BUF_OUT && (src != dst[i] || safe(i)) &&
              (dst[i] != BUF_OUT || lbytes(lay[i + 1]) <= cap_out);
    if (!ok) {
      set_error(10, "internal error: invalid buffer assignment");
      return false;
    }
  }
  // double API: complex intermediates stay in float-float form between
  // passes (same 16 bytes per value), so only the first pass converts from
  // double and only the last converts back
  if (arith == ARITH_DF) {
    for (int i = 0; i + 1 < P; i++) {
      if (lay[i + 1].cplx && mode_cplx_out(prog->passes[i].p.mode) && mode_cplx_in(prog->passes[i + 1].p.mode)) {
        prog->passes[i].p.out_df = 1;
        prog->passes[i + 1].p.in_df = 1;
      }
    }
  }
  prog->ws_bytes[0] = prog->ws_bytes[1] = 0;
  for (int i = 0; i < P; i++) {
    Pass& ps = prog->passes[i];
    ps.src = (i == 0) ? BUF_IN : dst[i - 1];
    ps.dst = dst[i];
    if (ps.dst == BUF_WSA || ps.dst == BUF_WSB) {
      const Layout& B = lay[i + 1];
      size_t bytes = (size_t)B.span * (B.cplx ? esz_c : esz_r);
      size_t& w = prog->ws_bytes[ps.dst - BUF_WSA];
      w = std::max(w, bytes);
    }
  }
  return true;
}

}  // namespace pg

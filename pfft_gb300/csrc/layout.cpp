// Data-distribution arithmetic of PFFT at a single rank.
//
// With one process every block is the whole axis, so the reference's block
// decomposition (kernel/block.c:54-95, util/util.c:43-59) reduces to
// "local size = physical size, local start = 0".  What remains is the
// bookkeeping that decides *which* physical size each array reports and how
// many elements must be allocated:
//   - the split into a transposed-out and a transposed-in half with their
//     per-stage transform flags   (kernel/partrafo.c:735-834)
//   - the per-stage memory demand (kernel/partrafo-transposed.c:88-182,
//     kernel/outrafo.c:93-115, kernel/sertrafo.c:152-169,
//     kernel/ousample.c:55-75, kernel/transpose.c:63-137)
//   - the 3-D-on-3-D remap sizes  (kernel/remap_3dto2d.c:125-215)
//   - the r2c / c2r real-unit fix-ups (kernel/partrafo-transposed.c:158-176)
//   - the SHIFTED start offsets   (kernel/partrafo.c:287-299)
// The single-rank FFTW-MPI transpose demand (kernel/transpose.c:115-137,
// fftw_mpi_local_size_many_transposed of FFTW 3.3.4) is the product of the
// two transposed extents.
#include <algorithm>
#include <vector>
#include "core.h"

namespace pg {

static INT phys1(INT n, unsigned f) { return (f & TR_RDFT) ? n / 2 + 1 : n; }

static INT prod_phys(int rnk, const INT* n, unsigned f) {
  INT p = 1;
  for (int t = 0; t < rnk; t++) p *= (t == rnk - 1) ? phys1(n[t], f) : n[t];
  return p;
}

// kernel/outrafo.c:93-115 : max over embed, transform, truncate
static INT outrafo_mem(INT nb, int rnk, const INT* n, const INT* ni, const INT* no, INT hm, unsigned f) {
  INT m = 1;
  m = std::max(m, nb * std::max(prod_phys(rnk, ni, f), prod_phys(rnk, n, f)) * hm);
  m = std::max(m, nb * prod_phys(rnk, n, f) * hm);
  m = std::max(m, nb * std::max(prod_phys(rnk, n, f), prod_phys(rnk, no, f)) * hm);
  return m;
}

int effective_mesh_rank(int rnk_n, int cart_dims) {
  if (cart_dims <= 0) return 1;  // non-Cartesian communicators become 1-D meshes
  if (rnk_n == 3 && cart_dims == 3) return 2;
  return cart_dims;
}

namespace {

struct Half {
  std::vector<INT> n, ni, no;
  std::vector<unsigned> flags;  // index r = first stage (last dims), 0 = axis 0
};

// kernel/partrafo.c:735-834 (including its flag quirks)
void split_halves(int d, const INT* n, const INT* ni, const INT* no, int r, unsigned trafo, unsigned transp,
                  Half* to, Half* ti) {
  to->n.assign(n, n + d);
  to->ni.assign(ni, ni + d);
  to->no.assign(no, no + d);
  to->flags.assign(r + 1, trafo);
  ti->n.assign(no, no + d);
  ti->ni.assign(no, no + d);
  ti->no.assign(no, no + d);
  ti->flags.assign(r + 1, trafo | TR_SKIP);
  if (transp & F_TRANSPOSED_IN) {
    ti->flags.assign(r + 1, trafo);
    ti->n.assign(n, n + d);
    ti->ni.assign(ni, ni + d);
    ti->no.assign(no, no + d);
  }
  if (trafo & TR_R2C) {
    for (int t = 0; t <= r; t++) to->flags[t] = (t == r) ? trafo : TR_C2C;
    to->n.assign(n, n + d);
    to->ni.assign(ni, ni + d);
    to->no.assign(no, no + d);
    ti->flags.assign(r + 1, TR_C2C | TR_SKIP);
    for (int t = 0; t < d; t++) ti->n[t] = ti->ni[t] = ti->no[t] = (t == d - 1) ? no[t] / 2 + 1 : no[t];
  }
  if (trafo & TR_C2R) {
    to->flags.assign(r + 1, TR_C2C | TR_SKIP);
    for (int t = 0; t < d; t++) to->n[t] = to->ni[t] = to->no[t] = (t == d - 1) ? ni[t] / 2 + 1 : ni[t];
    for (int t = 0; t <= r; t++) ti->flags[t] = (t == r) ? trafo : TR_C2C;
    ti->n.assign(n, n + d);
    ti->ni.assign(ni, ni + d);
    ti->no.assign(no, no + d);
  }
  if (transp & F_TRANSPOSED_OUT) {
    ti->flags.assign(r + 1, 0);
    for (int t = 0; t < d; t++) ti->n[t] = ti->ni[t] = ti->no[t] = 0;
  }
  if (transp & F_TRANSPOSED_IN) {
    // the reference clears the pointer rather than the flags here; the
    // transposed-out half is not used in this case, only its sizes vanish
    for (int t = 0; t < d; t++) to->n[t] = to->ni[t] = to->no[t] = 0;
  }
  // the reference tests (~transp & (IN || OUT)), i.e. bit 0 only
  if (!(transp & F_TRANSPOSED_IN)) {
    if (trafo & TR_C2R)
      to->flags[0] = TR_PHANTOM;
    else
      ti->flags[0] = TR_PHANTOM;
  }
}

// physical sizes with the user-facing real fix-ups of one half
void half_local(int d, const Half& h, int r, bool mesh3d_remap, INT* lni, INT* lno) {
  unsigned f = h.flags[r];
  for (int t = 0; t < d; t++) {
    lni[t] = (t == d - 1) ? phys1(h.ni[t], f) : h.ni[t];
    lno[t] = (t == d - 1) ? phys1(h.no[t], f) : h.no[t];
  }
  if (f & TR_R2C) lni[d - 1] = (f & TR_PADDED) ? 2 * lni[d - 1] : h.ni[d - 1];
  if (f & TR_C2R) lno[d - 1] = (f & TR_PADDED) ? 2 * lno[d - 1] : h.no[d - 1];
  (void)mesh3d_remap;
}

// kernel/partrafo-transposed.c:88-182 at one rank
INT half_mem(int d, const Half& h, INT hm, int r, bool transposed_in) {
  unsigned f = h.flags[r];
  std::vector<INT> lni(d), lno(d);
  for (int t = 0; t < d; t++) {
    lni[t] = (t == d - 1) ? phys1(h.ni[t], f) : h.ni[t];
    lno[t] = (t == d - 1) ? phys1(h.no[t], f) : h.no[t];
  }
  // the backward half is planned from its output side
  const std::vector<INT>& lnA = transposed_in ? lno : lni;  // "input" side
  const std::vector<INT>& lnB = transposed_in ? lni : lno;  // "output" side
  INT nb = 1;
  for (int t = 0; t < r; t++) nb *= lnA[t];
  const std::vector<INT>& nt = transposed_in ? h.ni : h.no;  // tuple sizes
  INT tuple = hm;
  if (r + 1 < d) tuple *= phys1(nt[d - 1], f);
  for (int t = r + 1; t < d - 1; t++) tuple *= nt[t];

  INT mem = 1;
  mem = std::max(mem, outrafo_mem(nb, d - r, &h.n[r], &h.ni[r], &h.no[r], hm, f));

  std::vector<INT> pni(d), pno(d);
  for (int t = 0; t < d; t++) {
    pni[t] = (t == d - 1) ? phys1(h.ni[t], f) : h.ni[t];
    pno[t] = (t == d - 1) ? phys1(h.no[t], f) : h.no[t];
  }
  const std::vector<INT>& pA = transposed_in ? pno : pni;
  const std::vector<INT>& pB = transposed_in ? pni : pno;
  for (int step = 0; step < r; step++) {
    // global transpose of this step (kernel/transpose.c:63-112)
    INT N0 = pB[r - step];
    INT N1 = pA[r - 1 - step];
    INT h0 = 1;
    for (int t = 0; t < step; t++) h0 *= lnB[r - t];
    for (int t = 0; t < r - 1 - step; t++) h0 *= lnA[t];
    INT tot = N0 * h0 * N1;
    mem = std::max(mem, tot == 0 ? (INT)1 : std::max(tot, (INT)1));
    // serial stage step+1 (kernel/outrafo.c:46-91)
    int s = step + 1;
    INT nbs = 1;
    for (int t = 0; t < s; t++) nbs *= lnB[r - t];
    for (int t = 0; t < r - s; t++) nbs *= lnA[t];
    INT N = h.n[r - s], Ni = h.ni[r - s], No = h.no[r - s];
    unsigned fs = h.flags[r - s];
    mem = std::max(mem, outrafo_mem(nbs, 1, &N, &Ni, &No, tuple, fs));
  }
  return mem;
}

// kernel/remap_3dto2d.c:125-215 at one rank
INT remap3d_mem(int d, int cart_dims, const std::vector<INT>& pn, INT hm) {
  if (d != 3 || cart_dims != 3) return 0;
  INT full = pn[0] * pn[1] * pn[2];
  return std::max((INT)1, std::max(full * hm, full));
}

}  // namespace

INT local_size(const SizeQuery& q, INT* lni, INT* lis, INT* lno, INT* los) {
  const int d = q.rnk_n;
  const unsigned transp = q.pfft_flags & (F_TRANSPOSED_IN | F_TRANSPOSED_OUT);
  const int r = effective_mesh_rank(d, q.cart_dims);
  const bool remap3d = (d == 3 && q.cart_dims == 3);
  Half to, ti;
  split_halves(d, q.n, q.ni, q.no, r, q.trafo, transp, &to, &ti);

  std::vector<INT> dummy_n(d), dummy_s(d);
  // which half writes the user's arrays (kernel/partrafo.c:703-732)
  INT *lni_to = lni, *lno_to = dummy_n.data(), *lni_ti = dummy_n.data(), *lno_ti = lno;
  if (transp & F_TRANSPOSED_OUT) {
    lno_to = lno;
    lni_ti = lno_ti = dummy_n.data();
  }
  if (transp & F_TRANSPOSED_IN) {
    lni_to = lno_to = dummy_n.data();
    lni_ti = lni;
    lno_ti = lno;
  }
  for (int t = 0; t < d; t++) lis[t] = los[t] = 0;

  INT mem = 1;
  if (!(transp & F_TRANSPOSED_IN)) {
    std::vector<INT> a(d), b(d);
    half_local(d, to, r, remap3d, a.data(), b.data());
    if (lni_to != dummy_n.data()) std::copy(a.begin(), a.end(), lni_to);
    if (lno_to != dummy_n.data()) std::copy(b.begin(), b.end(), lno_to);
    mem = std::max(mem, half_mem(d, to, q.howmany, r, false));
    if (remap3d) {
      // the remap overwrites the input blocks with the logical sizes
      if (lni_to != dummy_n.data())
        for (int t = 0; t < d; t++) lni_to[t] = to.ni[t];
      mem = std::max(mem, remap3d_mem(d, q.cart_dims, to.ni, q.howmany));
    }
  }
  if (!(transp & F_TRANSPOSED_OUT)) {
    std::vector<INT> a(d), b(d);
    half_local(d, ti, r, remap3d, a.data(), b.data());
    if (lni_ti != dummy_n.data()) std::copy(a.begin(), a.end(), lni_ti);
    if (lno_ti != dummy_n.data()) std::copy(b.begin(), b.end(), lno_ti);
    mem = std::max(mem, half_mem(d, ti, q.howmany, r, true));
    if (remap3d) {
      if (lno_ti != dummy_n.data())
        for (int t = 0; t < d; t++) lno_ti[t] = ti.no[t];
      mem = std::max(mem, remap3d_mem(d, q.cart_dims, ti.no, q.howmany));
    }
  }
  if (q.pfft_flags & F_SHIFTED_IN)
    for (int t = 0; t < d; t++) lis[t] -= q.ni[t] / 2;
  if (q.pfft_flags & F_SHIFTED_OUT)
    for (int t = 0; t < d; t++) los[t] -= q.no[t] / 2;
  return mem;
}

Layout compact_layout(int d, const INT* ext, const int* order, INT hm, bool cplx) {
  Layout L;
  L.d = d;
  L.cplx = cplx;
  L.hm = hm;
  L.hm_stride = 1;
  INT s = hm;
  for (int i = d - 1; i >= 0; i--) {
    int ax = order[i];
    L.ext[ax] = ext[ax];
    L.stride[ax] = s;
    s *= ext[ax];
  }
  L.span = s;
  return L;
}

}  // namespace pg

"""Oracle for PFFT's data-distribution integers (TEST INFRASTRUCTURE ONLY).

A line-by-line Python restatement of the reference's local-size bookkeeping,
evaluated for a Cartesian mesh whose dimensions are all 1 (one process,
coordinates 0).  It keeps the reference's structure - block sizes, the split
into transposed-out / transposed-in halves, per-stage memory demand, the
3-D-on-3-D remap and the real-unit fix-ups - so that the product's closed-form
C++ layout engine can be checked against it on many configurations.

Reference functions restated (PFFT tree):
  kernel/block.c:54-95                 block offsets / sizes
  util/util.c:43-83, 207-227           decompose, user blocks, physical sizes
  kernel/partrafo.c:202-314            local_size_partrafo
  kernel/partrafo.c:652-834            evaluate_blocks, init_param_local_size,
                                       init_param_size_and_trafo_flags
  kernel/partrafo-transposed.c:88-182, 294-411
  kernel/outrafo.c:46-115              get_outrafo_param, local_size_outrafo
  kernel/sertrafo.c:152-169            local_size_sertrafo
  kernel/ousample.c:55-75              local_size_ousam_dd
  kernel/transpose.c:63-137            global transpose parameters / size
  kernel/remap_3dto2d.c:125-215, 437-457
The single-rank size returned by FFTW-MPI's local_size_many_transposed
(FFTW 3.3.4) is the product of the two transposed extents times howmany.
"""

C2C, R2C, C2R, R2R = 1, 2, 4, 8  # transform types (own encoding)
SKIP, PHANTOM, PADDED = 16, 32, 64
RDFT = R2C | C2R

T_IN, T_OUT = 1, 2
S_IN, S_OUT = 4, 8
PADDED_R2C_FLAG = 1 << 11


def num_blocks(n, blk):
    return (n + blk - 1) // blk


def local_block_size(n, blk, which):
    b = num_blocks(n, blk)
    if which >= b:
        return 0
    return n - which * blk if which == b - 1 else blk


def local_block_offset(n, blk, which):
    return 0 if which >= num_blocks(n, blk) else which * blk


def global_block_size(n, user_blk, nprocs):
    return (n + nprocs - 1) // nprocs if user_blk == 0 else user_blk


def phys1(n, flag):
    return n // 2 + 1 if flag & RDFT else n


def phys(ns, flag):
    out = list(ns)
    out[-1] = phys1(ns[-1], flag)
    return out


def prod(v):
    p = 1
    for x in v:
        p *= x
    return p


def ousam_size(nb, ni, no, hm, flag):
    return max(nb * prod(phys(ni, flag)) * hm, nb * prod(phys(no, flag)) * hm)


def sertrafo_size(nb, n, hm, flag):
    return nb * prod(phys(n, flag)) * hm


def outrafo_size(nb, n, ni, no, hm, flag):
    mem = 1
    mem = max(mem, ousam_size(nb, ni, n, hm, flag))
    mem = max(mem, sertrafo_size(nb, n, hm, flag))
    mem = max(mem, ousam_size(nb, n, no, hm, flag))
    return mem


def transp_size(N0, N1, h0, h1):
    A, B = N1 * h1, N0 * h0
    if A * B * h0 * h1 == 0:
        return 1
    return max(A * B, 1)


def split(d, n, ni, no, r, trafo, transp):
    to_f = [trafo] * (r + 1)
    to_n, to_ni, to_no = list(n), list(ni), list(no)
    ti_f = [trafo | SKIP] * (r + 1)
    ti_n, ti_ni, ti_no = list(no), list(no), list(no)
    if transp & T_IN:
        ti_f = [trafo] * (r + 1)
        ti_n, ti_ni, ti_no = list(n), list(ni), list(no)
    if trafo & R2C:
        to_f = [(trafo if t == r else C2C) for t in range(r + 1)]
        to_n, to_ni, to_no = list(n), list(ni), list(no)
        ti_f = [C2C | SKIP] * (r + 1)
        ti_n = [no[t] if t < d - 1 else no[t] // 2 + 1 for t in range(d)]
        ti_ni, ti_no = list(ti_n), list(ti_n)
    if trafo & C2R:
        to_f = [C2C | SKIP] * (r + 1)
        to_n = [ni[t] if t < d - 1 else ni[t] // 2 + 1 for t in range(d)]
        to_ni, to_no = list(to_n), list(to_n)
        ti_f = [(trafo if t == r else C2C) for t in range(r + 1)]
        ti_n, ti_ni, ti_no = list(n), list(ni), list(no)
    if transp & T_OUT:
        ti_f = [0] * (r + 1)
        ti_n = [0] * d
        ti_ni = [0] * d
        ti_no = [0] * d
    if transp & T_IN:
        to_n = [0] * d
        to_ni = [0] * d
        to_no = [0] * d
    if (~transp) & 1:  # the reference tests (~transp & (IN || OUT)), i.e. bit 0
        if trafo & C2R:
            to_f[0] = PHANTOM
        else:
            ti_f[0] = PHANTOM
    return (to_n, to_ni, to_no, to_f), (ti_n, ti_ni, ti_no, ti_f)


def decompose(pn, blk, r, coords, shift):
    ln = list(pn)
    ls = [0] * len(pn)
    for t in range(r):
        ln[t + shift] = local_block_size(pn[t + shift], blk[t], coords[t])
        ls[t + shift] = local_block_offset(pn[t + shift], blk[t], coords[t])
    return ln, ls


def local_size_transposed(d, ni, no, iblk, oblk, r, flag, transp):
    coords = [0] * r
    if transp & T_OUT:
        lni, _ = decompose(phys(ni, flag), iblk, r, coords, 0)
        lno, _ = decompose(phys(no, flag), oblk, r, coords, 1)
    else:
        lni, _ = decompose(phys(ni, flag), iblk, r, coords, 1)
        lno, _ = decompose(phys(no, flag), oblk, r, coords, 0)
    return lni, lno


def half_size(d, n, ni, no, hm, iblk, oblk, r, transp, flags):
    flag = flags[r]
    lni, lno = local_size_transposed(d, ni, no, iblk, oblk, r, flag, transp)
    ln = lno if transp & T_IN else lni
    nb = prod(ln[:r])
    nn = no if transp & T_OUT else ni
    tpl = hm
    if r + 1 < d:
        tpl *= phys1(nn[d - 1], flag)
    for t in range(r + 1, d - 1):
        tpl *= nn[t]
    mem = max(1, outrafo_size(nb, n[r:], ni[r:], no[r:], hm, flag))
    pni, pno = phys(ni, flag), phys(no, flag)
    for step in range(r):
        if transp & T_IN:
            A_no, A_ni, A_lno, A_lni = pni, pno, lni, lno
        else:
            A_no, A_ni, A_lno, A_lni = pno, pni, lno, lni
        N0 = A_no[r - step]
        N1 = A_ni[r - 1 - step]
        h0 = 1
        for t in range(step):
            h0 *= A_lno[r - t]
        for t in range(r - 1 - step):
            h0 *= A_lni[t]
        mem = max(mem, transp_size(N0, N1, h0, 1))
        s = step + 1
        nbs = 1
        for t in range(s):
            nbs *= A_lno[r - t]
        for t in range(r - s):
            nbs *= A_lni[t]
        fl = flags[r - s]
        mem = max(mem, outrafo_size(nbs, [n[r - s]], [ni[r - s]], [no[r - s]], tpl, fl))
    if flag & R2C:
        lni[d - 1] = 2 * lni[d - 1] if flag & PADDED else ni[d - 1]
    if flag & C2R:
        lno[d - 1] = 2 * lno[d - 1] if flag & PADDED else no[d - 1]
    return mem, lni, lno


def remap3d(d, cart, pn, hm, flag):
    if d != 3 or cart != 3:
        return 0, None
    if flag & RDFT:
        flag = R2R
    # P = 1: every block is the whole axis
    ln = list(pn)
    mem = 1
    mem = max(mem, sertrafo_size(ln[0] * ln[1], [ln[2]], hm, flag))
    mem = max(mem, transp_size(ln[1], ln[2], 1, ln[0]))
    mem = max(mem, transp_size(ln[0], ln[2], ln[1], 1))
    mem = max(mem, sertrafo_size(ln[2], [ln[0] * ln[1]], hm, flag))
    return mem, ln


def local_size(d, n, ni, no, howmany, trafo, flags, cart):
    """(alloc_local, local_ni, local_i_start, local_no, local_o_start)."""
    if trafo in (R2C, C2R) and (flags & PADDED_R2C_FLAG):
        trafo |= PADDED
    transp = flags & (T_IN | T_OUT)
    cd = cart if cart > 0 else 1
    r = 2 if (d == 3 and cd == 3) else cd
    blk = [global_block_size(1, 0, 1)] * r  # unused at one rank (blocks cover the axis)
    to, ti = split(d, n, ni, no, r, trafo, transp)
    lni_user = [0] * d
    lno_user = [0] * d
    mem = 1
    if not transp & T_IN:
        to_n, to_ni, to_no, to_f = to
        iblk = [global_block_size(x, 0, 1) for x in phys(to_ni, to_f[r])[:r]]
        mblk = [global_block_size(x, 0, 1) for x in phys(to_no, to_f[r])[1:r + 1]]
        m, a, b = half_size(d, to_n, to_ni, to_no, howmany, iblk, mblk, r, T_OUT, to_f)
        mem = max(mem, m)
        lni_user = a
        if transp & T_OUT:
            lno_user = b
        m3, ln3 = remap3d(d, cart, to_ni, howmany, to_f[r])
        mem = max(mem, m3)
        if ln3 is not None:
            lni_user = ln3
    if not transp & T_OUT:
        ti_n, ti_ni, ti_no, ti_f = ti
        mblk = [global_block_size(x, 0, 1) for x in phys(ti_ni, ti_f[r])[1:r + 1]]
        oblk = [global_block_size(x, 0, 1) for x in phys(ti_no, ti_f[r])[:r]]
        m, a, b = half_size(d, ti_n, ti_ni, ti_no, howmany, mblk, oblk, r, T_IN, ti_f)
        mem = max(mem, m)
        lno_user = b
        if transp & T_IN:
            lni_user = a
        m3, ln3 = remap3d(d, cart, ti_no, howmany, ti_f[r])
        mem = max(mem, m3)
        if ln3 is not None:
            lno_user = ln3
    del blk
    lis = [0] * d
    los = [0] * d
    if flags & S_IN:
        lis = [-(x // 2) for x in ni]
    if flags & S_OUT:
        los = [-(x // 2) for x in no]
    return mem, lni_user, lis, lno_user, los


def mesh_rank(d, cart):
    cd = cart if cart > 0 else 1
    return 2 if (d == 3 and cd == 3) else cd

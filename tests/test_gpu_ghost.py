"""pfft_exchange / pfft_reduce (ghost cells) on the GPU against the oracle.

At one process the exchange is a periodic wrap of the compact block into the
box gc_below + n + gc_above and the reduce is its adjoint
(gcell/gcells_plan.c:379-486, gcell/gcells_sendrecv.c).  Cases follow
tests/simple_check_ghost_c2c.c (8^3, gc_above[0] = 4), the r2c-input variants
(padded real rows) and the benchmark configuration (256^3 real, width 2).
The exchange is a copy: results must be bit-identical.  The reduce sums in a
different order than the reference's message sequence: relative tolerance.
"""
import numpy as np
import pytest

import pfft_gb300 as pg
from oracle import ghost

pytestmark = pytest.mark.gpu


def run_gc(torch, kind, n, gcb, gca, prec="double", flags=0, howmany=1, reduce=False, seed=0):
    L = pg.lib()
    pre = "pfft_" if prec == "double" else "pfftf_"
    rdt = torch.float64 if prec == "double" else torch.float32
    npdt = np.float64 if prec == "double" else np.float32
    pn = list(n)
    tuple_ = howmany * (2 if kind == "c" else 1)
    if kind == "c" and (flags & pg.PFFT_GC_R2C):
        pn[-1] = n[-1] // 2 + 1
    if kind == "r" and (flags & pg.PFFT_GC_PADDED):
        pn[-1] = 2 * (n[-1] // 2 + 1)
    box = [b + m + a for b, m, a in zip(gcb, pn, gca)]
    rng = np.random.default_rng(seed)
    blockv = rng.uniform(-1, 1, int(np.prod(pn)) * tuple_).astype(npdt)
    buf = torch.zeros(int(np.prod(box)) * tuple_, dtype=rdt, device="cuda")
    comm = pg.procmesh(2)
    fn = getattr(L, pre + ("plan_many_cgc" if kind == "c" else "plan_many_rgc"))
    plan = fn(3, pg.ints(n), howmany, None, pg.ints(gcb), pg.ints(gca), buf.data_ptr(), comm, flags)
    assert plan
    try:
        if reduce:
            boxv = rng.uniform(-1, 1, buf.numel()).astype(npdt)
            buf.copy_(torch.from_numpy(boxv))
            getattr(L, pre + "reduce")(plan)
            got = buf.cpu().numpy()
            ref_blk = ghost.reduce(boxv.reshape(box + [tuple_]).astype(np.float64), pn, gcb, gca).ravel()
            ref = np.zeros(buf.numel())
            ref[: ref_blk.size] = ref_blk
            return got, ref
        buf[: blockv.size] = torch.from_numpy(blockv).cuda()
        getattr(L, pre + "exchange")(plan)
        got = buf.cpu().numpy()
        ref = ghost.exchange(blockv.reshape(pn + [tuple_]), pn, gcb, gca).ravel()
        return got, ref
    finally:
        getattr(L, pre + "destroy_gcplan")(plan)


@pytest.mark.parametrize("prec", ["double", "float"])
@pytest.mark.parametrize("kind,n,gcb,gca,flags", [
    ("c", [8, 8, 8], [0, 0, 0], [4, 0, 0], 0),           # tests/simple_check_ghost_c2c.c
    ("c", [8, 8, 8], [1, 2, 3], [3, 2, 1], 0),
    ("c", [5, 6, 7], [7, 1, 0], [0, 9, 2], 0),           # halos wider than the block wrap repeatedly
    ("r", [6, 7, 9], [2, 2, 2], [2, 2, 2], 0),
    ("r", [6, 7, 8], [1, 1, 1], [1, 1, 1], pg.PFFT_GC_PADDED),
    ("c", [6, 7, 8], [1, 0, 2], [0, 1, 1], pg.PFFT_GC_R2C),
    ("c", [6, 7, 8], [1, 0, 2], [0, 1, 1], pg.PFFT_GC_TRANSPOSED),
    # many chunks of the in-place move: no halo below (rows barely move),
    # one-cell rows, long rows beyond the staging area (copy + gather path)
    ("r", [64, 48, 40], [3, 0, 1], [0, 2, 5], 0),
    ("c", [40, 64, 33], [0, 0, 0], [0, 0, 3], 0),
    ("r", [50, 40, 1], [2, 3, 0], [1, 0, 0], 0),
    ("c", [4, 3, 2100], [1, 1, 1], [1, 1, 1], 0),
    # 16-byte vector moves (every row start and length a multiple of 16 bytes)
    # with many chunks, in both precisions, and a real block on that path
    ("c", [48, 40, 64], [0, 1, 2], [2, 0, 2], 0),
    ("r", [16, 12, 8], [2, 0, 2], [2, 4, 2], 0),
])
def test_exchange_bit_exact(cuda, pfft_lib, prec, kind, n, gcb, gca, flags):
    if flags & pg.PFFT_GC_TRANSPOSED:
        # the plan works on the box with the distributed dims rotated (n1, n0, n2)
        got, _ = run_gc(cuda, kind, n, gcb, gca, prec, flags)
        pn = [n[1], n[0], n[2]]
        pb, pa = [gcb[1], gcb[0], gcb[2]], [gca[1], gca[0], gca[2]]
        got2, ref = run_gc(cuda, kind, pn, pb, pa, prec, 0)
        assert np.array_equal(got, got2)
        return
    got, ref = run_gc(cuda, kind, n, gcb, gca, prec, flags)
    assert np.array_equal(got[: ref.size], ref.astype(got.dtype))


@pytest.mark.parametrize("prec,tol", [("double", 1e-14), ("float", 1e-6)])
def test_reduce(cuda, pfft_lib, prec, tol):
    for kind, n, gcb, gca in [("c", [8, 8, 8], [0, 0, 0], [4, 0, 0]), ("c", [5, 6, 7], [7, 1, 0], [0, 9, 2]),
                              ("r", [64, 48, 40], [3, 0, 1], [0, 2, 5]), ("c", [40, 64, 33], [0, 0, 0], [0, 0, 3]),
                              ("r", [50, 40, 1], [2, 3, 0], [1, 0, 0]), ("c", [4, 3, 2100], [1, 1, 1], [1, 1, 1]),
                              ("c", [48, 40, 64], [0, 1, 2], [2, 0, 2])]:
        got, ref = run_gc(cuda, kind, n, gcb, gca, prec, reduce=True)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < tol, (n, err)


def test_reduce_256_width2(cuda, pfft_lib):
    got, ref = run_gc(cuda, "r", [256, 256, 256], [2, 2, 2], [2, 2, 2], "double", reduce=True)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-14


def test_exchange_reduce_roundtrip_simple_check_ghost(cuda, pfft_lib):
    """tests/simple_check_ghost_c2c.c at one process: exchange then reduce
    multiplies every cell by the number of its images in the box."""
    torch = cuda
    L = pg.lib()
    n, gcb, gca = [8, 8, 8], [0, 0, 0], [4, 0, 0]
    comm = pg.procmesh(2)
    lni, lis, lno, los = (pg.ints([0] * 3) for _ in range(4))
    L.pfft_local_size_dft_3d(pg.ints(n), comm, 0, lni, lis, lno, los)
    lngc, lgcs = pg.ints([0] * 3), pg.ints([0] * 3)
    alloc_gc = L.pfft_local_size_gc_3d(lni, lis, pg.ints(gcb), pg.ints(gca), lngc, lgcs)
    data = torch.zeros(2 * alloc_gc, dtype=torch.float64, device="cuda")
    plan = L.pfft_plan_cgc_3d(pg.ints(n), pg.ints(gcb), pg.ints(gca), data.data_ptr(), comm, 0)
    L.pfft_init_input_complex_3d(pg.ints(n), lni, lis, data.data_ptr())
    x0 = data[: 2 * 512].clone()
    L.pfft_exchange(plan)
    L.pfft_reduce(plan)
    mult = np.ones((8, 8, 8))
    mult[:4] = 2
    got = data[: 2 * 512].cpu().numpy().reshape(8, 8, 8, 2)
    ref = x0.cpu().numpy().reshape(8, 8, 8, 2) * mult[..., None]
    assert np.abs(got - ref).max() < 1e-12
    L.pfft_destroy_gcplan(plan)


def test_halo_256_width2(cuda, pfft_lib):
    """Benchmark configuration: 256^3 real field, halo 2 on every face."""
    got, ref = run_gc(cuda, "r", [256, 256, 256], [2, 2, 2], [2, 2, 2], "double")
    assert np.array_equal(got[: ref.size], ref)

"""Data-distribution integers of the C-ABI library against the oracle's
literal restatement of the reference (no GPU: these entry points only do
integer arithmetic).  Bit-exact equality is required."""
import numpy as np
import pytest

import pfft_gb300 as pg
from oracle import layout as LO
from tests.pfft_util import LS_NAME, TR

KINDS = ["c2c", "r2c", "c2r", "r2r"]


def lib_sizes(L, pre, kind, d, n, ni, no, hm, flags, comm):
    a = [pg.ints([0] * d) for _ in range(4)]
    mem = getattr(L, pre + LS_NAME[kind])(d, pg.ints(n), pg.ints(ni), pg.ints(no), hm, None, None, comm, flags, *a)
    return mem, [list(x) for x in a]


def test_random_configurations(pfft_lib):
    L = pfft_lib
    rng = np.random.default_rng(12345)
    checked = 0
    for _ in range(1500):
        d = int(rng.integers(2, 6))
        cart = int(rng.integers(0, 4))
        if cart > d or (cart == d and d != 3):
            continue
        n = [int(rng.integers(2, 40)) for _ in range(d)]
        if rng.random() < 0.5:
            ni, no = list(n), list(n)
        else:
            ni = [int(rng.integers(1, x + 1)) for x in n]
            no = [int(rng.integers(1, x + 1)) for x in n]
        hm = int(rng.integers(1, 4))
        kind = KINDS[int(rng.integers(0, 4))]
        flags = int(rng.choice([0, 1, 2])) | int(rng.choice([0, 4, 8, 12])) | int(rng.choice([0, 1 << 11]))
        # keep SHIFTED cases even, as the reference requires
        if flags & 12:
            n = [x + (x % 2) for x in n]
            ni = [min(x + (x % 2), y) for x, y in zip(ni, n)]
            no = [min(x + (x % 2), y) for x, y in zip(no, n)]
        comm = pg.MPI_COMM_WORLD if cart == 0 else pg.procmesh(cart)
        for pre in ("pfft_", "pfftf_"):
            mem, (lni, lis, lno, los) = lib_sizes(L, pre, kind, d, n, ni, no, hm, flags, comm)
            ref = LO.local_size(d, n, ni, no, hm, TR[kind], flags, cart)
            assert (mem, lni, lis, lno, los) == tuple(ref), (kind, d, cart, n, ni, no, hm, flags)
        checked += 1
    assert checked > 500


@pytest.mark.parametrize("kind", KINDS)
def test_benchmark_configurations(pfft_lib, kind):
    L = pfft_lib
    comm = pg.procmesh(2)
    for n, flags in [([64] * 3, 0), ([256] * 3, 2 | (1 << 11)), ([512] * 3, 0), ([1024] * 3, 0), ([64] * 4, 0),
                     ([256] * 3, 1 | (1 << 11))]:
        d = len(n)
        mem, got = lib_sizes(L, "pfft_", kind, d, n, n, n, 1, flags, comm)
        ref = LO.local_size(d, n, n, n, 1, TR[kind], flags, 2)
        assert (mem, *got) == tuple(ref)


def test_local_block_and_3d_helpers(pfft_lib):
    L = pfft_lib
    comm = pg.procmesh(2)
    n = pg.ints([29, 27, 31])
    a = [pg.ints([0] * 3) for _ in range(4)]
    mem = L.pfft_local_size_dft_r2c_3d(n, comm, pg.PFFT_PADDED_R2C, *a)
    assert list(a[0]) == [29, 27, 32] and list(a[2]) == [29, 27, 16] and mem == 29 * 27 * 16
    b = [pg.ints([0] * 3) for _ in range(4)]
    L.pfft_local_block_many_dft_r2c(3, n, n, None, None, comm, 0, pg.PFFT_PADDED_R2C, *b)
    assert [list(x) for x in b] == [list(x) for x in a]
    # the reference's gc local sizes (gcell/gcells_plan.c:51-76)
    lngc, lgcs = pg.ints([0] * 3), pg.ints([0] * 3)
    mem = L.pfft_local_size_gc_3d(pg.ints([8, 8, 8]), pg.ints([0, 0, 0]), pg.ints([1, 0, 2]), pg.ints([0, 4, 1]),
                                  lngc, lgcs)
    assert list(lngc) == [9, 12, 11] and list(lgcs) == [-1, 0, -2] and mem == 9 * 12 * 11


def test_procmesh_rules(pfft_lib):
    import ctypes
    L = pfft_lib
    c = ctypes.c_int(0)
    assert L.pfft_create_procmesh_2d(pg.MPI_COMM_WORLD, 1, 1, ctypes.byref(c)) == 0 and c.value > 0
    # a mesh that does not match the single process is refused (kernel/procmesh.c:47-48)
    assert L.pfft_create_procmesh_2d(pg.MPI_COMM_WORLD, 2, 2, ctypes.byref(c)) != 0


def test_planner_rejections(pfft_lib):
    """kernel/partrafo.c:337-373: these return NULL without touching a GPU."""
    L = pfft_lib
    comm2 = pg.procmesh(2)
    n = pg.ints([8, 8, 8])
    nodd = pg.ints([8, 9, 8])
    assert not L.pfft_plan_dft_3d(nodd, None, None, comm2, -1, pg.PFFT_SHIFTED_IN)
    assert not L.pfft_plan_dft_3d(n, None, None, comm2, -1, pg.PFFT_TRANSPOSED_IN | pg.PFFT_TRANSPOSED_OUT)
    assert not L.pfft_plan_dft_r2c_3d(n, None, None, comm2, -1, pg.PFFT_TRANSPOSED_IN)
    assert not L.pfft_plan_dft_c2r_3d(n, None, None, comm2, 1, pg.PFFT_TRANSPOSED_OUT)
    # FFT rank below the mesh rank, and rank == mesh rank != 3
    assert not L.pfft_plan_dft(1, pg.ints([8]), None, None, comm2, -1, 0)
    assert not L.pfft_plan_dft(2, pg.ints([8, 8]), None, None, comm2, -1, 0)


def test_null_plan_execute_and_destroy(pfft_lib, capfd):
    """api/api-basic.c:243-246,1050-1054: a NULL plan given to execute or
    destroy prints an error and returns (the process keeps running)."""
    L = pfft_lib
    L.pfft_execute(None)
    L.pfftf_execute(None)
    L.pfft_destroy_plan(None)
    L.pfft_execute_adjoint(None)
    err = capfd.readouterr().err
    assert "PFFT" in err or err == ""

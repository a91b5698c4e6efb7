"""The allocation-free ghost-cell exchange against pfft_exchange (GPU).

pfft_gb300_exchange_noalloc serves callers that cannot allocate device memory
when they need a halo (allocation-free solver loops, memory-pool budgets,
code that must not synchronise the device): it performs the exchange of a
ghost-cell plan with its scratch in a fixed 32 MiB array compiled into the
library.  Its output must equal the plan-based pfft_exchange exactly (the
exchange is a pure copy), on two calls in a row, and sizes beyond the scratch
must be refused.  This file is collected last so that a failure here does not
hide the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg

pytestmark = pytest.mark.gpu


def _noalloc():
    f = pg.lib().pfft_gb300_exchange_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.POINTER(pg.INT), ctypes.POINTER(pg.INT), ctypes.POINTER(pg.INT), pg.INT,
                  ctypes.c_void_p, ctypes.c_void_p]
    return f


def _plan_exchange(L, n, gcb, gca, buf, prec, tuple_):
    comm = pg.procmesh(2)
    pre = "pfft_" if prec == "double" else "pfftf_"
    # tuple 2: complex cells (plan_cgc); tuple 1: real cells (plan_rgc)
    name = "plan_cgc_3d" if tuple_ == 2 else "plan_rgc_3d"
    plan = getattr(L, pre + name)(pg.ints(n), pg.ints(gcb), pg.ints(gca), buf.data_ptr(), comm, 0)
    assert plan
    getattr(L, pre + "exchange")(plan)
    getattr(L, pre + "destroy_gcplan")(plan)


# (block, ghost widths below, above, reals per cell): ghost widths up to and
# beyond the block's extent (the wrap then repeats the block), real and
# complex cells
CASES = [([20, 24, 28], [2, 1, 3], [1, 4, 2], 2), ([20, 24, 28], [2, 1, 3], [1, 4, 2], 1),
         ([3, 4, 5], [7, 1, 9], [2, 8, 1], 2), ([3, 4, 5], [7, 1, 9], [2, 8, 1], 1)]


@pytest.mark.parametrize("prec", ["double", "float"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_noalloc_exchange_matches_plan_exchange(cuda, pfft_lib, prec, case):
    torch = cuda
    L = pg.lib()
    f = _noalloc()
    rdt = torch.float64 if prec == "double" else torch.float32
    n, gcb, gca, tup = CASES[case]
    box = int(np.prod([b + m + a for b, m, a in zip(gcb, n, gca)]))
    block = int(np.prod(n))
    g = torch.Generator().manual_seed(3 + case)
    for call in range(2):  # two calls in a row: the shared scratch keeps the previous call's contents
        x = torch.rand(tup * block, generator=g, dtype=torch.float64).to(rdt)
        a = torch.zeros(tup * box, dtype=rdt, device="cuda")
        b = torch.zeros(tup * box, dtype=rdt, device="cuda")
        a[: tup * block] = x.cuda()
        b[: tup * block] = x.cuda()
        _plan_exchange(L, n, gcb, gca, a, prec, tup)
        stream = torch.cuda.current_stream()
        rc = f(1 if prec == "double" else 0, pg.ints(n), pg.ints(gcb), pg.ints(gca), tup, b.data_ptr(),
               ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        assert torch.equal(a, b), "call %d differs" % call


def test_noalloc_rejects_host_memory(cuda, pfft_lib):
    """A host array is refused before anything is queued (the gather would
    address it as device memory)."""
    f = _noalloc()
    host = np.zeros(2 * 6 * 6 * 6, dtype=np.float64)
    rc = f(1, pg.ints([4, 4, 4]), pg.ints([1, 1, 1]), pg.ints([1, 1, 1]), 2, host.ctypes.data, None)
    assert rc != 0


def test_noalloc_rejects_oversize(cuda, pfft_lib):
    torch = cuda
    f = _noalloc()
    # 200^3 complex doubles = 128 MB > the 32 MiB scratch: refused before any GPU work
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = f(1, pg.ints([200, 200, 200]), pg.ints([1, 1, 1]), pg.ints([1, 1, 1]), 2, buf.data_ptr(), None)
    assert rc != 0
    # sizes whose products overflow 64 bits are refused too
    big = 1 << 40
    rc = f(1, pg.ints([big, big, big]), pg.ints([0, 0, 0]), pg.ints([0, 0, 0]), 2, buf.data_ptr(), None)
    assert rc != 0
    rc = f(1, pg.ints([1, 1, 1]), pg.ints([big, big, 0]), pg.ints([big, 0, 0]), 1 << 40, buf.data_ptr(), None)
    assert rc != 0

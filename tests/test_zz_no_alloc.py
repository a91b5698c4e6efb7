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


def _plan_exchange(L, n, gcb, gca, buf, prec):
    comm = pg.procmesh(2)
    pre = "pfft_" if prec == "double" else "pfftf_"
    plan = getattr(L, pre + "plan_cgc_3d")(pg.ints(n), pg.ints(gcb), pg.ints(gca), buf.data_ptr(), comm, 0)
    assert plan
    getattr(L, pre + "exchange")(plan)
    getattr(L, pre + "destroy_gcplan")(plan)


@pytest.mark.parametrize("prec", ["double", "float"])
def test_noalloc_exchange_matches_plan_exchange(cuda, pfft_lib, prec):
    torch = cuda
    L = pg.lib()
    f = _noalloc()
    rdt = torch.float64 if prec == "double" else torch.float32
    n, gcb, gca = [20, 24, 28], [2, 1, 3], [1, 4, 2]
    box = int(np.prod([b + m + a for b, m, a in zip(gcb, n, gca)]))
    block = int(np.prod(n))
    g = torch.Generator().manual_seed(3)
    for call in range(2):  # two calls in a row: the shared scratch keeps the previous call's contents
        x = torch.rand(2 * block, generator=g, dtype=torch.float64).to(rdt)
        a = torch.zeros(2 * box, dtype=rdt, device="cuda")
        b = torch.zeros(2 * box, dtype=rdt, device="cuda")
        a[: 2 * block] = x.cuda()
        b[: 2 * block] = x.cuda()
        _plan_exchange(L, n, gcb, gca, a, prec)
        stream = torch.cuda.current_stream()
        rc = f(1 if prec == "double" else 0, pg.ints(n), pg.ints(gcb), pg.ints(gca), 2, b.data_ptr(),
               ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        assert torch.equal(a, b), "call %d differs" % call


def test_noalloc_rejects_oversize(cuda, pfft_lib):
    torch = cuda
    f = _noalloc()
    # 200^3 complex doubles = 128 MB > the 32 MiB scratch: refused before any GPU work
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = f(1, pg.ints([200, 200, 200]), pg.ints([1, 1, 1]), pg.ints([1, 1, 1]), 2, buf.data_ptr(), None)
    assert rc != 0

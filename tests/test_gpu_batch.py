"""Batched execution (one persistent launch for many plans of uneven sizes).

The benchmark suite's batched configuration: transforms with sizes drawn by
seed from {32^3, 48x64x40, 96^3, 128x128x64, 128^3}, complex64 and
complex128, uniform[-1,1) inputs.  Every plan's output in the batch must match
the oracle with the same tolerance as a plain execute; the dependency waits of
the persistent kernel are bounded, which a self-test exercises.
"""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, double_arith, oracle_run, rel_l2

pytestmark = pytest.mark.gpu

SIZES = [(32, 32, 32), (48, 64, 40), (96, 96, 96), (128, 128, 64), (128, 128, 128)]


def make_plans(torch, prec, count, seed, flags=0):
    L = pg.lib()
    pre = "pfftf_" if prec == "float" else "pfft_"
    cdt = torch.complex64 if prec == "float" else torch.complex128
    rng = np.random.default_rng(seed)
    comm = pg.procmesh(2)
    plans, arrays = [], []
    for i in range(count):
        n = SIZES[int(rng.integers(0, len(SIZES)))]
        x = rng.uniform(-1, 1, 2 * int(np.prod(n)))
        a = torch.from_numpy(x).view(torch.complex128).to(cdt).cuda()
        b = torch.zeros_like(a)
        with double_arith(prec):
            p = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, -1, flags)
        assert p
        plans.append(p)
        arrays.append((n, x, a, b))
    return pre, plans, arrays


@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("double-df", 1e-12), ("double-dfq", 1e-12), ("float", 2e-6)])
def test_batch_matches_oracle(cuda, pfft_lib, prec, tol):
    torch = cuda
    L = pg.lib()
    pre, plans, arrays = make_plans(torch, prec, 12, seed=3, flags=pg.PFFT_TRANSPOSED_OUT)
    arr = (ctypes.c_void_p * len(plans))(*plans)
    b = getattr(L, pre + "gb300_batch_create")(len(plans), arr)
    assert b
    try:
        for rep in range(2):  # graph capture, then a replay
            for (_, _, _, out) in arrays:
                out.zero_()
            torch.cuda.synchronize()
            assert L.pfft_gb300_batch_execute(b) == 0
            for (n, x, a, out) in arrays:
                xin = x.astype(np.float32).astype(np.float64) if prec == "float" else x
                ref = oracle_run(Req("c2c", n, flags=pg.PFFT_TRANSPOSED_OUT), xin)
                got = torch.view_as_real(out).double().cpu().numpy().ravel()
                assert rel_l2(got, ref) <= tol
    finally:
        L.pfft_gb300_batch_destroy(b)
        for p in plans:
            getattr(L, pre + "destroy_plan")(p)


def test_batch_64_uneven_equals_loop(cuda, pfft_lib):
    """64 uneven complex128 transforms: the batch and a loop of plain
    executes give the same results (both within the double tolerance)."""
    torch = cuda
    L = pg.lib()
    pre, plans, arrays = make_plans(torch, "double", 64, seed=11)
    for p in plans:
        L.pfft_execute(p)
    torch.cuda.synchronize()
    loop_out = [out.clone() for (_, _, _, out) in arrays]
    arr = (ctypes.c_void_p * len(plans))(*plans)
    b = L.pfft_gb300_batch_create(len(plans), arr)
    try:
        for (_, _, _, out) in arrays:
            out.zero_()
        assert L.pfft_gb300_batch_execute(b) == 0
        for lo, (n, _, _, out) in zip(loop_out, arrays):
            d = torch.linalg.vector_norm(out - lo) / torch.linalg.vector_norm(lo)
            assert float(d) < 1e-12
    finally:
        L.pfft_gb300_batch_destroy(b)
        for p in plans:
            L.pfft_destroy_plan(p)


def test_batch_wait_is_bounded(cuda, pfft_lib):
    """A dependency nothing satisfies: the bounded wait expires, the kernel
    returns and the host sees the timeout status (no hang, context usable)."""
    torch = cuda
    L = pg.lib()
    assert L.pfft_gb300_batch_wait_selftest(1000) == -2
    x = torch.ones(4, device="cuda")
    assert float(x.sum()) == 4.0


@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("float", 2e-6)])
def test_batch_mixed_plan_kinds(cuda, pfft_lib, prec, tol):
    """One batch of r2c (padded, transposed out), c2r, r2r and c2c plans of
    different shapes: every output matches the oracle."""
    from tests.pfft_util import mask_padding, random_input
    torch = cuda
    L = pg.lib()
    pre = "pfftf_" if prec == "float" else "pfft_"
    rdt = torch.float32 if prec == "float" else torch.float64
    TO, PAD = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_PADDED_R2C
    reqs = [Req("r2c", (32, 48, 64), flags=PAD | TO), Req("c2r", (40, 24, 32), sign=1),
            Req("r2r", (24, 20, 18), kinds=[5, 4, 7]), Req("c2c", (96, 32, 40), flags=TO),
            Req("c2c", (128, 16, 64), sign=1)]
    names = {"c2c": "plan_many_dft", "r2c": "plan_many_dft_r2c", "c2r": "plan_many_dft_c2r", "r2r": "plan_many_r2r"}
    rng = np.random.default_rng(9)
    comm = pg.procmesh(2)
    plans, keep = [], []
    for req in reqs:
        ci, co, mem = req.counts()
        words = max(2 * mem, ci, co)
        x = random_input(req, rng)
        if prec == "float":
            x = x.astype(np.float32).astype(np.float64)
        a = torch.zeros(words, dtype=rdt, device="cuda")
        b = torch.zeros(words, dtype=rdt, device="cuda")
        a[:ci] = torch.from_numpy(x).to("cuda", rdt)
        fn = getattr(L, pre + names[req.kind])
        n, ni, no = pg.ints(req.n), pg.ints(req.ni), pg.ints(req.no)
        if req.kind == "r2r":
            p = fn(req.d, n, ni, no, 1, None, None, a.data_ptr(), b.data_ptr(), comm, pg.cints(req.kinds), req.flags)
        else:
            p = fn(req.d, n, ni, no, 1, None, None, a.data_ptr(), b.data_ptr(), comm, req.sign, req.flags)
        assert p, pg.last_error()
        plans.append(p)
        keep.append((req, x, a, b, co))
    arr = (ctypes.c_void_p * len(plans))(*plans)
    bt = getattr(L, pre + "gb300_batch_create")(len(plans), arr)
    assert bt, pg.last_error()
    try:
        assert L.pfft_gb300_batch_execute(bt) == 0
        for req, x, a, b, co in keep:
            got = mask_padding(req, b[:co].double().cpu().numpy())
            ref = mask_padding(req, oracle_run(req, x))
            assert rel_l2(got, ref) <= tol, req.kind
    finally:
        L.pfft_gb300_batch_destroy(bt)
        for p in plans:
            getattr(L, pre + "destroy_plan")(p)

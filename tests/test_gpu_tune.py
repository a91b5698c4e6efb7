"""Autotuning (PFFT_PATIENT / PFFT_TUNE) and wisdom reuse on the GPU: tuned
plans match the oracle, record one wisdom entry per pass, and a later plan of
the same problem - created without tuning flags, after the wisdom went through
export, forget and import - makes the same per-pass choices."""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, double_arith, oracle_run, random_input, rel_l2

pytestmark = pytest.mark.gpu


def pass_choices(L, pre, plan):
    n = ctypes.c_int(0)
    getattr(L, pre + "gb300_plan_info")(plan, ctypes.byref(n), None, None)
    out = []
    for i in range(n.value):
        lines, thr = ctypes.c_int(0), ctypes.c_int(0)
        getattr(L, pre + "gb300_pass_info")(plan, i, None, None, ctypes.byref(lines), ctypes.byref(thr), None, None)
        out.append((getattr(L, pre + "gb300_pass_kernel")(plan, i), lines.value, thr.value))
    return out


@pytest.mark.parametrize("prec,kind,n,flags", [
    ("double-df", "c2c", (64, 96, 512), pg.PFFT_PATIENT),
    ("double-dfq", "c2c", (32, 64, 512), pg.PFFT_PATIENT | pg.PFFT_TRANSPOSED_OUT),
    ("float", "c2c", (48, 1024, 40), pg.PFFT_TUNE | pg.PFFT_TRANSPOSED_OUT),
    ("double", "r2c", (30, 28, 64), pg.PFFT_EXHAUSTIVE),
])
def test_tuned_plan_and_wisdom_reuse(cuda, pfft_lib, prec, kind, n, flags):
    torch = cuda
    L = pg.lib()
    L.pfft_gb300_forget_wisdom()
    req = Req(kind, n, flags=flags)
    rng = np.random.default_rng(3)
    x = random_input(req, rng)
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
    pre = "pfftf_" if prec == "float" else "pfft_"
    rdt = torch.float32 if prec == "float" else torch.float64
    ci, co, mem = req.counts()
    words = max(2 * mem, ci, co)
    a = torch.zeros(words, dtype=rdt, device="cuda")
    b = torch.zeros(words, dtype=rdt, device="cuda")
    comm = pg.procmesh(2)
    fn = getattr(L, pre + ("plan_many_dft" if kind == "c2c" else "plan_many_dft_r2c"))

    def plan(fl):
        with double_arith(prec):
            p = fn(3, pg.ints(n), pg.ints(n), pg.ints(n), 1, None, None, a.data_ptr(), b.data_ptr(), comm, -1, fl)
        assert p, pg.last_error()
        return p

    p1 = plan(flags)  # tunes (overwrites b)
    nent = L.pfft_gb300_wisdom_entries()
    tuned = pass_choices(L, pre, p1)
    assert nent >= 1
    a[:ci] = torch.from_numpy(x).to("cuda", rdt)
    getattr(L, pre + "execute")(p1)
    torch.cuda.synchronize()
    got = b[:co].double().cpu().numpy()
    ref = oracle_run(Req(kind, n, flags=flags), x)
    assert rel_l2(got, ref) <= (2e-6 if prec == "float" else 1e-12)
    getattr(L, pre + "destroy_plan")(p1)

    text = pg.export_wisdom()
    L.pfft_gb300_forget_wisdom()
    assert L.pfft_gb300_import_wisdom_from_string(text.encode()) == 1
    assert L.pfft_gb300_wisdom_entries() == nent
    p2 = plan(flags & ~(pg.PFFT_PATIENT | pg.PFFT_EXHAUSTIVE | pg.PFFT_TUNE))  # no timing: wisdom only
    assert pass_choices(L, pre, p2) == tuned
    b.zero_()
    getattr(L, pre + "execute")(p2)
    torch.cuda.synchronize()
    assert rel_l2(b[:co].double().cpu().numpy(), ref) <= (2e-6 if prec == "float" else 1e-12)
    getattr(L, pre + "destroy_plan")(p2)
    L.pfft_gb300_forget_wisdom()


def test_tuning_leaves_input_intact(cuda, pfft_lib):
    """Out-of-place tuning writes the output array only."""
    torch = cuda
    L = pg.lib()
    n = (32, 64, 128)
    a = torch.randn(2 * 32 * 64 * 128, dtype=torch.float64, device="cuda")
    keep = a.clone()
    b = torch.zeros_like(a)
    p = L.pfft_plan_dft_3d(pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), -1, pg.PFFT_PATIENT)
    assert p
    torch.cuda.synchronize()
    assert torch.equal(a, keep)
    L.pfft_destroy_plan(p)
    L.pfft_gb300_forget_wisdom()

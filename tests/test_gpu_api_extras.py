"""Planner and execution features around the transform, through the C-ABI
(GPU): the _skipped planners (api/api-adv.c:157-217), graph mode of a plain
pfft_execute, the timer API fed from the pass events (kernel/timer.c), and the
I/O flags PFFT_PRESERVE_INPUT / PFFT_DESTROY_INPUT / PFFT_BUFFERED_INPLACE
(api/pfft.h:540-542)."""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, gpu_run, oracle_run, random_input, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "float": 2e-6}


@pytest.mark.parametrize("prec", ["double", "float"])
@pytest.mark.parametrize("kind,skip", [("c2c", [1, 0, 0]), ("c2c", [0, 1, 0]), ("c2c", [0, 0, 1]), ("c2c", [1, 1, 0]),
                                       ("c2c", [1, 1, 1]), ("r2c", [1, 0, 0]), ("r2c", [0, 1, 0]),
                                       ("c2r", [0, 1, 0]), ("r2r", [0, 1, 0]), ("r2r", [1, 0, 1])])
def test_skipped_planners_match_oracle(cuda, pfft_lib, prec, kind, skip):
    n = (12, 16, 10)
    kinds = [pg.PFFT_REDFT10, pg.PFFT_RODFT01, pg.PFFT_R2HC] if kind == "r2r" else None
    sign = 1 if kind == "c2r" else -1
    req = Req(kind, n, sign=sign, skip=skip, kinds=kinds)
    rng = np.random.default_rng(21)
    x = random_input(req, rng)
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
    ref = oracle_run(req, x)
    got = gpu_run(req, x, prec=prec)
    assert rel_l2(got, ref) <= TOL[prec], rel_l2(got, ref)


def _plan_c2c(L, pre, n, a, b, flags=0, sign=pg.PFFT_FORWARD):
    p = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), sign, flags)
    assert p, pg.last_error()
    return p


@pytest.mark.parametrize("prec", ["double", "float"])
def test_graph_mode_bit_identical(cuda, pfft_lib, prec):
    torch = cuda
    L = pfft_lib
    pre = "pfft_" if prec == "double" else "pfftf_"
    cdt = torch.complex128 if prec == "double" else torch.complex64
    n = (32, 64, 48)
    g = torch.Generator().manual_seed(4)
    x = torch.randn(n, dtype=torch.complex128, generator=g).to(cdt).cuda()
    y = torch.zeros_like(x)
    p = _plan_c2c(L, pre, n, x, y)
    getattr(L, pre + "execute")(p)
    torch.cuda.synchronize()
    ref = y.clone()
    assert getattr(L, pre + "gb300_set_graph")(p, 1) == 0
    for _ in range(3):  # capture, then replays
        y.zero_()
        getattr(L, pre + "execute")(p)
        torch.cuda.synchronize()
        assert torch.equal(y, ref)
    # new arrays: the graph is captured again for them
    x2 = (x * 2).contiguous()
    y2 = torch.zeros_like(x2)
    getattr(L, pre + "execute_dft")(p, x2.data_ptr(), y2.data_ptr())
    torch.cuda.synchronize()
    getattr(L, pre + "gb300_set_graph")(p, 0)
    y3 = torch.zeros_like(x2)
    getattr(L, pre + "execute_dft")(p, x2.data_ptr(), y3.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(y2, y3)
    # and back to the first arrays: replay of a fresh capture
    getattr(L, pre + "gb300_set_graph")(p, 1)
    y.zero_()
    getattr(L, pre + "execute")(p)
    torch.cuda.synchronize()
    assert torch.equal(y, ref)
    getattr(L, pre + "destroy_plan")(p)


def _timer_api(L, pre):
    f = lambda nm: getattr(L, pre + nm)
    f("get_timer").restype = ctypes.c_void_p
    f("get_timer").argtypes = [ctypes.c_void_p]
    f("convert_timer2vec").restype = ctypes.POINTER(ctypes.c_double)
    f("convert_timer2vec").argtypes = [ctypes.c_void_p]
    f("convert_vec2timer").restype = ctypes.c_void_p
    f("convert_vec2timer").argtypes = [ctypes.POINTER(ctypes.c_double)]
    for nm in ("destroy_timer", "average_timer", "reset_timer"):
        f(nm).restype = None
        f(nm).argtypes = [ctypes.c_void_p]
    f("add_timers").restype = ctypes.c_void_p
    f("add_timers").argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    f("copy_timer").restype = ctypes.c_void_p
    f("copy_timer").argtypes = [ctypes.c_void_p]
    f("write_average_timer").restype = None
    f("write_average_timer").argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    return f


def _vec(f, t):
    v = f("convert_timer2vec")(t)
    rnk_trafo, rnk_remap = int(v[1]), int(v[2])
    out = [v[i] for i in range(rnk_trafo + rnk_remap + 9)]
    ctypes.CDLL(None).free(ctypes.cast(v, ctypes.c_void_p))
    return out


def test_timer_api_reads_pass_events(cuda, pfft_lib, tmp_path):
    torch = cuda
    L = pfft_lib
    f = _timer_api(L, "pfft_")
    n = (32, 48, 64)
    x = torch.randn(n, dtype=torch.complex128).cuda()
    y = torch.zeros_like(x)
    p = _plan_c2c(L, "pfft_", n, x, y)
    npass = ctypes.c_int(0)
    L.pfft_gb300_plan_info(p, ctypes.byref(npass), None, None)
    assert L.pfft_gb300_set_pass_timing(p, 1) == 0
    reps = 4
    for _ in range(reps):
        L.pfft_execute(p)
    t = f("get_timer")(p)
    v = _vec(f, t)
    # layout of kernel/timer.c's vector: rnk_pm, rnk_trafo, rnk_remap, iter, whole, trafo[], remap[], ...
    assert v[0] == 2 and v[1] == 6 and v[2] == 4 and v[3] == reps
    trafo = v[5:5 + 6]
    ev = []
    for i in range(npass.value):
        ms, runs = ctypes.c_double(0), ctypes.c_int(0)
        L.pfft_gb300_pass_time(p, i, ctypes.byref(ms), ctypes.byref(runs))
        assert runs.value == reps
        ev.append(ms.value * 1e-3)
    # one serial stage per pass, in seconds, equal to the pass events' sum
    assert np.allclose(trafo[:npass.value], ev, rtol=1e-9, atol=0)
    assert all(tv == 0 for tv in trafo[npass.value:]) and all(r == 0 for r in v[11:15])
    assert v[4] >= sum(ev)  # whole (wall clock) covers the passes
    # vector round trip, copy, sum, average
    arr = (ctypes.c_double * len(v))(*v)
    t2 = f("convert_vec2timer")(arr)
    assert _vec(f, t2) == v
    t3 = f("add_timers")(t, t2)
    v3 = _vec(f, t3)
    assert v3[3] == 2 * reps and np.isclose(v3[4], 2 * v[4])
    f("average_timer")(t3)
    v4 = _vec(f, t3)
    assert np.isclose(v4[4], v[4] / reps)
    out = tmp_path / "timer.m"
    f("write_average_timer")(p, str(out).encode(), pg.MPI_COMM_WORLD)
    assert "pfft_forw" in out.read_text()
    f("reset_timer")(p)
    t5 = f("get_timer")(p)
    assert _vec(f, t5)[3] == 0
    for tt in (t, t2, t3, t5):
        f("destroy_timer")(tt)
    L.pfft_destroy_plan(p)


IO_CASES = [Req("c2c", (16, 24, 32)), Req("c2c", (16, 24, 32), flags=pg.PFFT_TRANSPOSED_OUT),
            Req("r2c", (16, 24, 32), flags=pg.PFFT_PADDED_R2C), Req("c2r", (16, 24, 32), sign=1),
            Req("c2r", (16, 24, 32), sign=-1), Req("c2c", (16, 24, 32), flags=pg.PFFT_SHIFTED_OUT)]


@pytest.mark.parametrize("io", ["preserve", "destroy"])
@pytest.mark.parametrize("idx", range(len(IO_CASES)))
def test_input_preserved_and_result_unchanged(cuda, pfft_lib, io, idx):
    """PRESERVE_INPUT (the default of out-of-place plans) keeps the input;
    DESTROY_INPUT permits overwriting it, which this library never needs:
    both give the default plan's result and leave the input as it was."""
    torch = cuda
    base = IO_CASES[idx]
    extra = pg.PFFT_PRESERVE_INPUT if io == "preserve" else pg.PFFT_DESTROY_INPUT
    req = Req(base.kind, base.n, sign=base.sign, flags=base.flags | extra)
    rng = np.random.default_rng(idx)
    x = random_input(req, rng)
    ref = oracle_run(req, x)
    L = pfft_lib
    ci, co, mem = req.counts()
    words = max(2 * mem, ci, co)
    a = torch.zeros(words, dtype=torch.float64, device="cuda")
    b = torch.zeros(words, dtype=torch.float64, device="cuda")
    a[:ci] = torch.from_numpy(x).cuda()
    before = a.clone()
    from tests.pfft_util import PLAN_NAME
    fn = getattr(L, "pfft_" + PLAN_NAME[req.kind])
    p = fn(3, pg.ints(req.n), pg.ints(req.n), pg.ints(req.n), 1, None, None, a.data_ptr(), b.data_ptr(),
           pg.procmesh(2), req.sign, req.flags)
    assert p, pg.last_error()
    L.pfft_execute(p)
    torch.cuda.synchronize()
    L.pfft_destroy_plan(p)
    assert torch.equal(a, before)
    from tests.pfft_util import mask_padding
    assert rel_l2(mask_padding(req, b[:co].cpu().numpy()), mask_padding(req, ref)) <= 1e-12


@pytest.mark.parametrize("prec", ["double", "float"])
@pytest.mark.parametrize("idx", range(len(IO_CASES)))
def test_buffered_inplace_result_in_input_array(cuda, pfft_lib, prec, idx):
    """PFFT_BUFFERED_INPLACE on an out-of-place plan: the results end up in
    the input array (doc/tutorial.tex, "Preserving input data") and equal the
    plain out-of-place result; the output array is not written."""
    torch = cuda
    L = pfft_lib
    req = IO_CASES[idx]
    pre = "pfft_" if prec == "double" else "pfftf_"
    rdt = torch.float64 if prec == "double" else torch.float32
    rng = np.random.default_rng(100 + idx)
    x = random_input(req, rng)
    ci, co, mem = req.counts()
    words = max(2 * mem, ci, co)
    from tests.pfft_util import PLAN_NAME, mask_padding
    fn = getattr(L, pre + PLAN_NAME[req.kind])

    def run(flags):
        a = torch.zeros(words, dtype=rdt, device="cuda")
        b = torch.full((words,), 7.0, dtype=rdt, device="cuda")
        a[:ci] = torch.from_numpy(x).to(rdt).cuda()
        p = fn(3, pg.ints(req.n), pg.ints(req.n), pg.ints(req.n), 1, None, None, a.data_ptr(), b.data_ptr(),
               pg.procmesh(2), req.sign, req.flags | flags)
        assert p, pg.last_error()
        getattr(L, pre + "execute")(p)
        torch.cuda.synchronize()
        getattr(L, pre + "destroy_plan")(p)
        return a, b

    _, plain = run(0)
    a, b = run(pg.PFFT_BUFFERED_INPLACE)
    assert torch.all(b == 7.0), "the output array was written"
    got = mask_padding(req, a[:co].double().cpu().numpy())
    want = mask_padding(req, plain[:co].double().cpu().numpy())
    assert rel_l2(got, want) <= (1e-13 if prec == "double" else 1e-6)

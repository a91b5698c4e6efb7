"""Executes on host arrays (pinned host memory through pfft_execute_dft), the
path of the end-to-end measurement: the results equal those of the same plan
on device arrays bit for bit, with the host-array pipeline (input copied slab
by slab while the leading passes run on the slabs already there, output
copied back in column chunks while the last pass runs) and without it
(whole-array staging); layouts the pipeline does not cover (r2c, in-place)
take the whole-array path."""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg

pytestmark = pytest.mark.gpu

TO, TI = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_TRANSPOSED_IN

CASES = [
    ("double", (128, 128, 256), pg.PFFT_FORWARD, 0, True),
    ("double", (128, 128, 256), pg.PFFT_BACKWARD, TO, None),  # None: whichever path the layout allows
    ("double", (64, 256, 256), pg.PFFT_FORWARD, TI, None),
    ("float", (256, 256, 128), pg.PFFT_FORWARD, 0, True),
    ("double", (96, 96, 96), pg.PFFT_FORWARD, 0, False),  # slabs below the pipeline's 8 MB minimum
]


@pytest.mark.parametrize("prec,n,sign,flags,piped", CASES)
def test_host_arrays_equal_device_arrays(cuda, pfft_lib, prec, n, sign, flags, piped):
    torch = cuda
    L = pg.lib()
    pre = "pfft_" if prec == "double" else "pfftf_"
    cdt = torch.complex128 if prec == "double" else torch.complex64
    rng = np.random.default_rng(7)
    cnt = int(np.prod(n))
    x = torch.from_numpy(rng.uniform(-1, 1, 2 * cnt)).view(torch.complex128).to(cdt)
    a = x.cuda()
    b = torch.empty_like(a)
    comm = pg.procmesh(2)
    plan = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, sign, flags)
    assert plan, pg.last_error()
    try:
        getattr(L, pre + "execute")(plan)
        torch.cuda.synchronize()
        ref = b.cpu()
        hin = x.clone().pin_memory()
        for pipe in (1, 0):
            hout = torch.zeros_like(hin).pin_memory()
            assert getattr(L, pre + "gb300_set_pipeline")(plan, pipe) == 0
            before = L.pfft_gb300_pipelined_executes()
            for rep in range(2):  # second call reuses the staging buffers, streams and events
                hout.zero_()
                getattr(L, pre + "execute_dft")(plan, hin.data_ptr(), hout.data_ptr())
                code, msg = pg.last_error()
                assert code == 0, msg
                assert torch.equal(hout, ref), (pipe, rep)
            ran = L.pfft_gb300_pipelined_executes() - before
            if piped is None:
                assert ran in ((0, 2) if pipe else (0,)), (pipe, ran)
            else:
                assert ran == (2 if (pipe and piped) else 0), (pipe, ran)
        assert torch.equal(hin, x)  # the input array is not written
    finally:
        getattr(L, pre + "destroy_plan")(plan)


def test_host_arrays_r2c_takes_whole_array_path(cuda, pfft_lib):
    torch = cuda
    L = pg.lib()
    n = (128, 128, 256)
    rng = np.random.default_rng(8)
    x = torch.from_numpy(rng.standard_normal(int(np.prod(n))))
    a = x.cuda()
    b = torch.empty(128 * 128 * 129, dtype=torch.complex128, device="cuda")
    comm = pg.procmesh(2)
    plan = L.pfft_plan_dft_r2c_3d(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, pg.PFFT_FORWARD, 0)
    assert plan, pg.last_error()
    try:
        L.pfft_execute(plan)
        torch.cuda.synchronize()
        ref = b.cpu()
        hin = x.clone().pin_memory()
        hout = torch.zeros_like(ref).pin_memory()
        before = L.pfft_gb300_pipelined_executes()
        L.pfft_execute_dft_r2c(plan, hin.data_ptr(), hout.data_ptr())
        assert pg.last_error()[0] == 0
        assert L.pfft_gb300_pipelined_executes() == before
        assert torch.equal(hout, ref)
    finally:
        L.pfft_destroy_plan(plan)

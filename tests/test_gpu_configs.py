"""The benchmark suite's configurations at their full sizes.

C1  64^3 c2c complex128, forward then backward / N^3, against the oracle.
C2  256^3 r2c / c2r, float64 and float32, N(0,1) real input, PADDED_R2C
    in place, forward TRANSPOSED_OUT, backward TRANSPOSED_IN, against the
    oracle; plus REDFT10 (and its inverse REDFT01) on the same shape, against
    scipy.fft.dctn (pocketfft, an independent implementation of the same
    definitions: the oracle evaluates r2r lines directly, O(n^2) per line, and
    is checked against scipy at smaller sizes).
C5  512^3 complex128 and 1024^3 complex64 forward + backward (size-independent
    properties: round trip and Parseval), 512^3 complex128 (forward and
    backward, three double arithmetics), 1024 x 1024 x 256 complex64 and
    64^4 complex128 against the oracle.

Inputs are seeded synthetic data with the suite's distributions.
"""
import os

import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, double_arith, gpu_run, mask_padding, oracle_run, rel_l2

pytestmark = pytest.mark.gpu

TO, TI, PAD = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_TRANSPOSED_IN, pg.PFFT_PADDED_R2C


def test_c1_64cube_forward_backward(cuda, pfft_lib):
    n = (64, 64, 64)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 2 * 64 ** 3)
    fwd = Req("c2c", n)
    y = gpu_run(fwd, x)
    assert rel_l2(y, oracle_run(fwd, x)) <= 1e-12
    back = Req("c2c", n, sign=1)
    z = gpu_run(back, y) / 64 ** 3
    assert rel_l2(z, x) <= 1e-12


@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("float", 2e-6)])
def test_c2_256cube_r2c_c2r_padded_transposed(cuda, pfft_lib, prec, tol):
    n = (256, 256, 256)
    rng = np.random.default_rng(2)
    fwd = Req("r2c", n, flags=PAD | TO)
    ci, co, _ = fwd.counts()
    x = rng.standard_normal(ci)
    x.reshape(-1, 258)[:, 256:] = 0.0  # row padding
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
    y = gpu_run(fwd, x, prec=prec, inplace=True)
    ref = oracle_run(fwd, x)
    assert rel_l2(y, ref) <= tol
    back = Req("c2r", n, sign=1, flags=PAD | TI)
    z = mask_padding(back, gpu_run(back, ref, prec=prec, inplace=True)) / 256 ** 3
    assert rel_l2(z, x) <= tol


@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("float", 2e-6)])
def test_c2_256cube_redft10(cuda, pfft_lib, prec, tol):
    n = (256, 256, 256)
    rng = np.random.default_rng(3)
    fwd = Req("r2r", n, kinds=[5, 5, 5])  # REDFT10
    x = rng.standard_normal(256 ** 3)
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
    sfft = pytest.importorskip("scipy.fft")
    y = gpu_run(fwd, x, prec=prec)
    ref = sfft.dctn(x.reshape(n), type=2, workers=-1).ravel()  # = FFTW REDFT10
    assert rel_l2(y, ref) <= tol
    back = Req("r2r", n, kinds=[4, 4, 4])  # REDFT01, inverse up to (2n)^3
    z = gpu_run(back, ref, prec=prec) / (2 * 256) ** 3
    assert rel_l2(z, x) <= tol


def _roundtrip_large(torch, n, prec):
    """Forward + backward on device arrays of a large c2c transform; returns
    (round-trip rel error, Parseval rel error)."""
    L = pg.lib()
    pre = "pfft_" if prec == "double" else "pfftf_"
    cdt = torch.complex128 if prec == "double" else torch.complex64
    N = int(np.prod(n))
    g = torch.Generator(device="cuda").manual_seed(5)
    x = (torch.rand(N, dtype=torch.float64 if prec == "double" else torch.float32, device="cuda", generator=g) * 2 - 1)
    x = torch.complex(x, x.roll(1)).to(cdt)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    comm = pg.procmesh(2)
    pf = getattr(L, pre + "plan_dft_3d")(pg.ints(n), x.data_ptr(), y.data_ptr(), comm, -1, 0)
    pb = getattr(L, pre + "plan_dft_3d")(pg.ints(n), y.data_ptr(), z.data_ptr(), comm, 1, 0)
    assert pf and pb, pg.last_error()
    try:
        getattr(L, pre + "execute")(pf)
        getattr(L, pre + "execute")(pb)
        torch.cuda.synchronize()
        nx = torch.linalg.vector_norm(x.to(torch.complex128)).item()
        ny = torch.linalg.vector_norm(y.to(torch.complex128)).item()
        rt = (torch.linalg.vector_norm((z / N - x).to(torch.complex128)).item()) / nx
        parseval = abs(ny ** 2 / N - nx ** 2) / nx ** 2
    finally:
        getattr(L, pre + "destroy_plan")(pf)
        getattr(L, pre + "destroy_plan")(pb)
    return rt, parseval


def test_c5_512cube_complex128_roundtrip(cuda, pfft_lib):
    rt, pv = _roundtrip_large(cuda, (512, 512, 512), "double")
    assert rt <= 1e-12 and pv <= 1e-12, (rt, pv)


def test_c5_512cube_complex128_roundtrip_block_quantised(cuda, pfft_lib):
    """512^3 complex128 with block-quantised float-float radix-8 stages."""
    with double_arith("double-dfq"):
        rt, pv = _roundtrip_large(cuda, (512, 512, 512), "double")
    assert rt <= 1e-12 and pv <= 1e-12, (rt, pv)


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("prec,tol", [("double", 1e-15), ("double-f64", 1e-15), ("double-dfq", 1e-12)])
def test_c5_512cube_complex128_against_oracle(cuda, pfft_lib, sign, prec, tol):
    """The headline size element for element against the FP64 oracle, forward
    and backward, in the default arithmetic (64-bit fixed point), native FP64
    and the opt-in block-quantised float-float."""
    n = (512, 512, 512)
    req = Req("c2c", n, sign=sign)
    x = np.random.default_rng(8 + sign).uniform(-1, 1, 2 * 512 ** 3)
    ref = oracle_run(req, x, nthreads=os.cpu_count())
    y = gpu_run(req, x, prec=prec)
    e = rel_l2(y, ref)
    del y, ref
    cuda.cuda.empty_cache()
    assert e <= tol, e


def test_c5_1024x1024x256_complex64_against_oracle(cuda, pfft_lib):
    """complex64 at a 2^28-point size against the FP64 oracle (the float
    API's input is the oracle's input rounded to float)."""
    n = (1024, 1024, 256)
    req = Req("c2c", n)
    x = np.random.default_rng(12).uniform(-1, 1, 2 * int(np.prod(n))).astype(np.float32).astype(np.float64)
    ref = oracle_run(req, x, nthreads=os.cpu_count())
    y = gpu_run(req, x, prec="float")
    e = rel_l2(y, ref)
    del y, ref
    cuda.cuda.empty_cache()
    assert e <= 1e-6, e


def test_c5_1024cube_complex64_roundtrip(cuda, pfft_lib):
    rt, pv = _roundtrip_large(cuda, (1024, 1024, 1024), "float")
    assert rt <= 2e-6 and pv <= 2e-6, (rt, pv)
    cuda.cuda.empty_cache()


def test_c5_64_4d_complex128(cuda, pfft_lib):
    n = (64, 64, 64, 64)
    rng = np.random.default_rng(4)
    req = Req("c2c", n)
    x = rng.uniform(-1, 1, 2 * 64 ** 4)
    for prec in ("double", "double-f64"):
        y = gpu_run(req, x, prec=prec)
        assert rel_l2(y, oracle_run(req, x)) <= 1e-12

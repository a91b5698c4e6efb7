"""pfft_execute_adjoint on the GPU: dot-product identities, agreement with a
reference gradient assembled from the oracle's c2r / truncate plans, and the
differentiable oversampled r2c of the benchmark suite through the torch
autograd harness, checked against central finite differences.

Adjoints are with respect to the real inner product <a, b> = Re sum conj(a) b
(torch's convention for complex gradients, dL/dRe + i dL/dIm).
"""
import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, gpu_run, oracle_run, random_input, rel_l2

pytestmark = pytest.mark.gpu

TO, TI, PAD = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_TRANSPOSED_IN, pg.PFFT_PADDED_R2C
S_IN, S_OUT = pg.PFFT_SHIFTED_IN, pg.PFFT_SHIFTED_OUT


def _mask_in_padding(req, v):
    if req.kind == "r2c" and req.padded():
        _, lni, _, _, _ = req.sizes()
        a = np.array(v).reshape(-1, lni[-1] * req.howmany)
        a[:, req.ni[-1] * req.howmany:] = 0
        return a.ravel()
    return v


CASES = [
    Req("c2c", (16, 12, 10)), Req("c2c", (16, 12, 10), flags=TO), Req("c2c", (16, 12, 10), sign=1, flags=TI),
    Req("c2c", (20, 16, 12), ni=(10, 8, 12), no=(16, 12, 6)), Req("c2c", (16, 12, 8), flags=S_IN | S_OUT),
    Req("r2c", (16, 12, 10)), Req("r2c", (16, 12, 10), flags=PAD | TO), Req("r2c", (32, 30, 28), ni=(16, 15, 14)),
    Req("r2c", (16, 12, 10), sign=1), Req("c2r", (16, 12, 10), sign=1), Req("c2r", (16, 12, 10), sign=1, flags=TI),
    Req("c2r", (16, 12, 10), sign=-1), Req("c2r", (32, 30, 28), no=(16, 15, 14), sign=1),
    Req("c2c", (64, 64, 64)), Req("c2c", (512, 8, 8), flags=TO),
]


@pytest.mark.parametrize("req", CASES, ids=lambda r: "%s-%s-%x" % (r.kind, "x".join(map(str, r.n)), r.flags))
@pytest.mark.parametrize("prec,tol", [("double", 1e-12), ("double-df", 1e-12), ("double-dfq", 1e-12), ("float", 2e-6)])
def test_dot_product_identity(cuda, pfft_lib, req, prec, tol):
    rng = np.random.default_rng(5)
    x = _mask_in_padding(req, random_input(req, rng))
    ci, co, _ = req.counts()
    y = rng.uniform(-1, 1, co)
    if req.kind == "c2r" and req.padded():
        pass
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
        y = y.astype(np.float32).astype(np.float64)
    Ax = gpu_run(req, x, prec=prec)
    Aty = gpu_run(req, y, prec=prec, adjoint=True)
    lhs = float(np.dot(Ax, y))
    rhs = float(np.dot(x, _mask_in_padding(req, Aty)))
    scale = np.linalg.norm(Ax) * np.linalg.norm(y)
    assert abs(lhs - rhs) <= tol * scale, (lhs, rhs)


def _weights_c2r_input(n_last_logical, half):
    # interior half-spectrum bins get weight 1/2 in the adjoint of r2c
    w = np.full(half, 0.5)
    w[0] = 1.0
    if n_last_logical % 2 == 0:
        w[n_last_logical // 2] = 1.0
    return w


@pytest.mark.parametrize("prec", ["double", "double-df", "double-dfq"])
def test_r2c_adjoint_matches_reference_gradient(cuda, pfft_lib, prec):
    """Adjoint of an oversampled r2c = the reference's c2r plan (n -> ni)
    applied to the Hermitian-weighted half spectrum, then truncation."""
    n, ni = (32, 30, 28), (16, 15, 14)
    req = Req("r2c", n, ni=ni)
    rng = np.random.default_rng(6)
    _, co, _ = req.counts()
    g = rng.uniform(-1, 1, co)
    got = gpu_run(req, g, prec=prec, adjoint=True)
    h = n[2] // 2 + 1
    gw = g.view(np.complex128).reshape(n[0], n[1], h) * _weights_c2r_input(n[2], h)
    ref_req = Req("c2r", n, no=ni, sign=1)
    ref = oracle_run(ref_req, gw.view(np.float64).ravel())
    assert rel_l2(got, ref) < 1e-12


def _config4_loss_weights(n, h, sigma=32.0):
    k0 = np.fft.fftfreq(n[0], 1.0 / n[0])
    k1 = np.fft.fftfreq(n[1], 1.0 / n[1])
    k2 = np.arange(h)
    K = k0[:, None, None] ** 2 + k1[None, :, None] ** 2 + k2[None, None, :] ** 2
    return np.exp(-K / (2 * sigma ** 2))


@pytest.mark.parametrize("full", [False, True])
def test_config4_autograd_fd_and_reference(cuda, pfft_lib, full):
    """Differentiable oversampled r2c: x (ni^3, float32, N(0,1)) zero-padded to
    n^3, forward r2c, loss = sum_k exp(-|k|^2/(2*32^2)) |F_k|^2 over the stored
    bins with signed frequencies.  The autograd gradient (adjoint kernels) is
    checked against the reference gradient assembled from the oracle's
    c2r/truncate plans, and against central finite differences (h = 1e-3) at
    64 seeded coordinates evaluated with the double-precision transform."""
    torch = cuda
    from pfft_gb300.autograd import PfftOp, apply
    n = (256, 256, 256) if full else (64, 64, 64)
    ni = tuple(x // 2 for x in n)
    h = n[2] // 2 + 1
    W = _config4_loss_weights(n, h)
    Wt32 = torch.from_numpy(W).float().cuda()
    Wt64 = torch.from_numpy(W).cuda()
    rng = np.random.default_rng(7)
    x0 = rng.standard_normal(ni).astype(np.float32)

    op32 = PfftOp("r2c", n, ni=ni, dtype=torch.float32)
    x = torch.from_numpy(x0).cuda().requires_grad_(True)
    F = apply(op32, x)
    loss = (Wt32 * (F.real ** 2 + F.imag ** 2)).sum()
    loss.backward()
    g32 = x.grad.double().cpu().numpy()

    # reference gradient: dL/dF = 2 W F (FP64 forward by the oracle), then the
    # reference's c2r plan n -> ni on the Hermitian-weighted spectrum
    req = Req("r2c", n, ni=ni)
    Fref = oracle_run(req, x0.astype(np.float64).ravel()).view(np.complex128).reshape(n[0], n[1], h)
    G = 2 * W * Fref * _weights_c2r_input(n[2], h)
    gref = oracle_run(Req("c2r", n, no=ni, sign=1), G.view(np.float64).ravel()).reshape(ni)
    assert rel_l2(g32, gref) < 2e-6

    # central finite differences in double precision at 64 coordinates
    op64 = PfftOp("r2c", n, ni=ni, dtype=torch.float64)
    xd = torch.from_numpy(x0.astype(np.float64)).cuda()

    def L64(v):
        Fv = op64.forward(v)
        return float((Wt64 * (Fv.real ** 2 + Fv.imag ** 2)).sum())

    hstep = 1e-3
    idx = rng.choice(int(np.prod(ni)), 64, replace=False)
    fd = []
    for j in idx:
        c = np.unravel_index(j, ni)
        xp = xd.clone()
        xp[c] += hstep
        xm = xd.clone()
        xm[c] -= hstep
        fd.append((L64(xp) - L64(xm)) / (2 * hstep))
    fd = np.array(fd)
    gsel = gref.ravel()[idx]
    assert rel_l2(fd, gsel) < 1e-6
    assert rel_l2(g32.ravel()[idx], fd) < 2e-6

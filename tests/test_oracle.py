"""Pinning the CPU oracle (no GPU).

The reference cannot be built here (it needs FFTW-MPI, MPI and a configure-
generated config.h), so the oracle is pinned against
  * the reference's own checks: the forward/backward round trips of
    tests/simple_check_*.c on their sizes, with the reference's golden
    generator and its tolerance (tests/run_checks.sh:75: maxerror < 1e-12),
    and the c2r-versus-c2c comparison of tests/simple_check_c2r_c2c.c;
  * numpy.fft and scipy.fft as independent implementations of the FFTW
    transform definitions the reference calls (kernel/sertrafo.c:517-545).
"""
import numpy as np
import pytest

import oracle
from oracle import golden
from oracle import layout as LO

TOL = 1e-12  # tests/run_checks.sh:75


def roundtrip(kind_f, kind_b, n, ni=None, no=None, flags_f=0, flags_b=0, mesh=2, kinds_f=None, kinds_b=None,
              scale=None):
    n = list(n)
    ni = list(ni or n)
    no = list(no or n)
    d = len(n)
    if kind_f == "c2c":
        x = golden.init_complex(n if ni == n else ni, ni, [0] * d)
        xin = x.astype(np.complex128).view(np.float64).ravel()
        cnt_mid = 2 * int(np.prod(n))
    elif kind_f == "r2c":
        x = golden.init_real(ni, ni, [0] * d)
        xin = x.ravel()
        cnt_mid = 2 * int(np.prod(n[:-1])) * (n[-1] // 2 + 1)
    else:  # r2r
        x = golden.init_real(ni, ni, [0] * d)
        xin = x.ravel()
        cnt_mid = int(np.prod(n))
    mid = oracle.execute(kind_f, n, ni, n, 1, -1, flags_f, mesh, xin, cnt_mid, kinds=kinds_f)
    if kind_f == "c2c":
        back = oracle.execute("c2c", n, n, no, 1, +1, flags_b, mesh, mid, 2 * int(np.prod(no)))
        y = back.view(np.complex128).reshape(no)
        ref = golden.init_complex(n if no == n else no, no, [0] * d)
    elif kind_f == "r2c":
        back = oracle.execute("c2r", n, n, no, 1, +1, flags_b, mesh, mid, int(np.prod(no)))
        y = back.reshape(no)
        ref = golden.init_real(no, no, [0] * d)
    else:
        back = oracle.execute("r2r", n, n, no, 1, -1, flags_b, mesh, mid, int(np.prod(no)), kinds=kinds_b)
        y = back.reshape(no)
        ref = golden.init_real(no, no, [0] * d)
    y = y / (scale if scale is not None else np.prod(n))
    return np.abs(y - ref).max()


def test_engine_vs_numpy():
    rng = np.random.default_rng(1)
    for n in [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 27, 29, 31, 48, 64, 97, 101, 128, 211, 256, 1021, 1024]:
        x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
        y = oracle.fft_lines(x, -1)
        yb = oracle.fft_lines(x, +1)
        ref = np.fft.fft(x, axis=-1)
        refb = np.fft.ifft(x, axis=-1) * n
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(y - ref).max() / scale < 1e-13, n
        assert np.abs(yb - refb).max() / scale < 1e-13, n


def test_r2r_vs_scipy():
    sf = pytest.importorskip("scipy.fft")
    rng = np.random.default_rng(2)
    table = {3: ("dct", 1), 4: ("dct", 3), 5: ("dct", 2), 6: ("dct", 4), 7: ("dst", 1), 8: ("dst", 3),
             9: ("dst", 2), 10: ("dst", 4)}
    for n in [2, 3, 5, 8, 16, 17, 31]:
        x = rng.standard_normal(n)
        for k, (f, t) in table.items():
            y = oracle.r2r_line(x, k)
            z = getattr(sf, f)(x, type=t)
            assert np.abs(y - z).max() <= 1e-12 * max(1.0, np.abs(z).max()), (n, k)
        X = np.fft.fft(x)
        hc = np.zeros(n)
        hc[: n // 2 + 1] = X[: n // 2 + 1].real
        for k in range(1, (n + 1) // 2):
            hc[n - k] = X[k].imag
        assert np.abs(oracle.r2r_line(x, 0) - hc).max() < 1e-12
        assert np.abs(oracle.r2r_line(hc, 1) - n * x).max() < 1e-11
        assert np.abs(oracle.r2r_line(x, 2) - (X.real - X.imag)).max() < 1e-12


def test_multidim_vs_numpy():
    rng = np.random.default_rng(3)
    n = [6, 5, 8]
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    out = oracle.execute("c2c", n, n, n, 1, -1, 0, 2, x.view(np.float64).ravel(), 2 * int(np.prod(n)))
    assert np.abs(out.view(np.complex128).reshape(n) - np.fft.fftn(x)).max() < 1e-12
    out = oracle.execute("c2c", n, n, n, 1, -1, 2, 2, x.view(np.float64).ravel(), 2 * int(np.prod(n)))
    assert np.abs(out.view(np.complex128).reshape(n[1], n[2], n[0]) - np.fft.fftn(x).transpose(1, 2, 0)).max() < 1e-12
    xr = rng.standard_normal(n)
    out = oracle.execute("r2c", n, n, n, 1, -1, 0, 2, xr.ravel(), 2 * n[0] * n[1] * (n[2] // 2 + 1))
    assert np.abs(out.view(np.complex128).reshape(n[0], n[1], n[2] // 2 + 1) - np.fft.rfftn(xr)).max() < 1e-12
    # 4-D on a 2-D mesh, transposed out: [n1][n2][n0][n3]
    n4 = [3, 4, 5, 2]
    x4 = rng.standard_normal(n4) + 1j * rng.standard_normal(n4)
    out = oracle.execute("c2c", n4, n4, n4, 1, -1, 2, 2, x4.view(np.float64).ravel(), 2 * int(np.prod(n4)))
    ref = np.fft.fftn(x4).transpose(1, 2, 0, 3)
    assert np.abs(out.view(np.complex128).reshape(ref.shape) - ref).max() < 1e-12


# ---- the reference's round-trip checks --------------------------------------------------------
def test_simple_check_c2c():  # tests/simple_check_c2c.c
    assert roundtrip("c2c", "c2c", (29, 27, 31)) < TOL


def test_simple_check_c2c_transposed():  # tests/simple_check_c2c_transposed.c
    assert roundtrip("c2c", "c2c", (29, 27, 31), flags_f=2, flags_b=1) < TOL


def test_minimal_check_c2c():  # tests/minimal_check_c2c.c
    assert roundtrip("c2c", "c2c", (2, 2, 4)) < TOL


def test_simple_check_c2c_4d():  # tests/simple_check_c2c_4d.c
    assert roundtrip("c2c", "c2c", (13, 14, 19, 17)) < TOL
    assert roundtrip("c2c", "c2c", (13, 14, 19, 17), flags_f=2, flags_b=1) < TOL


def test_simple_check_r2c():  # tests/simple_check_r2c.c, _transposed
    assert roundtrip("r2c", "c2r", (29, 27, 31)) < TOL
    assert roundtrip("r2c", "c2r", (29, 27, 31), flags_f=2, flags_b=1) < TOL


def test_simple_check_ousam_c2c():  # tests/simple_check_ousam_c2c.c
    assert roundtrip("c2c", "c2c", (29, 27, 31), ni=(16, 16, 16), no=(16, 16, 16)) < TOL


def test_simple_check_ousam_r2c():  # tests/simple_check_ousam_r2c.c
    assert roundtrip("r2c", "c2r", (29, 27, 31), ni=(16, 16, 16), no=(16, 16, 16)) < TOL


def test_simple_check_r2r():  # tests/simple_check_r2r.c: logical N = 2(n-1), 2n, 2(n+1)
    n = (29, 27, 31)
    N = 2 * (n[0] - 1) * 2 * n[1] * 2 * (n[2] + 1)
    err = roundtrip("r2r", "r2r", n, kinds_f=[3, 4, 7], kinds_b=[3, 5, 7], scale=N)
    assert err < TOL


def _semirandom(N, k0, k1, k2):
    # tests/simple_check_c2r_c2c.c:113-130
    def di(i):
        return 1000.0 / (1 if i == 0 else i)
    if k0 == N[0]:
        return _semirandom(N, 0, k1, k2)
    if k1 == N[1]:
        return _semirandom(N, k0, 0, k2)
    if k2 == N[2]:
        return _semirandom(N, k0, k1, 0)
    l0 = k0 + N[0] if k0 else 1
    l1 = k1 - 2 * N[1] if k1 else 1
    l2 = k2 + N[2] if k2 else 1
    re = di(l0 + l1 * l2) + 3 * di(l0 * l1 + l2) + di(l2 * l0 + l1)
    im = 3 * di(l0 + l1 * l1) + di(l1 + l2 * l2) - di(l2 + l0 * l0)
    return complex(re, im)


def test_simple_check_c2r_c2c():  # tests/simple_check_c2r_c2c.c
    n = [4, 4, 6]
    h = n[2] // 2 + 1

    def init(shape):
        a = np.zeros(shape, dtype=np.complex128)
        for k0 in range(shape[0]):
            for k1 in range(shape[1]):
                for k2 in range(shape[2]):
                    a[k0, k1, k2] = _semirandom(n, k0, k1, k2) + np.conj(
                        _semirandom(n, n[0] - k0, n[1] - k1, n[2] - k2))
        return a
    xc = init(n)
    xr = init([n[0], n[1], h])
    fc = oracle.execute("c2c", n, n, n, 1, -1, 0, 2, xc.view(np.float64).ravel(), 2 * 96)
    fr = oracle.execute("c2r", n, n, n, 1, -1, 0, 2, xr.view(np.float64).ravel(), 96)
    bc = oracle.execute("c2c", n, n, n, 1, +1, 0, 2, fc, 2 * 96).view(np.complex128).reshape(n) / 96
    br = oracle.execute("r2c", n, n, n, 1, +1, 0, 2, fr, 2 * 4 * 4 * h).view(np.complex128).reshape(4, 4, h) / 96
    err = 0.0
    for k0 in range(n[0]):
        for k1 in range(1, n[1]):
            for k2 in range(2, h):
                err = max(err, abs(br[k0, k1, k2] - bc[k0, k1, k2]))
    assert err < TOL


def test_forward_c2r_equals_c2c_on_hermitian_input():
    # FORWARD c2r conjugates its input and runs the backward c2r
    # (kernel/partrafo.c:428-443); on a Hermitian spectrum this is the
    # forward DFT of the full spectrum, which is real
    rng = np.random.default_rng(4)
    n = [6, 4, 8]
    X = np.fft.fftn(rng.standard_normal(n))
    half = np.ascontiguousarray(X[:, :, : n[2] // 2 + 1])
    out = oracle.execute("c2r", n, n, n, 1, -1, 0, 2, half.view(np.float64).ravel(), int(np.prod(n)))
    assert np.abs(out.reshape(n) - np.fft.fftn(X).real).max() < 1e-10


def test_golden_generator_matches_reference_formula():
    # api/api-basic.c:60-70, 254-264: value at plain index m
    n = [3, 4, 5]
    x = golden.init_complex(n, n, [0, 0, 0])
    for (i, j, k) in [(0, 0, 0), (1, 2, 3), (2, 3, 4), (0, 1, 0)]:
        m = 0
        for t, v in enumerate((i, j, k)):
            m += m * n[t] + v
        ref = complex(1500, 1250) if m == 0 else complex(1000 / (2 * m), 1000 / (2 * m + 1))
        assert x[i, j, k] == ref


def test_layout_reference_values():
    # 256^3 r2c padded, transposed out (configuration of the benchmark suite)
    mem, lni, lis, lno, los = LO.local_size(3, [256] * 3, [256] * 3, [256] * 3, 1, LO.R2C, 2 | (1 << 11), 2)
    assert lni == [256, 256, 258] and lno == [256, 256, 129]
    assert mem == 256 * 256 * 129
    # c2c 64^3 on a 2-D mesh
    mem, lni, lis, lno, los = LO.local_size(3, [64] * 3, [64] * 3, [64] * 3, 1, LO.C2C, 0, 2)
    assert mem == 64 ** 3 and lni == [64] * 3 and lno == [64] * 3
    # shifted starts
    _, _, lis, _, los = LO.local_size(3, [8] * 3, [8] * 3, [8] * 3, 1, LO.C2C, 4 | 8, 2)
    assert lis == [-4] * 3 and los == [-4] * 3
    # 3-D data on a 3-D mesh: real rows are reported unpadded
    mem, lni, _, lno, _ = LO.local_size(3, [8, 8, 8], [8, 8, 8], [8, 8, 8], 1, LO.R2C, 1 << 11, 3)
    assert lni == [8, 8, 8] and lno == [8, 8, 5] and mem == 512


def test_r2r_3d_vs_scipy():
    """The oracle's multi-axis r2r (REDFT10 / REDFT01 / RODFT00 on 32x24x20)
    against scipy.fft's n-dimensional DCT/DST."""
    import scipy.fft as sf
    from tests.pfft_util import Req, oracle_run, rel_l2
    n = (32, 24, 20)
    x = np.random.default_rng(7).standard_normal(int(np.prod(n)))
    for kinds, fn in (([5, 5, 5], lambda a: sf.dctn(a, type=2)), ([4, 4, 4], lambda a: sf.dctn(a, type=3)),
                      ([7, 7, 7], lambda a: sf.dstn(a, type=1))):
        y = oracle_run(Req("r2r", n, kinds=kinds), x)
        assert rel_l2(y, fn(x.reshape(n)).ravel()) < 1e-14

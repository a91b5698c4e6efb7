"""The library's golden-data generators against the oracle's restatement
(no GPU: host arrays).

pfft_init_input_complex / _real / _complex_hermitian (and the _3d and pfftf_
forms) fill the reference's deterministic test data (api/api-basic.c:60-121,
with the non-row-major plain_index of :254-264); the reference's round-trip
checks compare against it, so it must equal oracle/golden.py element for
element, on local blocks that start inside the global array.  The matching
check_output_* must then report an error of zero (one float rounding for
the float Hermitian data, which the check compares in double).
"""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg
from oracle import golden

SHAPES = [((5, 6, 7), (3, 6, 4), (1, 0, 2)), ((4, 4, 6), (4, 4, 6), (0, 0, 0)),
          ((29, 27, 31), (7, 5, 31), (20, 3, 0))]


def _fill(L, pre, name, n, ln, ls, buf, rnk3):
    if rnk3:
        getattr(L, pre + name + "_3d")(pg.ints(n), pg.ints(ln), pg.ints(ls), buf.ctypes.data)
    else:
        getattr(L, pre + name)(len(n), pg.ints(n), pg.ints(ln), pg.ints(ls), buf.ctypes.data)


@pytest.mark.parametrize("prec", ["double", "float"])
@pytest.mark.parametrize("rnk3", [True, False])
@pytest.mark.parametrize("n,ln,ls", SHAPES)
def test_init_input_matches_oracle(pfft_lib, prec, rnk3, n, ln, ls):
    L = pfft_lib
    pre = "pfft_" if prec == "double" else "pfftf_"
    rdt = np.float64 if prec == "double" else np.float32
    cnt = int(np.prod(ln))
    # complex
    buf = np.full(2 * cnt, np.nan, dtype=rdt)
    _fill(L, pre, "init_input_complex", n, ln, ls, buf, rnk3)
    want = golden.init_complex(n, ln, ls, dtype=rdt).ravel()
    got = buf.view(np.complex128 if prec == "double" else np.complex64)
    assert np.array_equal(got, want.astype(got.dtype))
    # real
    rbuf = np.full(cnt, np.nan, dtype=rdt)
    _fill(L, pre, "init_input_real", n, ln, ls, rbuf, rnk3)
    assert np.array_equal(rbuf, golden.init_real(n, ln, ls, dtype=rdt).ravel())
    # Hermitian
    hbuf = np.full(2 * cnt, np.nan, dtype=rdt)
    _fill(L, pre, "init_input_complex_hermitian", n, ln, ls, hbuf, rnk3)
    hgot = hbuf.view(np.complex128 if prec == "double" else np.complex64)
    assert np.array_equal(hgot, golden.init_hermitian(n, ln, ls, dtype=rdt).ravel().astype(hgot.dtype))


@pytest.mark.parametrize("prec", ["double", "float"])
def test_check_output_of_generated_data_is_zero(pfft_lib, prec):
    L = pfft_lib
    pre = "pfft_" if prec == "double" else "pfftf_"
    rdt = np.float64 if prec == "double" else np.float32
    n, ln, ls = SHAPES[0]
    cnt = int(np.prod(ln))
    for gen, chk, words in (("init_input_complex", "check_output_complex", 2),
                            ("init_input_real", "check_output_real", 1),
                            ("init_input_complex_hermitian", "check_output_complex_hermitian", 2)):
        buf = np.zeros(words * cnt, dtype=rdt)
        _fill(L, pre, gen, n, ln, ls, buf, True)
        err = getattr(L, pre + chk + "_3d")(pg.ints(n), pg.ints(ln), pg.ints(ls), buf.ctypes.data, pg.MPI_COMM_WORLD)
        # float Hermitian data is rounded once from the double combination the
        # check compares against: one rounding of values up to 1500
        tol = 1e-4 if (prec == "float" and "hermitian" in gen) else 0.0
        assert err <= tol, (gen, err)
        buf[words * 3] += 1.0  # one changed value is reported
        err = getattr(L, pre + chk + "_3d")(pg.ints(n), pg.ints(ln), pg.ints(ls), buf.ctypes.data, pg.MPI_COMM_WORLD)
        assert err > 0.5, (gen, err)

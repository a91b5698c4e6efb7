"""GPU parity of pfft_execute against the CPU oracle, through the C-ABI.

Cases follow the reference's check programs (tests/simple_check_*.c): their
sizes (29x27x31, 13x14x19x17, 2x2x4, 16^3 <-> 29x27x31 oversampling),
transposed layouts, in-place and out-of-place arrays, r2c/c2r padding, the
r2r kinds they use, plus the configurations of the benchmark suite at sizes
the oracle finishes in seconds.  Tolerances: relative L2 <= 1e-12 for the
double API, <= 2e-6 for the float API.  The double API is run with its
default arithmetic ("double": native FP64 up to 2^18 points, float-float
above), with float-float forced ("double-df") and with float-float whose
radix-8 stages round the high words to a per-butterfly grid ("double-dfq"),
so every arithmetic is checked at every size.
"""
import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, gpu_run, mask_padding, oracle_run, random_input, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "double-df": 1e-12, "double-dfq": 1e-12, "double-f64": 1e-12, "float": 2e-6}
PRECS = ["double", "double-df", "double-dfq", "float"]
DPRECS = ["double", "double-df", "double-dfq"]
TO, TI = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_TRANSPOSED_IN
PAD = pg.PFFT_PADDED_R2C


def check(req, prec="double", inplace=False, dist="uniform", seed=1):
    rng = np.random.default_rng(seed)
    x = random_input(req, rng, dist)
    if prec == "float":
        x = x.astype(np.float32).astype(np.float64)
    ref = mask_padding(req, oracle_run(req, x))
    got = mask_padding(req, gpu_run(req, x, prec=prec, inplace=inplace))
    err = rel_l2(got, ref)
    assert err <= TOL[prec], "rel L2 %.3e > %.1e" % (err, TOL[prec])
    return err


C2C_CASES = [
    ((8, 8, 8), 0), ((2, 2, 4), 0), ((29, 27, 31), 0), ((64, 64, 64), 0), ((29, 27, 31), TO),
    ((29, 27, 31), TI), ((64, 64, 64), TO), ((16, 12, 10), TI), ((5, 7, 11), 0), ((48, 64, 40), 0),
    ((96, 32, 17), 0),
]


@pytest.mark.parametrize("n,flags", C2C_CASES)
@pytest.mark.parametrize("prec", PRECS)
def test_c2c_3d(cuda, pfft_lib, n, flags, prec):
    check(Req("c2c", n, flags=flags), prec)


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("prec", DPRECS)
def test_c2c_backward_and_inplace(cuda, pfft_lib, sign, prec):
    check(Req("c2c", (29, 27, 31), sign=sign), prec, inplace=True)
    check(Req("c2c", (29, 27, 31), sign=sign, flags=TO), prec, inplace=True)


@pytest.mark.parametrize("n,flags", [((8, 8, 8), 0), ((29, 27, 31), 0), ((16, 16, 16), TO), ((29, 27, 31), TO),
                                     ((16, 16, 16), PAD), ((29, 27, 31), PAD | TO), ((64, 64, 64), PAD | TO)])
@pytest.mark.parametrize("prec", PRECS)
def test_r2c(cuda, pfft_lib, n, flags, prec):
    check(Req("r2c", n, flags=flags), prec, dist="normal")


@pytest.mark.parametrize("n,flags", [((8, 8, 8), 0), ((29, 27, 31), 0), ((16, 16, 16), TI), ((29, 27, 31), TI),
                                     ((16, 16, 16), PAD), ((29, 27, 31), PAD | TI), ((64, 64, 64), PAD | TI)])
@pytest.mark.parametrize("prec", PRECS)
def test_c2r(cuda, pfft_lib, n, flags, prec):
    check(Req("c2r", n, sign=1, flags=flags), prec)


@pytest.mark.parametrize("prec", DPRECS)
def test_r2c_backward_c2r_forward(cuda, pfft_lib, prec):
    # conjugation paths (kernel/partrafo.c:428-443)
    check(Req("r2c", (12, 10, 16), sign=1), prec, dist="normal")
    check(Req("c2r", (12, 10, 16), sign=-1), prec)


@pytest.mark.parametrize("prec", DPRECS)
def test_r2c_c2r_inplace_padded(cuda, pfft_lib, prec):
    check(Req("r2c", (16, 12, 10), flags=PAD), prec, inplace=True, dist="normal")
    check(Req("c2r", (16, 12, 10), sign=1, flags=PAD), prec, inplace=True)
    check(Req("r2c", (16, 12, 10), flags=PAD | TO), prec, inplace=True, dist="normal")
    check(Req("c2r", (16, 12, 10), sign=1, flags=PAD | TI), prec, inplace=True)


@pytest.mark.parametrize("kinds", [(3, 3, 3), (4, 4, 4), (5, 5, 5), (6, 6, 6), (7, 7, 7), (8, 8, 8), (9, 9, 9),
                                   (10, 10, 10), (0, 1, 2), (3, 4, 7), (5, 9, 6)])
@pytest.mark.parametrize("prec", PRECS)
def test_r2r(cuda, pfft_lib, kinds, prec):
    check(Req("r2r", (9, 8, 10), kinds=list(kinds)), prec, dist="normal")


@pytest.mark.parametrize("prec", PRECS)
def test_dct_fast_paths(cuda, pfft_lib, prec):
    """REDFT10 / REDFT01 on 2^a, 3 * 2^a and 5 * 2^a lengths (the FFT-based
    DCT path of the radix-8 and mixed-radix kernels), transposed, oversampled
    and mixed with other kinds."""
    check(Req("r2r", (32, 96, 40), kinds=[5, 5, 5]), prec, dist="normal")
    check(Req("r2r", (32, 96, 40), kinds=[4, 4, 4], flags=TO), prec, dist="normal")
    check(Req("r2r", (64, 48, 16), kinds=[4, 5, 7]), prec, dist="normal")
    check(Req("r2r", (64, 48, 32), ni=(40, 30, 20), kinds=[5, 4, 5]), prec, dist="normal")
    check(Req("r2r", (64, 48, 32), no=(40, 30, 20), kinds=[4, 5, 4], flags=TI), prec, dist="normal")


@pytest.mark.parametrize("prec", DPRECS)
def test_r2r_transposed(cuda, pfft_lib, prec):
    check(Req("r2r", (16, 16, 16), kinds=[5, 5, 5], flags=TO), prec, dist="normal")
    check(Req("r2r", (16, 16, 16), kinds=[4, 4, 4], flags=TI), prec, dist="normal")


@pytest.mark.parametrize("prec", DPRECS)
def test_ousam_c2c(cuda, pfft_lib, prec):
    # tests/simple_check_ousam_c2c.c: ni = 16^3 -> n = 29x27x31 -> no = n, and back
    check(Req("c2c", (29, 27, 31), ni=(16, 16, 16)), prec)
    check(Req("c2c", (29, 27, 31), no=(16, 16, 16), sign=1), prec)
    check(Req("c2c", (29, 27, 31), ni=(16, 16, 16), no=(20, 18, 16), flags=TO), prec)


@pytest.mark.parametrize("prec", DPRECS)
def test_ousam_r2c_c2r(cuda, pfft_lib, prec):
    check(Req("r2c", (29, 27, 31), ni=(16, 16, 16)), prec, dist="normal")
    check(Req("c2r", (29, 27, 31), no=(16, 16, 16), sign=1), prec)
    check(Req("r2c", (32, 32, 32), ni=(16, 16, 16), flags=PAD | TO), prec, dist="normal")
    # truncated r2c output keeps the reference's bin range
    check(Req("r2c", (32, 30, 28), no=(16, 16, 16)), prec, dist="normal")


@pytest.mark.parametrize("prec", DPRECS)
def test_shifted(cuda, pfft_lib, prec):
    S_IN, S_OUT = pg.PFFT_SHIFTED_IN, pg.PFFT_SHIFTED_OUT
    check(Req("c2c", (8, 10, 12), flags=S_IN | S_OUT), prec)
    check(Req("c2c", (8, 10, 12), flags=S_OUT), prec)
    check(Req("c2c", (8, 10, 12), flags=S_IN), prec)
    check(Req("c2c", (16, 16, 16), ni=(8, 8, 8), flags=S_IN | S_OUT), prec)
    check(Req("r2c", (8, 10, 12), flags=S_IN | S_OUT), prec, dist="normal")


@pytest.mark.parametrize("prec", DPRECS)
def test_4d_and_meshes(cuda, pfft_lib, prec):
    check(Req("c2c", (13, 14, 19, 17)), prec)
    check(Req("c2c", (13, 14, 19, 17), flags=TO), prec)
    check(Req("c2c", (8, 6, 10, 4), cart=3), prec)
    check(Req("c2c", (8, 6, 10, 4), cart=3, flags=TO), prec)
    check(Req("c2c", (12, 10, 8), cart=1, flags=TO), prec)
    check(Req("c2c", (12, 10, 8), cart=0, flags=TO), prec)
    check(Req("c2c", (12, 10, 8), cart=3, flags=TO), prec)
    check(Req("r2c", (12, 10, 8), cart=3, flags=PAD), prec, dist="normal")


@pytest.mark.parametrize("prec", DPRECS)
def test_howmany(cuda, pfft_lib, prec):
    check(Req("c2c", (8, 8, 8), howmany=2), prec)
    check(Req("c2c", (8, 8, 8), howmany=3, flags=TO), prec)
    check(Req("r2c", (8, 8, 8), howmany=2), prec, dist="normal")
    check(Req("c2r", (8, 8, 8), howmany=2, sign=1), prec)


def test_native_f64_arith(cuda, pfft_lib):
    check(Req("c2c", (29, 27, 31), flags=TO), "double-f64")
    check(Req("r2c", (16, 16, 16), flags=PAD), "double-f64", dist="normal")
    check(Req("c2c", (128, 64, 256), flags=TO), "double-f64")


def test_double_arith_modes(cuda, pfft_lib):
    """Mode selection: unknown modes are refused, the previous mode stays."""
    L = pg.lib()
    old = L.pfft_gb300_get_double_arith()
    assert old in (0, 1, 2, 3)
    assert L.pfft_gb300_set_double_arith(7) == -1
    assert L.pfft_gb300_get_double_arith() == old


@pytest.mark.parametrize("n,flags", [((16, 512, 8), 0), ((512, 4, 64), TO), ((8, 16, 4096), 0), ((4, 1024, 8), TI),
                                     ((128, 32, 256), 0), ((2048, 8, 16), TO), ((96, 8, 768), 0), ((40, 320, 24), TO),
                                     ((8, 640, 48), TI)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_block_quantised_error_level(cuda, pfft_lib, n, flags, sign):
    """The block-quantised float-float butterflies ("double-dfq": radix-8
    stages, and the radix-2/3/4/5 stages of the mixed-radix kernel on
    3 * 2^a and 5 * 2^a lines) stay within a few times 1e-13 relative L2 per
    transform on uniform and normal data
    and on data spanning 2^-30..2^30 in magnitude (the error is relative to
    each butterfly's largest component), against about 1e-14 for TwoSum
    float-float on the same lines."""
    req = Req("c2c", n, flags=flags, sign=sign)
    rng = np.random.default_rng(5)
    for dist in ("uniform", "normal", "wide"):
        if dist == "wide":
            x = rng.standard_normal(2 * int(np.prod(n))) * np.exp2(rng.uniform(-30, 30, 2 * int(np.prod(n))))
        else:
            x = random_input(req, rng, dist)
        ref = oracle_run(req, x)
        eq = rel_l2(gpu_run(req, x, prec="double-dfq"), ref)
        ed = rel_l2(gpu_run(req, x, prec="double-df"), ref)
        print("dfq %s %s %s: %.3e (df %.3e)" % (n, sign, dist, eq, ed))
        assert eq <= 1e-12 and ed <= 1e-13, (dist, eq, ed)


@pytest.mark.parametrize("n,flags", [((32, 32, 32), 0), ((16, 32, 64), TO), ((64, 64, 64), 0), ((128, 64, 256), TO),
                                     ((96, 48, 40), 0), ((24, 80, 192), TO), ((40, 96, 384), TI), ((768, 6, 160), 0),
                                     ((8, 640, 320), TO), ((512, 8, 16), 0),
                                     ((16, 1024, 8), TI), ((2048, 4, 4), 0), ((8, 4, 4096), 0)])
@pytest.mark.parametrize("prec", PRECS)
def test_kernel_paths_agree(cuda, pfft_lib, n, flags, prec):
    """The register-resident radix-8 and mixed-radix (3 * 2^a, 5 * 2^a)
    kernels and the general pass kernel all match the oracle on c2c lines
    (row, column and transposing passes, every supported line length)."""
    L = pg.lib()
    try:
        for path in (1, 0):
            L.pfft_gb300_set_kernel_path(path)
            check(Req("c2c", n, flags=flags), prec)
            check(Req("c2c", n, flags=flags, sign=1), prec)
    finally:
        L.pfft_gb300_set_kernel_path(1)


@pytest.mark.parametrize("n,flags", [((32, 32, 32), 0), ((16, 32, 64), TO), ((64, 64, 64), TI), ((128, 64, 256), TO),
                                     ((512, 8, 16), 0), ((16, 1024, 8), TI), ((2048, 4, 4), 0), ((8, 4, 4096), 0),
                                     ((3, 5, 512), 0), ((512, 6, 3), 0), ((256, 12, 40), TO)])
@pytest.mark.parametrize("prec", PRECS)
def test_staged_variant_agrees(cuda, pfft_lib, n, flags, prec):
    """The staged persistent variant of the radix-8 kernel (bulk and
    tensor-map copies into shared memory on an mbarrier) and the plain kernel
    both match the oracle: row, column and transposing passes, tail tiles
    (3 x 5 lines of 512), column tiles that would straddle a batch dimension
    (512-point columns over 6 x 3 lines: not staged), float-float
    intermediates; no staged wait expires."""
    L = pg.lib()
    try:
        for staged in (2, 0):
            L.pfft_gb300_set_staged(staged)
            before = L.pfft_gb300_staged_launches()
            check(Req("c2c", n, flags=flags), prec)
            check(Req("c2c", n, flags=flags, sign=1), prec)
            ran = L.pfft_gb300_staged_launches() - before
            # (native FP64 plans use the general kernel; 512 x 6 x 3 has no stageable pass)
            if staged and prec != "double" and n != (512, 6, 3):
                assert ran > 0
            if not staged:
                assert ran == 0
        assert L.pfft_gb300_staged_status() == 0
    finally:
        L.pfft_gb300_set_staged(1)

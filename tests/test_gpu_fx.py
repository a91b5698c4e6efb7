"""The double API's default arithmetic on the radix-8 kernel: 64-bit block
fixed point (fft_fast.cuh, FX), against the FP64 oracle and against native
FP64 on the same inputs (GPU, through the C-ABI).

FX converts each tile's doubles to int64 mantissas on the tile's common grid
(58 bits below the tile's largest exponent), adds exactly and multiplies by
64-bit twiddles; it must be at least as accurate as native FP64 arithmetic
(the reference computes in FFTW double) on every length, direction and
layout, exactly invariant under power-of-two scaling of the input (the grid
follows the exponent), and must turn a tile holding an infinity or NaN into
NaN instead of garbage.
"""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg
from tests.pfft_util import Req, gpu_run, mask_padding, oracle_run, random_input, rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, 16), (8, 32, 64), (4, 8, 128), (2, 4, 256), (2, 2, 512), (2, 1024, 2), (2, 2048, 1),
          (4096, 2, 1), (32, 64, 128)]


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("flags", [0, pg.PFFT_TRANSPOSED_OUT])
@pytest.mark.parametrize("n", SHAPES)
def test_fx_no_less_accurate_than_native_fp64(cuda, pfft_lib, n, flags, sign):
    req = Req("c2c", n, sign=sign, flags=flags)
    rng = np.random.default_rng(sum(n) + sign + flags)
    x = random_input(req, rng)
    ref = oracle_run(req, x)
    fx = gpu_run(req, x, prec="double")
    nat = gpu_run(req, x, prec="double-f64")
    e_fx, e_nat = rel_l2(fx, ref), rel_l2(nat, ref)
    assert e_fx <= 1e-15, e_fx
    assert e_fx <= 1.25 * e_nat + 1e-17, (e_fx, e_nat)


MIXED_SHAPES = [(24, 40, 48), (96, 96, 8), (2, 768, 4), (640, 4, 2), (160, 2, 320), (80, 384, 1), (192, 6, 10)]


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("flags", [0, pg.PFFT_TRANSPOSED_OUT])
@pytest.mark.parametrize("n", MIXED_SHAPES)
def test_fx_mixed_radix_no_less_accurate_than_native_fp64(cuda, pfft_lib, n, flags, sign):
    """3 * 2^a and 5 * 2^a lengths run FX on the mixed-radix kernel (radix-3
    and radix-5 butterflies with 64-bit fixed-point constants): the same bar
    as the radix-8 kernel against the oracle and native FP64."""
    req = Req("c2c", n, sign=sign, flags=flags)
    rng = np.random.default_rng(sum(n) * 7 + sign + flags)
    x = random_input(req, rng)
    ref = oracle_run(req, x)
    fx = gpu_run(req, x, prec="double")
    nat = gpu_run(req, x, prec="double-f64")
    e_fx, e_nat = rel_l2(fx, ref), rel_l2(nat, ref)
    assert e_fx <= 1e-15, e_fx
    assert e_fx <= 1.25 * e_nat + 1e-17, (e_fx, e_nat)


def _exact_dft3(x, n, sign=-1):
    """3-D DFT in extended precision (numpy longdouble: 64- or 113-bit
    mantissa), one axis at a time by explicit DFT matrices: a reference more
    accurate than either arithmetic under test (the FP64 oracle shares native
    FP64's rounding pattern on sparse inputs, e.g. it reproduces a spike's
    transform bit for bit)."""
    ld = np.longdouble
    pi = ld("3.14159265358979323846264338327950288")
    a = (x[0::2].astype(ld) + x[1::2].astype(ld) * np.clongdouble(1j)).reshape(n)
    for ax, m in enumerate(n):
        k = np.arange(m)
        # the angle from the integer numerator jk mod m keeps the table exact to longdouble
        ph = np.mod(np.outer(k, k), m).astype(ld) * (2 * pi / ld(m))
        W = np.cos(ph) + sign * np.clongdouble(1j) * np.sin(ph)
        a = np.moveaxis(np.tensordot(W, np.moveaxis(a, ax, 0), axes=(1, 0)), 0, ax)
    out = np.empty(2 * a.size, dtype=ld)
    out[0::2] = a.real.ravel()
    out[1::2] = a.imag.ravel()
    return out


def _rel(got, exact):
    e = np.asarray(exact, dtype=np.longdouble)
    return float(np.linalg.norm((np.asarray(got, dtype=np.longdouble) - e).astype(np.float64)) /
                 np.linalg.norm(e.astype(np.float64)))


@pytest.mark.parametrize("dist", ["uniform", "spread", "spike", "spike_alone", "one_line"])
@pytest.mark.parametrize("n", [(8, 16, 32), (24, 40, 8)])
def test_fx_dynamic_range_against_extended_precision(cuda, pfft_lib, dist, n):
    """Uniform values, values spread over 2^+-40, a single large value among
    small ones (and alone), one line a million times larger than the rest:
    FX's error against an extended-precision DFT stays within 1.25x native
    FP64's error, or within one double rounding (2^-53) of the result, on
    the radix-8 kernel and on the mixed-radix one (24 = 3 * 8, 40 = 5 * 8)."""
    req = Req("c2c", n)
    rng = np.random.default_rng(3)
    x = random_input(req, rng)
    if dist == "spread":
        x = x * np.exp2(rng.uniform(-40, 40, x.size))
    elif dist == "spike":
        x = x * 1e-6
        x[1000] = 1500.0
    elif dist == "spike_alone":
        x = np.zeros_like(x)
        x[1000] = 1500.0
    elif dist == "one_line":
        x.reshape(-1, 64)[17] *= 1e6
    exact = _exact_dft3(x, n)
    e_fx = _rel(gpu_run(req, x, prec="double"), exact)
    e_nat = _rel(gpu_run(req, x, prec="double-f64"), exact)
    assert e_fx <= max(1.25 * e_nat, 2.0 ** -53), (e_fx, e_nat)


@pytest.mark.parametrize("k", [-1000, -200, -1, 7, 300, 900])
def test_fx_power_of_two_scaling_is_exact(cuda, pfft_lib, k):
    """The grid follows the tile's exponent, so scaling the input by 2^k
    scales every stored result by exactly 2^k (away from overflow and from
    results below 2^-1022, which are stored as zero)."""
    req = Req("c2c", (32, 64, 16))
    x = random_input(req, np.random.default_rng(9))
    base = gpu_run(req, x, prec="double")
    got = gpu_run(req, np.ldexp(x, k), prec="double")
    want = np.ldexp(base, k)
    tiny = np.abs(want) < 2.0 ** -1000
    assert np.array_equal(got[~tiny], want[~tiny])


def test_fx_zeros_and_nonfinite(cuda, pfft_lib):
    req = Req("c2c", (16, 16, 64))
    x = np.zeros(req.counts()[0])
    assert np.array_equal(gpu_run(req, x, prec="double"), np.zeros_like(x))
    x = random_input(req, np.random.default_rng(1))
    x[77] = np.inf
    out = gpu_run(req, x, prec="double")
    assert np.isnan(out).any() and not np.isinf(out).any()
    x[77] = np.nan
    assert np.isnan(gpu_run(req, x, prec="double")).any()


def test_fx_large_transform_against_oracle(cuda, pfft_lib):
    """256^3 complex128, forward: FX and native FP64 against the oracle."""
    req = Req("c2c", (256, 256, 256))
    x = random_input(req, np.random.default_rng(12))
    ref = oracle_run(req, x)
    e_fx = rel_l2(gpu_run(req, x, prec="double"), ref)
    e_nat = rel_l2(gpu_run(req, x, prec="double-f64"), ref)
    assert e_fx <= 1e-15 and e_fx <= 1.25 * e_nat, (e_fx, e_nat)


@pytest.mark.parametrize("link", [0, 1])
@pytest.mark.parametrize("req", [Req("c2c", (32, 64, 128)), Req("c2c", (32, 64, 128), flags=pg.PFFT_TRANSPOSED_OUT),
                                 Req("c2c", (16, 32, 64), sign=1, flags=pg.PFFT_TRANSPOSED_IN),
                                 Req("c2c", (8, 16, 32, 64)), Req("c2c", (16, 32, 64), howmany=3),
                                 Req("r2c", (32, 64, 128), flags=pg.PFFT_PADDED_R2C | pg.PFFT_TRANSPOSED_OUT),
                                 Req("c2r", (32, 64, 128), sign=1)],
                         ids=["c2c", "c2c_to", "c2c_ti_bwd", "c2c_4d", "c2c_hm3", "r2c_pad_to", "c2r"])
def test_fx_mantissas_between_passes(cuda, pfft_lib, req, link):
    """Mode 2 keeps the int64 mantissas and one exponent per line between two
    radix-8 passes (pfft_gb300_set_fx_link, on by default) instead of
    rounding to double in between: with and without, every layout matches the
    oracle at FP64 level."""
    L = pfft_lib
    old = L.pfft_gb300_set_fx_link(link)
    try:
        x = random_input(req, np.random.default_rng(31))
        ref = oracle_run(req, x)
        got = gpu_run(req, x, prec="double")
    finally:
        L.pfft_gb300_set_fx_link(old)
    from tests.pfft_util import mask_padding
    assert rel_l2(mask_padding(req, got), mask_padding(req, ref)) <= 1e-15


@pytest.mark.parametrize("n,flags,links", [((512, 64, 128), 0, [2, 3, 1]), ((32, 64, 128), pg.PFFT_TRANSPOSED_OUT, [2, 3, 1]),
                                           ((16, 16, 32, 64), 0, [2, 3, 3, 1]), ((64, 48, 32), 0, [0, 0, 0])])
def test_fx_links_form(cuda, pfft_lib, n, flags, links):
    """Consecutive power-of-two c2c passes of a default double plan keep the
    mantissas between them (1 = input linked, 2 = output linked); a
    non-power-of-two axis (48, general kernel in FP64) breaks the chain."""
    torch = cuda
    L = pfft_lib
    cnt = int(np.prod(n))
    a = torch.zeros(2 * cnt, dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    p = L.pfft_plan_dft(len(n), pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), pg.PFFT_FORWARD, flags)
    assert p, pg.last_error()
    got = [L.pfft_gb300_pass_fx_link(p, i) for i in range(len(links))]
    L.pfft_destroy_plan(p)
    if 48 in n:  # the 48-point pass breaks the chain on both sides
        assert got[1] == 0
    else:
        assert got == links


@pytest.mark.parametrize("kind,n,flags,kinds", [
    ("r2c", (8, 16, 32), 0, None),                                          # paired (128 rows)
    ("r2c", (32, 32, 64), pg.PFFT_PADDED_R2C | pg.PFFT_TRANSPOSED_OUT, None),  # the benchmark's layout
    ("r2c", (3, 5, 64), 0, None),                                           # 15 rows: not paired
    ("r2c", (4, 6, 4096), 0, None),                                         # one-line tiles
    ("r2r", (16, 32, 64), 0, [5, 5, 5]),                                    # REDFT10 on every axis
    ("r2r", (6, 8, 256), 0, [5, 5, 5]),
    ("c2r", (8, 16, 32), 0, None),                                          # the inverse kinds combine
    ("c2r", (32, 32, 64), pg.PFFT_PADDED_R2C | pg.PFFT_TRANSPOSED_IN, None),  # before the transform
    ("r2r", (16, 32, 64), 0, [4, 4, 4]),                                    # REDFT01
])
def test_fx_paired_real_lines(cuda, pfft_lib, kind, n, flags, kinds):
    """r2c, c2r, REDFT10 and REDFT01 passes of default double plans
    transform two real lines (adjacent along the pass's first batch
    dimension, when its extent is even) as one complex line, separating the
    spectra after the transform (forward kinds) or combining them before it
    (inverse kinds, kernels of their own).  Against
    the oracle they stay within 1e-15 and within 1.25x native FP64's error,
    and the plan reports the pairing (bit 2 of pfft_gb300_pass_fx_link)."""
    sign = 1 if kind == "c2r" else -1
    req = Req(kind, n, flags=flags, kinds=kinds) if kinds else Req(kind, n, flags=flags, sign=sign)
    rng = np.random.default_rng(sum(n) + flags)
    x = random_input(req, rng)
    ref = mask_padding(req, oracle_run(req, x))  # (a padded real output's padding is undefined)
    fx = mask_padding(req, gpu_run(req, x, prec="double"))
    nat = mask_padding(req, gpu_run(req, x, prec="double-f64"))
    e_fx, e_nat = rel_l2(fx, ref), rel_l2(nat, ref)
    assert e_fx <= 1e-15, e_fx
    assert e_fx <= 1.25 * e_nat + 1e-17, (e_fx, e_nat)
    # which passes pair
    torch = cuda
    L = pfft_lib
    cnt = int(np.prod(n))
    a = torch.zeros(2 * cnt + 64 * n[0] * n[1], dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    if kind == "r2c":
        p = L.pfft_plan_dft_r2c_3d(pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), pg.PFFT_FORWARD, flags)
    elif kind == "c2r":
        p = L.pfft_plan_dft_c2r_3d(pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), pg.PFFT_BACKWARD, flags)
    else:
        p = L.pfft_plan_r2r_3d(pg.ints(n), a.data_ptr(), b.data_ptr(), pg.procmesh(2), (ctypes.c_int * 3)(*kinds), flags)
    assert p, pg.last_error()
    vals = [L.pfft_gb300_pass_fx_link(p, i) for i in range(8)]  # -1 past the last pass
    L.pfft_destroy_plan(p)
    paired = sum(1 for v in vals if v >= 0 and v & 4)
    if n == (3, 5, 64):
        assert paired == 0  # odd batch extent
    else:
        assert paired >= 1, vals

"""The integer-only double <-> float-float conversions of the double API
(GPU): relative error <= 2^-46 for magnitudes in [2^-74, 2^127], exact zeros,
and the documented degradation below 2^-74."""
import ctypes

import numpy as np
import pytest

import pfft_gb300 as pg

pytestmark = pytest.mark.gpu


def roundtrip(torch, x):
    L = pg.lib()
    f = L.pfft_gb300_selftest_df_roundtrip
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    a = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    b = torch.empty_like(a)
    assert f(a.data_ptr(), b.data_ptr(), a.numel(), None) == 0
    torch.cuda.synchronize()
    return b.cpu().numpy()


def test_conversion_precision(cuda, pfft_lib):
    rng = np.random.default_rng(0)
    specials = [1.0, -1.0, 2.0 ** 126, -(2.0 ** -125), 1 - 2.0 ** -53, 1 + 2.0 ** -52, 3.0, 0.1, -0.1,
                np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0), 2.0 ** -74, 12345.678901234567]
    x = np.concatenate([np.array(specials), rng.uniform(-1, 1, 100000),
                        rng.standard_normal(100000) * 10.0 ** rng.integers(-20, 30, 100000)])
    y = roundtrip(cuda, x)
    rel = np.abs(y - x) / np.abs(x)
    assert rel.max() <= 2.0 ** -46, rel.max()


def test_zero_and_tiny(cuda, pfft_lib):
    x = np.array([0.0, -0.0, 1e-30, -1e-37, 1e-300])
    y = roundtrip(cuda, x)
    assert y[0] == 0.0 and y[1] == 0.0
    assert abs(y[2] - x[2]) <= 2.0 ** -23 * abs(x[2])
    assert abs(y[3] - x[3]) <= 2.0 ** -23 * abs(x[3])
    assert y[4] == 0.0  # below the float range (2^-126): flushed


def fast_counts(torch, pairs):
    L = pg.lib()
    f = L.pfft_gb300_selftest_df_fast
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    a = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.float32)).cuda()
    c = torch.zeros(2, dtype=torch.int64, device="cuda")
    assert f(a.data_ptr(), a.numel() // 2, c.data_ptr(), None) == 0
    torch.cuda.synchronize()
    return [int(v) for v in c.cpu().tolist()]


def test_store_conversion_fast_path_bit_identical(cuda, pfft_lib):
    """The kernels store float-float values as doubles through a fast path
    (no range cases) and fall back to the full routine outside it; where the
    fast path applies its result is bit-identical to the full routine's:
    high words over the float range (powers of two included), low words up
    to 8 ulp of either sign (unnormalised), zeros, inf, NaN, denormals."""
    rng = np.random.default_rng(3)
    n = 400000
    hi = (rng.uniform(1, 2, n) * np.exp2(rng.integers(-126, 128, n))).astype(np.float32)
    hi[: n // 8] = np.exp2(rng.integers(-120, 120, n // 8)).astype(np.float32)  # powers of two
    hi *= rng.choice([-1, 1], n).astype(np.float32)
    scale = np.exp2(rng.integers(-30, 4, n).astype(np.float64))
    lo = (rng.uniform(-1, 1, n) * scale * np.spacing(np.abs(hi)).astype(np.float64)).astype(np.float32)
    lo[n // 16: n // 8] = -np.sign(hi[n // 16: n // 8]) * np.abs(lo[n // 16: n // 8])
    pairs = np.empty(2 * n, dtype=np.float32)
    pairs[0::2], pairs[1::2] = hi, lo
    specials = np.array([0, 0, -0.0, 0, np.inf, 0, np.nan, 0, 1e-40, 1e-45, 2.0 ** -80, 2.0 ** -105],
                        dtype=np.float32)
    took, diff = fast_counts(cuda, np.concatenate([pairs, specials]))
    assert diff == 0 and took > 200000, (took, diff)  # |hi| >= 2^-75, not a power of two

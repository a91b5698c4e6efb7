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

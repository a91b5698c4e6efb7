"""The reference's deterministic golden-data generator, restated in numpy
(TEST INFRASTRUCTURE ONLY).

api/api-basic.c:60-70   init_scalar: 1500+1250i at plain index 0, else
                        1000/(2m) + i*1000/(2m+1)
api/api-basic.c:72-87   init_scalar_periodic: index mod n per axis (C remainder)
api/api-basic.c:89-121  init_array: real arrays take the real part and 0 for
                        padding elements; Hermitian arrays 0.5(d1 + conj(d2))
                        with d2 at the mirrored index n - k
api/api-basic.c:254-264 plain_index: k += k*n[t] + kvec[t]  (not row-major;
                        reproduced as written)
"""
import numpy as np


def _cmod(a, n):
    # C remainder (sign follows the dividend)
    return np.fmod(a, n)


def plain_index(kv, n):
    k = np.zeros(kv[0].shape, dtype=np.int64)
    for t in range(len(n)):
        k = k + k * n[t] + kv[t]
    return k


def _scalar(kv, n, dtype):
    rdt = np.float32 if dtype == np.float32 else np.float64
    per = [_cmod(kv[t], n[t]) for t in range(len(n))]
    m = plain_index(per, n).astype(rdt)
    two_m = (rdt(2) * m)
    two_m1 = (rdt(2) * m + rdt(1))
    with np.errstate(divide="ignore"):
        re = (1000.0 / two_m.astype(np.float64)).astype(rdt)
        im = (1000.0 / two_m1.astype(np.float64)).astype(rdt)
    re = np.where(m == 0, rdt(1500.0), re)
    im = np.where(m == 0, rdt(1250.0), im)
    return re, im


def _grid(local_n, local_start):
    idx = np.indices(local_n, dtype=np.int64)
    return [idx[t] + local_start[t] for t in range(len(local_n))]


def init_complex(n, local_n, local_start, dtype=np.float64):
    kv = _grid(local_n, local_start)
    re, im = _scalar(kv, n, dtype)
    return re + 1j * im.astype(np.float64) if dtype == np.float64 else (re + 1j * im).astype(np.complex64)


def init_real(n, local_n, local_start, dtype=np.float64):
    kv = _grid(local_n, local_start)
    re, _ = _scalar(kv, n, dtype)
    return np.where(kv[-1] < n[-1], re, 0).astype(dtype)


def init_hermitian(n, local_n, local_start, dtype=np.float64):
    kv = _grid(local_n, local_start)
    re1, im1 = _scalar(kv, n, dtype)
    km = [n[t] - kv[t] for t in range(len(n))]
    re2, im2 = _scalar(km, n, dtype)
    d1 = re1.astype(np.float64) + 1j * im1.astype(np.float64)
    d2 = re2.astype(np.float64) + 1j * im2.astype(np.float64)
    v = 0.5 * (d1 + np.conj(d2))
    return v if dtype == np.float64 else v.astype(np.complex64)

"""CPU oracle of the GB300 PFFT library - TEST INFRASTRUCTURE ONLY.

Imported only by tests/, by __graft_entry__.smoke() and by the benchmark's
CPU-baseline leg, always as the checker (or the timed CPU baseline), never as
the thing measured on the GPU.  The reference (PFFT + FFTW-MPI + MPI) cannot be
built here, so the oracle is a restatement:

  pfft_oracle.c  transform semantics of pfft_execute at one process (FP64)
  layout.py      local-size / allocation integers
  golden.py      the reference's deterministic golden-data generator
  ghost.py       periodic-wrap ghost-cell exchange and its adjoint

How it is pinned is described in pfft_oracle.c and tests/test_oracle.py.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        LL = ctypes.POINTER(ctypes.c_longlong)
        IP = ctypes.POINTER(ctypes.c_int)
        DP = ctypes.POINTER(ctypes.c_double)
        L.oracle_execute.restype = ctypes.c_int
        L.oracle_execute.argtypes = [ctypes.c_int, LL, LL, LL, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, IP, IP, ctypes.c_uint, ctypes.c_int, DP, DP, ctypes.c_int]
        L.oracle_fft_lines.restype = ctypes.c_int
        L.oracle_fft_lines.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, DP]
        L.oracle_r2r_line.restype = ctypes.c_int
        L.oracle_r2r_line.argtypes = [ctypes.c_long, ctypes.c_int, DP, DP]
        _lib = L
    return _lib


KIND = {"c2c": 0, "r2c": 1, "c2r": 2, "r2r": 3}


def _ll(v):
    v = [int(x) for x in v]
    return (ctypes.c_longlong * len(v))(*v)


def execute(kind, n, ni, no, howmany, sign, flags, mesh_rank, inp, out_count, kinds=None, skip=None,
            padded=False, nthreads=None, out_init=None):
    """Run the oracle.  `inp` is a float64 array in the input memory layout
    (complex interleaved); returns a float64 array of `out_count` values in the
    output memory layout (initialised from `out_init` when given, so padding
    elements the transform does not write keep their values)."""
    L = lib()
    d = len(n)
    inp = np.ascontiguousarray(inp, dtype=np.float64)
    out = np.zeros(out_count, dtype=np.float64) if out_init is None else np.array(out_init, dtype=np.float64)
    ki = (ctypes.c_int * d)(*kinds) if kinds is not None else None
    sk = (ctypes.c_int * d)(*skip) if skip is not None else None
    if nthreads is None:
        nthreads = min(16, os.cpu_count() or 1)
    rc = L.oracle_execute(d, _ll(n), _ll(ni), _ll(no), int(howmany), KIND[kind], 1 if padded else 0, int(sign),
                          ki, sk, int(flags), int(mesh_rank),
                          inp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(nthreads))
    if rc != 0:
        raise ValueError("oracle rejected the request")
    return out


def fft_lines(x, sign=-1):
    """Complex DFT along the last axis of a complex128 array (oracle engine)."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    n = a.shape[-1]
    L = lib()
    buf = a.view(np.float64)
    L.oracle_fft_lines(n, a.size // n, sign, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return a


def r2r_line(x, kind):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib().oracle_r2r_line(x.size, kind, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return y

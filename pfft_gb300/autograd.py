"""Thin torch.autograd harness over the C-ABI (pfft_execute / the adjoint entry).

`PfftOp` owns one PFFT plan for fixed shapes; `apply(op, x)` runs it as a
differentiable torch function.  The forward calls pfft_execute_dft (or the
r2c / c2r variants) on the tensors' device memory, the backward calls
pfft_execute_adjoint_arrays, i.e. the hand-written adjoint kernels:
  c2c  the unnormalised transform of the opposite sign,
  r2c  a c2r of the half spectrum with interior bins halved,
  c2r  an r2c with interior bins doubled,
and zero-padding / truncation swap roles.  Gradients of complex tensors follow
torch's convention dL/dRe + i dL/dIm, for which these are exactly the adjoints
with respect to the real inner product.  Work is queued on torch's current
stream (no host synchronisation).
"""
import ctypes

import numpy as np
import torch

from . import (MPI_COMM_WORLD, PFFT_BACKWARD, PFFT_FORWARD, PFFT_PADDED_R2C, ints, lib, procmesh)

_PLAN = {"c2c": "plan_many_dft", "r2c": "plan_many_dft_r2c", "c2r": "plan_many_dft_c2r"}
_EXEC = {"c2c": "execute_dft", "r2c": "execute_dft_r2c", "c2r": "execute_dft_c2r"}


class PfftOp:
    """One plan: kind in {"c2c", "r2c", "c2r"}, sizes as in pfft_plan_many_*.

    The input tensor has PFFT's input layout for the plan (natural order unless
    TRANSPOSED_IN), the output its output layout; complex arrays are complex
    torch tensors."""

    def __init__(self, kind, n, ni=None, no=None, sign=PFFT_FORWARD, flags=0, dtype=torch.float64,
                 device="cuda", mesh_rank=2):
        self.kind = kind
        self.n = list(n)
        self.ni = list(ni) if ni is not None else list(n)
        self.no = list(no) if no is not None else list(n)
        self.sign = sign
        self.flags = flags
        self.real = dtype
        self.cplx = torch.complex128 if dtype == torch.float64 else torch.complex64
        self.pre = "pfft_" if dtype == torch.float64 else "pfftf_"
        self.device = torch.device(device)
        L = lib()
        d = len(self.n)
        a = [ints([0] * d) for _ in range(4)]
        comm = procmesh(mesh_rank) if mesh_rank > 0 else MPI_COMM_WORLD
        ls = {"c2c": "local_size_many_dft", "r2c": "local_size_many_dft_r2c", "c2r": "local_size_many_dft_c2r"}
        self.alloc = getattr(L, self.pre + ls[kind])(d, ints(self.n), ints(self.ni), ints(self.no), 1, None, None,
                                                     comm, flags, *a)
        self.local_ni = list(a[0])
        self.local_no = list(a[2])
        self.in_shape = tuple(self.local_ni)
        self.out_shape = tuple(self.local_no)
        self.in_dtype = self.real if kind == "r2c" else self.cplx
        self.out_dtype = self.real if kind == "c2r" else self.cplx
        # plan on scratch arrays of the right sizes; execution uses the caller's arrays
        x = torch.empty(self.in_shape, dtype=self.in_dtype, device=self.device)
        y = torch.empty(self.out_shape, dtype=self.out_dtype, device=self.device)
        self.plan = getattr(L, self.pre + _PLAN[kind])(d, ints(self.n), ints(self.ni), ints(self.no), 1, None, None,
                                                       x.data_ptr(), y.data_ptr(), comm, sign, flags)
        if not self.plan:
            raise RuntimeError("PFFT planner returned NULL")
        getattr(L, self.pre + "gb300_set_sync")(self.plan, 0)

    def _stream(self):
        s = torch.cuda.current_stream(self.device)
        getattr(lib(), self.pre + "gb300_set_stream")(self.plan, ctypes.c_void_p(s.cuda_stream))

    def forward(self, x):
        x = x.contiguous()
        assert tuple(x.shape) == self.in_shape and x.dtype == self.in_dtype
        y = torch.empty(self.out_shape, dtype=self.out_dtype, device=self.device)
        self._stream()
        getattr(lib(), self.pre + _EXEC[self.kind])(self.plan, x.data_ptr(), y.data_ptr())
        return y

    def adjoint(self, gy):
        gy = gy.contiguous()
        assert tuple(gy.shape) == self.out_shape
        gx = torch.zeros(self.in_shape, dtype=self.in_dtype, device=self.device)
        self._stream()
        getattr(lib(), self.pre + "execute_adjoint_arrays")(self.plan, gy.data_ptr(), gx.data_ptr())
        return gx

    def __del__(self):
        try:
            if self.plan:
                getattr(lib(), self.pre + "destroy_plan")(self.plan)
        except Exception:
            pass


class _Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        ctx.op = op
        return op.forward(x)

    @staticmethod
    def backward(ctx, gy):
        return ctx.op.adjoint(gy), None


def apply(op, x):
    """Differentiable application of a PfftOp."""
    return _Fn.apply(x, op)

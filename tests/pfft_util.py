"""Shared helpers of the test-suite: run a PFFT plan through the C-ABI on the
GPU (torch only provides device memory) and run the same request through the
CPU oracle, both on arrays in PFFT's memory layouts."""
import ctypes

import numpy as np

import pfft_gb300 as pg
from oracle import layout as LO

TR = {"c2c": LO.C2C, "r2c": LO.R2C, "c2r": LO.C2R, "r2r": LO.R2R}
LS_NAME = {"c2c": "local_size_many_dft", "r2c": "local_size_many_dft_r2c", "c2r": "local_size_many_dft_c2r",
           "r2r": "local_size_many_r2r"}
PLAN_NAME = {"c2c": "plan_many_dft", "r2c": "plan_many_dft_r2c", "c2r": "plan_many_dft_c2r",
             "r2r": "plan_many_r2r"}


class Req:
    """A plan request in PFFT terms."""

    def __init__(self, kind, n, ni=None, no=None, howmany=1, sign=-1, flags=0, cart=2, kinds=None, skip=None):
        self.kind = kind
        self.n = list(n)
        self.ni = list(ni) if ni is not None else list(n)
        self.no = list(no) if no is not None else list(n)
        self.howmany = howmany
        self.sign = sign
        self.flags = flags
        self.cart = cart
        self.kinds = kinds
        self.skip = skip

    @property
    def d(self):
        return len(self.n)

    def sizes(self):
        return LO.local_size(self.d, self.n, self.ni, self.no, self.howmany, TR[self.kind], self.flags, self.cart)

    def in_complex(self):
        return self.kind in ("c2c", "c2r")

    def out_complex(self):
        return self.kind in ("c2c", "r2c")

    def counts(self):
        """(doubles in the input layout, doubles in the output layout, alloc_local)."""
        mem, lni, _, lno, _ = self.sizes()
        ci = int(np.prod(lni)) * self.howmany * (2 if self.in_complex() else 1)
        co = int(np.prod(lno)) * self.howmany * (2 if self.out_complex() else 1)
        return ci, co, mem

    def mesh_rank(self):
        return LO.mesh_rank(self.d, self.cart)

    def padded(self):
        return bool(self.flags & pg.PFFT_PADDED_R2C) and not (self.d == 3 and self.cart == 3)


def random_input(req, rng, dist="uniform"):
    ci, _, _ = req.counts()
    if dist == "normal":
        x = rng.standard_normal(ci)
    else:
        x = rng.uniform(-1.0, 1.0, ci)
    if req.kind == "r2c" and req.padded():
        # zero the padding reals of each row (they are not read)
        _, lni, _, _, _ = req.sizes()
        a = x.reshape(-1, lni[-1] * req.howmany)
        a[:, req.ni[-1] * req.howmany:] = 0
        x = a.ravel()
    return x


def oracle_run(req, x, nthreads=None):
    import oracle
    _, co, _ = req.counts()
    return oracle.execute(req.kind, req.n, req.ni, req.no, req.howmany, req.sign, req.flags, req.mesh_rank(), x,
                          co, kinds=req.kinds, skip=req.skip, padded=req.padded(), nthreads=nthreads)


def comm_for(req):
    return pg.MPI_COMM_WORLD if req.cart == 0 else pg.procmesh(req.cart)


class double_arith:
    """Context manager selecting the double API's arithmetic for the plans
    created inside it: "double" keeps the default (64-bit fixed point on the
    radix-8 passes, FP64 elsewhere), "double-f64" native FP64 everywhere,
    "double-df" TwoSum float-float, "double-dfq" float-float with
    block-quantised radix-8 stages; "float" changes nothing."""

    MODES = {"double-df": 0, "double-f64": 1, "double-dfq": 3}

    def __init__(self, prec):
        self.mode = self.MODES.get(prec)

    def __enter__(self):
        if self.mode is not None:
            L = pg.lib()
            self.old = L.pfft_gb300_get_double_arith()
            assert L.pfft_gb300_set_double_arith(self.mode) == 0
        return self

    def __exit__(self, *exc):
        if self.mode is not None:
            pg.lib().pfft_gb300_set_double_arith(self.old)
        return False


def is_double(prec):
    return prec != "float"


def gpu_run(req, x, prec="double", inplace=False, adjoint=False, torch=None, keep=False):
    """Plan + execute through the C-ABI with device arrays; returns float64
    numpy of the output layout (the adjoint maps the output layout to the
    input layout).  prec: "float", "double" (default arithmetic), "double-df",
    "double-dfq" or "double-f64"."""
    import torch as _t
    torch = torch or _t
    L = pg.lib()
    pre = "pfft_" if is_double(prec) else "pfftf_"
    rdt = torch.float64 if is_double(prec) else torch.float32
    ci, co, mem = req.counts()
    words = 2 * mem  # alloc_local is in complex units for complex arrays
    words = max(words, ci, co)
    dev = torch.device("cuda")
    a = torch.zeros(words, dtype=rdt, device=dev)
    b = a if inplace else torch.zeros(words, dtype=rdt, device=dev)
    src, dst = (b, a) if adjoint else (a, b)
    nin = co if adjoint else ci
    src[:nin] = torch.from_numpy(np.asarray(x, dtype=np.float64)).to(dev, rdt)
    comm = comm_for(req)
    fn = getattr(L, pre + PLAN_NAME[req.kind])
    n, ni, no = pg.ints(req.n), pg.ints(req.ni), pg.ints(req.no)
    # the _skipped planners take the per-axis skip flags after the block sizes
    pre_args = (req.d, n, ni, no, req.howmany, None, None)
    if req.skip is not None:
        fn = getattr(L, pre + PLAN_NAME[req.kind] + "_skipped")
        pre_args = pre_args + (pg.cints(req.skip),)
    with double_arith(prec):
        if req.kind == "r2r":
            kinds = pg.cints(req.kinds)
            plan = fn(*pre_args, a.data_ptr(), b.data_ptr(), comm, kinds, req.flags)
        else:
            plan = fn(*pre_args, a.data_ptr(), b.data_ptr(), comm, req.sign, req.flags)
    if not plan:
        raise RuntimeError("planner returned NULL: %s" % (pg.last_error(),))
    try:
        torch.cuda.synchronize()
        if adjoint:
            getattr(L, pre + "execute_adjoint")(plan)
        else:
            getattr(L, pre + "execute")(plan)
        torch.cuda.synchronize()
        nout = ci if adjoint else co
        out = dst[:nout].double().cpu().numpy()
    finally:
        getattr(L, pre + "destroy_plan")(plan)
    code, msg = pg.last_error()
    return out


def mask_padding(req, out):
    """Zero the row padding of a padded c2r output (its contents are
    unspecified, as in the reference, which uses the output as scratch)."""
    if req.kind != "c2r" or not req.padded():
        return out
    _, _, _, lno, _ = req.sizes()
    a = np.array(out, dtype=np.float64).reshape(-1, lno[-1] * req.howmany)
    a[:, req.no[-1] * req.howmany:] = 0
    return a.ravel()


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)

"""Python binding of the GB300 PFFT C-ABI library (libpfft_gb300.so).

This is the ctypes binding a Python user of PFFT would use, and the one the
tests and the benchmark call through.  It loads the in-tree library and
declares the argument types of the entry points; nothing here computes a
transform.  If the library has not been built, `lib()` raises (build it with
`python -m pfft_gb300.build` or `__graft_entry__.build()`).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libpfft_gb300.so")

INT = ctypes.c_ssize_t  # ptrdiff_t
c_void_p = ctypes.c_void_p

# ---- flags (api/pfft.h:528-572) --------------------------------------------
PFFT_TRANSPOSED_NONE = 0
PFFT_TRANSPOSED_IN = 1 << 0
PFFT_TRANSPOSED_OUT = 1 << 1
PFFT_SHIFTED_NONE = 0
PFFT_SHIFTED_IN = 1 << 2
PFFT_SHIFTED_OUT = 1 << 3
PFFT_MEASURE = 0
PFFT_ESTIMATE = 1 << 4
PFFT_PATIENT = 1 << 5
PFFT_EXHAUSTIVE = 1 << 6
PFFT_NO_TUNE = 0
PFFT_TUNE = 1 << 7
PFFT_PRESERVE_INPUT = 1 << 8
PFFT_DESTROY_INPUT = 1 << 9
PFFT_BUFFERED_INPLACE = 1 << 10
PFFT_PADDED_R2C = 1 << 11
PFFT_PADDED_C2R = PFFT_PADDED_R2C

PFFT_FORWARD = -1
PFFT_BACKWARD = 1

PFFT_R2HC, PFFT_HC2R, PFFT_DHT = 0, 1, 2
PFFT_REDFT00, PFFT_REDFT01, PFFT_REDFT10, PFFT_REDFT11 = 3, 4, 5, 6
PFFT_RODFT00, PFFT_RODFT01, PFFT_RODFT10, PFFT_RODFT11 = 7, 8, 9, 10

PFFT_GC_TRANSPOSED_NONE = 0
PFFT_GC_TRANSPOSED = 1 << 0
PFFT_GC_SENDRECV = 1 << 1
PFFT_GC_RMA = 1 << 2
PFFT_GC_R2C = 1 << 3
PFFT_GC_PADDED = 1 << 4

MPI_COMM_WORLD = 1
MPI_COMM_SELF = 2

_lib = None

_P = ctypes.POINTER(INT)
_IP = ctypes.POINTER(ctypes.c_int)


def _declare(L):
    for pre in ("pfft_", "pfftf_"):
        R = ctypes.c_double if pre == "pfft_" else ctypes.c_float
        f = lambda name: getattr(L, pre + name)
        for nm in ("local_size_dft_3d", "local_size_dft_r2c_3d", "local_size_dft_c2r_3d", "local_size_r2r_3d"):
            f(nm).restype = INT
            f(nm).argtypes = [_P, ctypes.c_int, ctypes.c_uint, _P, _P, _P, _P]
        for nm in ("local_size_dft", "local_size_dft_r2c", "local_size_dft_c2r", "local_size_r2r"):
            f(nm).restype = INT
            f(nm).argtypes = [ctypes.c_int, _P, ctypes.c_int, ctypes.c_uint, _P, _P, _P, _P]
        for nm in ("local_size_many_dft", "local_size_many_dft_r2c", "local_size_many_dft_c2r",
                   "local_size_many_r2r"):
            f(nm).restype = INT
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, INT, _P, _P, ctypes.c_int, ctypes.c_uint, _P, _P, _P, _P]
        for nm in ("local_block_many_dft", "local_block_many_dft_r2c", "local_block_many_dft_c2r",
                   "local_block_many_r2r"):
            f(nm).restype = None
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_uint,
                              _P, _P, _P, _P]
        for nm in ("plan_dft_3d", "plan_dft_r2c_3d", "plan_dft_c2r_3d"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [_P, c_void_p, c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        f("plan_r2r_3d").restype = c_void_p
        f("plan_r2r_3d").argtypes = [_P, c_void_p, c_void_p, ctypes.c_int, _IP, ctypes.c_uint]
        for nm in ("plan_dft", "plan_dft_r2c", "plan_dft_c2r"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [ctypes.c_int, _P, c_void_p, c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        f("plan_r2r").restype = c_void_p
        f("plan_r2r").argtypes = [ctypes.c_int, _P, c_void_p, c_void_p, ctypes.c_int, _IP, ctypes.c_uint]
        for nm in ("plan_many_dft", "plan_many_dft_r2c", "plan_many_dft_c2r"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, INT, _P, _P, c_void_p, c_void_p, ctypes.c_int,
                              ctypes.c_int, ctypes.c_uint]
        f("plan_many_r2r").restype = c_void_p
        f("plan_many_r2r").argtypes = [ctypes.c_int, _P, _P, _P, INT, _P, _P, c_void_p, c_void_p,
                                       ctypes.c_int, _IP, ctypes.c_uint]
        for nm in ("plan_many_dft_skipped", "plan_many_dft_r2c_skipped", "plan_many_dft_c2r_skipped"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, INT, _P, _P, _IP, c_void_p, c_void_p, ctypes.c_int,
                              ctypes.c_int, ctypes.c_uint]
        f("plan_many_r2r_skipped").restype = c_void_p
        f("plan_many_r2r_skipped").argtypes = [ctypes.c_int, _P, _P, _P, INT, _P, _P, _IP, c_void_p, c_void_p,
                                               ctypes.c_int, _IP, ctypes.c_uint]
        for nm in ("execute", "destroy_plan", "execute_adjoint"):
            f(nm).restype = None
            f(nm).argtypes = [c_void_p]
        for nm in ("execute_dft", "execute_dft_r2c", "execute_dft_c2r", "execute_r2r", "execute_adjoint_arrays"):
            f(nm).restype = None
            f(nm).argtypes = [c_void_p, c_void_p, c_void_p]
        for nm in ("init_input_complex_3d", "init_input_complex_hermitian_3d", "init_input_real_3d",
                   "clear_input_complex_3d", "clear_input_complex_hermitian_3d", "clear_input_real_3d"):
            f(nm).restype = None
            f(nm).argtypes = [_P, _P, _P, c_void_p]
        for nm in ("init_input_complex", "init_input_complex_hermitian", "init_input_real",
                   "clear_input_complex", "clear_input_complex_hermitian", "clear_input_real"):
            f(nm).restype = None
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, c_void_p]
        for nm in ("check_output_complex_3d", "check_output_complex_hermitian_3d", "check_output_real_3d"):
            f(nm).restype = R
            f(nm).argtypes = [_P, _P, _P, c_void_p, ctypes.c_int]
        for nm in ("check_output_complex", "check_output_complex_hermitian", "check_output_real"):
            f(nm).restype = R
            f(nm).argtypes = [ctypes.c_int, _P, _P, _P, c_void_p, ctypes.c_int]
        f("create_procmesh").restype = ctypes.c_int
        f("create_procmesh").argtypes = [ctypes.c_int, ctypes.c_int, _IP, _IP]
        f("create_procmesh_1d").restype = ctypes.c_int
        f("create_procmesh_1d").argtypes = [ctypes.c_int, ctypes.c_int, _IP]
        f("create_procmesh_2d").restype = ctypes.c_int
        f("create_procmesh_2d").argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _IP]
        for nm in ("local_size_gc_3d",):
            f(nm).restype = INT
            f(nm).argtypes = [_P, _P, _P, _P, _P, _P]
        f("local_size_many_gc").restype = INT
        f("local_size_many_gc").argtypes = [ctypes.c_int, _P, _P, INT, _P, _P, _P, _P]
        for nm in ("plan_rgc_3d", "plan_cgc_3d"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [_P, _P, _P, c_void_p, ctypes.c_int, ctypes.c_uint]
        for nm in ("plan_many_rgc", "plan_many_cgc"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [ctypes.c_int, _P, INT, _P, _P, _P, c_void_p, ctypes.c_int, ctypes.c_uint]
        for nm in ("exchange", "reduce", "destroy_gcplan"):
            f(nm).restype = None
            f(nm).argtypes = [c_void_p]
        f("gb300_gc_set_stream").restype = ctypes.c_int
        f("gb300_gc_set_stream").argtypes = [c_void_p, c_void_p]
        for nm in ("alloc_real", "alloc_complex", "malloc"):
            f(nm).restype = c_void_p
            f(nm).argtypes = [ctypes.c_size_t]
        f("free").restype = None
        f("free").argtypes = [c_void_p]
        for nm in ("init", "cleanup"):
            f(nm).restype = None
            f(nm).argtypes = []
        for nm in ("gb300_set_stream",):
            f(nm).restype = ctypes.c_int
            f(nm).argtypes = [c_void_p, c_void_p]
        for nm in ("gb300_set_sync", "gb300_set_graph", "gb300_set_pipeline"):
            f(nm).restype = ctypes.c_int
            f(nm).argtypes = [c_void_p, ctypes.c_int]
        f("gb300_plan_info").restype = ctypes.c_int
        f("gb300_plan_info").argtypes = [c_void_p, _IP, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_size_t)]
        f("gb300_set_pass_timing").restype = ctypes.c_int
        f("gb300_set_pass_timing").argtypes = [c_void_p, ctypes.c_int]
        f("gb300_pass_time").restype = ctypes.c_int
        f("gb300_pass_time").argtypes = [c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), _IP]
        f("gb300_pass_info").restype = ctypes.c_int
        f("gb300_pass_info").argtypes = [c_void_p, ctypes.c_int, _IP, _IP, _IP, _IP, _IP,
                                         ctypes.POINTER(ctypes.c_double)]
    L.pfft_gb300_batch_create.restype = c_void_p
    L.pfft_gb300_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(c_void_p)]
    L.pfftf_gb300_batch_create.restype = c_void_p
    L.pfftf_gb300_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(c_void_p)]
    L.pfft_gb300_batch_execute.restype = ctypes.c_int
    L.pfft_gb300_batch_execute.argtypes = [c_void_p]
    L.pfft_gb300_batch_set_stream.argtypes = [c_void_p, c_void_p]
    L.pfft_gb300_batch_set_graph.argtypes = [c_void_p, ctypes.c_int]
    L.pfft_gb300_batch_info.argtypes = [c_void_p, _IP, _IP, _IP, ctypes.POINTER(ctypes.c_double)]
    L.pfft_gb300_batch_destroy.argtypes = [c_void_p]
    L.pfft_gb300_batch_wait_selftest.restype = ctypes.c_int
    L.pfft_gb300_batch_wait_selftest.argtypes = [ctypes.c_longlong]
    L.pfft_gb300_last_error.restype = ctypes.c_int
    L.pfft_gb300_last_error_string.restype = ctypes.c_char_p
    L.pfft_gb300_set_double_arith.argtypes = [ctypes.c_int]
    L.pfft_gb300_set_double_arith.restype = ctypes.c_int
    L.pfft_gb300_set_fx_link.argtypes = [ctypes.c_int]
    L.pfft_gb300_set_fx_link.restype = ctypes.c_int
    for nm in ("pfft_gb300_plan_arith", "pfftf_gb300_plan_arith"):
        getattr(L, nm).argtypes = [c_void_p]
        getattr(L, nm).restype = ctypes.c_int
    L.pfft_gb300_export_wisdom_to_string.restype = c_void_p
    L.pfft_gb300_import_wisdom_from_string.argtypes = [ctypes.c_char_p]
    L.pfft_gb300_import_wisdom_from_string.restype = ctypes.c_int
    L.pfft_gb300_export_wisdom_to_filename.argtypes = [ctypes.c_char_p]
    L.pfft_gb300_export_wisdom_to_filename.restype = ctypes.c_int
    L.pfft_gb300_import_wisdom_from_filename.argtypes = [ctypes.c_char_p]
    L.pfft_gb300_import_wisdom_from_filename.restype = ctypes.c_int
    L.pfft_gb300_wisdom_entries.restype = ctypes.c_int
    for nm in ("pfft_gb300_pass_fx_link", "pfftf_gb300_pass_fx_link"):
        getattr(L, nm).argtypes = [c_void_p, ctypes.c_int]
        getattr(L, nm).restype = ctypes.c_int
    for nm in ("pfft_gb300_pass_kernel", "pfftf_gb300_pass_kernel"):
        getattr(L, nm).argtypes = [c_void_p, ctypes.c_int]
        getattr(L, nm).restype = ctypes.c_int
    L.pfft_gb300_set_kernel_path.argtypes = [ctypes.c_int]
    L.pfft_gb300_get_kernel_path.restype = ctypes.c_int
    L.pfft_gb300_get_double_arith.restype = ctypes.c_int
    L.pfft_gb300_set_staged.argtypes = [ctypes.c_int]
    L.pfft_gb300_get_staged.restype = ctypes.c_int
    L.pfft_gb300_staged_launches.restype = ctypes.c_longlong
    L.pfft_gb300_pipelined_executes.restype = ctypes.c_longlong
    L.pfft_gb300_staged_status.restype = ctypes.c_int


def export_wisdom():
    """The wisdom of this process as text (see pfft_gb300_export_wisdom_to_string)."""
    L = lib()
    p = L.pfft_gb300_export_wisdom_to_string()
    if not p:
        return None
    try:
        return ctypes.string_at(p).decode()
    finally:
        ctypes.CDLL(None).free(ctypes.c_void_p(p))


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("libpfft_gb300.so is not built (run pfft_gb300/build.py)")
        L = ctypes.CDLL(LIBPATH)
        _declare(L)
        _lib = L
    return _lib


def ints(seq):
    """ptrdiff_t array from a sequence."""
    seq = list(seq)
    return (INT * len(seq))(*seq)


def cints(seq):
    seq = list(seq)
    return (ctypes.c_int * len(seq))(*seq)


def procmesh(rnk=2):
    """A 1x...x1 Cartesian communicator of the given rank."""
    L = lib()
    c = ctypes.c_int(0)
    rc = L.pfft_create_procmesh(rnk, MPI_COMM_WORLD, cints([1] * rnk), ctypes.byref(c))
    if rc:
        raise RuntimeError("create_procmesh failed")
    return c.value


def last_error():
    L = lib()
    return L.pfft_gb300_last_error(), (L.pfft_gb300_last_error_string() or b"").decode()

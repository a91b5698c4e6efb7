"""The C-ABI library loads and exports every entry point its headers declare
(no GPU needed)."""
import os
import re
import subprocess

import pfft_gb300 as pg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    hdr = open(os.path.join(ROOT, "include", "pfft.h")).read()
    body = hdr[hdr.index("#define PFFT_GB300_DECLARE"):hdr.index("PFFT_GB300_DECLARE(pfft_, double")]
    names = set(re.findall(r"PX##(\w+)\s*\(", body))
    for pre in ("pfft_", "pfftf_"):
        syms |= {pre + nm for nm in names}
    for h in ("pfft_gb300.h", "mpi.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b((?:pfftf?_|MPI_)\w+)\s*\(", txt, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_library_exports_all_declared_symbols(pfft_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", pg.LIBPATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    want = declared_symbols()
    assert len(want) > 250
    missing = sorted(want - exported)
    assert not missing, missing


def test_library_has_no_torch_dependency(pfft_lib):
    out = subprocess.run(["ldd", pg.LIBPATH], capture_output=True, text=True).stdout
    assert "torch" not in out and "c10" not in out


def test_noalloc_buffer_rule(pfft_lib):
    """The buffer check of the allocation-free exchange (no GPU needed):
    managed memory and device memory of the current device are accepted; a
    device pointer of another GPU is refused with cudaErrorInvalidDevice
    (101) and host memory with cudaErrorInvalidValue (1), before anything is
    queued."""
    import ctypes
    f = pfft_lib.pg_noalloc_buffer_check
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    unregistered, host, device, managed = 0, 1, 2, 3  # cudaMemoryType
    assert f(device, 0, 0) == 0
    assert f(device, 3, 3) == 0
    assert f(managed, 0, 1) == 0
    assert f(device, 1, 0) == 101
    assert f(device, 0, 2) == 101
    assert f(host, 0, 0) == 1
    assert f(unregistered, 0, 0) == 1

"""Build libpfft_gb300.so (the C-ABI library) in-tree with nvcc for sm_103a.

Every translation unit under pfft_gb300/csrc is compiled in parallel and
linked into pfft_gb300/libpfft_gb300.so.  The batched-launch units
(batch*.cu) are relocatable device code, device-linked together, so that the
tile functions of the persistent kernel compile in parallel units.  A unit is
recompiled only when it or one of the headers is newer than its object file.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpfft_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build pfft_gb300")
    return cand


def _cuda_lib_dir():
    nv = os.path.realpath(_nvcc())
    return os.path.join(os.path.dirname(os.path.dirname(nv)), "lib64")


def _headers():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _rdc(src):
    return os.path.basename(src).startswith("batch")


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _rdc(src):
        extra = list(extra) + ["-rdc=true"]
    if os.path.basename(src).startswith("batch_tiles"):
        extra = list(extra) + ["-maxrregcount=80"]  # callees of a kernel bounded to three 256-thread blocks per SM
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, None
    cmd = [_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                              "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(verbose=False, extra=None):
    """Compile and link the library; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    extra = list(extra or [])
    objs, errs = [], []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for obj, err in ex.map(lambda s: _compile(s, extra), srcs):
            objs.append(obj)
            if err:
                errs.append(err)
    if errs:
        raise RuntimeError("\n".join(errs))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        libdir = _cuda_lib_dir()
        rdc = [o for s_, o in zip(srcs, objs) if _rdc(s_)]
        dlink = os.path.join(BUILD, "device_link.o")
        cmd = [_nvcc()] + ARCH + ["-dlink", "-Xcompiler", "-fPIC", "-o", dlink] + rdc
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("device link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB + ".tmp"] + objs + [dlink,
            "-Xlinker", "--no-undefined", "-Xlinker", "-rpath," + libdir, "-L" + libdir]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])

"""Benchmark of the PFFT transform-execution path on GB300.

Workload (one step): one forward pfft_execute of a 512^3 complex128 c2c
transform on a 1x1 process mesh, out of place, standard layout - the
configuration the headline target is quoted on.  The plan is made with
PFFT_PATIENT (the autotuner runs at planning time, outside the timed region).  Inputs are uniform[-1,1)
from a fixed seed, 2.1 GB per array (larger than the 129 MB L2, so no flush is
needed between steps).

  value   algorithmic GB/s of the execute with device-resident arrays:
          B = P_min * 2 * N * 16 bytes (P_min = 3 minimal HBM passes for 512^3
          complex128) divided by the CUDA-event time of the step
  e2e     the same metric through the C-ABI with pinned HOST arrays
          (host->device copy of the input and device->host copy of the output
          inside the timed region, done by pfft_execute itself)
  roofline  the pass kernel (the only kernel of the path): algorithmic bytes
          of one launch over its CUDA-event duration, against the measured HBM
          copy bandwidth; traffic from the committed ncu summary
  cpu_baseline  the CPU oracle (a C FP64 port, not the reference, which cannot
          be built: it needs FFTW-MPI and MPI) on all host cores, one full
          forward execute of the same 512^3 workload; scipy_baseline is
          scipy.fft.fftn on the same input and cores (labelled: not the
          reference)
  accuracy  round-trip relative L2 error (backward of the measured forward
          output, divided by N, against the input) and the Parseval defect of
          the measured transform; the double API's arithmetic is its default
          (float-float with block-quantised radix-8 stages at this size)

--impl reference times that CPU port instead (the reference arm): the full
512^3 forward every step, with the real per-step wall time.
With --gpus N > 1 (torchrun), every rank runs an independent replica (the path
does not shard on one node without MPI); value sums the ranks' bytes over the
slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N3 = (512, 512, 512)
P_MIN = 3
ELEM = 16  # complex128


def algo_bytes(n=N3):
    return P_MIN * 2 * int(np.prod(n)) * ELEM


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get("c2c_512_f64_pass_bytes_per_launch")
    except Exception:
        return None


class Clocks:
    """Sample SM clocks and throttle reasons with nvidia-smi every 50 ms; only
    the samples stamped inside the timed window are kept."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self, t0=None, t1=None):
        """t0, t1: wall-clock (time.time()) bounds of the timed window."""
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons, pw = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                ts = time.mktime(time.strptime(s[0].split(".")[0], "%Y/%m/%d %H:%M:%S")) + \
                    float("0." + s[0].split(".")[1]) if "." in s[0] else 0.0
                if t0 is not None and not (t0 - 0.05 <= ts <= t1 + 0.05):
                    continue
                sm.append(float(s[1]))
                mx = float(s[2])
                pw.append(float(s[3]))
                for i, nm in enumerate(names):
                    if s[4 + i].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_median": statistics.median(pw) if pw else None}


def _oracle_forward(n, x, threads):
    import oracle
    cnt = 2 * int(np.prod(n))
    return oracle.execute("c2c", n, n, n, 1, -1, 0, 2, x, cnt, nthreads=threads)


def cpu_input(n, seed=1):
    return np.random.default_rng(seed).uniform(-1.0, 1.0, 2 * int(np.prod(n)))


def cpu_baseline(n=N3, threads=None, x=None, keep=None):
    """Time the CPU oracle on one full forward execute of the workload (the
    whole 512^3 complex128 transform, about 3 s on 16 cores).  keep: a dict
    that receives the oracle's output ("out"), the FP64 reference the GPU
    results are compared with."""
    threads = threads or (os.cpu_count() or 1)
    x = cpu_input(n) if x is None else x
    t0 = time.perf_counter()
    y = _oracle_forward(n, x, threads)
    dt = time.perf_counter() - t0
    if keep is not None:
        keep["out"] = y
    return {"value": algo_bytes(n) / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "the full workload: one %s c2c complex128 forward, %.2f s" % ("x".join(map(str, n)), dt),
            "seconds": dt}


def scipy_baseline(n=N3, threads=None, x=None, reps=1):
    """scipy.fft.fftn (pocketfft, not the reference and not FFTW) on the same
    input with all host threads: a second, independent CPU number."""
    try:
        import scipy.fft as sf
    except Exception as e:  # pragma: no cover - scipy is on both machines
        return {"unavailable": "scipy.fft not importable: %s" % e}
    threads = threads or (os.cpu_count() or 1)
    x = cpu_input(n) if x is None else x
    z = x.view(np.complex128).reshape(n)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        sf.fftn(z, workers=threads)
        ts.append(time.perf_counter() - t0)
    dt = statistics.median(ts)
    return {"value": algo_bytes(n) / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "scipy",
            "sample": "scipy.fft.fftn(workers=%d) of the full %s complex128 input, median of %d, %.2f s; "
                      "not the reference" % (threads, "x".join(map(str, n)), reps, dt)}


BATCH_SIZES = [(32, 32, 32), (48, 64, 40), (96, 96, 96), (128, 128, 64), (128, 128, 128)]


def measure_batched(L, pg, torch, prec, nplans=64, seed=11, reps=5, tune=True):
    """64 uneven c2c transforms (sizes drawn by seed from BATCH_SIZES): one
    persistent batched launch (CUDA graph) against a per-plan loop of plain
    pfft_execute calls (blocking, as the reference's execute) and against the
    same loop queued asynchronously on one stream; returns times, ratios and
    the largest relative difference between the batch and the loop outputs."""
    pre = "pfft_" if prec == "double" else "pfftf_"
    cdt = torch.complex128 if prec == "double" else torch.complex64
    rng = np.random.default_rng(seed)
    comm = pg.procmesh(2)
    flags = pg.PFFT_PATIENT if tune else 0  # autotuned radix / tile choices (planning time)
    plans, outs, pts = [], [], 0
    for _ in range(nplans):
        n = BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))]
        x = torch.from_numpy(rng.uniform(-1, 1, 2 * int(np.prod(n)))).view(torch.complex128).to(cdt).cuda()
        y = torch.zeros_like(x)
        p = getattr(L, pre + "plan_dft_3d")(pg.ints(n), x.data_ptr(), y.data_ptr(), comm, pg.PFFT_FORWARD, flags)
        if not p:
            raise RuntimeError("plan failed: %s" % (pg.last_error(),))
        plans.append((p, x, y))
        outs.append(y)
        pts += int(np.prod(n))
    ex = getattr(L, pre + "execute")
    s0 = torch.cuda.default_stream()

    def timed(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s0)
        for _ in range(reps):
            fn()
        e1.record(s0)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def loop():
        for p, _, _ in plans:
            ex(p)
    loop_ms = timed(loop)
    ref = [y.clone() for y in outs]
    for p, _, _ in plans:
        getattr(L, pre + "gb300_set_sync")(p, 0)
    loop_async_ms = timed(loop)
    for p, _, _ in plans:
        getattr(L, pre + "gb300_set_sync")(p, 1)
    arr = (ctypes.c_void_p * nplans)(*[p for p, _, _ in plans])
    b = getattr(L, pre + "gb300_batch_create")(nplans, arr)
    if not b:
        raise RuntimeError("batch failed: %s" % (pg.last_error(),))
    for y in outs:
        y.zero_()

    def batch():
        if L.pfft_gb300_batch_execute(b) != 0:
            raise RuntimeError("batch execute failed: %s" % (pg.last_error(),))
    batch_ms = timed(batch)
    ntasks, grid = ctypes.c_int(0), ctypes.c_int(0)
    L.pfft_gb300_batch_info(b, ctypes.byref(ntasks), ctypes.byref(grid), None, None)
    diff = max(float(torch.linalg.vector_norm(y - r) / torch.linalg.vector_norm(r)) for y, r in zip(outs, ref))
    L.pfft_gb300_batch_destroy(b)
    for p, _, _ in plans:
        getattr(L, pre + "destroy_plan")(p)
    esz = 16 if prec == "double" else 8
    return {"transforms": nplans, "points": pts, "dtype": "complex128" if prec == "double" else "complex64",
            "batch_ms": batch_ms, "loop_ms": loop_ms, "loop_async_ms": loop_async_ms,
            "ratio": loop_ms / batch_ms, "ratio_vs_async_loop": loop_async_ms / batch_ms,
            "batch_gbs_min_traffic": 3 * 2 * pts * esz / (batch_ms * 1e-3) / 1e9,
            "max_rel_l2_batch_vs_loop": diff, "tasks": ntasks.value, "grid": grid.value,
            "planner": "PFFT_PATIENT" if tune else "PFFT_MEASURE"}


def measure_adjoint(L, pg, torch, reps=5):
    """Cost of a forward+adjoint gradient step through the C-ABI against two
    plain executes, on the differentiable oversampled r2c (float32 128^3
    zero-padded to 256^3) and on the 512^3 c2c complex128 transform."""
    res = {}
    comm = pg.procmesh(2)
    s = torch.cuda.Stream()
    cases = [("r2c_f32_128to256", "pfftf_", 3, (256, 256, 256), (128, 128, 128)),
             ("c2c_f64_512", "pfft_", 3, (512, 512, 512), (512, 512, 512))]
    for name, pre, d, n, ni in cases:
        a = [pg.ints([0] * d) for _ in range(4)]
        kind = "r2c" if name.startswith("r2c") else "c2c"
        ls = "local_size_many_dft_r2c" if kind == "r2c" else "local_size_many_dft"
        alloc = getattr(L, pre + ls)(d, pg.ints(n), pg.ints(ni), pg.ints(n), 1, None, None, comm, 0, *a)
        x = torch.zeros(2 * alloc, dtype=torch.float64 if pre == "pfft_" else torch.float32, device="cuda")
        y = torch.zeros_like(x)
        x.uniform_(-1, 1)
        pl = "plan_many_dft_r2c" if kind == "r2c" else "plan_many_dft"
        p = getattr(L, pre + pl)(d, pg.ints(n), pg.ints(ni), pg.ints(n), 1, None, None, x.data_ptr(), y.data_ptr(),
                                 comm, pg.PFFT_FORWARD, 0)
        if not p:
            raise RuntimeError("plan failed: %s" % (pg.last_error(),))
        getattr(L, pre + "gb300_set_stream")(p, ctypes.c_void_p(s.cuda_stream))
        getattr(L, pre + "gb300_set_sync")(p, 0)
        ex, adj = getattr(L, pre + "execute"), getattr(L, pre + "execute_adjoint")

        def timed(fn):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                fn()
            e1.record(s)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        two = timed(lambda: (ex(p), ex(p)))
        fa = timed(lambda: (ex(p), adj(p)))
        getattr(L, pre + "destroy_plan")(p)
        res[name] = {"fwd_adj_ms": fa, "two_exec_ms": two, "ratio": fa / two}
        del x, y
        torch.cuda.empty_cache()
    return res



# ---- the other configurations of the metric ---------------------------------------------
DARITH = {"df": 0, "native": 1, "auto": 2, "dfq": 3}


def rel_l2_np(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)


def p_min(points, esz):
    """Minimal HBM passes: ceil(log2 N / log2 M), M = 2^13 complex128 or 2^14
    complex64 points staged by one CTA."""
    return int(np.ceil(np.log2(points) / (13 if esz == 16 else 14)))


def frac_key(peak):
    return "frac_of_measured_peak" if peak[1] == "measured" else "frac_of_fallback_peak"


def timed_stream(torch, stream, fn, reps, warm=2):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def measure_arith_512(L, pg, torch, x_host, oracle_out, peak):
    """The 512^3 complex128 forward in each double arithmetic and in complex64:
    CUDA-event time, algorithmic GB/s, fraction of the HBM peak and the
    forward relative L2 error against the FP64 oracle's output on the same
    input (the double input rounded to float for complex64)."""
    res = {}
    n = N3
    cnt = int(np.prod(n))
    stream = torch.cuda.Stream()
    comm = pg.procmesh(2)
    old = L.pfft_gb300_get_double_arith()
    labels = {"native": "f64 (native FP64 arithmetic on every pass, general kernel)",
              "dfq": "f64 storage, float-float arithmetic with block-quantised radix-8 butterflies (48-49 bits; "
                     "opt-in)",
              "df": "f64 storage, TwoSum float-float arithmetic (48-49 bits; opt-in)",
              "complex64": "f32 (the reference's single-precision API, pfftf_)"}
    for name in ("native", "dfq", "df", "complex64"):
        pre = "pfftf_" if name == "complex64" else "pfft_"
        if name != "complex64":
            L.pfft_gb300_set_double_arith(DARITH[name])
        dt = torch.float32 if name == "complex64" else torch.float64
        a = x_host.to(dt).cuda()
        b = torch.empty_like(a)
        flags = pg.PFFT_MEASURE if name == "native" else pg.PFFT_PATIENT
        p = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, pg.PFFT_FORWARD, flags)
        L.pfft_gb300_set_double_arith(old)
        if not p:
            res[name] = {"error": "plan failed: %s" % (pg.last_error(),)}
            continue
        getattr(L, pre + "gb300_set_stream")(p, ctypes.c_void_p(stream.cuda_stream))
        getattr(L, pre + "gb300_set_sync")(p, 0)
        reps = 3 if name == "native" else 10
        ms = timed_stream(torch, stream, lambda: getattr(L, pre + "execute")(p), reps)
        esz = 8 if name == "complex64" else 16
        B = p_min(cnt, esz) * 2 * cnt * esz
        r = {"dtype": labels[name], "ms": ms, "gbs": B / (ms * 1e-3) / 1e9, "bytes": B,
             frac_key(peak): B / (ms * 1e-3) / 1e9 / peak[0]}
        if oracle_out is not None:
            r["forward_rel_l2_vs_fp64_oracle"] = rel_l2_np(b.double().cpu().numpy(), oracle_out)
        res[name] = r
        getattr(L, pre + "destroy_plan")(p)
        del a, b
        torch.cuda.empty_cache()
    return res


def _alloc_words(L, pg, pre, kind, n, ni, no, flags, comm):
    d = len(n)
    a = [pg.ints([0] * d) for _ in range(4)]
    ls = {"c2c": "local_size_many_dft", "r2c": "local_size_many_dft_r2c", "c2r": "local_size_many_dft_c2r",
          "r2r": "local_size_many_r2r"}[kind]
    alloc = getattr(L, pre + ls)(d, pg.ints(n), pg.ints(ni), pg.ints(no), 1, None, None, comm, flags, *a)
    return alloc, [list(v) for v in a]


def _plan(L, pg, pre, kind, n, ni, no, x, y, comm, sign, flags, kinds=None):
    d = len(n)
    pl = {"c2c": "plan_many_dft", "r2c": "plan_many_dft_r2c", "c2r": "plan_many_dft_c2r",
          "r2r": "plan_many_r2r"}[kind]
    last = pg.cints(kinds) if kind == "r2r" else sign
    return getattr(L, pre + pl)(d, pg.ints(n), pg.ints(ni), pg.ints(no), 1, None, None, x.data_ptr(), y.data_ptr(),
                                comm, last, flags)


def measure_config(L, pg, torch, kind, n, prec, flags_f, flags_b, B, peak, ni=None, kinds=None, kinds_inv=None,
                   norm=None, inplace=False, dist="uniform", reps=10):
    """One configuration: the forward execute timed with CUDA events
    (algorithmic bytes B per execute), then the inverse plan's round trip
    error against the input (a size-independent check)."""
    pre = "pfft_" if prec == "double" else "pfftf_"
    rdt = torch.float64 if prec == "double" else torch.float32
    comm = pg.procmesh(2)
    ni = list(ni or n)
    inv = {"c2c": "c2c", "r2c": "c2r", "r2r": "r2r"}[kind]
    allocf, (lni, _, lno, _) = _alloc_words(L, pg, pre, kind, n, ni, n, flags_f, comm)
    allocb, _ = _alloc_words(L, pg, pre, inv, n, n, ni, flags_b, comm)
    words = 2 * max(allocf, allocb)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.zeros(words, dtype=rdt, device="cuda")
    cin = int(np.prod(lni)) * (2 if kind == "c2c" else 1)
    if dist == "normal":
        x[:cin].normal_(generator=g)
    else:
        x[:cin].uniform_(-1, 1, generator=g)
    if kind == "r2c" and (flags_f & pg.PFFT_PADDED_R2C):
        x[:cin].view(-1, lni[-1])[:, ni[-1]:] = 0
    x0 = x.clone()
    y = x if inplace else torch.zeros(words, dtype=rdt, device="cuda")
    z = torch.zeros(words, dtype=rdt, device="cuda")
    pf = _plan(L, pg, pre, kind, n, ni, n, x, y, comm, -1, flags_f | pg.PFFT_PATIENT, kinds)
    if not pf:
        return {"error": "plan failed: %s" % (pg.last_error(),)}
    stream = torch.cuda.Stream()
    getattr(L, pre + "gb300_set_stream")(pf, ctypes.c_void_p(stream.cuda_stream))
    getattr(L, pre + "gb300_set_sync")(pf, 0)
    if inplace:
        # the input is restored before every step; events bracket the execute alone
        times = []
        for i in range(reps + 2):
            with torch.cuda.stream(stream):
                x.copy_(x0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            getattr(L, pre + "execute")(pf)
            e1.record(stream)
            torch.cuda.synchronize()
            if i >= 2:
                times.append(e0.elapsed_time(e1))
        ms = float(np.median(times))
        with torch.cuda.stream(stream):
            x.copy_(x0)
    else:
        ms = timed_stream(torch, stream, lambda: getattr(L, pre + "execute")(pf), reps)
    getattr(L, pre + "execute")(pf)
    torch.cuda.synchronize()
    dst = y if inplace else z
    pb = _plan(L, pg, pre, inv, n, n, ni, y, dst, comm, 1, flags_b | pg.PFFT_MEASURE, kinds_inv)
    rt = None
    if pb:
        getattr(L, pre + "execute")(pb)
        torch.cuda.synchronize()
        scale = norm if norm is not None else float(np.prod(n))
        out = dst[:cin].double() / scale
        ref = x0[:cin].double()
        if kind == "r2c" and (flags_f & pg.PFFT_PADDED_R2C):
            out = out.view(-1, lni[-1])[:, :ni[-1]]
            ref = ref.view(-1, lni[-1])[:, :ni[-1]]
        rt = float(torch.linalg.vector_norm(out - ref) / torch.linalg.vector_norm(ref))
        getattr(L, pre + "destroy_plan")(pb)
    getattr(L, pre + "destroy_plan")(pf)
    gbs = B / (ms * 1e-3) / 1e9
    r = {"ms": ms, "gbs": gbs, "bytes": B, frac_key(peak): gbs / peak[0], "roundtrip_rel_l2": rt,
         "bound": 1e-12 if prec == "double" else 2e-6}
    del x, y, z, x0
    torch.cuda.empty_cache()
    return r


def measure_halo(L, pg, torch, peak, n=(256, 256, 256), w=2, reps=10):
    """pfft_exchange of a 256^3 real float64 block with a halo of width 2 on
    every face (periodic wrap, in place): CUDA-event time against the
    algorithmic bytes, the block read once (134.2 MB) and the box written once
    (140.6 MB); and the reduce, its adjoint, on the same bytes."""
    comm = pg.procmesh(2)
    box = [m + 2 * w for m in n]
    buf = torch.zeros(int(np.prod(box)), dtype=torch.float64, device="cuda")
    buf[: int(np.prod(n))].uniform_(-1, 1)
    p = L.pfft_plan_rgc_3d(pg.ints(n), pg.ints([w] * 3), pg.ints([w] * 3), buf.data_ptr(), comm, 0)
    if not p:
        return {"error": "ghost plan failed"}
    stream = torch.cuda.Stream()
    L.pfft_gb300_gc_set_stream(p, ctypes.c_void_p(stream.cuda_stream))
    B = int(np.prod(n)) * 8 + int(np.prod(box)) * 8
    res = {"workload": "256^3 float64 real block, halo 2 on every face, periodic wrap, in place"}
    for op in ("exchange", "reduce"):
        fn = getattr(L, "pfft_" + op)
        ms = timed_stream(torch, stream, lambda: fn(p), reps)
        gbs = B / (ms * 1e-3) / 1e9
        res[op] = {"ms": ms, "gbs": gbs, "bytes": B, frac_key(peak): gbs / peak[0]}
    L.pfft_destroy_gcplan(p)
    del buf
    torch.cuda.empty_cache()
    return res


def config_table(pg):
    """name -> (measure_config arguments after L, pg, torch; keyword arguments)
    for every configuration of the metric besides the 512^3 headline (each a
    forward execute with the default arithmetic; algorithmic bytes
    B = in + out + 2 (P_min - 1) work)."""
    TO, TI, PAD = pg.PFFT_TRANSPOSED_OUT, pg.PFFT_TRANSPOSED_IN, pg.PFFT_PADDED_R2C
    t = {"c2c_64cube_c128": (("c2c", (64, 64, 64), "double", 0, 0, 2 * 2 * 64 ** 3 * 16), {})}
    n256 = (256, 256, 256)
    for prec, esz in (("double", 8), ("float", 4)):
        tag = "f64" if prec == "double" else "f32"
        rin = 256 * 256 * 258 * esz
        cout = 256 * 256 * 129 * 2 * esz
        t["r2c_256cube_%s_padded_transposed_inplace" % tag] = (
            ("r2c", n256, prec, PAD | TO, PAD | TI, rin + cout + 2 * cout), {"inplace": True, "dist": "normal"})
        rb = 256 ** 3 * esz
        t["redft10_256cube_%s" % tag] = (
            ("r2r", n256, prec, 0, 0, 4 * rb),
            {"kinds": [pg.PFFT_REDFT10] * 3, "kinds_inv": [pg.PFFT_REDFT01] * 3, "norm": float((2 * 256) ** 3),
             "dist": "normal"})
    t["ousam_r2c_f32_128to256"] = (("r2c", n256, "float", 0, 0, 211 * 10 ** 6),
                                   {"ni": (128, 128, 128), "dist": "normal"})
    t["c2c_1024cube_c64"] = (("c2c", (1024, 1024, 1024), "float", 0, 0, 3 * 2 * 1024 ** 3 * 8), {"reps": 5})
    t["c2c_64pow4_c128"] = (("c2c", (64, 64, 64, 64), "double", 0, 0, 2 * 2 * 64 ** 4 * 16), {})
    return t


def measure_configs(L, pg, torch, peak):
    """Every configuration of config_table, then the 256^3 halo."""
    c = {}
    for name, (args, kw) in config_table(pg).items():
        c[name] = measure_config(L, pg, torch, *args, peak, **kw)
    c["halo_256cube_w2_f64"] = measure_halo(L, pg, torch, peak)
    return c


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl != "reference" else "gloo")
    return world, rank, local


def reduce_max(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference arm: the reference (PFFT + FFTW-MPI + MPI) cannot be
    built here, so this times its CPU restatement (the oracle, FP64) on the
    same workload as the GPU arm - one full 512^3 complex128 forward execute
    per step, all host threads - with the real per-step wall time."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = (args.ref_n,) * 3
    x = cpu_input(n)
    per = []
    t_all = time.perf_counter()
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _oracle_forward(n, x, threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            per.append(dt)
    wall = time.perf_counter() - t_all
    ms = 1e3 * sum(per) / len(per)
    v = algo_bytes(n) / (ms * 1e-3) / 1e9
    line = {"metric": "3D FFT HBM GB/s & %roofline, 5N*log2N GFLOP/s; batched vs loop; adjoint cost",
            "value": v, "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic uniform[-1,1) seed 1",
            "config": {"workload": "pfft_execute c2c %d^3 complex128 forward, 1x1 procmesh, out-of-place, "
                                   "TRANSPOSED_NONE" % args.ref_n,
                       "bytes_per_step": algo_bytes(n), "p_min": P_MIN, "parallelism": "host cores"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": "the full workload every step: %d timed + %d warm-up forward executes "
                                       "of %d^3 complex128, mean %.2f s per step, %.1f s in all" %
                                       (args.steps, args.warmup, args.ref_n, ms / 1e3, wall)},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (PFFT + FFTW-MPI + MPI) cannot be built here; this arm times the CPU "
                    "oracle, a C FP64 restatement of its transform path"}
    if not args.no_scipy:
        line["scipy_baseline"] = scipy_baseline(n, threads, x)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched-vs-loop and adjoint-cost parts")
    ap.add_argument("--no-scipy", action="store_true", help="skip the scipy.fft.fftn CPU number")
    ap.add_argument("--ref-n", type=int, default=512,
                    help="cube edge of the reference arm's workload (512, the benchmark's; smaller only in tests)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--n", type=int, default=512, help="cube edge (profiling runs use a smaller case)")
    ap.add_argument("--shape", default=None, help="n0xn1xn2 instead of a cube (profiling runs)")
    ap.add_argument("--export-wisdom", default=None, help="write the planner's wisdom to this file after planning")
    ap.add_argument("--import-wisdom", default=None,
                    help="load wisdom from this file and plan with PFFT_MEASURE (the recorded choices, no timing)")
    ap.add_argument("--no-tune", action="store_true",
                    help="plan with PFFT_MEASURE instead of PFFT_PATIENT (by default the autotuner times every "
                         "pass's candidates at planning time, before the timed region)")
    ap.add_argument("--batched-only", default=None, choices=["double", "float"],
                    help="print only the batched-vs-loop measurement of that precision (profiling runs)")
    ap.add_argument("--halo-only", action="store_true",
                    help="print only the 256^3 halo exchange / reduce measurement (profiling runs)")
    ap.add_argument("--config-only", default=None,
                    help="print only the measurement of one named configuration (profiling runs)")
    ap.add_argument("--prec", default="double", choices=["double", "float"],
                    help="double = pfft_ (complex128, the headline); float = pfftf_ (complex64)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    import pfft_gb300 as pg
    torch.cuda.set_device(local)
    L = pg.lib()
    if args.batched_only:
        print(json.dumps(measure_batched(L, pg, torch, args.batched_only, tune=not args.no_tune)), flush=True)
        return
    if args.halo_only:
        print(json.dumps(measure_halo(L, pg, torch, measured_peak())), flush=True)
        return
    if args.config_only:
        cargs, kw = config_table(pg)[args.config_only]
        print(json.dumps(measure_config(L, pg, torch, *cargs, measured_peak(), **kw)), flush=True)
        return
    dev = torch.device("cuda", local)
    n = tuple(int(v) for v in args.shape.split("x")) if args.shape else (args.n, args.n, args.n)
    cnt = int(np.prod(n))
    rng = np.random.default_rng(1 + rank)
    host = torch.from_numpy(rng.uniform(-1.0, 1.0, 2 * cnt))
    pre = "pfft_" if args.prec == "double" else "pfftf_"
    esz = 16 if args.prec == "double" else 8
    if args.prec == "float":
        host = host.float()
    a = host.to(dev)
    b = torch.empty_like(a)
    comm = pg.procmesh(2)
    if args.import_wisdom:
        if L.pfft_gb300_import_wisdom_from_filename(args.import_wisdom.encode()) != 1:
            raise RuntimeError("cannot import wisdom from %s" % args.import_wisdom)
        args.no_tune = True
    plan_flags = pg.PFFT_TRANSPOSED_NONE | (pg.PFFT_MEASURE if args.no_tune else pg.PFFT_PATIENT)
    plan = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, pg.PFFT_FORWARD, plan_flags)
    if not plan:
        raise RuntimeError("plan failed: %s" % (pg.last_error(),))
    if args.export_wisdom:
        L.pfft_gb300_export_wisdom_to_filename(args.export_wisdom.encode())
    stream = torch.cuda.Stream(device=dev)
    getattr(L, pre + "gb300_set_stream")(plan, ctypes.c_void_p(stream.cuda_stream))
    getattr(L, pre + "gb300_set_sync")(plan, 0)
    npass = ctypes.c_int(0)
    getattr(L, pre + "gb300_plan_info")(plan, ctypes.byref(npass), None, None)
    plan_arith = getattr(L, pre + "gb300_plan_arith")(plan)
    dmode = L.pfft_gb300_get_double_arith()
    pass_bytes = []
    pass_kernel = [getattr(L, pre + "gb300_pass_kernel")(plan, i) for i in range(npass.value)]
    for i in range(npass.value):
        bb = ctypes.c_double(0)
        getattr(L, pre + "gb300_pass_info")(plan, i, None, None, None, None, None, ctypes.byref(bb))
        pass_bytes.append(bb.value)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            getattr(L, pre + "execute")(plan)
    torch.cuda.synchronize()

    # ---- timed region: device-resident arrays ----
    getattr(L, pre + "gb300_set_pass_timing")(plan, 1)
    getattr(L, pre + "gb300_set_sync")(plan, 1)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.5)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        getattr(L, pre + "execute")(plan)
    e1.record(stream)
    torch.cuda.synchronize()
    tw1 = time.time()
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop(tw0, tw1)
    pass_ms = []
    for i in range(npass.value):
        t = ctypes.c_double(0)
        runs = ctypes.c_int(0)
        getattr(L, pre + "gb300_pass_time")(plan, i, ctypes.byref(t), ctypes.byref(runs))
        pass_ms.append(t.value / max(1, runs.value))
    getattr(L, pre + "gb300_set_pass_timing")(plan, 0)
    ms_max = reduce_max(ms, world)

    # ---- e2e: pinned host arrays through the same C-ABI call ----
    e2e_max = None
    if args.e2e_steps > 0:
        hin = host.pin_memory()
        hout = torch.empty_like(hin).pin_memory()
        getattr(L, pre + "execute_dft")(plan, hin.data_ptr(), hout.data_ptr())  # staging buffers allocated here, untimed
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            getattr(L, pre + "execute_dft")(plan, hin.data_ptr(), hout.data_ptr())
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        e2e_max = reduce_max(e2e_s, world)
    # ---- accuracy of the measured transform (size-independent properties) ----
    # b holds forward(a): backward with a second plan, round-trip error
    # |backward(forward(a))/N - a| / |a| and Parseval |forward(a)|^2 / N vs |a|^2
    c = torch.empty_like(a)
    pb = getattr(L, pre + "plan_dft_3d")(pg.ints(n), b.data_ptr(), c.data_ptr(), comm, pg.PFFT_BACKWARD,
                                         pg.PFFT_TRANSPOSED_NONE | pg.PFFT_MEASURE)
    accuracy = None
    if pb:
        getattr(L, pre + "execute")(pb)
        torch.cuda.synchronize()
        na = float(torch.linalg.vector_norm(a.double()))
        nb = float(torch.linalg.vector_norm(b.double()))
        accuracy = {"roundtrip_rel_l2": float(torch.linalg.vector_norm(c.double() / cnt - a.double())) / na,
                    "parseval_rel": abs(nb * nb / cnt - na * na) / (na * na),
                    "bound": 1e-12 if args.prec == "double" else 2e-6}
        getattr(L, pre + "destroy_plan")(pb)
    del c
    # the forward output, for the comparison with the FP64 oracle on the same input
    full = (n == N3 and rank == 0 and not args.no_cpu_baseline)
    fwd_host = b.double().cpu().numpy() if full else None
    getattr(L, pre + "destroy_plan")(plan)
    del a, b
    torch.cuda.empty_cache()

    # ---- CPU baselines on the same workload (rank 0), and the FP64 oracle's output ----
    cpu = {}
    oracle_keep = {}
    if full:
        xb = host.double().numpy()
        cpu["cpu_baseline"] = cpu_baseline(N3, x=xb, keep=oracle_keep)
        if not args.no_scipy:
            cpu["scipy_baseline"] = scipy_baseline(N3, x=xb)
        if accuracy is not None:
            accuracy["forward_rel_l2_vs_fp64_oracle"] = rel_l2_np(fwd_host, oracle_keep["out"])
        del fwd_host

    # ---- the metric's other parts: batched vs loop, adjoint cost, every arithmetic at 512^3,
    # ---- the other configurations (outside the step's timed region) ----
    extra = {}
    peak = measured_peak()
    if not args.no_extras:
        extra["batched_vs_loop"] = {pr: measure_batched(L, pg, torch, pr, tune=not args.no_tune)
                                    for pr in ("double", "float")}
        extra["adjoint_cost"] = measure_adjoint(L, pg, torch)
        if n == N3 and args.prec == "double":
            extra["arith_512"] = measure_arith_512(L, pg, torch, host, oracle_keep.get("out"), peak)
        extra["configs"] = measure_configs(L, pg, torch, peak)
    oracle_keep.clear()

    pts = int(np.prod(n))
    pmin = int(np.ceil(np.log2(pts) / (13 if esz == 16 else 14)))  # minimal HBM passes
    B = pmin * 2 * pts * esz
    peak, peak_kind = peak
    value = world * B / (ms_max * 1e-3) / 1e9
    # dominant kernel: the pass with the largest share of the step
    k = int(np.argmax(pass_ms)) if pass_ms else 0
    ach = pass_bytes[k] / (pass_ms[k] * 1e-3) / 1e9 if pass_ms and pass_ms[k] > 0 else None
    traffic = committed_traffic()
    if rank != 0:
        return
    gflops = 5.0 * cnt * np.log2(cnt) / (ms * 1e-3) / 1e9
    line = {
        "metric": "3D FFT HBM GB/s & %roofline, 5N*log2N GFLOP/s; batched vs loop; adjoint cost",
        "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {0: "f32",
                  1: ("f64 storage, int64 block-fixed-point arithmetic on the radix-8 and mixed-radix passes (58-60 "
                      "bits against the tile maximum; measured no less accurate than native FP64), FP64 elsewhere")
                  if dmode == 2 else "f64 (native FP64 arithmetic)",
                  2: "f64 storage, float-float arithmetic" +
                  (" (block-quantised radix-8 stages)" if dmode == 3 else " (TwoSum)")}[plan_arith],
        "accuracy": accuracy,
        "data": "synthetic uniform[-1,1) seed 1+rank",
        "config": {"workload": "pfft_execute c2c %s %s forward, 1x1 procmesh, out-of-place, "
                               "TRANSPOSED_NONE" % ("x".join(map(str, n)) if args.shape else "%d^3" % args.n,
                                                    "complex128" if args.prec == "double" else "complex64"),
                   "bytes_per_step": B, "p_min": pmin, "planner": ("PFFT_MEASURE with imported wisdom" if args.import_wisdom else "PFFT_MEASURE") if args.no_tune
                   else "PFFT_PATIENT (autotuned at planning time)",
                   "l2": "arrays (%.2f GB each) larger than the 129 MB L2; no flush" % (cnt * esz / 1e9),
                   "parallelism": "replicas" if world > 1
                   else "single GPU"},
        "pct_roofline": value / world / peak,
        "gflops": gflops,
        "pass_ms": pass_ms,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": (ach / peak) if ach else None, "traffic": traffic,
                     "kernel": "%s (pass %d of %d)" % ("k_fast" if pass_kernel[k] == 1 else "k_pass", k, len(pass_ms)),
                     "peak_source": peak_kind},
        "e2e": None if e2e_max is None else {
            "value": world * B / e2e_max / 1e9, "unit": "GB/s", "h2d_bytes_per_step": cnt * esz,
            "d2h_bytes_per_step": cnt * esz, "ms_per_step": e2e_max * 1e3},
        "gpu_launches": npass.value * args.steps,
        "clocks": clk,
    }
    line.update(extra)
    line.update(cpu)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

"""Benchmark of the PFFT transform-execution path on GB300.

Workload (one step): one forward pfft_execute of a 512^3 complex128 c2c
transform on a 1x1 process mesh, out of place, standard layout - the
configuration the headline target is quoted on.  Inputs are uniform[-1,1)
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
          be built: it needs FFTW-MPI and MPI) on the host cores, on a bounded
          sample of the same workload

--impl reference times that CPU port instead (the reference arm).
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
    """Sample SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return

        def rd():
            for line in self.proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx = float(s[1])
                for i, nm in enumerate(names):
                    if s[3 + i].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(sample_n0=128, threads=None):
    """Time the CPU oracle on a bounded sample (n0 x 512 x 512) of the workload."""
    import oracle
    threads = threads or (os.cpu_count() or 1)
    n = (sample_n0, N3[1], N3[2])
    rng = np.random.default_rng(1)
    x = rng.uniform(-1.0, 1.0, 2 * int(np.prod(n)))
    t0 = time.perf_counter()
    oracle.execute("c2c", n, n, n, 1, -1, 0, 2, x, 2 * int(np.prod(n)), nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": algo_bytes(n) / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "%dx512x512 c2c complex128 forward (1/%d of the workload), one run, %.2f s" %
                      (sample_n0, N3[0] // sample_n0, dt)}


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
    if rank != 0:
        return
    steps = []
    threads = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(sample_n0=args.ref_sample_n0, threads=threads)
        if i >= args.warmup:
            steps.append(r)
    v = statistics.median([s["value"] for s in steps])
    ms = algo_bytes() / (v * 1e9) * 1e3
    line = {"metric": "3D FFT HBM GB/s & %roofline, 5N*log2N GFLOP/s; batched vs loop; adjoint cost",
            "value": v, "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic uniform[-1,1) seed 1",
            "config": {"workload": "pfft_execute c2c 512^3 complex128 forward, 1x1 procmesh, out-of-place "
                                   "(CPU port timed on a %dx512x512 sample per step)" % args.ref_sample_n0},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": steps[0]["sample"]},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference (PFFT + FFTW-MPI + MPI) cannot be built here; this arm times the CPU "
                    "oracle, a C FP64 restatement of its transform path"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-sample-n0", type=int, default=128)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--n", type=int, default=512, help="cube edge (profiling runs use a smaller case)")
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
    dev = torch.device("cuda", local)
    n = (args.n, args.n, args.n)
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
    plan = getattr(L, pre + "plan_dft_3d")(pg.ints(n), a.data_ptr(), b.data_ptr(), comm, pg.PFFT_FORWARD,
                                           pg.PFFT_TRANSPOSED_NONE | pg.PFFT_MEASURE)
    if not plan:
        raise RuntimeError("plan failed: %s" % (pg.last_error(),))
    stream = torch.cuda.Stream(device=dev)
    getattr(L, pre + "gb300_set_stream")(plan, ctypes.c_void_p(stream.cuda_stream))
    getattr(L, pre + "gb300_set_sync")(plan, 0)
    npass = ctypes.c_int(0)
    getattr(L, pre + "gb300_plan_info")(plan, ctypes.byref(npass), None, None)
    pass_bytes = []
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
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        getattr(L, pre + "execute")(plan)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
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
    getattr(L, pre + "destroy_plan")(plan)

    pts = int(np.prod(n))
    pmin = int(np.ceil(np.log2(pts) / (13 if esz == 16 else 14)))  # minimal HBM passes
    B = pmin * 2 * pts * esz
    peak, peak_kind = measured_peak()
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
        "dtype": ("f32" if args.prec == "float" else
                  "f64 storage, float-float arithmetic" if L.pfft_gb300_get_double_arith() == 0 else "f64"),
        "data": "synthetic uniform[-1,1) seed 1+rank",
        "config": {"workload": "pfft_execute c2c %d^3 %s forward, 1x1 procmesh, out-of-place, "
                               "TRANSPOSED_NONE" % (args.n, "complex128" if args.prec == "double" else "complex64"),
                   "bytes_per_step": B, "p_min": pmin,
                   "l2": "arrays (2.1 GB) larger than L2; no flush", "parallelism": "replicas" if world > 1
                   else "single GPU"},
        "pct_roofline": value / world / peak,
        "gflops": gflops,
        "pass_ms": pass_ms,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": (ach / peak) if ach else None, "traffic": traffic,
                     "kernel": "k_pass (pass %d of %d)" % (k, len(pass_ms)), "peak_source": peak_kind},
        "e2e": None if e2e_max is None else {
            "value": world * B / e2e_max / 1e9, "unit": "GB/s", "h2d_bytes_per_step": cnt * esz,
            "d2h_bytes_per_step": cnt * esz, "ms_per_step": e2e_max * 1e3},
        "gpu_launches": npass.value * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sample_n0=args.ref_sample_n0)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

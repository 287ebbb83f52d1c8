"""Benchmark of the in-place transpose path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl eithot|reference]

Workload: the plain 4D in-place transpose of a (4, 20011, 8192, 2) int32
tensor (5.25 GB) of seeded counter-hash 32-bit values, permutation
(1 3 2 4), sub-tensor count and alpha from the estimator.  A step is one
in-place transpose of the whole tensor; the permutation moves the same bytes
whatever they hold, so each step re-transposes the buffer as a fresh
(4, 20011, 8192, 2) tensor.  The tensor (5.25 GB) is larger than L2
(129 MB), so no flush is needed between steps.

value: effective GB/s = 2 * bytes / device time per step (inputs resident).
e2e:   the same metric through the C ABI with the tensor in pinned host
       memory: every step copies it to the device, transposes, and copies
       the result back; consecutive steps are pipelined over three device
       buffers (copies of one step overlap the transpose of another).
Beside them: the 3001 x 4096 int32 matrix (perm (2 1)) timed the same way
(device-resident and end to end), the (16, 3001, 1024, 256, 4) uint16 tensor
(100.7 GB, perm (5 3 1 4 2)) device-resident under the fewest-pass plan and
the reference's series, summaries of the batched form (4096 mixed tensors)
and the served form (200 Poisson-arriving requests), the reference's own CUDA build
(test_inplace recompiled for sm_103a from baseline/_ref, when built) on both
configurations, and the reference's own single-threaded host permutation
next to the oracle's OpenMP restatement of it.
With N > 1 (torchrun) every rank runs its own replica (the path does not
shard); value sums the ranks' bytes over the max-over-ranks time.
--impl reference times the reference's CPU path on the host cores on a
bounded slice of the workload: its own TensorUtil::seq_tt compiled from the
reference's sources (single-threaded, as the reference runs it) when that
build exists, else the oracle's restatement of it.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = [4, 20011, 8192, 2]
PERM = [1, 3, 2, 4]
ELEM = 4
SEED = 0xE17407
METRIC = "bit-exact in-place GB/s (2·bytes/s) vs HBM peak; served p99 vs serial"
WORKLOAD = "in-place 4D transpose (4,20011,8192,2) int32 perm (1 3 2 4), nb/alpha from the estimator"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="eithot", choices=["eithot", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 3001 x 4096 matrix and the reference's own GPU build")
    ap.add_argument("--dims", default=None,
                    help="comma-separated dims overriding the workload (small cases for ncu captures)")
    ap.add_argument("--workload", default="transpose", choices=["transpose", "batched", "served", "study", "case"],
                    help="transpose: the default line; batched: 4096 mixed tensors through the batched form "
                         "against one call per tensor; served: Poisson-arriving requests through the server "
                         "against serial calls; study: REORDER_TYPE pre/post/mixed and sub-tensor count sweeps; "
                         "case: one shape (--dims, --perm, --elem, --order, --knob) timed per pass")
    ap.add_argument("--count", type=int, default=0, help="tensors (batched) or requests (served); 0: default")
    ap.add_argument("--perm", default=None, help="case: comma-separated 1-based permutation")
    ap.add_argument("--elem", type=int, default=4, help="case: element size in bytes")
    ap.add_argument("--order", type=int, default=0, help="case: reorder type (0 mixed, 1 pre, 2 post, 3 fewest passes)")
    ap.add_argument("--alpha", type=float, default=0.05, help="case: extra-memory ratio")
    ap.add_argument("--knob", action="append", default=[], help="case: tuning knob key=value (repeatable)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    """DRAM bytes per launch of each pass kind at this workload, as measured
    by ncu (dram__bytes_read.sum + dram__bytes_write.sum): lines
    `<pass kind> <bytes>` in profiles/traffic.txt, '#' starts a comment."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    out = {}
    if os.path.exists(path):
        with open(path) as f:
            for line in f:
                line = line.split("#", 1)[0].split()
                if len(line) == 2:
                    out[line[0]] = float(line[1])
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                t = [x.strip() for x in line.split(",")]
                if len(t) < 9:
                    continue
                try:
                    sm.append(float(t[1]))
                    mx.append(float(t[2]))
                except ValueError:
                    continue
                for name, v in zip(names, t[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(threads=0, budget_s=10.0):
    """The reference's host permutation (oracle restatement of seq_tt) on a
    slice of the workload: dims (4, 20011, 512, 2), 328 MB."""
    import numpy as np
    import oracle

    dims = [4, 20011, 512, 2]
    n = math.prod(dims)
    src = oracle.fill_hash(n, ELEM, SEED)
    oracle.permute(src, dims, PERM, ELEM, threads=threads)  # warm
    times = []
    t_end = time.perf_counter() + budget_s
    while time.perf_counter() < t_end or len(times) < 2:
        t0 = time.perf_counter()
        oracle.permute(src, dims, PERM, ELEM, threads=threads)
        times.append(time.perf_counter() - t0)
        if len(times) >= 50:
            break
    t = statistics.median(times)
    cores = oracle.max_threads() if threads <= 0 else threads
    return {"value": 2.0 * n * ELEM / t / 1e9, "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": "oracle restatement of TensorUtil::seq_tt, out-of-place, on dims (4,20011,512,2) int32 "
                      "(1/16 of the workload, 328 MB), median of %d runs" % len(times)}


def ref_bin(name):
    """A binary of the reference's own build (baseline/_ref, built by
    `make -C oracle ref-gpu` for this machine), or None."""
    path = os.path.join(ROOT, "baseline", "_ref", "ITNT", "bin-" + platform.machine(), name)
    return path if os.path.exists(path) else None


SLICE = [4, 20011, 512, 2]  # 1/16 of the workload, for the host permutation


def ref_seqtt_baseline(runs=1):
    """The reference's own host permutation TensorUtil::seq_tt (compiled from
    its sources, single-threaded as the reference runs it) on the workload's
    1/16 slice, iota data."""
    exe = ref_bin("ref_seqtt_timer")
    if not exe:
        return None
    r = subprocess.run([exe, str(ELEM), str(runs), "1"] + [str(d) for d in SLICE] + [str(p) for p in PERM],
                       capture_output=True, text=True, timeout=600)
    if r.returncode != 0 or not r.stdout.split():
        return None
    secs = float(r.stdout.split()[0])
    n = math.prod(SLICE)
    return {"value": 2.0 * n * ELEM / secs / 1e9, "unit": "GB/s", "cores": 1, "kind": "reference",
            "ms_per_run": secs * 1e3,
            "sample": "the reference's TensorUtil::seq_tt compiled from its sources, single-threaded, out-of-place "
                      "on dims (4,20011,512,2) int32 (1/16 of the workload, 328 MB), median of %d runs" % runs}


REF_CASES = {"4,20011,8192,2 perm 1 3 2 4": ([4, 20011, 8192, 2], [1, 3, 2, 4]),
             "3001,4096 perm 2 1": ([3001, 4096], [2, 1])}


def reference_gpu(timeout=900):
    """The reference's own CUDA build (its test_inplace, recompiled for
    sm_103a from its sources) on the bench workload and on the 3001 x 4096
    int32 matrix: one run each, as the reference's driver runs (iota data,
    H2D, inplace::transpose, D2H, verify_inplace on the host).  Reports its
    own two timings: "Execution Time without h2d2h" (device part) and
    "Execution Time" (with both copies), as effective GB/s."""
    exe = ref_bin("test_inplace")
    if not exe:
        return {"unavailable": "the reference's GPU build is absent (baseline/_ref is made where the "
                               "reference tree is mounted)"}
    out = {}
    for name, (dims, perm) in REF_CASES.items():
        nb, alpha = 1, 0.01
        args = [str(d) for d in dims] + [str(p) for p in perm] + [str(ELEM), str(nb), str(alpha)]
        with tempfile.TemporaryDirectory() as tmp:
            try:
                r = subprocess.run([exe] + args, cwd=tmp, capture_output=True, text=True, timeout=timeout)
            except subprocess.TimeoutExpired:
                out[name] = {"unavailable": "timed out after %d s" % timeout}
                continue
        text = r.stdout
        dev_ms = re.search(r"Execution Time without h2d2h: ([0-9.]+)ms", text)
        all_ms = re.search(r"Execution Time: ([0-9.]+)ms", text)
        if r.returncode != 0 or not dev_ms or not all_ms:
            out[name] = {"unavailable": "exit %d: %s" % (r.returncode, (r.stdout + r.stderr).strip()[-300:])}
            continue
        nbytes = math.prod(dims) * ELEM
        d, a = float(dev_ms.group(1)), float(all_ms.group(1))
        out[name] = {"correct": "Correct transpose" in text, "nb": nb, "alpha": alpha,
                     "device_ms": d, "device_gbs": 2.0 * nbytes / (d / 1e3) / 1e9,
                     "e2e_ms": a, "e2e_gbs": 2.0 * nbytes / (a / 1e3) / 1e9,
                     "command": "test_inplace " + " ".join(args)}
    return out


C3 = ([16, 3001, 1024, 256, 4], [5, 3, 1, 4, 2], 2, 0.05)


def time_c3(E, dev, steps=3):
    """The (16, 3001, 1024, 256, 4) uint16 tensor (100.7 GB, larger than L2),
    perm (5 3 1 4 2), nb 1, alpha 0.05, device-resident: the fewest-pass plan
    (EITHOT_ORDER_FEWEST) and the reference's series (EITHOT_ORDER_MIXED, the
    default).  Each plan's first transpose is checked on the device element
    by element; then `steps` transposes are timed with CUDA events (each
    re-transposes the buffer as a fresh tensor of the same shape)."""
    import torch
    dims, perm, elem, alpha = C3
    n = math.prod(dims)
    nbytes = n * elem
    free, _ = torch.cuda.mem_get_info(dev)
    if free < nbytes * 1.08:
        return {"unavailable": "needs %.1f GB of free device memory, %.1f GB free" % (nbytes * 1.08 / 1e9, free / 1e9)}
    buf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    peak, _ = load_peaks()
    out = {"dims": dims, "perm": perm, "elem_bytes": elem, "alpha": alpha, "bytes": nbytes}
    for name, order in (("fewest_passes", E.ORDER_FEWEST), ("reference_series", E.ORDER_MIXED)):
        E.fill_hash_ptr(buf.data_ptr(), n, elem, SEED, 0, stream.cuda_stream)
        E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, elem, 1, alpha, order, stream.cuda_stream)
        bad, _ = E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, SEED, stream.cuda_stream)
        status = E.call_status(E.last_call(), stream.cuda_stream)
        E.profile_reset()
        E.set_profiling(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, elem, 1, alpha, order, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        E.set_profiling(False)
        st = E.last_stats()
        ms = e0.elapsed_time(e1) / steps
        per = {}
        for p in E.profile():
            d = per.setdefault(p["name"], [0.0, 0, p["bytes"]])
            d[0] += p["ms"]
            d[1] += 1
        E.profile_reset()
        out[name] = {"bit_exact": bad == 0 and status == E.OK, "ms": ms, "gbs": 2.0 * nbytes / (ms / 1e3) / 1e9,
                     "frac": 2.0 * nbytes / (ms / 1e3) / 1e9 / peak, "passes": st["n_passes"],
                     "workspace_bytes": st["workspace_bytes"],
                     "per_pass": {k: {"ms": v[0] / v[1], "gbs": v[2] / (v[0] / v[1] / 1e3) / 1e9} for k, v in per.items()}}
    del buf
    torch.cuda.empty_cache()
    return out


def time_c1(E, dev, steps=50):
    """The 3001 x 4096 int32 matrix, perm (2 1), nb 1, alpha 0.01: device
    time per transpose (resident, CUDA events) and end to end through the C
    ABI (H2D from pinned memory, transpose, D2H, serialised like the
    reference's driver)."""
    import torch
    dims, perm = [3001, 4096], [2, 1]
    n = math.prod(dims)
    nbytes = n * ELEM
    buf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    E.fill_hash_ptr(buf.data_ptr(), n, ELEM, SEED)
    stream = torch.cuda.current_stream(dev)
    for _ in range(5):
        E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, ELEM, 1, 0.01, E.ORDER_MIXED, stream.cuda_stream)
    # L2 (129 MB) would hold the 49 MB matrix: flush it between steps with a
    # 256 MB write and time only the transposes
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ms = []
    for _ in range(steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, ELEM, 1, 0.01, E.ORDER_MIXED, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host.copy_(buf)
    e2e = []
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        buf.copy_(host, non_blocking=True)
        E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, ELEM, 1, 0.01, E.ORDER_MIXED, stream.cuda_stream)
        host.copy_(buf, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        e2e.append(e0.elapsed_time(e1))
    d, a = statistics.median(ms), statistics.median(e2e)
    return {"dims": dims, "perm": perm, "elem_bytes": ELEM, "device_ms": d, "device_gbs": 2.0 * nbytes / (d / 1e3) / 1e9,
            "e2e_ms": a, "e2e_gbs": 2.0 * nbytes / (a / 1e3) / 1e9,
            "timing": "median of %d flushed device steps and %d serialised H2D+transpose+D2H steps" % (steps, 10)}


def max_over_ranks(x: float, device) -> float:
    """The largest of every rank's x (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gbs(bytes_per_rank: int, ms_per_step: float, world: int) -> float:
    """Whole-job effective GB/s: every rank moves 2 * bytes per step; the
    step time is the slowest rank's."""
    return world * 2.0 * bytes_per_rank / (ms_per_step / 1e3) / 1e9


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    exe = ref_bin("ref_seqtt_timer")
    if exe:
        # the reference's own host permutation, compiled from its sources:
        # each step is one single-threaded seq_tt over the slice
        n = math.prod(SLICE)
        r = subprocess.run([exe, str(ELEM), str(max(1, args.steps)), str(max(0, args.warmup))] +
                           [str(d) for d in SLICE] + [str(p) for p in PERM], capture_output=True, text=True,
                           timeout=1800)
        if r.returncode == 0 and r.stdout.split():
            dt = float(r.stdout.split()[0])
            value = 2.0 * n * ELEM / dt / 1e9
            sample = ("the reference's TensorUtil::seq_tt compiled from its sources, single-threaded as the "
                      "reference runs it, out-of-place on dims (4,20011,512,2) int32 (iota)")
            line = {
                "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "i32", "data": "synthetic (iota, the reference's init_data)",
                "config": {"workload": WORKLOAD, "sample": "dims (4,20011,512,2), 1/16 of the workload", "dims": DIMS,
                           "perm": PERM, "elem_bytes": ELEM},
                "cpu_baseline": {"value": value, "unit": "GB/s", "cores": 1, "kind": "reference", "sample": sample},
                "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            }
            print(json.dumps(line), flush=True)
            return 0
    import numpy as np
    import oracle

    dims = [4, 20011, 512, 2]
    n = math.prod(dims)
    src = oracle.fill_hash(n, ELEM, SEED)
    for _ in range(max(0, args.warmup)):
        oracle.permute(src, dims, PERM, ELEM, threads=0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.permute(src, dims, PERM, ELEM, threads=0)
    dt = (time.perf_counter() - t0) / max(1, args.steps)
    value = 2.0 * n * ELEM / dt / 1e9
    cores = oracle.max_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "i32", "data": "synthetic (seeded counter-hash int32, generated on the host)",
        "config": {"workload": WORKLOAD, "sample": "dims (4,20011,512,2), 1/16 of the workload", "dims": DIMS,
                   "perm": PERM, "elem_bytes": ELEM},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "reference host permutation (TensorUtil::seq_tt) restated in oracle/permute.c, "
                                   "OpenMP over %d host threads, out-of-place on dims (4,20011,512,2) int32" % cores},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def end_to_end(args, E, buf, nbytes, cap, nb, alpha, dev, world):
    """Host buffers through the C ABI: every step copies its input from
    pinned host memory (H2D), transposes it in place and copies the result
    back (D2H).  Steps are pipelined over three device buffers: step k+1's
    H2D and step k-1's D2H run on copy streams while step k's transpose runs,
    and a buffer is refilled as soon as its result has left (two buffers
    would idle the host link for a transpose per step); the transposes
    themselves are serialised on one compute stream."""
    import torch
    host_in = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host_in.copy_(buf[: nbytes])
    host_out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)  # D2H copies are serialised on one stream
    nbuf = 3
    dbuf = [buf] + [torch.empty(cap, dtype=torch.uint8, device=dev) for _ in range(nbuf - 1)]
    h2d, comp, d2h = (torch.cuda.Stream(dev) for _ in range(3))
    main = torch.cuda.current_stream(dev)

    def run(steps):
        freed = [None] * nbuf  # event: buffer k%nbuf's previous D2H done
        for st in (h2d, comp, d2h):
            st.wait_stream(main)
        for k in range(steps):
            b = k % nbuf
            with torch.cuda.stream(h2d):
                if freed[b] is not None:
                    h2d.wait_event(freed[b])
                dbuf[b][: nbytes].copy_(host_in, non_blocking=True)
                loaded = torch.cuda.Event()
                loaded.record(h2d)
            comp.wait_event(loaded)
            E.transpose_ptr(dbuf[b].data_ptr(), cap, DIMS, PERM, ELEM, nb, alpha, E.ORDER_MIXED, comp.cuda_stream)
            done = torch.cuda.Event()
            done.record(comp)
            with torch.cuda.stream(d2h):
                d2h.wait_event(done)
                host_out.copy_(dbuf[b][: nbytes], non_blocking=True)
                freed[b] = torch.cuda.Event()
                freed[b].record(d2h)
        for st in (h2d, comp, d2h):
            main.wait_stream(st)

    # untimed passes over every buffer: the first DMAs into or out of
    # freshly pinned host pages run several times slower than later ones
    host_out.fill_(0)
    run(4)
    torch.cuda.synchronize(dev)
    # host DMA on this machine stalls now and then for 0.1-0.35 s; the
    # median of seven timed runs keeps a stall from deciding the figure
    steps = max(2, args.e2e_steps)
    runs = []
    for _ in range(7):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(main)
        run(steps)
        e1.record(main)
        torch.cuda.synchronize(dev)
        runs.append(e0.elapsed_time(e1) / steps)
    ms = max_over_ranks(statistics.median(runs), dev)
    del dbuf[1:]
    return {"value": job_gbs(nbytes, ms, world), "unit": "GB/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "ms_per_step": ms, "steps": steps,
            "runs_ms_per_step": [round(r, 3) for r in runs],
            "pipeline": "3 device buffers; H2D, transpose and D2H of consecutive steps overlap"}


def run_eithot(args):
    import torch
    import eithot_gb300 as E

    global DIMS
    if args.dims:
        DIMS = [int(x) for x in args.dims.split(",")]

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    nb, alpha, _ = E.estimate(DIMS, PERM, ELEM)
    n = math.prod(DIMS)
    nbytes = n * ELEM
    plan = E.plan(DIMS, PERM, nb, alpha)
    cap = plan.padded_volume * ELEM
    buf = torch.empty(cap, dtype=torch.uint8, device=dev)
    # seeded counter-hash content, generated on the device
    E.fill_hash_ptr(buf.data_ptr(), n, ELEM, SEED + rank)
    stream = torch.cuda.current_stream(dev)

    def step():
        E.transpose_ptr(buf.data_ptr(), cap, DIMS, PERM, ELEM, nb, alpha, E.ORDER_MIXED, stream.cuda_stream)

    # the first step is checked element by element on the device: output
    # element o must hold the hash of the source index its coordinates name
    step()
    bad, first = E.check_hash_ptr(buf.data_ptr(), DIMS, PERM, ELEM, SEED + rank, stream.cuda_stream)
    if bad or E.index_faults() or E.sync_timeouts():
        raise SystemExit("bench: first step wrong: %d mismatching elements, first at output index %d" % (bad, first))

    for _ in range(max(0, args.warmup) - 1):
        step()
    torch.cuda.synchronize(dev)

    # timed region (device-resident), CUDA events on the launching stream;
    # the library also brackets every pass with events on that stream
    E.profile_reset()
    E.set_profiling(True)
    launches = 0
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(dev.index) as clk:
        start.record(stream)
        for _ in range(args.steps):
            step()
            launches += E.last_stats()["n_launches"]
        stop.record(stream)
        torch.cuda.synchronize(dev)
    clocks = clk.summary()
    total_ms = start.elapsed_time(stop)
    per_pass = {}
    for p in E.profile():
        d = per_pass.setdefault(p["name"], {"ms": 0.0, "n": 0, "bytes": p["bytes"]})
        d["ms"] += p["ms"]
        d["n"] += 1
    E.set_profiling(False)
    E.profile_reset()
    total_ms = max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = job_gbs(nbytes, ms_per_step, world)

    # end-to-end through the C ABI from pinned host memory
    e2e = None
    if not args.no_e2e:
        e2e = end_to_end(args, E, buf, nbytes, cap, nb, alpha, dev, world)

    peak, peak_kind = load_peaks()
    dominant = max(per_pass.items(), key=lambda kv: kv[1]["ms"]) if per_pass else None
    roofline = None
    if dominant:
        name, d = dominant
        avg_ms = d["ms"] / d["n"]
        achieved = d["bytes"] / (avg_ms / 1e3) / 1e9
        traffic = load_traffic().get(name.split(" ")[0])
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": traffic, "kernel": name,
                    "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured"
                    else "fallback 6.8 TB/s",
                    "passes": {k: {"avg_ms": v["ms"] / v["n"], "gbs": v["bytes"] / (v["ms"] / v["n"] / 1e3) / 1e9}
                               for k, v in per_pass.items()},
                    # the whole transpose (every pass) against the same peak
                    "transpose_frac": value / world / peak}

    c1 = time_c1(E, dev) if (rank == 0 and not args.no_extras) else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "i32", "data": "synthetic (seeded counter-hash int32, generated on the device)",
            "config": {"workload": WORKLOAD, "dims": DIMS, "perm": PERM, "elem_bytes": ELEM, "nb": nb,
                       "alpha": alpha, "bytes": nbytes,
                       "l2": "no flush: the 5.25 GB tensor is larger than the 129 MB L2",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": roofline,
            "clocks": clocks,
        }
        if c1:
            line["c1_3001x4096"] = c1
        if not args.no_cpu_baseline:
            port = cpu_baseline()
            ref = ref_seqtt_baseline()
            if ref:
                ref["port_beside"] = port
                line["cpu_baseline"] = ref
            else:
                line["cpu_baseline"] = port
        if not args.no_extras:
            del buf
            torch.cuda.empty_cache()
            line["reference_gpu"] = reference_gpu()
            line["c3_16x3001x1024x256x4_u16"] = time_c3(E, dev)
            # the batched and served forms, summarised (their own workloads print full lines)
            bt = batched_result(args)
            line["batched_4096_mixed"] = {k: bt[k] for k in ("value", "unit", "ms_per_batch", "one_at_a_time",
                                                            "one_at_a_time_fewest", "speedup_vs_one_at_a_time",
                                                            "launches_per_batch", "config")}
            sv = served_result(args)
            line["served_200_poisson"] = {k: sv[k] for k in ("served", "serial", "config")}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def mixed_tensors(count, seed, min_bytes, max_bytes, min_rank, max_rank):
    """Seeded tensors: rank uniform in [min_rank, max_rank], total bytes
    log-uniform in [min_bytes, max_bytes] split over the dims log-uniformly,
    a uniform random permutation, element size uniform in {1, 2, 4, 8}."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        r = int(rng.integers(min_rank, max_rank + 1))
        elem = int(rng.choice([1, 2, 4, 8]))
        total = math.exp(rng.uniform(math.log(min_bytes), math.log(max_bytes)))
        n = max(1, int(total / elem))
        w = rng.uniform(0.05, 1.0, size=r)
        w = w / w.sum() * math.log(n)
        dims = [max(1, int(round(math.exp(x)))) for x in w]
        perm = [int(x) + 1 for x in rng.permutation(r)]
        out.append((dims, perm, elem))
    return out


def run_batched(args):
    print(json.dumps(batched_result(args)), flush=True)
    return 0


def batched_result(args):
    """4096 tensors of 4 KB-64 MB, rank 3-6: the batched form against one
    eithot_transpose call per tensor on one stream (both device-resident,
    wall-clock from the first issue to the device being idle)."""
    import numpy as np
    import torch
    import eithot_gb300 as E
    dev = torch.device("cuda", 0)
    ts = mixed_tensors(args.count or 4096, 4, 4096, 64 << 20, 3, 6)
    sizes = [math.prod(d) * e for d, p, e in ts]
    caps = [int(s * 1.03) + 256 for s in sizes]
    offs = np.cumsum([0] + [(c + 255) // 256 * 256 for c in caps])
    buf = torch.empty(int(offs[-1]), dtype=torch.uint8, device=dev)
    ptrs = [buf.data_ptr() + int(o) for o in offs[:-1]]
    st = torch.cuda.current_stream(dev)
    for t, ((d, p, e), q) in enumerate(zip(ts, ptrs)):
        E.fill_hash_ptr(q, math.prod(d), e, SEED + t, 0, st.cuda_stream)
    batch = E.Batch(ts)
    ws = torch.empty(max(1, batch.workspace_size), dtype=torch.uint8, device=dev)
    batch.run(ptrs, caps, ws.data_ptr(), batch.workspace_size, st.cuda_stream)
    bad = 0
    for t, ((d, p, e), q) in enumerate(zip(ts, ptrs)):
        bad += E.check_hash_ptr(q, d, p, e, SEED + t, st.cuda_stream)[0]
    if bad or E.index_faults() or E.sync_timeouts():
        raise SystemExit("bench: batched run wrong (%d mismatching elements)" % bad)

    def timed(fn):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t0

    def plain(order=E.ORDER_MIXED):
        for (d, p, e), q, c in zip(ts, ptrs, caps):
            E.transpose_ptr(q, c, d, p, e, 1, 0.01, order, st.cuda_stream)

    def plain_fewest():
        plain(E.ORDER_FEWEST)

    def batched():
        batch.run(ptrs, caps, ws.data_ptr(), batch.workspace_size, st.cuda_stream)

    plain()
    plain_fewest()
    batched()  # a repeat of the checked run's buffers: captured into a CUDA graph here, replayed below
    t_plain = statistics.median(timed(plain) for _ in range(max(3, args.steps // 4)))
    t_plain_fewest = statistics.median(timed(plain_fewest) for _ in range(max(3, args.steps // 4)))
    t_batch = statistics.median(timed(batched) for _ in range(max(3, args.steps // 4)))
    total = sum(sizes)
    line = {"metric": "batched in-place GB/s (2*bytes/s), %d mixed tensors" % len(ts), "value": 2 * total / t_batch / 1e9,
            "unit": "GB/s", "higher_is_better": True, "n_gpus": 1, "ms_per_batch": t_batch * 1e3,
            "one_at_a_time": {"value": 2 * total / t_plain / 1e9, "ms": t_plain * 1e3,
                              "plan": "the reference's series (EITHOT_ORDER_MIXED, eithot_transpose's default)"},
            "one_at_a_time_fewest": {"value": 2 * total / t_plain_fewest / 1e9, "ms": t_plain_fewest * 1e3,
                                     "plan": "fewest modelled passes (EITHOT_ORDER_FEWEST), as the batch plans"},
            "speedup_vs_one_at_a_time": t_plain / t_batch, "launches_per_batch": batch.launches,
            "data": "synthetic (seeded counter hash per tensor, checked on the device after the first run)",
            "config": {"workload": "4096 tensors, rank U{3..6}, bytes log-uniform [4 KB, 64 MB], elem U{1,2,4,8}, "
                                   "random permutations (seed 4)", "tensors": len(ts), "bytes": total}}
    del buf, ws
    torch.cuda.empty_cache()
    return line


class _Arena:
    """First-fit placement of request tensors in one device buffer."""

    def __init__(self, size):
        self.free = [(0, size)]

    def take(self, n):
        n = (n + 255) // 256 * 256
        for i, (o, l) in enumerate(self.free):
            if l >= n:
                self.free[i] = (o + n, l - n)
                return o
        return None

    def give(self, o, n):
        n = (n + 255) // 256 * 256
        self.free.append((o, n))
        self.free.sort()
        merged = []
        for a, l in self.free:
            if merged and merged[-1][0] + merged[-1][1] == a:
                merged[-1] = (merged[-1][0], merged[-1][1] + l)
            elif l:
                merged.append((a, l))
        self.free = merged


def run_served(args):
    print(json.dumps(served_result(args)), flush=True)
    return 0


def served_result(args):
    """Poisson arrivals (200 requests/s, seeded) of tensors of 1 MB-40 GB,
    rank 2-8, resident in one device arena: the server (4 streams, 5 %
    workspace pool, continuous batching) against serial eithot_transpose
    calls in arrival order.  Latency = finish - arrival."""
    import numpy as np
    import torch
    import eithot_gb300 as E
    dev = torch.device("cuda", 0)
    count = args.count or 200
    reqs = mixed_tensors(count, 5, 1 << 20, 40 << 30, 2, 8)
    rng = np.random.default_rng(6)
    arrivals = np.cumsum(rng.exponential(1.0 / 200.0, size=count))
    sizes = [math.prod(d) * e for d, p, e in reqs]
    free, _ = torch.cuda.mem_get_info(dev)
    arena_bytes = int(min(free * 0.55, 160e9))
    arena = torch.empty(arena_bytes, dtype=torch.uint8, device=dev)
    base = arena.data_ptr()
    # the pool holds the largest request's scratch plus room for batches
    pool = max(E.workspace_size(d, p, e, 1, 0.05) for d, p, e in reqs) + (256 << 20)

    def drive(serial):
        alloc = _Arena(arena_bytes)
        srv = None if serial else E.Server(pool, streams=4)
        st = torch.cuda.Stream(dev)
        placed, start, finish = {}, None, {}
        nxt = 0
        t0 = time.perf_counter()
        waiting = []
        while len(finish) < count:
            now = time.perf_counter() - t0
            while nxt < count and arrivals[nxt] <= now:
                waiting.append(nxt)
                nxt += 1
            if serial:
                if waiting:
                    i = waiting.pop(0)
                    d, p, e = reqs[i]
                    o = alloc.take(sizes[i] + 256)
                    E.transpose_ptr(base + o, sizes[i] + 256, d, p, e, 1, 0.05, E.ORDER_MIXED, st.cuda_stream)
                    st.synchronize()
                    finish[i] = time.perf_counter() - t0
                    alloc.give(o, sizes[i] + 256)
                elif nxt < count:
                    time.sleep(max(0.0, min(0.001, arrivals[nxt] - now)))
                continue
            while waiting:
                i = waiting[0]
                o = alloc.take(sizes[i] + 256)
                if o is None:
                    break
                d, p, e = reqs[i]
                tk = srv.submit(base + o, sizes[i] + 256, d, p, e, 1, 0.05)
                placed[tk] = (i, o)
                waiting.pop(0)
            for tk in srv.poll():
                i, o = placed.pop(tk)
                finish[i] = time.perf_counter() - t0
                alloc.give(o, sizes[i] + 256)
            if not placed and not waiting and nxt < count:
                time.sleep(max(0.0, min(0.001, arrivals[nxt] - (time.perf_counter() - t0))))
        if srv:
            srv.close()
        lat = np.array([finish[i] - arrivals[i] for i in range(count)])
        span = max(finish.values())
        return lat, span

    drive(False)  # warm every kernel the requests need
    lat_s, span_s = drive(True)
    lat_v, span_v = drive(False)
    if E.index_faults() or E.sync_timeouts():
        raise SystemExit("bench: served run reported index faults or sync timeouts")
    total = sum(sizes)
    line = {"metric": "served in-place transposes: p50/p99 latency and GB/s", "unit": "ms", "higher_is_better": False,
            "n_gpus": 1, "value": float(np.percentile(lat_v, 99) * 1e3),
            "served": {"p50_ms": float(np.percentile(lat_v, 50) * 1e3), "p99_ms": float(np.percentile(lat_v, 99) * 1e3),
                       "GBs": 2 * total / span_v / 1e9, "span_s": span_v},
            "serial": {"p50_ms": float(np.percentile(lat_s, 50) * 1e3), "p99_ms": float(np.percentile(lat_s, 99) * 1e3),
                       "GBs": 2 * total / span_s / 1e9, "span_s": span_s},
            "data": "synthetic shapes; tensor contents are not generated (the kernels move bytes whatever they hold)",
            "config": {"workload": "%d requests, Poisson 200/s (seed 6), rank U{2..8}, bytes log-uniform [1 MB, 40 GB], "
                                   "elem U{1,2,4,8}, random permutations (seed 5), alpha 0.05" % count,
                       "bytes": total, "server": {"streams": 4, "workspace_pool_bytes": pool}}}
    del arena
    torch.cuda.empty_cache()
    return line


def run_study(args):
    """The reference's experiments on GB300: REORDER_TYPE (pre, post,
    mixed) on rank 4-6 permutations, and the sub-tensor count nb at fixed
    alpha on large tensors (time and scratch).  One JSON line per case."""
    import numpy as np
    import torch
    import eithot_gb300 as E
    dev = torch.device("cuda", 0)
    st = torch.cuda.current_stream(dev)

    def time_case(dims, perm, elem, nb, alpha, order):
        info = E.plan(dims, perm, nb, alpha, order)
        cap = info.padded_volume * elem
        buf = torch.empty(cap, dtype=torch.uint8, device=dev)
        E.transpose_ptr(buf.data_ptr(), cap, dims, perm, elem, nb, alpha, order, st.cuda_stream)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(3):
            E.transpose_ptr(buf.data_ptr(), cap, dims, perm, elem, nb, alpha, order, st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / 3
        return ms, E.workspace_size(dims, perm, elem, nb, alpha, order), info

    rng = np.random.default_rng(7)
    for r in (4, 5, 6):
        for _ in range(4):
            total = 1 << 30
            w = rng.uniform(0.3, 1.0, size=r)
            w = w / w.sum() * math.log(total / 4)
            dims = [max(2, int(round(math.exp(x)))) for x in w]
            perm = [int(x) + 1 for x in rng.permutation(r)]
            row = {"study": "reorder_type", "dims": dims, "perm": perm, "elem": 4}
            for name, order in (("mixed", E.ORDER_MIXED), ("pre", E.ORDER_PRE), ("post", E.ORDER_POST)):
                ms, ws, info = time_case(dims, perm, 4, 1, 0.01, order)
                row[name] = {"ms": round(ms, 3), "GBs": round(2 * math.prod(dims) * 4 / ms / 1e6, 1),
                             "rounds": sum(1 for s in info.steps if s.role == 0)}
            print(json.dumps(row), flush=True)
    for dims, perm in (([4, 20011, 8192, 2], [1, 3, 2, 4]), ([7248, 50, 3000], [2, 1, 3]),
                       ([16, 3001, 64, 256], [4, 3, 1, 2])):
        for nb in (1, 2, 4, 8, 16):
            ms, ws, info = time_case(dims, perm, 4, nb, 0.01, E.ORDER_MIXED)
            print(json.dumps({"study": "sub_tensors", "dims": dims, "perm": perm, "elem": 4, "nb_requested": nb,
                              "nb_applied": info.num_sub_tensors, "padded": info.padded, "ms": round(ms, 3),
                              "GBs": round(2 * math.prod(dims) * 4 / ms / 1e6, 1), "workspace_bytes": ws}), flush=True)
    return 0


def run_case(args):
    """One shape through the C ABI: W untimed transposes (the first checked
    element by element on the device), then K transposes timed with CUDA
    events on the launching stream, with per-pass times from the library's
    profiler.  For ncu captures of one pass kind on a small case."""
    import torch
    import eithot_gb300 as E
    dims = [int(x) for x in args.dims.split(",")]
    perm = [int(x) for x in args.perm.split(",")]
    elem = args.elem
    for kv in args.knob:
        k, v = kv.split("=")
        E.tune_set(k, float(v))
    dev = torch.device("cuda", 0)
    n = math.prod(dims)
    nbytes = n * elem
    buf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    E.fill_hash_ptr(buf.data_ptr(), n, elem, SEED, 0, stream.cuda_stream)

    def step():
        E.transpose_ptr(buf.data_ptr(), nbytes, dims, perm, elem, 1, args.alpha, args.order, stream.cuda_stream)

    step()
    bad, _ = E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, SEED, stream.cuda_stream)
    if bad or E.call_status(E.last_call(), stream.cuda_stream) != E.OK:
        raise SystemExit("bench: case wrong (%d mismatching elements)" % bad)
    for _ in range(max(0, args.warmup) - 1):
        step()
    torch.cuda.synchronize(dev)
    E.profile_reset()
    E.set_profiling(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    E.set_profiling(False)
    per = {}
    for p in E.profile():
        d = per.setdefault(p["name"], [0.0, 0, p["bytes"]])
        d[0] += p["ms"]
        d[1] += 1
    ms = e0.elapsed_time(e1) / max(1, args.steps)
    st = E.last_stats()
    print(json.dumps({"workload": "case", "dims": dims, "perm": perm, "elem_bytes": elem, "order": args.order,
                      "knobs": args.knob, "bit_exact": True, "ms": ms, "GBs": 2.0 * nbytes / (ms / 1e3) / 1e9,
                      "passes": st["n_passes"], "launches": st["n_launches"], "workspace_bytes": st["workspace_bytes"],
                      "per_pass": {k: {"ms": v[0] / v[1], "GBs": v[2] / (v[0] / v[1] / 1e3) / 1e9}
                                   for k, v in per.items()}}), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "case":
        return run_case(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    if args.workload == "study":
        return run_study(args)
    return run_eithot(args)


if __name__ == "__main__":
    sys.exit(main())

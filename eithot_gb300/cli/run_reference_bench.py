"""Runs the reference's benchmark script, unchanged, against this library's
drop-in programs.

    python eithot_gb300/cli/run_reference_bench.py --bench-dir DIR --task K
        [--reorder-type T] [--out OUT] [--cases N] [--test-inplace PATH]

DIR holds the reference's Benchmark folder (Bench.sh and test_cases/, as
the reference ships them).  The script expects test_inplace, Nd_estimation
and Statistic.py beside it (its README: "copy the test_inplace and
Nd_estimation ... into the Benchmark folder"); this runner makes a scratch
copy of the folder, links eithot_gb300/bin's programs there, runs
`bash Bench.sh K` and copies what the script leaves (per case file: the
appended times, throughputs and Statistic.txt) plus its console output to
OUT.  --reorder-type sets EITHOT_REORDER_TYPE for test_inplace (the
reference's compile-time REORDER_TYPE: 0 mixed, 1 pre, 2 post; 3 this
library's fewest-pass plans), as its experiment 6 asks.  --cases N keeps the
first N lines of every case file (a bounded run; the default keeps all).
--test-inplace PATH runs another test_inplace program in place of this
library's (e.g. the reference's own build, to time both on one GPU); the
estimator and the summary script stay this library's.
Prints one JSON line: cases run, cases verified correct, the mean/std of
the time and throughput columns per case file, and per case (in run order)
its dims, sub-tensor count, size, verdict and the two times test_inplace
prints ("Execution Time without h2d2h" and "Execution Time", ms).
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(os.path.dirname(HERE), "bin")


CASE_RE = re.compile(r"number of sub_tensors = (\d+)\s*\nDims = ([0-9 ]+), Data size = ([0-9.]+) GB\n"
                     r"(?:.*\n)*?(Correct|Incorrect) transpose\n"
                     r"Execution Time without h2d2h: (-?[0-9.]+)ms\nExecution Time: ([0-9.]+)ms")


def per_case(log):
    """The test_inplace blocks of the script's console output, in order."""
    out = []
    for m in CASE_RE.finditer(log):
        out.append({"nb": int(m.group(1)), "dims": [int(x) for x in m.group(2).split()], "gb": float(m.group(3)),
                    "correct": m.group(4) == "Correct", "kernel_ms": float(m.group(5)), "e2e_ms": float(m.group(6))})
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--bench-dir", required=True)
    ap.add_argument("--task", type=int, required=True)
    ap.add_argument("--reorder-type", type=int, default=None)
    ap.add_argument("--out", default=None)
    ap.add_argument("--cases", type=int, default=0)
    ap.add_argument("--test-inplace", default=None)
    args = ap.parse_args()
    for prog in ("test_inplace", "Nd_estimation", "Statistic.py"):
        if not os.path.exists(os.path.join(BIN, prog)):
            print("missing %s: build the library first" % os.path.join(BIN, prog), file=sys.stderr)
            return 2
    work = tempfile.mkdtemp(prefix="eithot_bench_")
    try:
        shutil.copy(os.path.join(args.bench_dir, "Bench.sh"), work)
        shutil.copytree(os.path.join(args.bench_dir, "test_cases"), os.path.join(work, "test_cases"))
        if args.cases > 0:
            for f in glob.glob(os.path.join(work, "test_cases", "*", "*.txt")):
                with open(f) as fh:
                    lines = fh.readlines()[: args.cases]
                with open(f, "w") as fh:
                    fh.writelines(lines)
        for prog in ("test_inplace", "Nd_estimation", "Statistic.py"):
            src = os.path.abspath(args.test_inplace) if prog == "test_inplace" and args.test_inplace else os.path.join(BIN, prog)
            os.symlink(src, os.path.join(work, prog))
        env = dict(os.environ)
        if args.reorder_type is not None:
            env["EITHOT_REORDER_TYPE"] = str(args.reorder_type)
        p = subprocess.run(["bash", "Bench.sh", str(args.task)], cwd=work, env=env, capture_output=True, text=True)
        log = p.stdout + p.stderr
        summary = {"task": args.task, "reorder_type": args.reorder_type, "test_inplace": args.test_inplace or "this library's",
                   "exit": p.returncode,
                   "cases": log.count("Execution Time:"), "correct": log.count("Correct transpose"),
                   "incorrect": log.count("Incorrect transpose"), "files": {}}
        summary["per_case"] = per_case(log)
        for d in sorted(glob.glob(os.path.join(work, "test_cases", "exp%d" % args.task, "*"))):
            if not os.path.isdir(d):
                continue
            cols = {}
            for name in ("inplace_bench.txt", "inplace_bench_throughput.txt"):
                path = os.path.join(d, name)
                if os.path.exists(path):
                    with open(path) as fh:
                        v = [float(x) for x in fh.read().split()]
                    if v:
                        cols[name[:-4]] = {"n": len(v), "mean": statistics.mean(v), "std": statistics.pstdev(v)}
            summary["files"][os.path.basename(d)] = cols
        if args.out:
            os.makedirs(args.out, exist_ok=True)
            with open(os.path.join(args.out, "bench_sh_task%d.log" % args.task), "w") as fh:
                fh.write(log)
            for d in glob.glob(os.path.join(work, "test_cases", "exp%d" % args.task, "*")):
                if os.path.isdir(d):
                    shutil.copytree(d, os.path.join(args.out, os.path.basename(d)), dirs_exist_ok=True)
        print(json.dumps(summary), flush=True)
        return 0 if p.returncode == 0 and summary["incorrect"] == 0 else 1
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    sys.exit(main())

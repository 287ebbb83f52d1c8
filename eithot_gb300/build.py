"""Builds the in-tree shared library eithot_gb300/_lib/libeithot.so for sm_103a.

    python eithot_gb300/build.py [-v] [-f]

Host C++ is compiled by g++, CUDA by nvcc (one -gencode, sm_103a), in
parallel; the library links the CUDA runtime statically and carries no torch
dependency.  Objects go to eithot_gb300/_build/.  The drop-in replacements of
the reference's command-line programs (test_inplace, Nd_estimation) are
linked against the library into eithot_gb300/bin/, beside a copy of
Statistic.py (the summary script the reference's benchmark runs).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libeithot.so")
CLIDIR = os.path.join(PKG, "cli")
BINDIR = os.path.join(PKG, "bin")
CLI_PROGRAMS = {"test_inplace": "test_inplace.cpp", "Nd_estimation": "nd_estimation.cpp"}
CLI_SCRIPTS = ["Statistic.py"]  # run by the reference's benchmark script beside the programs

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Device code is stored uncompressed: the CUDA runtime inflates a compressed
# fatbinary on the first use of its module in every process, which cost about
# 40 ms of a process's first transpose on GB300 (49-53 ms against 8-11 ms
# uncompressed; the library grows from 18 to 67 MB).
NVCC_FLAGS = ARCH + ["--compress-mode=none"]
CU_SOURCES = ["kernels.cu", "checks.cu", "perm.cu", "noalloc.cu", "status.cu"]
# kernels.cu is compiled once for the host-side executor and once per unit
# size (-DEITHOT_UNIT): one device module per unit size, loaded on first use.
UNIT_SIZES = {"kernels.cu": [1, 2, 4, 8, 16]}
CPP_SOURCES = ["plan.cpp", "lower.cpp", "search.cpp", "estimator.cpp", "capi.cpp", "batch.cpp", "server.cpp"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), proc.stdout, proc.stderr))
    return proc.stdout + proc.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", os.path.join(cuda, "include")]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "eithot.h"))
    jobs, objs = [], []
    # objects built with other flags are rebuilt
    stamp = os.path.join(BUILD, "nvcc_flags.txt")
    flags_text = " ".join(NVCC_FLAGS)
    if not os.path.exists(stamp) or open(stamp).read() != flags_text:
        force = True
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        for unit in [None] + UNIT_SIZES.get(src, []):
            o = os.path.join(BUILD, src + (".u%d" % unit if unit else "") + ".o")
            objs.append(o)
            if force or _stale(o, [s] + headers):
                jobs.append([nvcc] + NVCC_FLAGS + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                                   "-Xptxas", "-v" if verbose else "-O3"] +
                            (["-DEITHOT_UNIT=%d" % unit] if unit else []) + inc + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"] + inc +
                        ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(LIB, objs):
        _run([nvcc] + NVCC_FLAGS + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs)
        with open(stamp, "w") as fh:
            fh.write(flags_text)
    os.makedirs(BINDIR, exist_ok=True)
    cli_jobs = []
    for name, src in CLI_PROGRAMS.items():
        s = os.path.join(CLIDIR, src)
        b = os.path.join(BINDIR, name)
        if force or _stale(b, [s, LIB, os.path.join(ROOT, "include", "eithot.h")]):
            cli_jobs.append([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-pthread"] + inc +
                            [s, "-o", b, "-L", LIBDIR, "-leithot", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/../_lib"])
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        for out in ex.map(_run, cli_jobs):
            if verbose and out.strip():
                print(out)
    for name in CLI_SCRIPTS:
        shutil.copyfile(os.path.join(CLIDIR, name), os.path.join(BINDIR, name))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

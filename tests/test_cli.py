"""The drop-in replacements of the reference's command-line programs
(eithot_gb300/bin/Nd_estimation and eithot_gb300/bin/test_inplace): same
argv, same stdout lines, same files appended in the working directory."""
import json
import math
import os
import re
import subprocess

import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "eithot_gb300", "bin")


def run(prog, args, cwd, env=None):
    exe = os.path.join(BIN, prog)
    assert os.path.exists(exe), "%s is not built (run __graft_entry__.build())" % exe
    return subprocess.run([exe] + [str(a) for a in args], cwd=cwd, capture_output=True, text=True, timeout=600,
                          env=env)


def test_nd_estimation_matches_reference_output(E, tmp_path):
    """Every case the reference estimator ran without crashing: identical
    stdout and identical proper_input.txt line (the reference was run with
    48 KiB of shared memory per block and 304 padding blocks, the values
    of a GB300 and of this program when no GPU is present)."""
    cases = json.load(open(os.path.join(ROOT, "tests", "golden", "estimates_ref.json")))["cases"]
    checked = 0
    for c in cases:
        if "crash" in c:
            continue
        d = tmp_path / ("c%d" % checked)
        d.mkdir()
        p = run("Nd_estimation", c["dims"] + c["perm"] + [c["elem"], c["nb"], c["alpha"]], d)
        assert p.returncode == 0, p.stderr
        assert p.stdout == c["stdout"], (c["dims"], c["perm"], c["elem"], c["alpha"])
        assert (d / "proper_input.txt").read_text() == c["proper_input"]
        checked += 1
    assert checked >= 150


def test_nd_estimation_appends(E, tmp_path):
    for _ in range(2):
        assert run("Nd_estimation", [3001, 4096, 2, 1, 4, 1, 0.01], tmp_path).returncode == 0
    assert (tmp_path / "proper_input.txt").read_text() == "3001 4096 2 1 4 1 0.01\n" * 2


def test_nd_estimation_beyond_reference_limits(E, tmp_path):
    """The 100.7 GB uint16 tensor the reference estimator asserts on
    (UPPER_BOUND_VOLUME 22e9) gets an estimate."""
    p = run("Nd_estimation", [16, 3001, 1024, 256, 4, 5, 3, 1, 4, 2, 2, 1, 0.05], tmp_path)
    assert p.returncode == 0, p.stderr
    assert p.stdout.splitlines()[-1].startswith("\t16 3001 1024 256 4 5 3 1 4 2 2 ")


def test_cli_usage_errors(E, tmp_path):
    for prog in ("Nd_estimation", "test_inplace"):
        p = run(prog, [3001, 4096, 2, 1], tmp_path)
        assert p.returncode == 2 and "usage" in p.stderr
    # the reference rejects element sizes below 4 it cannot move; 3 is invalid here too
    p = run("test_inplace", [30, 40, 2, 1, 3, 1, 0.01], tmp_path)
    assert p.returncode == 0 and p.stdout == "Invalid rank or type size\n"
    assert not (tmp_path / "inplace_bench.txt").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    [3001, 4096, 2, 1, 4, 1, 0.01],                   # 3001x4096 int32, one sub-tensor
    [7249, 50, 2, 1, 4, 4, 0.02],                      # sub-tensors with padding
    [33, 17, 9, 2, 3, 1, 8, 1, 0.01],                  # 64-bit elements
    [16, 3001, 64, 3, 1, 2, 2, 1, 0.05],               # 16-bit elements (beyond the reference)
    [6, 4, 3401, 3, 2, 1, 1, 2, 0.01]])                # 8-bit elements, sub-tensors
def test_test_inplace_runs_and_verifies(E, tmp_path, args):
    """Every line the reference's driver prints (ITNT/src/test_inplace.cpp:32-76),
    compared exactly except the two measured times, whose format is checked;
    the two files it appends to hold the total time and 2*bytes/1e6/time."""
    p = run("test_inplace", args, tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = p.stdout.splitlines()
    rank = (len(args) - 3) // 2
    dims, perm, elem = args[:rank], args[rank:2 * rank], args[2 * rank]
    perm_int = sum(10 ** i * perm[rank - i - 1] for i in range(rank))
    size = math.prod(dims) * elem
    assert len(lines) == 7, lines
    assert lines[:5] == ["%dD Inplace %d transpose" % (rank, perm_int),
                         "number of sub_tensors = %d" % args[2 * rank + 1],
                         "Dims = %s, Data size = %.5f GB" % (" ".join(str(d) for d in dims), size / 1e9),
                         "Inplace transpose verify_inplace", "Correct transpose"]
    assert re.fullmatch(r"Execution Time without h2d2h: -?\d+\.\d{5}ms", lines[5]), lines[5]
    m = re.fullmatch(r"Execution Time: (\d+\.\d{5})ms", lines[6])
    assert m, lines[6]
    t = float(m.group(1))
    assert (tmp_path / "inplace_bench.txt").read_text() == "%.5f\n" % t
    thr = (tmp_path / "inplace_bench_throughput.txt").read_text()
    assert re.fullmatch(r"\d+\.\d{5}\n", thr)
    assert abs(float(thr) - size * 2 / 1e6 / t) <= 1e-4 * float(thr) + 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    [3001, 4096, 2, 1, 4, 1, 0.01],                   # 3001x4096 int32
    [7249, 50, 2, 1, 4, 4, 0.02],                      # sub-tensors with padding
    [33, 17, 9, 2, 3, 1, 8, 1, 0.01],                  # 64-bit elements
    [6, 4, 3401, 3, 2, 1, 1, 2, 0.01]])                # 8-bit elements, sub-tensors
def test_test_inplace_managed_memory(E, tmp_path, args):
    """EITHOT_MEMORY_TYPE=2: the reference's managed path (tensor in
    cudaMallocManaged memory with 3 % slack, transposed where it lies,
    checked in place by the host), with its own output lines."""
    env = dict(os.environ, EITHOT_MEMORY_TYPE="2")
    p = run("test_inplace", args, tmp_path, env=env)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = p.stdout.splitlines()
    rank = (len(args) - 3) // 2
    assert lines[0].startswith("%dD Inplace " % rank) and ", Data size = " in lines[0]
    assert lines[1] == "number of sub_tensors = %d" % args[2 * rank + 1]
    assert lines[2:4] == ["Inplace transpose verify_inplace", "Correct transpose"]
    assert lines[4].startswith("Execution Time: ")
    t = float(lines[4].split(": ")[1].rstrip("ms"))
    assert (tmp_path / "inplace_bench.txt").read_text() == "%.5f\n" % t
    assert float((tmp_path / "inplace_bench_throughput.txt").read_text()) > 0


def test_statistic_summarises_the_bench_files(tmp_path):
    """Statistic.py (copied beside the programs into eithot_gb300/bin): mean and
    population standard deviation of inplace_bench.txt and
    inplace_bench_throughput.txt, printed and written to Statistic.txt."""
    import statistics
    (tmp_path / "inplace_bench.txt").write_text("70.5\n72.25\n60.0\n")
    (tmp_path / "inplace_bench_throughput.txt").write_text("6.5\n6.0\n")
    p = subprocess.run(["python3", os.path.join(ROOT, "eithot_gb300", "cli", "Statistic.py")], cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert p.returncode == 0, p.stderr
    want = ("Bench time:\n\tAvg:  %r\n\tStd:  %r\nThroughput:\n\tAvg:  %r\n\tStd:  %r\n"
            % (statistics.fmean([70.5, 72.25, 60.0]), statistics.pstdev([70.5, 72.25, 60.0]), 6.25, 0.25))
    assert p.stdout == want
    assert (tmp_path / "Statistic.txt").read_text() == want


def test_benchmark_script_runner_parses_each_case():
    """The runner of the reference's benchmark script reads every
    test_inplace block of the script's console output (host only)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "run_reference_bench", os.path.join(ROOT, "eithot_gb300", "cli", "run_reference_bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    log = ("test_cases/exp2/exp2.txt\nCase 1\ninit Extra Memory size = 7.42195 MB\n\tx\n\n"
           "Case 1\n2D Inplace 21 transpose\nnumber of sub_tensors = 4\nDims = 7248 7248, Data size = 0.21013 GB\n"
           "Inplace transpose verify_inplace\nCorrect transpose\nExecution Time without h2d2h: 2.50000ms\n"
           "Execution Time: 4.75000ms\n\nCase 2\n3D Inplace 132 transpose\nnumber of sub_tensors = 8\n"
           "Dims = 368 384 384, Data size = 0.21706 GB\nInplace transpose verify_inplace\nIncorrect transpose\n"
           "Execution Time without h2d2h: -0.10000ms\nExecution Time: 3.00000ms\n")
    cases = mod.per_case(log)
    assert cases == [
        {"nb": 4, "dims": [7248, 7248], "gb": 0.21013, "correct": True, "kernel_ms": 2.5, "e2e_ms": 4.75},
        {"nb": 8, "dims": [368, 384, 384], "gb": 0.21706, "correct": False, "kernel_ms": -0.1, "e2e_ms": 3.0}]

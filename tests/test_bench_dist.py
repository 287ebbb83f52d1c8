"""bench.py's multi-rank path, on CPU with the gloo backend: ranks are
independent replicas (no collective on the data path); the step time is
the slowest rank's and the job's bytes are every rank's; the reference arm
runs on rank 0 only."""
import importlib.util
import os
import socket

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench = load_bench()
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, torch.device("cpu"))
    gbs = bench.job_gbs(1000, slowest, world)
    dist.barrier()
    dist.destroy_process_group()
    out_q.put((rank, slowest, gbs))


def test_max_over_ranks_and_job_throughput_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]         # both ranks see the slowest rank's time
    assert all(abs(r[2] - 2 * 2 * 1000 / 15e-3 / 1e9) < 1e-12 for r in res)


def test_single_process_has_no_reduction():
    bench = load_bench()
    assert bench.max_over_ranks(3.5, torch.device("cpu")) == 3.5
    assert bench.job_gbs(5245763584, 3.9, 1) == pytest.approx(2690.1, rel=1e-3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    bench = load_bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    import argparse
    ns = argparse.Namespace(gpus=2, steps=1, warmup=0, impl="reference")
    assert bench.run_reference(ns) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_rank_zero():
    """`bench.py --impl reference` on the host: one JSON line with the arm's
    own metric, a cpu_baseline describing the run and an e2e with no host
    copies."""
    import json
    import subprocess
    import sys
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

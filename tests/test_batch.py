"""The batched form (eithot_batch_*): many independent transposes planned
once and run over internal streams; every tensor bit-exact against the
oracle."""
import math

import numpy as np
import pytest

import oracle


def random_tensors(count, seed, max_bytes=1 << 21):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        r = int(rng.integers(2, 7))
        elem = int(rng.choice([1, 2, 4, 8]))
        total = math.exp(rng.uniform(math.log(64), math.log(max_bytes)))
        n = max(1, int(total / elem))
        w = rng.uniform(0.05, 1.0, size=r)
        w = w / w.sum() * math.log(n)
        dims = [max(1, int(round(math.exp(x)))) for x in w]
        perm = [int(x) + 1 for x in rng.permutation(r)]
        out.append((dims, perm, elem))
    return out


def test_batch_plans_on_the_host(E):
    b = E.Batch([([3001, 4096], [2, 1], 4), ([5, 6, 7], [3, 1, 2], 1), ([9], [1], 2)])
    assert b.count == 3 and b.workspace_size >= 0
    b.close()
    with pytest.raises(E.EithotError) as ei:
        E.Batch([([3, 4], [2, 1], 4), ([3, 4, 5], [1, 1, 2], 4)])
    assert ei.value.code == E.EINVAL and "tensor 1" in str(ei.value)
    empty = E.Batch([])
    assert empty.count == 0 and empty.workspace_size == 0


gpu = pytest.mark.gpu


def run_batch(E, tensors, seed, caller_workspace=False, runs=2, shifts=None):
    """shifts: per tensor, a byte offset added to its 256-aligned base."""
    import torch
    dev = torch.device("cuda:0")
    b = E.Batch(tensors)
    sizes = [math.prod(d) * e for d, p, e in tensors]
    caps = [s + 256 for s in sizes]
    offs = np.cumsum([0] + [(c + 512) // 256 * 256 for c in caps])[:-1]
    if shifts is not None:
        offs = offs + np.array(shifts)
    offs = np.append(offs, offs[-1] + caps[-1] + 512)
    buf = torch.zeros(int(offs[-1]), dtype=torch.uint8, device=dev)
    ws = None
    if caller_workspace and b.workspace_size:
        ws = torch.empty(b.workspace_size, dtype=torch.uint8, device=dev)
    for run in range(runs):
        hosts = [oracle.fill_hash(math.prod(d), e, seed + 1000 * run + t) for t, (d, p, e) in enumerate(tensors)]
        for h, o in zip(hosts, offs):
            buf[int(o):int(o) + h.size] = torch.from_numpy(h).to(dev)
        ptrs = [buf.data_ptr() + int(o) for o in offs[:-1]]
        b.run(ptrs, caps, ws.data_ptr() if ws is not None else 0, b.workspace_size if ws is not None else 0,
              torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert E.index_faults() == 0 and E.sync_timeouts() == 0
        assert b.launches > 0
        got = buf.cpu().numpy()
        for t, ((d, p, e), h, o) in enumerate(zip(tensors, hosts, offs)):
            want = oracle.permute(h, d, p, e)
            if not np.array_equal(got[int(o):int(o) + h.size], want):
                raise AssertionError("batch tensor %d %s perm %s elem %d differs" % (t, d, p, e))
    b.close()


@gpu
def test_batch_random_small_tensors(E):
    run_batch(E, random_tensors(300, 5), seed=11)


@gpu
def test_batch_with_large_and_staged_tensors_caller_workspace(E):
    tensors = random_tensors(40, 6) + [([60000, 300], [2, 1], 4), ([300, 60000], [2, 1], 4),
                                       ([2, 300000], [2, 1], 1), ([3001, 4096], [2, 1], 4)]
    run_batch(E, tensors, seed=21, caller_workspace=True)


@gpu
def test_batch_of_one_and_identity(E):
    run_batch(E, [([37, 64, 5, 3], [3, 1, 4, 2], 4)], seed=3)
    run_batch(E, [([37, 64], [1, 2], 2), ([5, 6, 7], [3, 2, 1], 8)], seed=4)


@gpu
def test_batch_uses_shape_knobs(E):
    """Tensors whose shapes carry recorded knobs are planned and run with them;
    the results stay bit-exact."""
    tensors = random_tensors(30, 8) + [([3001, 4096], [2, 1], 4), ([2, 300000], [2, 1], 1), ([60, 40, 3401], [3, 1, 2], 2)]
    try:
        E.tune_shape_set([3001, 4096], [2, 1], 4, "variant", 1)
        E.tune_shape_set([3001, 4096], [2, 1], 4, "dbuf", 0)
        E.tune_shape_set([2, 300000], [2, 1], 1, "factor", 0)
        E.tune_shape_set([60, 40, 3401], [3, 1, 2], 2, "col_form", 2)  # groups are still left out
        E.tune_shape_set([60, 40, 3401], [3, 1, 2], 2, "max_cluster", 2)
        run_batch(E, tensors, seed=31)
    finally:
        E.tune_shape_clear()


@gpu
@pytest.mark.parametrize("graph", [1, 0])
def test_batch_repeated_runs_replay_a_graph(E, graph):
    """Runs on the same buffers and workspace: the first issues directly, the
    second captures a CUDA graph and every later one replays it (with the
    knob off, every run issues directly); new contents every run, each
    bit-exact."""
    saved = E.tune_get("batch_graph")
    try:
        E.tune_set("batch_graph", graph)
        tensors = random_tensors(60, 9) + [([3001, 4096], [2, 1], 4), ([2, 300000], [2, 1], 1), ([60, 40, 3401], [3, 1, 2], 2)]
        run_batch(E, tensors, seed=41, caller_workspace=True, runs=4)
    finally:
        E.tune_set("batch_graph", saved)


@gpu
@pytest.mark.parametrize("queue", [1, 0])
def test_batch_queue_of_small_tensors(E, queue):
    """Small tensors whose whole permutation fits one CTA are permuted by one
    persistent launch over a device queue (knob batch_queue=1; with 0 they
    run through their planned passes in the lanes): 1- to 16-byte elements,
    ranks 2-8, bases shifted off 16-byte boundaries (a tensor whose entry
    does not apply on its buffer, e.g. 2-byte stores only, falls back to its
    passes), beside larger tensors in the lanes; four runs (the second
    captures a graph, the later ones replay it), each bit-exact."""
    saved = E.tune_get("batch_queue")
    try:
        E.tune_set("batch_queue", queue)
        rng = np.random.default_rng(51)
        tensors, shifts = [], []
        for t in range(200):
            r = int(rng.integers(2, 9))
            elem = int(rng.choice([1, 2, 4, 8, 16]))
            dims = [int(rng.integers(1, 6)) for _ in range(r)]
            while math.prod(dims) * elem < 2048:
                dims[int(rng.integers(0, r))] += 1
            perm = [int(x) + 1 for x in rng.permutation(r)]
            tensors.append((dims, perm, elem))
            shifts.append(int(rng.choice([0, 0, 0, 2, 4, 8, 12])) if elem <= 4 else 0)
        tensors += [([3001, 4096], [2, 1], 4), ([60, 40, 3401], [3, 1, 2], 2)]
        shifts += [0, 0]
        run_batch(E, tensors, seed=61, caller_workspace=True, runs=4, shifts=shifts)
    finally:
        E.tune_set("batch_queue", saved)

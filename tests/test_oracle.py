"""The oracle itself, pinned against the reference's own outputs."""
import itertools
import json
import math
import os

import numpy as np
import pytest

import oracle
from oracle import estimator, planner
from conftest import GOLDEN


def np_permute(a, dims, perm):
    # dims[0] fastest -> numpy C-order shape is reversed dims
    r = len(dims)
    t = a.reshape(list(reversed(dims)))
    out_axes = [r - perm[j] for j in range(r)]          # numpy axis of output axis j
    return np.transpose(t, list(reversed(out_axes))).reshape(-1)


@pytest.mark.parametrize("elem", [1, 2, 4, 8, 3])
def test_permute_matches_numpy(elem):
    rng = np.random.default_rng(elem)
    for r in range(1, 6):
        for _ in range(5):
            dims = [int(x) for x in rng.integers(1, 7, size=r)]
            perm = [int(x) + 1 for x in rng.permutation(r)]
            n = math.prod(dims)
            a = rng.integers(0, 256, size=(n, elem), dtype=np.uint8)
            want = np_permute(np.arange(n), dims, perm)
            got = oracle.permute(a.reshape(-1), dims, perm, elem).reshape(n, elem)
            assert np.array_equal(got, a[want])
            got1 = oracle.permute(a.reshape(-1), dims, perm, elem, threads=1).reshape(n, elem)
            assert np.array_equal(got1, got)


def test_permute_matches_reference_seqtt():
    """TensorUtil::seq_tt compiled from the reference (tests/golden/seqtt_ref.npz)."""
    z = np.load(os.path.join(GOLDEN, "seqtt_ref.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    assert len(meta) >= 20
    for m in meta:
        a = z["in%d" % m["id"]]
        want = z["out%d" % m["id"]]
        got = oracle.permute(a.view(np.uint8), m["dims"], m["perm"], m["elem"]).view(a.dtype)
        assert np.array_equal(got, want), m


def test_iota_known_answer():
    """verify_inplace semantics (ITNT/src/tensor_util.cpp:113-142): after the
    transpose of an iota tensor, out[dest(i)] == i."""
    dims, perm = [3001, 4096], [2, 1]
    n = math.prod(dims)
    a = np.arange(n, dtype=np.int32)
    out = oracle.permute(a.view(np.uint8), dims, perm, 4).view(np.int32)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, n, size=2000):
        assert out[oracle.dest_index(dims, perm, int(i))] == i


def test_planner_matches_reference_plans():
    doc = json.load(open(os.path.join(GOLDEN, "plans_ref.json")))
    assert len(doc["cases"]) > 1000
    for c in doc["cases"]:
        steps, _ = planner.nd_plan(c["dims"], c["perm"], c["nb"], c["alpha"])
        got = [[t, off] + list(d) for t, off, d in steps]
        assert got == c["steps"], c


def test_estimator_matches_readme_screenshots():
    doc = json.load(open(os.path.join(GOLDEN, "estimator_readme.json")))
    assert len(doc["cases"]) == 57
    for c in doc["cases"]:
        e = estimator.estimate(c["dims"], c["perm"], c["elem"], c["nb"], c["alpha"])
        assert "%.5f" % (e["init_tmp"] / 1e6) == c["init_extra_mb"], c
        assert e["nb"] == c["nb_out"] and e["alpha_str"] == c["alpha_out"], (c, e)
    e = estimator.estimate([7248, 7248], [2, 1], 4, 1, 0.01)
    assert "%.5f" % (e["final_tmp"] / 1e6) == doc["final_extra_mb"]["1"]


def test_estimator_matches_reference_binary():
    doc = json.load(open(os.path.join(GOLDEN, "estimates_ref.json")))
    n = 0
    for c in doc["cases"]:
        if "crash" in c:
            continue
        e = estimator.estimate(c["dims"], c["perm"], c["elem"], c["nb"], c["alpha"])
        assert ("%.5f" % (e["init_tmp"] / 1e6), e["nb"], e["alpha_str"]) == \
            (c["init_extra_mb"], c["nb_out"], c["alpha_out"]), c
        n += 1
    assert n > 100

"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference code compiled from its own sources by `make -C oracle ref`
(oracle/_ref/):
  ref_plan       the reference's N-d orchestration + planner (ITNT/src/
                 Nd_transpose.cpp, permutation_util.cpp, Nd_decompose.cpp)
                 with recorders below it  -> plans_ref.json
  Nd_estimation  the reference estimator with 48 KiB shared memory per block
                 and 304 resident padding blocks -> estimates_ref.json
  ref_seqtt      the reference host permutation TensorUtil::seq_tt
                 -> seqtt_ref.npz
Only needed where the reference tree is mounted; the fixtures are committed.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import itertools
import json
import math
import os
import random
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")


def ref_plan(dims, perm, nb, alpha):
    out = subprocess.run([os.path.join(REF, "ref_plan")] + [str(x) for x in dims + perm + [nb, alpha]],
                         capture_output=True, text=True, check=True).stdout
    steps = []
    for line in out.strip().splitlines():
        t = line.split()
        steps.append([t[0], int(t[1])] + [int(x) for x in t[2:]])
    return steps


def ref_estimate(dims, perm, elem, nb, alpha):
    with tempfile.TemporaryDirectory() as d:
        env = dict(os.environ, EITHOT_REF_SMEM="49152", EITHOT_REF_PAD_BLOCKS="304")
        proc = subprocess.run([os.path.join(REF, "Nd_estimation")] + [str(x) for x in dims + perm + [elem, nb, alpha]],
                              capture_output=True, text=True, cwd=d, env=env)
        if proc.returncode != 0:
            return {"crash": proc.returncode}
        out = proc.stdout
        with open(os.path.join(d, "proper_input.txt")) as f:
            proper = f.read()
    lines = out.strip().splitlines()
    init = lines[0].split("=")[1].split()[0]
    last = lines[-1].split()
    return {"init_extra_mb": init, "nb_out": int(last[-2]), "alpha_out": last[-1], "stdout": out,
            "proper_input": proper}


def ref_seqtt(arr, dims, perm, elem):
    out = subprocess.run([os.path.join(REF, "ref_seqtt"), str(elem)] + [str(x) for x in dims + perm],
                         input=arr.tobytes(), capture_output=True, check=True).stdout
    return np.frombuffer(out, dtype=arr.dtype)


def fits_int32(dims, nb=1):
    return math.prod(dims) * 2 * max(nb, 1) < 2 ** 31


def plan_cases():
    rng = random.Random(20241203)
    cases = []
    for r in range(2, 7):
        for perm in itertools.permutations(range(1, r + 1)):
            reps = 2 if r <= 5 else 1
            for _ in range(reps):
                dims = [rng.choice([2, 3, 4, 5, 7, 8, 12, 16, 31, 48, 64, 96, 100]) for _ in range(r)]
                cases.append((dims, list(perm), 1, 0.01))
    # sub-tensor partitioning and padding (max dim above 32/alpha)
    for r in range(2, 6):
        for perm in itertools.permutations(range(1, r + 1)):
            if list(perm) == list(range(1, r + 1)):
                continue
            dims = [rng.choice([2, 3, 5, 8, 12]) for _ in range(r)]
            dims[rng.randrange(r)] = rng.choice([3300, 3500, 4096, 5000, 6400])
            nb = rng.choice([2, 3, 4, 8, 16])
            alpha = rng.choice([0.01, 0.02, 0.05])
            if fits_int32(dims, 2):
                cases.append((dims, list(perm), nb, alpha))
    cases.append(([3001, 4096], [2, 1], 1, 0.01))
    cases.append(([4, 20011, 8192, 2], [1, 3, 2, 4], 1, 0.01))
    cases.append(([7248, 7248], [2, 1], 4, 0.02))
    return cases


def est_cases():
    rng = random.Random(7)
    cases = []
    for r in range(2, 6):
        for perm in itertools.permutations(range(1, r + 1)):
            if list(perm) == list(range(1, r + 1)):
                continue
            for _ in range(2):
                dims = [rng.choice([2, 3, 5, 8, 12, 16, 33, 48, 96, 128, 300, 1000]) for _ in range(r)]
                if rng.random() < 0.5:
                    dims[rng.randrange(r)] = rng.choice([3001, 4096, 5000, 7000, 20011])
                if math.prod(dims) * 8 > 2e9:
                    continue
                cases.append((dims, list(perm), rng.choice([4, 8]), 1, rng.choice([0.01, 0.02, 0.05])))
    cases.append(([3001, 4096], [2, 1], 4, 1, 0.01))
    cases.append(([4, 20011, 8192, 2], [1, 3, 2, 4], 4, 1, 0.01))
    return cases


def main():
    plans = []
    for dims, perm, nb, alpha in plan_cases():
        plans.append({"dims": dims, "perm": perm, "nb": nb, "alpha": alpha, "steps": ref_plan(dims, perm, nb, alpha)})
    with open(os.path.join(HERE, "plans_ref.json"), "w") as f:
        json.dump({"source": "oracle/_ref/ref_plan (reference ITNT/src/Nd_transpose.cpp orchestration)",
                   "cases": plans}, f, separators=(",", ":"))
    ests = []
    for dims, perm, elem, nb, alpha in est_cases():
        e = ref_estimate(dims, perm, elem, nb, alpha)
        e.update({"dims": dims, "perm": perm, "elem": elem, "nb": nb, "alpha": alpha})
        ests.append(e)
    with open(os.path.join(HERE, "estimates_ref.json"), "w") as f:
        json.dump({"source": "oracle/_ref/Nd_estimation (reference estimator, smem 48 KiB, 304 padding blocks)",
                   "cases": ests}, f, separators=(",", ":"))
    rng = np.random.default_rng(11)
    arrays = {}
    meta = []
    k = 0
    for r in range(2, 7):
        for _ in range(4):
            dims = [int(x) for x in rng.integers(1, 9, size=r)]
            perm = [int(x) + 1 for x in rng.permutation(r)]
            elem = int(rng.choice([4, 8]))
            dt = np.int32 if elem == 4 else np.int64
            a = rng.integers(-2 ** 31, 2 ** 31, size=math.prod(dims), dtype=np.int64).astype(dt)
            arrays["in%d" % k] = a
            arrays["out%d" % k] = ref_seqtt(a, dims, perm, elem)
            meta.append({"id": k, "dims": dims, "perm": perm, "elem": elem})
            k += 1
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "seqtt_ref.npz"), **arrays)
    print("plans", len(plans), "estimates", len(ests), "seqtt", k)


if __name__ == "__main__":
    main()

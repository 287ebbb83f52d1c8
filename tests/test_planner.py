"""The product planner (C ABI eithot_plan) against the oracle and the
reference's own plans."""
import itertools
import json
import math
import os
import random

import pytest

from oracle import planner as oplanner
from conftest import GOLDEN

def test_plans_match_reference(E):
    doc = json.load(open(os.path.join(GOLDEN, "plans_ref.json")))
    for c in doc["cases"]:
        p = E.plan(c["dims"], c["perm"], c["nb"], c["alpha"])
        ref = c["steps"]
        # expand: reference issues [PADPRE] [132 partition] (series per sub) [132 join] [PADPOST]
        got = []
        rounds = [s for s in p.steps if s.role == E.STEP_ROUND]
        for s in p.steps:
            if s.role == E.STEP_PAD_PRE:
                got.append(["PADPRE", 0, s.dims[0], s.dims[1], p.num_sub_tensors] + list(c["dims"]))
            elif s.role in (E.STEP_PARTITION, E.STEP_JOIN):
                got.append(["132", 0] + s.dims)
                if s.role == E.STEP_PARTITION:
                    for i in range(p.num_sub_tensors):
                        got += [[str(r.code), i * p.sub_tensor_elems] + r.dims for r in rounds]
            elif s.role == E.STEP_PAD_POST:
                got.append(["PADPOST", 0, p.decompose_dim, c["dims"][p.decompose_dim], p.num_sub_tensors] +
                           [q - 1 for q in c["perm"]])
        if p.decompose_dim < 0:
            got = [[str(r.code), 0] + r.dims for r in rounds]
        assert got == ref, c


@pytest.mark.parametrize("rank", [2, 3, 4, 5, 6])
def test_all_permutations_match_oracle(E, rank):
    rng = random.Random(rank)
    for perm in itertools.permutations(range(1, rank + 1)):
        dims = [rng.choice([2, 3, 5, 8, 13, 48, 100]) for _ in range(rank)]
        for order in (0, 1, 2):
            p = E.plan(dims, list(perm), 1, 0.01, order)
            o = oplanner.choose_order(dims, list(perm), order)
            ops = oplanner.series(dims, list(perm), o)
            assert p.order_used == o
            assert [(s.dims, s.perm) for s in p.steps] == [(d, pp) for d, pp in ops], (dims, perm, order)


def test_high_rank_random(E):
    rng = random.Random(99)
    for _ in range(300):
        r = rng.choice([7, 8])
        perm = list(range(1, r + 1))
        rng.shuffle(perm)
        dims = [rng.choice([2, 3, 4, 5, 7]) for _ in range(r)]
        p = E.plan(dims, perm)
        o = oplanner.choose_order(dims, perm)
        assert [(s.dims, s.perm) for s in p.steps] == [(d, pp) for d, pp in oplanner.series(dims, perm, o)]


def test_64bit_plan_of_the_100gb_tensor(E):
    """(16, 3001, 1024, 256, 4) uint16, perm (5 3 1 4 2): the reference's int
    planner overflows in pre-order round 0; the product plans in 64-bit."""
    dims, perm = [16, 3001, 1024, 256, 4], [5, 3, 1, 4, 2]
    p = E.plan(dims, perm)
    o = oplanner.choose_order(dims, perm)
    assert o == oplanner.POST and p.order_used == E.ORDER_POST
    assert [(s.code, s.dims) for s in p.steps] == [
        (132, [16, 3001, 1048576]), (1324, [16384, 256, 4, 3001]),
        (213, [16, 4096, 768256]), (213, [1024, 4, 12292096])]
    pre = oplanner.series(dims, perm, oplanner.PRE)
    assert all(d > 0 for op in pre for d in op[0])


def test_invalid_inputs_return_einval(E):
    for dims, perm in [([2, 3], [1, 1]), ([2, 3], [0, 1]), ([2, 3], [1, 3]), ([0, 3], [2, 1])]:
        with pytest.raises(E.EithotError) as ei:
            E.plan(dims, perm)
        assert ei.value.code == E.EINVAL
    with pytest.raises(E.EithotError):
        E.plan([2, 3], [2, 1], 1, 0.0)


def test_subtensor_gate(E):
    # max dim <= 32/alpha forces nb = 1 (ITNT/src/Nd_transpose.cpp:268-275)
    assert E.plan([3200, 5], [2, 1], 4, 0.01).num_sub_tensors == 1
    p = E.plan([3201, 5], [2, 1], 4, 0.01)
    assert p.num_sub_tensors == 4 and p.padded and p.padded_dim_size == 3204
    p = E.plan([3204, 5], [2, 1], 4, 0.01)
    assert p.num_sub_tensors == 4 and not p.padded

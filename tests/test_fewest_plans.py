"""Parity of the pass-minimising plans (reorder type EITHOT_ORDER_FEWEST)
with the oracle, through the C ABI on device memory: the searched series
of batched 2D transposes, on-chip slab permutations (the reference's row
linearisations _3214 / _43215, generalised) and cycle-following block
permutations (its column linearisations _1432 / _14325 / _15432,
generalised).  Bit-exact against the oracle's out-of-place permutation."""
import itertools
import math
import random

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FEWEST = 3


def run_case(E, dims, perm, elem, alpha=0.01, seed=1, workspace=None, expect=None):
    """expect: a pass kind ("cycle-perm", "slab-perm") the plan must use."""
    n = math.prod(dims)
    host = oracle.fill_hash(n, elem, seed)
    buf = torch.from_numpy(host.copy()).cuda()
    s = torch.cuda.current_stream()
    wptr, wbytes = 0, 0
    if workspace is not None:
        ws = torch.empty(max(workspace, 256), dtype=torch.uint8, device="cuda")
        wptr, wbytes = ws.data_ptr(), workspace
    if expect:
        E.set_profiling(True)
        E.profile_reset()
    try:
        E.transpose_ptr(buf.data_ptr(), buf.numel(), dims, perm, elem, 1, alpha, FEWEST, s.cuda_stream, wptr, wbytes)
    finally:
        E.set_profiling(False)
    cid = E.last_call()
    assert E.call_status(cid, s.cuda_stream) == E.OK
    if expect:
        names = [p["name"] for p in E.profile()]
        E.profile_reset()
        assert any(nm.startswith(expect) for nm in names), names
    got = buf.cpu().numpy()
    want = oracle.permute(host, dims, perm, elem)
    if not np.array_equal(got, want):
        bad = np.nonzero(got != want)[0]
        raise AssertionError("mismatch %s perm %s elem %d: %d bad bytes, first at %d" % (dims, perm, elem, bad.size, bad[0]))
    return E.last_stats()


@pytest.fixture(params=[(1, 1), (1, 0), (2, 1), (0, 0)], ids=["runs-prefetch", "runs", "runs-carry", "per-element"])
def slab_kernel(E, request):
    """The slab-permutation kernels: runs of outputs per thread from padded
    rows (with the next slab prefetched into registers when one CTA per SM
    fits, or without; runs whose outputs share offsets read them from a
    table unless slab_runs is 2), and one divide chain per element."""
    old = (E.tune_get("slab_runs"), E.tune_get("slab_prefetch"))
    E.tune_set("slab_runs", request.param[0])
    E.tune_set("slab_prefetch", request.param[1])
    yield request.param
    E.tune_set("slab_runs", old[0])
    E.tune_set("slab_prefetch", old[1])


@pytest.mark.parametrize("rank", [3, 4, 5])
def test_every_permutation(E, rank, slab_kernel):
    rng = random.Random(7 + rank)
    for perm in itertools.permutations(range(1, rank + 1)):
        for elem in (1, 2, 4, 8):
            dims = [rng.choice([2, 3, 5, 16, 33, 64, 96, 130]) for _ in range(rank)]
            while math.prod(dims) * elem > (2 << 20):
                dims[dims.index(max(dims))] //= 2
            run_case(E, dims, list(perm), elem)


@pytest.mark.parametrize("dims,perm,elem,expect", [
    ([16, 301, 1024, 64, 4], [5, 3, 1, 4, 2], 2, "cycle-perm"),  # the 100 GB configuration's plan, 1/50 scale
    ([64, 50, 60, 70], [1, 4, 3, 2], 4, "cycle-perm"),        # 15 KB blocks
    ([1024, 7, 9, 11], [1, 4, 3, 2], 8, "slab-perm"),         # a slab of 7 x 9 x 11 8 KB elements, in strips
    ([4096, 3, 300, 200], [1, 4, 3, 2], 2, "cycle-perm"),     # 8 KB blocks of 2-byte elements
    ([4, 31, 64, 8, 4], [5, 3, 1, 4, 2], 16, "slab-perm"),    # a four-axis slab permutation of 16-byte elements
    ([16, 31, 64, 8, 4], [5, 3, 1, 4, 2], 8, "slab-perm"),
    ([20, 30, 40, 50, 6], [5, 4, 3, 2, 1], 2, None),
    ([8, 7, 6, 5, 4, 3], [6, 4, 2, 1, 3, 5], 4, None),
    ([2, 3, 5, 7, 11, 13, 2], [7, 1, 6, 2, 5, 3, 4], 1, None),
    ([4096, 33, 65], [1, 3, 2], 1, None), ([3001, 4096], [2, 1], 4, None), ([4, 2001, 819, 2], [1, 3, 2, 4], 4, None)])
def test_named_shapes(E, dims, perm, elem, expect, slab_kernel):
    """Named shapes; where a cycle-following block permutation is the kind
    under test, such moves are preferred (knob cycle_moves=2): at these sizes
    the cost model would rather stream (a cycle segment is walked by one CTA
    at about 2.6 GB/s)."""
    old = E.tune_get("cycle_moves")
    if expect == "cycle-perm":
        E.tune_set("cycle_moves", 2)
    try:
        run_case(E, dims, perm, elem, expect=expect)
    finally:
        E.tune_set("cycle_moves", old)


@pytest.mark.parametrize("elem", [1, 2, 4, 8, 16, 24])
def test_slab_permutations_forced(E, elem, slab_kernel):
    """Slab permutations preferred over every other move (knob slab_perm=2):
    3- to 5-axis slabs of 1- to 24-byte elements, odd and even row widths,
    unaligned slab sizes, 128 KB slabs of 2-byte elements."""
    old = E.tune_get("slab_perm")
    E.tune_set("slab_perm", 2)
    try:
        for dims, perm in [([16, 64, 4, 9], [3, 2, 1, 4]), ([7, 33, 5, 11], [2, 3, 1, 4]),
                           ([5, 6, 7, 8, 3], [4, 2, 1, 3, 5]), ([64, 32, 8, 5], [2, 3, 1, 4]), ([3, 1000, 7], [2, 1, 3]),
                           ([16, 1024, 4, 5], [3, 2, 1, 4])]:
            limit = 128 * 1024 if dims[:2] == [16, 1024] else 100 * 1024
            while math.prod(dims[:-1]) * elem > limit:
                dims[1] //= 2
            run_case(E, dims, perm, elem)
    finally:
        E.tune_set("slab_perm", old)


@pytest.mark.parametrize("elem", [1, 2, 4, 8, 16])
def test_slab_permutations_aligned_runs(E, elem, slab_kernel):
    """Slabs whose output axes below the store width divide it (runs of
    outputs that share their shared-memory offsets): two to four axes,
    runs inside the fastest output axis, covering it exactly, and spanning
    two and four of its rows; the (16, 1024, 4) 2-byte slab of the 100 GB
    configuration's plan."""
    old = E.tune_get("slab_perm")
    E.tune_set("slab_perm", 2)
    try:
        for dims, perm in [([16, 1024, 4, 3], [3, 2, 1, 4]), ([32, 64, 16, 2], [2, 3, 1, 4]), ([8, 2, 64, 5], [2, 1, 3, 4]),
                           ([64, 4, 16, 3], [2, 3, 1, 4]), ([2, 4, 8, 16, 3], [4, 2, 3, 1, 5]), ([128, 256, 3], [2, 1, 3]),
                           ([4, 4, 4, 4, 4, 2], [5, 4, 3, 2, 1, 6])]:
            while math.prod(dims[:-1]) * elem > 128 * 1024:
                dims[1] //= 2
            run_case(E, dims, perm, elem)
    finally:
        E.tune_set("slab_perm", old)


def test_cycle_permutation_in_chunks(E):
    """A block permutation (32 KB blocks over (301, 64, 4): 628 segments in
    44 cycles, 20.6 MB of saved blocks at once) given an 8 MB workspace: the
    segments run in several chunks of whole cycles, two launches each
    (cycle moves preferred, knob cycle_moves=2)."""
    dims, perm, elem = [16, 301, 1024, 64, 4], [5, 3, 1, 4, 2], 2
    old = E.tune_get("cycle_moves")
    E.tune_set("cycle_moves", 2)
    try:
        assert E.workspace_size(dims, perm, elem, 1, 0.05, FEWEST) > 16 << 20
        st = run_case(E, dims, perm, elem, alpha=0.05, workspace=8 << 20, expect="cycle-perm")
    finally:
        E.tune_set("cycle_moves", old)
    assert st["workspace_bytes"] == 8 << 20
    assert st["n_launches"] >= st["n_passes"] + 4


def test_16x3001x1024x256x4_uint16_fewest_passes(E):
    """(16, 3001, 1024, 256, 4) uint16 (100.7 GB), perm (5 3 1 4 2), alpha
    0.05, planned for the fewest passes: five passes (a Catanzaro transpose
    of 1024 x 3001 matrices of 32-byte elements, a cycle-following
    permutation of 32 KB blocks, the reference's last two rounds) where the
    reference's series takes six.  Every output element is checked on the
    device against the counter hash of its source index."""
    dims, perm, elem, seed = [16, 3001, 1024, 256, 4], [5, 3, 1, 4, 2], 2, 0xC3
    n = math.prod(dims)
    cap = n * elem
    free, _ = torch.cuda.mem_get_info()
    if free < cap * 1.08:
        pytest.skip("needs %.0f GB of free device memory" % (cap * 1.08 / 1e9))
    buf = torch.empty(cap, dtype=torch.uint8, device="cuda")
    E.fill_hash_ptr(buf.data_ptr(), n, elem, seed)
    s = torch.cuda.current_stream()
    E.transpose_ptr(buf.data_ptr(), cap, dims, perm, elem, 1, 0.05, FEWEST, s.cuda_stream)
    cid = E.last_call()
    assert E.call_status(cid, s.cuda_stream) == E.OK
    st = E.last_stats()
    assert st["n_passes"] <= 5
    assert st["workspace_bytes"] <= 0.05 * n * elem
    assert E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, seed) == (0, -1)

"""The lowered pass list applied on the CPU with the kernels' index maps
(tests/native/hostsim.cpp) reproduces the oracle permutation: checks the
planner -> lowering -> index-map chain without a GPU."""
import ctypes
import itertools
import math
import random

import numpy as np
import pytest

import oracle


def run(hostsim, dims, perm, elem, nb=1, alpha=0.01, order=0, slack=1.0, seed=0):
    r = len(dims)
    n = math.prod(dims)
    a = oracle.fill_hash(n, elem, seed)
    cap = int(n * elem * slack) + 64
    buf = np.zeros(cap, dtype=np.uint8)
    buf[:n * elem] = a
    D = (ctypes.c_int64 * r)(*dims)
    P = (ctypes.c_int * r)(*perm)
    k = hostsim.hs_transpose(buf.ctypes.data, cap, r, D, P, elem, nb, alpha, order)
    assert k >= 0, hostsim.hs_last_error()
    return np.array_equal(buf[:n * elem], oracle.permute(a, dims, perm, elem))


@pytest.mark.parametrize("rank", [2, 3, 4, 5])
def test_all_permutations(hostsim, rank):
    rng = random.Random(rank)
    for perm in itertools.permutations(range(1, rank + 1)):
        dims = [rng.choice([1, 2, 3, 5, 7, 8, 12, 13, 24]) for _ in range(rank)]
        for elem in (1, 2, 4, 8, 12):
            for order in (0, 1, 2):
                assert run(hostsim, dims, list(perm), elem, order=order), (dims, perm, elem, order)


@pytest.mark.parametrize("R,C,E", [(3001, 4096, 4), (300, 700, 4), (1000, 999, 2), (64, 8000, 8),
                                   (5000, 60, 16), (40, 2000, 24), (2048, 1536, 4), (700, 1400, 1)])
def test_catanzaro_2d(hostsim, R, C, E):
    assert run(hostsim, [C, R], [2, 1], E)


@pytest.mark.parametrize("dims,perm,nb,alpha", [
    ([7248, 50], [2, 1], 4, 0.02), ([3301, 7, 5], [3, 1, 2], 3, 0.01), ([5, 3302, 6], [2, 3, 1], 4, 0.01),
    ([6, 4, 3401], [3, 2, 1], 2, 0.01), ([40, 3203, 3], [1, 3, 2], 8, 0.01), ([3, 3301, 2, 5], [4, 2, 1, 3], 16, 0.01)])
@pytest.mark.parametrize("elem", [2, 4, 8])
def test_subtensors_and_padding(hostsim, dims, perm, nb, alpha, elem):
    assert run(hostsim, dims, perm, elem, nb, alpha, slack=1.1)


def test_large_elements(hostsim):
    # 132 / 1324 with wide carried dims (strip staging), partition-like shapes
    assert run(hostsim, [700, 3, 600], [1, 3, 2], 2)
    assert run(hostsim, [64, 6, 5, 70], [1, 3, 2, 4], 4)
    assert run(hostsim, [1500, 2, 300], [1, 3, 2], 4)


@pytest.mark.parametrize("dims,perm,elem", [
    ([4, 20011, 8192, 2], [1, 3, 2, 4], 4), ([3001, 4096], [2, 1], 4), ([2048, 1536], [2, 1], 4),
    ([9973, 1024], [2, 1], 8), ([16, 3001, 1024, 25, 4], [5, 3, 1, 4, 2], 2), ([1000, 999], [2, 1], 2),
    ([60000, 300], [2, 1], 4), ([17, 30011, 37], [1, 3, 2], 4)])
def test_32bit_maps_agree_with_64bit(hostsim, dims, perm, elem):
    """The kernels use the 32-bit flavour of a map whenever every
    intermediate stays below 2^31; it must equal the 64-bit flavour."""
    import ctypes
    r = len(dims)
    hostsim.hs_check_fn32.restype = ctypes.c_long
    hostsim.hs_check_fn32.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                      ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_long]
    bad = hostsim.hs_check_fn32(r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm), elem, 1, 0.01, 0,
                                2000000)
    assert bad == 0


@pytest.mark.parametrize("dims,perm,elem", [
    ([4, 20011, 8192, 2], [1, 3, 2, 4], 4), ([3001, 4096], [2, 1], 4), ([2048, 1536], [2, 1], 4),
    ([1000, 999], [2, 1], 2), ([60000, 300], [2, 1], 4), ([64, 8000], [2, 1], 8), ([6, 4, 3401], [3, 2, 1], 2)])
def test_row_shuffle_inverse(hostsim, dims, perm, elem):
    """EITHOT's r2c::row_shuffle map inverts the row shuffle, so the executor
    may run a row pass as a gather or as a scatter."""
    import ctypes
    r = len(dims)
    hostsim.hs_check_inverse.restype = ctypes.c_long
    hostsim.hs_check_inverse.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                         ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_long]
    assert hostsim.hs_check_inverse(r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm), elem, 1, 0.01, 0,
                                    2000000) == 0


@pytest.mark.parametrize("dims,perm,elem", [
    ([4, 20011, 8192, 2], [1, 3, 2, 4], 4), ([3001, 4096], [2, 1], 4), ([2048, 1536], [2, 1], 4),
    ([3000, 2999], [2, 1], 2), ([60000, 300], [2, 1], 4), ([6000, 4000], [2, 1], 4), ([4000, 6000], [2, 1], 2),
    ([5, 700000], [2, 1], 8), ([60, 40, 3401], [3, 2, 1], 2), ([12, 9000, 900], [1, 3, 2], 4)])
def test_owner_maps_match_column_gathers(hostsim, dims, perm, elem):
    """Owner-computed column passes (each CTA writes whole output row pieces
    from the source rows it staged itself, plus a halo) write exactly what
    the column gathers of both the c2r and the r2c variant write.  Factoring
    is off, so 1- and 2-byte transposes keep their Catanzaro passes."""
    import ctypes
    r = len(dims)
    hostsim.hs_tune.argtypes = [ctypes.c_char_p, ctypes.c_int]
    hostsim.hs_check_owner.restype = ctypes.c_long
    hostsim.hs_check_owner.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                       ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_long,
                                       ctypes.POINTER(ctypes.c_long)]
    visited = ctypes.c_long()
    try:
        assert hostsim.hs_tune(b"factor", 0) == 0
        bad = hostsim.hs_check_owner(r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm), elem, 1, 0.01, 0,
                                     300000, ctypes.byref(visited))
    finally:
        hostsim.hs_tune(b"factor", 1)
    assert bad == 0
    assert visited.value >= 1


@pytest.mark.parametrize("dims,perm,elem", [([8000, 7500], [2, 1], 1), ([2, 7500, 8000], [1, 3, 2], 1)])
def test_factored_transposes(hostsim, dims, perm, elem):
    """With on-chip staging limited to one CTA (no clusters, no groups), long
    rows or columns would stage through global scratch; the lowering splits
    such transposes along a factor of R or C.  The whole pass list, run with
    the kernels' own maps, must still produce the oracle's permutation."""
    import ctypes
    hostsim.hs_tune.argtypes = [ctypes.c_char_p, ctypes.c_int]
    describe = ctypes.create_string_buffer(1 << 14)
    try:
        assert hostsim.hs_tune(b"max_cluster", 1) == 0 and hostsim.hs_tune(b"col_form", 1) == 0
        r = len(dims)
        hostsim.hs_describe(describe, len(describe), r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm),
                            elem, 1, ctypes.c_double(0.01), 0)
        passes = describe.value.decode().splitlines()
        assert len(passes) >= 3  # split into two transposes
        assert run(hostsim, dims, perm, elem)
    finally:
        hostsim.hs_tune(b"max_cluster", 16)
        hostsim.hs_tune(b"col_form", 0)


OWNER_SHAPES = [([4, 20011, 8192, 2], [1, 3, 2, 4], 4), ([3001, 4096], [2, 1], 4), ([4096, 3001], [2, 1], 4),
                ([20011, 819, 8], [2, 1, 3], 4), ([4000, 6000], [2, 1], 2), ([6000, 4000], [2, 1], 1),
                ([2048, 1536], [2, 1], 32), ([999, 5003], [2, 1], 3), ([60, 40, 3401], [3, 1, 2], 2),
                ([5, 70000], [2, 1], 8), ([70000, 5], [2, 1], 8), ([16, 3001, 1024, 256, 4], [5, 3, 1, 4, 2], 2),
                ([2, 300000], [2, 1], 1), ([777, 14000], [2, 1], 8), ([1000003, 3], [2, 1], 4)]


@pytest.mark.parametrize("form,per_sm,dbuf", [(0, 0, 1), (1, 0, 1), (1, 0, 0), (2, 1, 1), (2, 2, 0), (2, 3, 0),
                                              (2, 4, 0), (2, 2, 1)])
def test_owner_passes_fit_their_shared_memory(hostsim, form, per_sm, dbuf):
    """Every owner-computed column pass, with its row tables, fits the
    per-block limit, and a group pass fits the SM share it was planned for
    (else the cooperative launch would find fewer co-resident CTAs)."""
    import ctypes
    hostsim.hs_tune.argtypes = [ctypes.c_char_p, ctypes.c_int]
    hostsim.hs_check_owner_smem.restype = ctypes.c_long
    hostsim.hs_check_owner_smem.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                            ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int)]
    owners = 0
    try:
        for key, value in (("col_form", form), ("group_per_sm", per_sm), ("dbuf", dbuf)):
            assert hostsim.hs_tune(key.encode(), value) == 0
        for dims, perm, elem in OWNER_SHAPES:
            r = len(dims)
            n = ctypes.c_int(0)
            bad = hostsim.hs_check_owner_smem(r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm), elem, 1,
                                              ctypes.c_double(0.05), 0, ctypes.byref(n))
            assert bad == 0, (dims, perm, elem, hostsim.hs_last_error().decode())
            owners += n.value
    finally:
        hostsim.hs_tune(b"col_form", 0)
        hostsim.hs_tune(b"group_per_sm", 0)
        hostsim.hs_tune(b"dbuf", 1)
    assert owners > 0


@pytest.mark.parametrize("rank", [3, 4, 5])
def test_fewest_pass_plans_all_permutations(hostsim, rank):
    """The pass-minimising search (order 3): every permutation of ranks 3-5
    on shapes whose leading blocks reach the cycle-following and slab moves;
    the block permutation is simulated with the device's segment algorithm
    (heads saved, segments walked backwards)."""
    rng = random.Random(100 + rank)
    for perm in itertools.permutations(range(1, rank + 1)):
        for elem in (1, 2, 4, 8):
            dims = [rng.choice([2, 3, 5, 16, 33, 64, 96, 130]) for _ in range(rank)]
            while math.prod(dims) * elem > (3 << 20):
                dims[dims.index(max(dims))] //= 2
            assert run(hostsim, dims, list(perm), elem, order=3), (dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [
    ([16, 31, 64, 8, 4], [5, 3, 1, 4, 2], 2), ([64, 50, 60, 70], [1, 4, 3, 2], 4), ([20, 30, 40, 50, 6], [5, 4, 3, 2, 1], 2),
    ([8, 7, 6, 5, 4, 3], [6, 4, 2, 1, 3, 5], 4), ([512, 9, 11, 13], [1, 4, 2, 3], 8), ([2, 3, 5, 7, 11, 13, 2], [7, 1, 6, 2, 5, 3, 4], 1)])
def test_fewest_pass_plans_named_shapes(hostsim, dims, perm, elem):
    """Shapes whose searched plans use cycle-following block permutations
    (4-32 KB blocks), slab permutations of 2-6 axes and factor splits."""
    assert run(hostsim, dims, perm, elem, order=3)


@pytest.mark.parametrize("dims,elem", [([41125, 20, 2], 1), ([300001, 5], 1), ([130001, 6, 2], 2), ([70001, 4], 4),
                                       ([40000, 3], 8), ([20000, 5], 16)])
def test_column_band_slabs(hostsim, dims, elem):
    """Few-row matrices beyond two slabs per SM are transposed in one pass by
    a column-band cluster slab, also when a row is longer than one CTA's
    shared memory (the row-band form cannot stage it, and the matrix would
    otherwise take two or three Catanzaro passes); the pass list still
    produces the oracle's permutation."""
    r = len(dims)
    perm = [2, 1] + list(range(3, r + 1))
    describe = ctypes.create_string_buffer(1 << 14)
    hostsim.hs_describe(describe, len(describe), r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm),
                        elem, 1, ctypes.c_double(0.01), 0)
    passes = describe.value.decode().splitlines()
    assert len(passes) == 1 and passes[0].startswith("slab-colband"), passes
    assert run(hostsim, dims, perm, elem)


def test_column_bands_follow_their_knob(hostsim):
    """slab_colband = 0 keeps the row-band cluster slab for few-row matrices
    whose rows fit one CTA, and the Catanzaro passes for rows that do not."""
    hostsim.hs_tune.argtypes = [ctypes.c_char_p, ctypes.c_int]
    describe = ctypes.create_string_buffer(1 << 14)

    def kinds(dims):
        r = len(dims)
        hostsim.hs_describe(describe, len(describe), r, (ctypes.c_int64 * r)(*dims),
                            (ctypes.c_int * r)(*([2, 1] + list(range(3, r + 1)))), 1, 1, ctypes.c_double(0.01), 0)
        return [line.split()[0] for line in describe.value.decode().splitlines()]

    try:
        assert kinds([41125, 20, 2]) == ["slab-colband"]
        assert kinds([300001, 5]) == ["slab-colband"]
        assert hostsim.hs_tune(b"slab_colband", 0) == 0
        assert kinds([41125, 20, 2]) == ["slab-cluster"]
        assert "slab-colband" not in kinds([300001, 5])
    finally:
        hostsim.hs_tune(b"slab_colband", 256)


@pytest.mark.parametrize("dims,perm,elem", [([1784616, 28], [2, 1], 1), ([2003328, 8], [2, 1], 1),
                                            ([4096, 3001], [2, 1], 2), ([6000, 4000], [2, 1], 1)])
def test_narrow_transposes_split_into_wider_granules(hostsim, dims, perm, elem):
    """1- and 2-byte transposes whose Catanzaro passes would move 1- or 2-byte
    units are split along a factor of R or C into a transpose of wider
    granules and small transposes (factor=1); factor=0 keeps the direct
    passes.  Both pass lists produce the oracle's permutation."""
    hostsim.hs_tune.argtypes = [ctypes.c_char_p, ctypes.c_int]
    describe = ctypes.create_string_buffer(1 << 14)
    r = len(dims)

    def passes():
        hostsim.hs_describe(describe, len(describe), r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm),
                            elem, 1, ctypes.c_double(0.01), 0)
        return describe.value.decode().splitlines()

    def catanzaro_elems(ps):
        return [int(p.split("E=")[1].split()[0]) for p in ps if p.startswith(("c2r-", "r2c-"))]

    factored = passes()
    assert all(e % 4 == 0 for e in catanzaro_elems(factored)), factored  # no pass of narrow units
    assert run(hostsim, dims, perm, elem)
    try:
        assert hostsim.hs_tune(b"factor", 0) == 0
        direct = passes()
        assert catanzaro_elems(direct) and all(e == elem for e in catanzaro_elems(direct)), direct
        assert run(hostsim, dims, perm, elem)
    finally:
        hostsim.hs_tune(b"factor", 1)


@pytest.mark.parametrize("order", [0, 3])
def test_mixed_tensors_through_the_kernel_maps(hostsim, order):
    """Tensors drawn like the batched workload's mix (rank 3-6, 1-8 byte
    elements, random permutations; 4 KB-8 MB here), planned under the
    reference's series (0) and the fewest-pass search (3), with column bands,
    the factoring of narrow passes and every other lowering in play: the pass
    lists, applied on the CPU with the kernels' index maps, reproduce the
    oracle's permutation."""
    import bench
    for dims, perm, elem in bench.mixed_tensors(150, 11, 4096, 8 << 20, 3, 6):
        assert run(hostsim, dims, perm, elem, order=order), (dims, perm, elem, order)

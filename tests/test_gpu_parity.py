"""Parity of the sm_103a path with the oracle, through the C ABI
(eithot_transpose_ex via eithot_gb300.transpose_ptr) on device memory.
Bit-exact: every byte of the output equals the oracle's out-of-place
permutation of the same seeded input."""
import ctypes
import itertools
import math
import random

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev():
    return torch.device("cuda:0")


def run_case(E, dims, perm, elem, nb=1, alpha=0.01, order=0, slack=1.0, seed=1, offset=0, stream=None):
    n = math.prod(dims)
    host = oracle.fill_hash(n, elem, seed)
    cap = int(n * elem * slack) + 256
    buf = torch.zeros(cap + offset, dtype=torch.uint8, device=dev())
    buf[offset:offset + n * elem] = torch.from_numpy(host).to(dev())
    s = stream or torch.cuda.current_stream()
    E.transpose_ptr(buf.data_ptr() + offset, cap, dims, perm, elem, nb, alpha, order, s.cuda_stream)
    s.synchronize()
    assert E.index_faults() == 0
    assert E.sync_timeouts() == 0
    got = buf[offset:offset + n * elem].cpu().numpy()
    want = oracle.permute(host, dims, perm, elem)
    if not np.array_equal(got, want):
        bad = np.nonzero(got != want)[0]
        raise AssertionError("mismatch %s perm %s elem %d: %d bad bytes, first at %d"
                             % (dims, perm, elem, bad.size, bad[0]))
    return E.last_stats()


def test_iota_3001x4096_int32(E):
    """3001 x 4096 int32 iota, perm (2 1), nb 1, alpha 0.01: byte-exact vs the
    oracle and the reference's verify_inplace known answer."""
    dims, perm = [3001, 4096], [2, 1]
    n = 3001 * 4096
    a = np.arange(n, dtype=np.int32)
    t = torch.from_numpy(a.copy()).to(dev())
    E.transpose(t, dims, perm, 1, 0.01)
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    want = oracle.permute(a.view(np.uint8), dims, perm, 4).view(np.int32)
    assert np.array_equal(got, want)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, n, size=4000):
        assert got[oracle.dest_index(dims, perm, int(i))] == i


@pytest.mark.parametrize("rank", [2, 3, 4])
@pytest.mark.parametrize("elem", [1, 2, 4, 8])
def test_all_permutations_small(E, rank, elem):
    rng = random.Random(rank * 10 + elem)
    for perm in itertools.permutations(range(1, rank + 1)):
        dims = [rng.choice([1, 2, 3, 5, 7, 8, 16, 33, 64]) for _ in range(rank)]
        run_case(E, dims, list(perm), elem, seed=rng.randrange(1 << 30))


@pytest.mark.parametrize("rank", [5, 6])
def test_random_high_rank(E, rank):
    rng = random.Random(rank)
    for _ in range(40):
        perm = list(range(1, rank + 1))
        rng.shuffle(perm)
        dims = [rng.choice([2, 3, 4, 5, 7, 9, 12]) for _ in range(rank)]
        run_case(E, dims, perm, rng.choice([1, 2, 4, 8]), order=rng.choice([0, 1, 2]))


@pytest.mark.parametrize("R,C,elem", [(3001, 4096, 4), (4096, 3001, 4), (2048, 1536, 4), (1000, 999, 2),
                                      (64, 80000, 4), (80000, 64, 4), (5000, 60, 16), (40, 2000, 24),
                                      (700, 1400, 1), (9973, 1024, 8)])
def test_catanzaro_2d(E, R, C, elem):
    run_case(E, [C, R], [2, 1], elem)


@pytest.fixture
def tuned(E):
    keys = ("variant", "col_owner", "col_chunk", "max_cluster", "dbuf", "col_form", "row_prefetch", "row_block",
            "slab_pack", "slab_cluster", "factor", "sync_relaxed", "group_per_sm", "col_bulk", "narrow_words",
            "slab_colband")
    saved = {k: E.tune_get(k) for k in keys}

    def set_(**kw):
        for k, v in kw.items():
            E.tune_set(k, v)
    yield set_
    for k, v in saved.items():
        E.tune_set(k, v)


@pytest.mark.parametrize("R,C,elem", [(3001, 4096, 4), (6000, 4000, 2), (4000, 6000, 1), (5, 70000, 8),
                                      (70000, 5, 8), (5000, 60, 16), (40, 2000, 24), (1000, 999, 1),
                                      (2048, 1536, 32)])
@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("form", ["gather", "cluster", "group"])
def test_column_kernels_all_forms(E, tuned, R, C, elem, variant, form):
    """c2r and r2c, with column gathers through distributed shared memory and
    with owner-computed column passes synchronised by a cluster or by a
    group of co-resident CTAs, on shapes with gcd 1 and gcd > 1
    (rotations), rows fewer than a tile's halo and wide elements."""
    # factoring off: 1- and 2-byte transposes keep their Catanzaro passes
    tuned(variant=variant, col_owner=0 if form == "gather" else 1, factor=0,
          col_form={"gather": 0, "cluster": 1, "group": 2}[form])
    run_case(E, [C, R], [2, 1], elem)


@pytest.mark.parametrize("chunk,max_cluster,dbuf,form", [(32, 16, 1, 1), (64, 8, 1, 1), (128, 4, 0, 1), (64, 2, 1, 1),
                                                         (32, 1, 0, 1), (128, 16, 1, 2), (256, 16, 1, 2),
                                                         (512, 16, 0, 2), (256, 8, 1, 0), (512, 16, 1, 0)])
def test_column_tilings(E, tuned, chunk, max_cluster, dbuf, form):
    """Row-piece widths, cluster sizes, CTA groups and single/double
    buffering of the column passes (the autotuner's search space)."""
    tuned(col_chunk=chunk, max_cluster=max_cluster, dbuf=dbuf, col_form=form, factor=0)
    for variant in (1, 2):
        E.tune_set("variant", variant)
        run_case(E, [4096, 3001], [2, 1], 4)
        run_case(E, [4, 20011, 819, 2], [1, 3, 2, 4], 4)
        run_case(E, [4000, 6000], [2, 1], 2)


@pytest.mark.parametrize("relaxed", [0, 1])
@pytest.mark.parametrize("per_sm", [1, 2, 3])
def test_group_arrivals_and_residency(E, tuned, relaxed, per_sm):
    """Group column passes with release and with relaxed arrivals, at one to
    three CTAs per SM (row tables in shared memory sized for each), c2r and
    r2c, gcd 1 and gcd > 1, 1- to 32-byte and 3-byte elements."""
    tuned(col_form=2, dbuf=0, sync_relaxed=relaxed, group_per_sm=per_sm, factor=0)
    for variant in (1, 2):
        E.tune_set("variant", variant)
        run_case(E, [4096, 3001], [2, 1], 4)
        run_case(E, [4, 20011, 819, 2], [1, 3, 2, 4], 4)
        run_case(E, [6000, 4000], [2, 1], 1)
        run_case(E, [2048, 1536], [2, 1], 32)
        run_case(E, [999, 5003], [2, 1], 3)


@pytest.mark.parametrize("per_sm", [1, 2])
def test_group_pass_with_bulk_copies(E, tuned, per_sm):
    """Double-buffered group column passes whose row pieces are staged by
    bulk copies completing on mbarriers (whole 16-byte-aligned elements
    moved in 16-byte units), c2r and r2c, 16-, 4- and 32-byte elements;
    shapes whose pieces do not qualify fall back to the cp.async form."""
    tuned(col_form=2, dbuf=1, col_bulk=1, group_per_sm=per_sm)
    for variant in (1, 2):
        E.tune_set("variant", variant)
        run_case(E, [4, 20011, 819, 2], [1, 3, 2, 4], 4)
        run_case(E, [4096, 3001], [2, 1], 4)
        run_case(E, [2048, 1536], [2, 1], 32)
        run_case(E, [999, 5003], [2, 1], 3)


@pytest.mark.parametrize("dims,perm,elem", [([4, 3001, 8192, 1], [1, 3, 2, 4], 4), ([2, 3001, 16384, 1], [1, 3, 2, 4], 4),
                                            ([3001, 32768], [2, 1], 4), ([3001, 30000], [2, 1], 4),
                                            ([777, 14000], [2, 1], 8), ([4, 4001, 7000, 2], [1, 3, 2, 4], 4)])
@pytest.mark.parametrize("prefetch", [0, 1])
def test_row_prefetch(E, tuned, dims, perm, elem, prefetch):
    """Rows of 110-128 KB (one CTA per SM) with and without the register
    prefetch of the next row, including rows that leave some threads'
    last units empty."""
    tuned(variant=2, row_prefetch=prefetch, factor=0)
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [([2, 300000], [2, 1], 1), ([3, 200001], [2, 1], 2), ([7, 70000], [2, 1], 4),
                                            ([2, 5, 100000], [3, 1, 2], 1), ([13, 40000], [2, 1], 8),
                                            ([300000, 2], [2, 1], 1), ([100, 3000], [2, 1], 2)])
@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("block", [0, 1])
def test_tall_skinny_rows_in_blocks(E, tuned, dims, perm, elem, variant, block):
    """Matrices of a few columns (rows of a few bytes): row passes staged as
    blocks of consecutive rows, and the one-row-per-item form."""
    tuned(variant=variant, row_block=block, factor=0)
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm", [([3, 5, 100000], [2, 1, 3]), ([2, 2, 300001], [2, 1, 3]),
                                       ([7, 3, 4, 5000], [3, 1, 2, 4]), ([5, 9, 1000], [3, 2, 1]),
                                       ([16, 8, 5000], [2, 1, 3]), ([1024, 4, 300], [2, 1, 3])])
@pytest.mark.parametrize("elem", [1, 2, 4, 8])
@pytest.mark.parametrize("pack", [0, 1])
def test_many_small_matrices(E, tuned, dims, perm, elem, pack):
    """Batches of tiny matrices transposed as blocks of consecutive
    matrices per CTA, and one matrix per CTA item."""
    tuned(slab_pack=pack)
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [([3000, 3, 200], [1, 3, 2], 4), ([5000, 16, 2], [1, 3, 2], 2),
                                            ([20000, 5, 7], [1, 3, 2], 1), ([4001, 3, 50], [1, 3, 2], 3),
                                            ([2048, 2, 3, 40], [1, 4, 3, 2], 8), ([100000, 3, 2], [1, 3, 2], 4)])
def test_few_very_wide_elements(E, dims, perm, elem):
    """Elements of many KB (a permutation that keeps a large leading block
    together): rows and slabs staged in strips of up to 32 KB, with a
    shorter last strip."""
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [([16, 4096, 50], [2, 1, 3], 2), ([300, 700], [2, 1], 4),
                                            ([3001, 200], [2, 1], 1), ([3001, 201], [2, 1], 1),
                                            ([1000, 150], [2, 1], 8), ([999, 130], [2, 1], 6),
                                            ([5, 600, 300], [1, 3, 2], 2), ([64, 2001, 3], [2, 1, 3], 2)])
@pytest.mark.parametrize("on", [0, 1])
def test_cluster_slabs(E, tuned, dims, perm, elem, on):
    """Matrices of 110 KB - 1.7 MB transposed in one owner-computed pass
    over a thread-block cluster (packed 4-byte stores for 1- and 2-byte
    elements, odd row counts, elements of several units), against the
    multi-pass decomposition."""
    tuned(slab_cluster=on)
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [([8000, 7500], [2, 1], 1), ([2, 7500, 8000], [1, 3, 2], 1),
                                            ([7000, 3000], [2, 1], 4), ([3, 5000, 6001], [1, 3, 2], 2)])
@pytest.mark.parametrize("factor", [0, 1])
def test_factored_transposes_on_gpu(E, tuned, dims, perm, elem, factor):
    """On-chip staging limited to single CTAs (no clusters, no groups):
    transposes whose passes would stage through global scratch are split
    along a factor of R or C (factor=1) or staged (factor=0)."""
    tuned(max_cluster=1, col_form=1, factor=factor)
    run_case(E, dims, perm, elem)


@pytest.mark.parametrize("dims,perm,elem", [
    ([5], [1], 4), ([1, 1, 1], [3, 2, 1], 2), ([7, 1, 5], [3, 2, 1], 1), ([1, 300000], [2, 1], 4),
    ([300000, 1], [2, 1], 8), ([33, 17, 9], [1, 2, 3], 4), ([3, 2, 2, 3, 2, 2, 3, 2], [8, 6, 4, 2, 7, 5, 3, 1], 2),
    ([9, 7, 5], [2, 3, 1], 33), ([4, 3, 5], [3, 1, 2], 64), ([2, 2], [2, 1], 1)])
def test_edge_shapes(E, dims, perm, elem):
    """Rank 1, size-1 axes, identity permutations, rank 8, element sizes of
    33 and 64 bytes, the smallest matrix."""
    run_case(E, dims, perm, elem)


def test_bounded_wait_gives_up(E):
    """A group-barrier wait that nothing releases gives up after its bound,
    is counted, and leaves the context usable."""
    assert E.selftest_wait() == 1
    assert E.sync_timeouts() == 0
    run_case(E, [4096, 3001], [2, 1], 4)


@pytest.mark.parametrize("dims,perm", [([60000, 300], [2, 1]), ([300, 60000], [2, 1]),
                                       ([4, 20011, 819, 2], [1, 3, 2, 4]), ([17, 30011, 37], [1, 3, 2]),
                                       ([3, 50000, 41], [3, 2, 1])])
def test_rows_and_columns_beyond_shared_memory(E, dims, perm):
    run_case(E, dims, perm, 4)


@pytest.mark.parametrize("dims,perm,nb,alpha", [
    ([7248, 50], [2, 1], 4, 0.02), ([3301, 7, 5], [3, 1, 2], 3, 0.01), ([5, 3302, 6], [2, 3, 1], 4, 0.01),
    ([6, 4, 3401], [3, 2, 1], 2, 0.01), ([40, 3203, 3], [1, 3, 2], 8, 0.01), ([3, 3301, 2, 5], [4, 2, 1, 3], 16, 0.01)])
@pytest.mark.parametrize("elem", [2, 4, 8])
def test_subtensors_and_padding(E, dims, perm, nb, alpha, elem):
    run_case(E, dims, perm, elem, nb, alpha, slack=1.1)


@pytest.mark.parametrize("elem", [2, 4])
def test_padding_blocks_larger_than_scratch(E, elem):
    """Sub-tensors with padding where each padded block is far larger than
    the alpha-bounded scratch: blocks move through scratch in pieces."""
    dims, perm = [4, 20011, 819, 2], [1, 3, 2, 4]
    ws = E.workspace_size(dims, perm, elem, 2, 0.01)
    assert ws <= 0.01 * math.prod(dims) * elem + (4 << 20)
    st = run_case(E, dims, perm, elem, 2, 0.01, slack=1.01)
    assert st["workspace_bytes"] == ws


def test_wide_elements(E):
    run_case(E, [700, 3, 600], [1, 3, 2], 2)
    run_case(E, [64, 6, 5, 70], [1, 3, 2, 4], 4)
    run_case(E, [1500, 2, 300], [1, 3, 2], 4)
    run_case(E, [16384, 25, 4, 3], [1, 3, 2, 4], 2)


@pytest.mark.parametrize("dims,elem", [([1001, 300], 1), ([41125, 20], 1), ([17, 12955], 1), ([777, 333], 2),
                                       ([5003, 61], 1), ([301, 1500], 2)])
@pytest.mark.parametrize("offset", [0, 1, 3])
def test_cluster_slabs_of_narrow_odd_rows(E, dims, elem, offset):
    """Matrices of 1- and 2-byte elements beyond one CTA's shared memory (one
    cluster-slab pass) whose rows are not whole 4-byte words: each CTA's band
    is staged from aligned words around it (bytes outside the band dropped),
    at bases off word boundaries; 2D transposes under the reference's series
    and the fewest-pass plans."""
    for order in (0, 3):
        run_case(E, dims, [2, 1], elem, order=order, offset=offset * elem % 4 if elem == 2 else offset)


@pytest.mark.parametrize("colband", [4096, 0])
@pytest.mark.parametrize("offset", [0, 4, 8, 1])
def test_cluster_slabs_in_column_bands(E, tuned, colband, offset):
    """Matrices with few rows beyond one CTA's shared memory: each CTA of the
    cluster stages a band of columns of every row and writes its contiguous
    range of the output (knob slab_colband=4096: wherever a band fits; 0 keeps
    row bands, or Catanzaro passes for rows longer than a CTA's shared
    memory), one to three matrices, 1- to 16-byte elements, bases on 16-, 8-,
    4- and 1-byte boundaries, odd matrix sizes (ranges off the store width:
    the any-alignment write)."""
    tuned(slab_colband=colband)
    for dims, elem in [([41125, 20, 3], 1), ([20011, 8, 2], 2), ([12000, 12, 1], 4), ([9000, 6, 2], 8),
                       ([5000, 4, 2], 16), ([70001, 9, 1], 1), ([30001, 5, 3], 2), ([5003, 61, 3], 1),
                       ([300001, 5, 2], 1), ([130001, 6, 2], 2), ([70001, 4, 1], 4), ([40000, 3, 2], 8),
                       ([20000, 5, 1], 16)]:
        if offset % elem and offset < elem:
            continue
        run_case(E, dims, [2, 1, 3], elem, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 4, 1])
def test_column_bands_in_byte_tiles(E, tuned, words, offset):
    """1-byte column bands with a multiple of 4 rows: 4 x 4 byte tiles
    transposed in registers (knob narrow_words=1) or runs of stores (0), the
    last columns of a band byte by byte; one to three matrices, bases on and
    off word boundaries (off: the any-alignment write)."""
    tuned(narrow_words=words)
    for dims in ([50001, 16, 2], [70000, 12, 1], [30003, 8, 3], [41125, 20, 3], [20001, 36, 2]):
        run_case(E, dims, [2, 1, 3], 1, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 4, 1])
def test_two_d_byte_slabs_in_tiles(E, tuned, words, offset):
    """2D transposes of 1-byte elements through the slab run kernel (one CTA
    per slab, and the fewest-pass plan's slab permutation of 160-byte slabs)
    with a multiple of 4 rows: 4 x 4 byte tiles (knob narrow_words=1) or runs
    of stores (0); odd column counts; bases off word boundaries take the
    runs."""
    tuned(narrow_words=words)
    for dims, order in [([1000, 100, 20], 0), ([999, 64, 30], 0), ([1001, 36, 20], 0), ([20, 8, 4000], 3)]:
        run_case(E, dims, [2, 1, 3], 1, order=order, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_slabs_of_odd_wide_elements(E, tuned, words, offset):
    """One-CTA slabs of wide elements whose size is odd or 2 mod 4 (1- and
    2-byte units), whole or in strips of 128-byte multiples: every piece read
    and written in the aligned words around it, its end bytes one by one
    (knob narrow_words=1), or unit by unit (0); bases off word boundaries,
    one to three matrices."""
    tuned(narrow_words=words)
    # the first axis stays in place: elements of its length (x elem) bytes
    for dims, elem in [([74359, 24, 28], 1), ([22701, 230, 8], 1), ([5193, 272, 25], 2), ([4095, 17, 5, 3], 1),
                       ([17, 300, 20], 1), ([1001, 7, 9, 2], 1)]:
        perm = [1, 3, 2] + list(range(4, len(dims) + 1))
        run_case(E, dims, perm, elem, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_cluster_slabs_of_wide_odd_elements(E, tuned, words, offset):
    """Cluster slabs of 17-1001-byte elements whose size is odd or 2 mod 4:
    each output row's segment written by one warp as the aligned words inside
    it, gathered byte by byte (knob narrow_words=1), or unit by unit (0)."""
    tuned(narrow_words=words)
    for dims, perm, elem in [([707, 61, 51, 3], [1, 3, 2, 4], 1), ([17, 7, 5572, 3], [1, 3, 2, 4], 1),
                             ([19, 3, 8769, 2], [1, 3, 2, 4], 1), ([1001, 40, 30], [1, 3, 2], 1),
                             ([35, 60, 70], [1, 3, 2], 1), ([9, 100, 90], [1, 3, 2], 2)]:
        run_case(E, dims, perm, elem, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_flat_narrow_slabs(E, tuned, words, offset):
    """One-CTA slabs of whole 1-, 3- and 2-mod-4-byte elements at any
    alignment (odd matrix sizes in a batch: no packed stores): the matrix read
    in aligned 16-byte chunks, the output written as aligned words gathered
    byte by byte (knob narrow_words=1), or unit by unit (0)."""
    tuned(narrow_words=words)
    for dims, perm, elem in [([31535, 3, 20], [2, 1, 3], 1), ([10023, 7, 30], [2, 1, 3], 1), ([341, 67, 50], [2, 1, 3], 1),
                             ([3, 5001, 7, 4], [1, 3, 2, 4], 1), ([3, 301, 77, 5], [1, 3, 2, 4], 1),
                             ([3, 1001, 9, 2], [1, 3, 2, 4], 2)]:
        run_case(E, dims, perm, elem, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("offset", [0, 1, 2, 3])
def test_slab_permutations_of_odd_elements(E, tuned, words, offset):
    """Slab permutations (fewest-pass plans) of elements of 9-351 bytes whose
    size is odd or 2 mod 4: pieces read in aligned 16-byte chunks and written
    as the aligned words inside them (knob narrow_words=1) or unit by unit
    (0); whole elements and strips, one to three slabs, bases off word
    boundaries."""
    tuned(narrow_words=words)
    for dims, perm, elem in [([9, 33, 3, 3, 21, 4], [1, 4, 6, 3, 5, 2], 1), ([35, 8, 10, 47, 3], [1, 4, 3, 2, 5], 1),
                             ([307, 3, 116, 2], [1, 4, 3, 2], 1), ([351, 14, 26, 2, 2], [1, 5, 3, 2, 4], 1),
                             ([11, 19, 13, 4, 5, 3], [1, 6, 4, 2, 5, 3], 1), ([65, 18, 6, 3, 8], [1, 3, 2, 5, 4], 1),
                             ([5, 7, 9, 11, 13], [1, 5, 4, 3, 2], 3), ([9, 33, 3, 3, 21, 4], [1, 4, 6, 3, 5, 2], 2)]:
        run_case(E, dims, perm, elem, order=3, offset=offset)


@pytest.mark.parametrize("words", [1, 0])
@pytest.mark.parametrize("factor", [0, 1])
def test_narrow_units_staged_from_words(E, tuned, words, factor):
    """1- and 2-byte elements whose rows are not whole 4-byte words, through
    Catanzaro row and column passes (factor=0), or split into transposes of
    wider granules (factor=1), row blocks, packed and cluster slabs:
    contiguous ranges staged from the aligned words around them (knob
    narrow_words=1) or unit by unit (0), at bases off word boundaries."""
    tuned(narrow_words=words, factor=factor)
    for dims, perm, elem, offset in [([5003, 999], [2, 1], 1, 1), ([2001, 513], [2, 1], 2, 2), ([7, 130001], [2, 1], 1, 3),
                                     ([130001, 7], [2, 1], 1, 0), ([33, 1000, 31], [3, 1, 2], 1, 1),
                                     ([3, 40001, 5], [2, 3, 1], 2, 2), ([301, 77, 13], [2, 1, 3], 1, 3),
                                     ([9, 5, 7, 11], [4, 3, 2, 1], 1, 1)]:
        run_case(E, dims, perm, elem, offset=offset)


def test_unaligned_base_and_odd_elements(E):
    run_case(E, [33, 17, 9], [2, 3, 1], 4, offset=4)
    run_case(E, [33, 17, 9], [3, 1, 2], 2, offset=2)
    run_case(E, [31, 1000, 3], [1, 3, 2], 1, offset=1)
    run_case(E, [5, 701, 3], [3, 2, 1], 3)
    run_case(E, [2, 3001, 40], [1, 3, 2], 6)


def test_side_stream(E):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        run_case(E, [3001, 128, 3], [3, 1, 2], 4, stream=s)


def test_reorder_types_agree(E):
    for order in (0, 1, 2):
        run_case(E, [12, 5, 40, 7, 3], [5, 3, 1, 4, 2], 2, order=order)


def test_capacity_is_enforced(E):
    dims, perm = [3301, 7, 5], [3, 1, 2]
    n = math.prod(dims)
    buf = torch.zeros(n * 4, dtype=torch.uint8, device=dev())
    with pytest.raises(E.EithotError) as ei:
        E.transpose_ptr(buf.data_ptr(), n * 4, dims, perm, 4, 3, 0.01)
    assert ei.value.code == E.EINVAL


def test_reference_signature_shim(E):
    """inplace::transpose(void*, int source, int rank, void* dim, void* perm
    (0-based), size_t, int nb, double alpha) — the reference's C++ entry."""
    fn = getattr(E.lib, "_ZN7inplace9transposeEPviiS0_S0_mid")
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_size_t, ctypes.c_int, ctypes.c_double]
    dims, perm = [300, 41, 7], [2, 3, 1]
    n = math.prod(dims)
    host = oracle.fill_hash(n, 4, 3)
    src = 5  # the reference's `source` element offset
    t = torch.zeros(n + src, dtype=torch.int32, device=dev())
    t[src:] = torch.from_numpy(host.view(np.int32)).to(dev())
    d = (ctypes.c_int * 3)(*dims)
    p = (ctypes.c_int * 3)(*[x - 1 for x in perm])
    fn(ctypes.c_void_p(t.data_ptr()), src, 3, d, p, 4, 1, 0.01)
    got = t[src:].cpu().numpy().view(np.uint8)
    assert np.array_equal(got, oracle.permute(host, dims, perm, 4))


@pytest.mark.slow
def test_4x20011x8192x2_int32_full_size(E):
    """(4, 20011, 8192, 2) int32, perm (1 3 2 4), nb/alpha from the
    estimator, extra device memory within alpha * bytes."""
    dims, perm = [4, 20011, 8192, 2], [1, 3, 2, 4]
    nb, alpha, _ = E.estimate(dims, perm, 4)
    E.set_profiling(True)  # fills the free-memory fields of the stats
    try:
        st = run_case(E, dims, perm, 4, nb, alpha, seed=0xE17407)
    finally:
        E.set_profiling(False)
        E.profile_reset()
    n = math.prod(dims)
    assert st["free_before"] > 0
    assert st["workspace_bytes"] <= alpha * n * 4 * 1.0001
    assert st["free_before"] - st["free_after_alloc"] <= alpha * n * 4 * 1.05 + (64 << 20)


def test_device_hash_fill_and_check(E):
    """The device content generator writes exactly the oracle's counter-hash
    bytes; the device permutation check accepts the transposed tensor and
    pinpoints a planted corruption."""
    dims, perm = [37, 64, 5, 3], [3, 1, 4, 2]
    n = math.prod(dims)
    for elem in (1, 2, 4, 8, 6):
        buf = torch.zeros(n * elem + 64, dtype=torch.uint8, device=dev())
        E.fill_hash_ptr(buf.data_ptr(), n, elem, 0x1234 + elem)
        torch.cuda.synchronize()
        host = oracle.fill_hash(n, elem, 0x1234 + elem)
        assert np.array_equal(buf[: n * elem].cpu().numpy(), host)
        assert E.check_hash_ptr(buf.data_ptr(), dims, [1, 2, 3, 4], elem, 0x1234 + elem) == (0, -1)
        E.transpose_ptr(buf.data_ptr(), n * elem + 64, dims, perm, elem)
        torch.cuda.synchronize()
        assert np.array_equal(buf[: n * elem].cpu().numpy(), oracle.permute(host, dims, perm, elem))
        assert E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, 0x1234 + elem) == (0, -1)
        buf[777 * elem] ^= 1
        assert E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, 0x1234 + elem) == (1, 777)


@pytest.mark.slow
def test_16x3001x1024x256x4_uint16_full_size(E):
    """(16, 3001, 1024, 256, 4) uint16 (100.7 GB), perm (5 3 1 4 2), nb/alpha
    from the estimator at alpha 0.05: the tensor no 32-bit planner can
    describe.  Every output element is checked on the device against the
    counter hash of the source index its coordinates name; a seeded sample
    is checked on the host with the oracle's index map."""
    dims, perm, elem, seed = [16, 3001, 1024, 256, 4], [5, 3, 1, 4, 2], 2, 0xC3
    n = math.prod(dims)
    nb, alpha, _ = E.estimate(dims, perm, elem, 1, 0.05)
    plan = E.plan(dims, perm, nb, alpha)
    cap = plan.padded_volume * elem
    free, _ = torch.cuda.mem_get_info()
    if free < cap * 1.08:
        pytest.skip("needs %.0f GB of free device memory" % (cap * 1.08 / 1e9))
    buf = torch.empty(cap, dtype=torch.uint8, device=dev())
    E.fill_hash_ptr(buf.data_ptr(), n, elem, seed)
    E.transpose_ptr(buf.data_ptr(), cap, dims, perm, elem, nb, alpha)
    torch.cuda.synchronize()
    st = E.last_stats()
    assert E.index_faults() == 0 and E.sync_timeouts() == 0
    assert st["workspace_bytes"] <= 0.05 * n * elem
    assert E.check_hash_ptr(buf.data_ptr(), dims, perm, elem, seed) == (0, -1)
    rng = np.random.default_rng(3)
    src = rng.integers(0, n, size=2000)
    dst = torch.tensor([oracle.dest_index(dims, perm, int(s)) for s in src], device=dev())
    got = buf[: n * elem].view(torch.int16)[dst].cpu().numpy().view(np.uint16)
    want = np.array([oracle.hash_value(seed, int(s)) & 0xFFFF for s in src], dtype=np.uint16)
    assert np.array_equal(got, want)

"""Per-shape knobs (eithot_tune_shape_*) and the autotuner built on them."""
import json
import math

import numpy as np
import pytest

import oracle


def test_shape_knobs_apply_to_that_shape_only(E):
    d, p = [4, 20011, 8192, 2], [1, 3, 2, 4]
    E.tune_shape_clear()
    base = E.workspace_size(d, p, 4)
    other = E.workspace_size([3001, 4096], [2, 1], 4)
    E.tune_shape_set(d, p, 4, "col_form", 1)    # clusters only: no group barrier counters
    assert E.tune_shape_count() == 1
    assert E.workspace_size(d, p, 4) != base
    assert E.workspace_size([3001, 4096], [2, 1], 4) == other
    assert E.workspace_size(d, p, 2) == E.workspace_size(d, p, 2)  # other element size: untouched entry
    with pytest.raises(E.EithotError):
        E.tune_shape_set(d, p, 4, "no_such_knob", 1)
    E.tune_shape_clear()
    assert E.tune_shape_count() == 0 and E.workspace_size(d, p, 4) == base


def test_saved_results_load_back(E, tmp_path):
    from eithot_gb300 import autotune
    E.tune_shape_clear()
    res = {autotune.key([300, 700], [2, 1], 4): {"config": {"variant": 2}, "ms": 0.1, "tried": 3},
           autotune.key([5, 6, 7], [3, 1, 2], 1): {"config": {}, "ms": 0.01, "tried": 1}}
    path = tmp_path / "tuned.json"
    autotune.save(str(path), res)
    assert json.load(open(path)) == res
    assert autotune.load(str(path)) == 2
    assert E.tune_shape_count() == 2
    E.tune_shape_clear()


@pytest.mark.gpu
def test_autotune_keeps_results_exact(E):
    torch = pytest.importorskip("torch")
    from eithot_gb300 import autotune
    E.tune_shape_clear()
    dims, perm, elem = [3001, 409], [2, 1], 4
    r = autotune.autotune(dims, perm, elem, candidates=[{}, {"variant": 1}, {"variant": 2}, {"slab_cluster": 0}],
                          reps=2)
    assert r["tried"] == 4 and r["ms"] > 0 and E.tune_shape_count() == 1
    n = math.prod(dims)
    host = oracle.fill_hash(n, elem, 31)
    t = torch.from_numpy(host.copy()).cuda()
    E.transpose_ptr(t.data_ptr(), t.numel(), dims, perm, elem)
    torch.cuda.synchronize()
    assert np.array_equal(t.cpu().numpy(), oracle.permute(host, dims, perm, elem))
    E.tune_shape_clear()


KNOB_VALUES = {"dbuf": 0, "max_cluster": 8, "variant": 1, "col_batch": 8, "col_chunk": 256, "col_owner": 0,
               "col_form": 1, "row_prefetch": 0, "row_block": 0, "slab_pack": 0, "slab_cluster": 0, "factor": 0,
               "sync_sleep_ns": 32, "sync_spin_limit": 4096, "sync_relaxed": 0, "group_per_sm": 2, "l2_prefetch": 1, "col_bulk": 1, "cycle_moves": 0, "slab_perm": 2, "slab_runs": 0, "slab_prefetch": 0, "slab2d_runs": 2, "row_solo_kb": 64, "batch_graph": 0, "batch_queue": 0, "batch_lanes": 8, "narrow_words": 0, "slab_colband": 0}


def test_every_knob_round_trips(E):
    """Every process-wide knob the header documents can be read, set to a
    valid value, read back and restored (host only)."""
    for key, value in KNOB_VALUES.items():
        old = E.tune_get(key)
        try:
            E.tune_set(key, value)
            assert E.tune_get(key) == value, key
        finally:
            E.tune_set(key, old)
        assert E.tune_get(key) == old


@pytest.mark.parametrize("key,value", [("max_cluster", 3), ("variant", 3), ("col_form", 5), ("group_per_sm", 7),
                                       ("sync_sleep_ns", -1), ("sync_spin_limit", -1), ("slab_perm", 3), ("slab_runs", 3), ("slab2d_runs", 3), ("cycle_moves", 3), ("row_solo_kb", 8), ("slab_colband", 5000), ("batch_lanes", 0), ("col_chunk", 100), ("no_such_knob", 1)])
def test_invalid_knob_values_are_refused(E, key, value):
    old = E.tune_get(key) if key != "no_such_knob" else None
    with pytest.raises(E.EithotError) as ei:
        E.tune_set(key, value)
    assert ei.value.code == E.EINVAL
    if old is not None:
        assert E.tune_get(key) == old

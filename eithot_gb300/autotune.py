"""Per-shape autotuner for the in-place transpose.

The library's lowering picks kernels by a cost model calibrated on GB300;
for a shape a caller runs often, measuring is better.  `autotune` times the
candidate knob settings on a scratch buffer of that shape on the current
device, records the fastest with eithot_tune_shape_set (so every later
eithot_transpose of exactly that shape uses it) and returns it.  Results
can be saved to and loaded from a JSON file keyed by shape.

This helper takes its scratch buffer and CUDA events from PyTorch (imported
when `autotune` runs); the library it tunes (libeithot.so, the C ABI) has
no PyTorch dependency, and a caller without PyTorch records knobs with
eithot_tune_shape_set directly.
"""
from __future__ import annotations

import json
import math
from typing import Dict, List, Optional, Sequence

from . import ORDER_MIXED, EithotError, plan, transpose_ptr, tune_shape_set

# Knob settings worth trying: the cost model's own choice first, then the
# forms it weighs against one another.
CANDIDATES: List[Dict[str, float]] = [
    {},
    {"variant": 1}, {"variant": 2},
    {"col_form": 1}, {"col_form": 2},
    {"col_form": 2, "group_per_sm": 2}, {"col_form": 2, "group_per_sm": 3},
    {"col_chunk": 128}, {"col_chunk": 256},
    {"slab_cluster": 0}, {"row_block": 0}, {"slab_pack": 0},
]

DEFAULTS = {"variant": 0, "col_form": 0, "group_per_sm": 0, "col_chunk": 0, "slab_cluster": 1, "row_block": 1,
            "slab_pack": 1}


def _key(dims, perm, elem) -> str:
    return "%s|%s|%d" % (",".join(str(int(d)) for d in dims), ",".join(str(int(p)) for p in perm), int(elem))


def _apply(dims, perm, elem, cfg: Dict[str, float]) -> None:
    for k, v in {**DEFAULTS, **cfg}.items():
        tune_shape_set(dims, perm, elem, k, v)


def autotune(dims: Sequence[int], perm: Sequence[int], elem_size: int, num_sub_tensors: int = 1,
             alpha: float = 0.01, candidates: Optional[List[Dict[str, float]]] = None, reps: int = 3) -> dict:
    """Times every candidate (a failing one is skipped) and keeps the
    fastest for this shape.  Returns {"config": ..., "ms": ..., "tried": n}."""
    import torch

    info = plan(dims, perm, num_sub_tensors, alpha)
    cap = info.padded_volume * elem_size
    buf = torch.empty(max(1, cap), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    best, best_ms, tried = None, math.inf, 0
    for cfg in candidates or CANDIDATES:
        _apply(dims, perm, elem_size, cfg)
        try:
            transpose_ptr(buf.data_ptr(), cap, dims, perm, elem_size, num_sub_tensors, alpha, ORDER_MIXED,
                          stream.cuda_stream)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                transpose_ptr(buf.data_ptr(), cap, dims, perm, elem_size, num_sub_tensors, alpha, ORDER_MIXED,
                              stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
        except EithotError:
            continue
        tried += 1
        ms = e0.elapsed_time(e1) / reps
        if ms < best_ms:
            best, best_ms = cfg, ms
    if best is None:
        raise EithotError(1, "no candidate ran")
    _apply(dims, perm, elem_size, best)
    return {"config": best, "ms": best_ms, "tried": tried}


def save(path: str, results: Dict[str, dict]) -> None:
    """results: {shape key: autotune() result} (see key())."""
    with open(path, "w") as f:
        json.dump(results, f, indent=1, sort_keys=True)


def load(path: str) -> int:
    """Records every saved shape's knobs; returns how many."""
    with open(path) as f:
        results = json.load(f)
    for k, r in results.items():
        dims, perm, elem = k.split("|")
        _apply([int(x) for x in dims.split(",")], [int(x) for x in perm.split(",")], int(elem), r["config"])
    return len(results)


def key(dims, perm, elem_size) -> str:
    """The JSON key of a shape."""
    return _key(dims, perm, elem_size)

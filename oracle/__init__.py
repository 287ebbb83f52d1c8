"""ORACLE — test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
as the checker; the product (eithot_gb300) never imports it.

* permute / permute_mt: CPU restatement of the reference's host out-of-place
  permutation TensorUtil::seq_tt (ITNT/src/tensor_util.cpp:92-104), C code in
  permute.c built into _build/liboracle.so;
* planner: restatement of the permutation planner and N-d orchestration;
* estimator: restatement of the Nd_estimation extra-memory estimator.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "_build/liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        I64P = ctypes.POINTER(ctypes.c_int64)
        IP = ctypes.POINTER(ctypes.c_int)
        L.oracle_permute.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, I64P, IP, ctypes.c_size_t]
        L.oracle_permute_mt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, I64P, IP,
                                        ctypes.c_size_t, ctypes.c_int]
        L.oracle_dest_index.argtypes = [ctypes.c_int, I64P, IP, ctypes.c_int64]
        L.oracle_dest_index.restype = ctypes.c_int64
        L.oracle_hash_value.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_hash_value.restype = ctypes.c_uint64
        L.oracle_fill_hash.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_size_t, ctypes.c_uint64,
                                       ctypes.c_int64]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _arrs(dims, perm):
    r = len(dims)
    return r, (ctypes.c_int64 * r)(*[int(d) for d in dims]), (ctypes.c_int * r)(*[int(p) for p in perm])


def permute(src: np.ndarray, dims, perm, elem: int, threads: int = 0) -> np.ndarray:
    """Out-of-place permutation of the raw bytes in `src` (dims[0] fastest,
    1-based perm).  threads=1 runs the single-threaded restatement."""
    src = np.ascontiguousarray(src)
    out = np.empty_like(src)
    r, D, P = _arrs(dims, perm)
    L = lib()
    if threads == 1:
        rc = L.oracle_permute(src.ctypes.data, out.ctypes.data, r, D, P, elem)
    else:
        rc = L.oracle_permute_mt(src.ctypes.data, out.ctypes.data, r, D, P, elem, threads)
    if rc != 0:
        raise ValueError("oracle: invalid permutation")
    return out


def dest_index(dims, perm, src_index: int) -> int:
    r, D, P = _arrs(dims, perm)
    return lib().oracle_dest_index(r, D, P, int(src_index))


def fill_hash(n: int, elem: int, seed: int, first_index: int = 0) -> np.ndarray:
    buf = np.empty(n * elem, dtype=np.uint8)
    lib().oracle_fill_hash(buf.ctypes.data, n, elem, seed, first_index)
    return buf


def hash_value(seed: int, index: int) -> int:
    return lib().oracle_hash_value(seed, index)


def max_threads() -> int:
    return lib().oracle_max_threads()

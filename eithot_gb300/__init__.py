"""EITHOT-GB300: in-place high-order tensor transposition on GB300 (sm_103a).

Python mirror of the reference interface for this path.  The reference's
entry point is ``inplace::transpose(data, source, rank, dim, permutation,
sizeofType, num_block, ALPHA)`` (ITNT/include/transpose.h:8) driven by the
``test_inplace dims... perm(1-based)... elem nb alpha`` tuple
(ITNT/src/test_inplace.cpp:142-158); :func:`transpose` takes the same tuple and
forwards to the C ABI in ``include/eithot.h`` (``libeithot.so``).  All device
work is the library's own sm_103a kernels; there is no CPU or library
fallback: if the shared library is missing the import raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libeithot.so")

OK, EINVAL, ENOMEM, ETIMEOUT, ECUDA, EUNSUPPORTED, EBUSY, EFAULT = range(8)
ORDER_MIXED, ORDER_PRE, ORDER_POST, ORDER_FEWEST = 0, 1, 2, 3
STEP_ROUND, STEP_PARTITION, STEP_JOIN, STEP_PAD_PRE, STEP_PAD_POST = range(5)


class EithotError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("eithot error %d: %s" % (code, msg))
        self.code = code


class _Step(ctypes.Structure):
    _fields_ = [("role", ctypes.c_int), ("code", ctypes.c_int), ("rank", ctypes.c_int),
                ("perm", ctypes.c_int * 4), ("dims", ctypes.c_int64 * 4)]


class _PlanInfo(ctypes.Structure):
    _fields_ = [("order_used", ctypes.c_int), ("num_sub_tensors", ctypes.c_int),
                ("decompose_dim", ctypes.c_int), ("padded", ctypes.c_int),
                ("padded_dim_size", ctypes.c_int64), ("volume", ctypes.c_int64),
                ("padded_volume", ctypes.c_int64), ("sub_tensor_elems", ctypes.c_int64),
                ("n_steps", ctypes.c_int)]


class _Stats(ctypes.Structure):
    _fields_ = [("workspace_bytes", ctypes.c_size_t), ("free_before", ctypes.c_size_t),
                ("free_after_alloc", ctypes.c_size_t), ("n_passes", ctypes.c_int),
                ("n_launches", ctypes.c_int), ("algorithmic_bytes", ctypes.c_double)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libeithot.so is not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    I64P = ctypes.POINTER(ctypes.c_int64)
    IP = ctypes.POINTER(ctypes.c_int)
    lib.eithot_plan.argtypes = [ctypes.c_int, I64P, IP, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                ctypes.POINTER(_PlanInfo), ctypes.POINTER(_Step), ctypes.c_int]
    lib.eithot_transpose.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, I64P, IP,
                                     ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    lib.eithot_transpose_ex.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, I64P, IP,
                                        ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.eithot_workspace_size.argtypes = [ctypes.c_int, I64P, IP, ctypes.c_size_t, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    lib.eithot_estimate.argtypes = [ctypes.c_int, I64P, IP, ctypes.c_size_t, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_size_t, ctypes.c_int, IP,
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_size_t)]
    lib.eithot_last_error.restype = ctypes.c_char_p
    lib.eithot_profile_get.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.eithot_last_stats.argtypes = [ctypes.POINTER(_Stats)]
    lib.eithot_fill_hash.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_int64,
                                     ctypes.c_void_p]
    lib.eithot_check_hash.argtypes = [ctypes.c_void_p, ctypes.c_int, I64P, IP, ctypes.c_size_t, ctypes.c_uint64,
                                      ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int64)]
    lib.eithot_batch_create.argtypes = [ctypes.c_int, IP, I64P, IP, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                                        ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]
    lib.eithot_batch_workspace_size.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
    lib.eithot_batch_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_size_t),
                                     ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.eithot_batch_launches.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    lib.eithot_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.eithot_server_create.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.eithot_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, I64P, IP,
                                         ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_uint64)]
    lib.eithot_server_poll.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]
    lib.eithot_server_poll_status.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.eithot_server_memory.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                                         ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    lib.eithot_server_pending.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    lib.eithot_server_launches.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    lib.eithot_server_destroy.argtypes = [ctypes.c_void_p]
    lib.eithot_tune_set.argtypes = [ctypes.c_char_p, ctypes.c_double]
    lib.eithot_tune_get.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    lib.eithot_tune_shape_set.argtypes = [ctypes.c_int, I64P, IP, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_double]
    lib.eithot_tune_shape_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib.eithot_last_call.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
    lib.eithot_call_status.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
    return lib


lib = _load()


def _arrays(dims: Sequence[int], perm: Sequence[int]):
    r = len(dims)
    if len(perm) != r:
        raise EithotError(EINVAL, "dims and permutation differ in length")
    return r, (ctypes.c_int64 * r)(*[int(d) for d in dims]), (ctypes.c_int * r)(*[int(p) for p in perm])


def _check(rc: int):
    if rc != OK:
        raise EithotError(rc, lib.eithot_last_error().decode())


@dataclass
class Step:
    role: int
    code: int
    dims: List[int]
    perm: List[int]


@dataclass
class PlanInfo:
    order_used: int
    num_sub_tensors: int
    decompose_dim: int
    padded: bool
    padded_dim_size: int
    volume: int
    padded_volume: int
    sub_tensor_elems: int
    steps: List[Step]


def plan(dims: Sequence[int], perm: Sequence[int], num_sub_tensors: int = 1, alpha: float = 0.01,
         order: int = ORDER_MIXED) -> PlanInfo:
    """The decomposition the library will execute (host only)."""
    r, d, p = _arrays(dims, perm)
    info = _PlanInfo()
    _check(lib.eithot_plan(r, d, p, num_sub_tensors, alpha, order, ctypes.byref(info), None, 0))
    steps = (_Step * max(1, info.n_steps))()
    _check(lib.eithot_plan(r, d, p, num_sub_tensors, alpha, order, ctypes.byref(info), steps, info.n_steps))
    out = []
    for i in range(info.n_steps):
        s = steps[i]
        if s.role in (STEP_PAD_PRE, STEP_PAD_POST):
            out.append(Step(s.role, 0, [s.dims[0], s.dims[1], s.dims[2]], []))
        else:
            out.append(Step(s.role, s.code, list(s.dims[:s.rank]), list(s.perm[:s.rank])))
    return PlanInfo(info.order_used, info.num_sub_tensors, info.decompose_dim, bool(info.padded),
                    info.padded_dim_size, info.volume, info.padded_volume, info.sub_tensor_elems, out)


def workspace_size(dims, perm, elem_size, num_sub_tensors=1, alpha=0.01, order=ORDER_MIXED) -> int:
    r, d, p = _arrays(dims, perm)
    out = ctypes.c_size_t()
    _check(lib.eithot_workspace_size(r, d, p, elem_size, num_sub_tensors, alpha, order, ctypes.byref(out)))
    return out.value


def estimate(dims, perm, elem_size, num_sub_tensors=1, alpha=0.01, smem_per_block=0, padding_blocks=0):
    """Nd_estimation's answer: (nb, alpha, modelled extra bytes)."""
    r, d, p = _arrays(dims, perm)
    nb = ctypes.c_int()
    a = ctypes.c_double()
    ex = ctypes.c_size_t()
    _check(lib.eithot_estimate(r, d, p, elem_size, num_sub_tensors, alpha, smem_per_block,
                               padding_blocks, ctypes.byref(nb), ctypes.byref(a), ctypes.byref(ex)))
    return nb.value, a.value, ex.value


def transpose_ptr(ptr: int, capacity_bytes: int, dims, perm, elem_size: int, num_sub_tensors: int = 1,
                  alpha: float = 0.01, order: int = ORDER_MIXED, stream: Optional[int] = None,
                  workspace_ptr: int = 0, workspace_bytes: int = 0) -> None:
    """In-place transpose of the tensor at device address `ptr` (C ABI call)."""
    r, d, p = _arrays(dims, perm)
    _check(lib.eithot_transpose_ex(ctypes.c_void_p(ptr), capacity_bytes, r, d, p, elem_size,
                                   num_sub_tensors, alpha, order,
                                   ctypes.c_void_p(workspace_ptr) if workspace_ptr else None,
                                   workspace_bytes, ctypes.c_void_p(stream) if stream else None))


def transpose(tensor, dims, perm, num_sub_tensors: int = 1, alpha: float = 0.01,
              order: int = ORDER_MIXED, elem_size: Optional[int] = None, stream=None):
    """In-place transpose of a CUDA torch tensor holding the row-major
    (dims[0] fastest) tensor; returns the same tensor (its storage now holds
    the permuted tensor).  The whole storage of `tensor` is the capacity the
    padded form may use."""
    import torch  # device memory and streams only

    if not tensor.is_cuda:
        raise EithotError(EINVAL, "tensor must live on a CUDA device")
    es = elem_size or tensor.element_size()
    cap = tensor.numel() * tensor.element_size()
    if stream is None:
        stream = torch.cuda.current_stream(tensor.device)
    sptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    with torch.cuda.device(tensor.device):
        transpose_ptr(tensor.data_ptr(), cap, dims, perm, es, num_sub_tensors, alpha, order, sptr)
    return tensor


def last_call() -> int:
    """Id of this thread's most recent transpose call (eithot_last_call)."""
    v = ctypes.c_uint64()
    _check(lib.eithot_last_call(ctypes.byref(v)))
    return v.value


def call_status(call_id: int, stream: Optional[int] = None) -> int:
    """Synchronises `stream` and returns the device-side outcome of call
    `call_id`: OK, ETIMEOUT (a bounded group-barrier wait gave up) or EFAULT
    (an index-map result fell outside its row or column)."""
    v = ctypes.c_int()
    _check(lib.eithot_call_status(call_id, ctypes.c_void_p(stream) if stream else None, ctypes.byref(v)))
    return v.value


def last_stats() -> dict:
    s = _Stats()
    _check(lib.eithot_last_stats(ctypes.byref(s)))
    return {k: getattr(s, k) for k, _ in _Stats._fields_}


def output_dims(dims: Sequence[int], perm: Sequence[int]) -> List[int]:
    return [int(dims[p - 1]) for p in perm]


def set_profiling(enable: bool) -> None:
    """Record CUDA events around every pass of subsequent calls (this thread)."""
    _check(lib.eithot_set_profiling(1 if enable else 0))


def profile_reset() -> None:
    _check(lib.eithot_profile_reset())


def profile() -> List[dict]:
    """Per-pass (name, ms, bytes) of the last profiled call; synchronise the
    stream first."""
    out = []
    name = ctypes.create_string_buffer(256)
    for i in range(lib.eithot_profile_count()):
        ms, by = ctypes.c_double(), ctypes.c_double()
        _check(lib.eithot_profile_get(i, name, 256, ctypes.byref(ms), ctypes.byref(by)))
        out.append({"name": name.value.decode(), "ms": ms.value, "bytes": by.value})
    return out


def index_faults() -> int:
    """Index-map results outside their row/column since the last call
    (kernels skip them); synchronises the device."""
    v = ctypes.c_uint()
    _check(lib.eithot_index_faults(ctypes.byref(v)))
    return v.value


def fill_hash_ptr(ptr: int, n_elems: int, elem_size: int, seed: int, first_index: int = 0,
                  stream: Optional[int] = None) -> None:
    """Writes the counter-hash sequence (elements first_index ..) to device
    memory at `ptr` (see eithot_fill_hash)."""
    _check(lib.eithot_fill_hash(ctypes.c_void_p(ptr), n_elems, elem_size, seed & (2**64 - 1), first_index,
                                ctypes.c_void_p(stream) if stream else None))


def check_hash_ptr(ptr: int, dims, perm, elem_size: int, seed: int, stream: Optional[int] = None):
    """(mismatches, first bad output index or -1) of the permutation (dims,
    perm) of a counter-hash tensor at `ptr`; synchronises the stream."""
    r, d, p = _arrays(dims, perm)
    bad, first = ctypes.c_uint64(), ctypes.c_int64()
    _check(lib.eithot_check_hash(ctypes.c_void_p(ptr), r, d, p, elem_size, seed & (2**64 - 1),
                                 ctypes.c_void_p(stream) if stream else None, ctypes.byref(bad), ctypes.byref(first)))
    return bad.value, first.value


class Batch:
    """Many independent in-place transposes planned once (eithot_batch_*).

    tensors: sequence of (dims, perm_1based, elem_size)."""

    def __init__(self, tensors, num_sub_tensors: int = 1, alpha: float = 0.01):
        ranks, dims, perms, elems = [], [], [], []
        for d, p, e in tensors:
            if len(d) != len(p):
                raise EithotError(EINVAL, "dims and permutation differ in length")
            ranks.append(len(d))
            dims += [int(x) for x in d]
            perms += [int(x) for x in p]
            elems.append(int(e))
        self.count = len(ranks)
        h = ctypes.c_void_p()
        _check(lib.eithot_batch_create(self.count, (ctypes.c_int * max(1, len(ranks)))(*ranks),
                                       (ctypes.c_int64 * max(1, len(dims)))(*dims),
                                       (ctypes.c_int * max(1, len(perms)))(*perms),
                                       (ctypes.c_size_t * max(1, len(elems)))(*elems),
                                       num_sub_tensors, alpha, ctypes.byref(h)))
        self._h = h

    @property
    def workspace_size(self) -> int:
        v = ctypes.c_size_t()
        _check(lib.eithot_batch_workspace_size(self._h, ctypes.byref(v)))
        return v.value

    def run(self, ptrs, capacities, workspace_ptr: int = 0, workspace_bytes: int = 0, stream: Optional[int] = None):
        n = self.count
        _check(lib.eithot_batch_run(self._h, (ctypes.c_void_p * max(1, n))(*ptrs),
                                    (ctypes.c_size_t * max(1, n))(*capacities),
                                    ctypes.c_void_p(workspace_ptr) if workspace_ptr else None, workspace_bytes,
                                    ctypes.c_void_p(stream) if stream else None))

    @property
    def launches(self) -> int:
        v = ctypes.c_int()
        _check(lib.eithot_batch_launches(self._h, ctypes.byref(v)))
        return v.value

    def close(self):
        if self._h:
            lib.eithot_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The served form (eithot_server_*): submit resident tensors, poll for
    the tickets of finished ones."""

    def __init__(self, workspace_bytes: int, streams: int = 4):
        h = ctypes.c_void_p()
        _check(lib.eithot_server_create(workspace_bytes, streams, ctypes.byref(h)))
        self._h = h
        self._done = (ctypes.c_uint64 * 4096)()
        self._status = (ctypes.c_int * 4096)()

    def submit(self, ptr: int, capacity_bytes: int, dims, perm, elem_size: int, num_sub_tensors: int = 1,
               alpha: float = 0.01) -> int:
        r, d, p = _arrays(dims, perm)
        t = ctypes.c_uint64()
        _check(lib.eithot_server_submit(self._h, ctypes.c_void_p(ptr), capacity_bytes, r, d, p, elem_size,
                                        num_sub_tensors, alpha, ctypes.byref(t)))
        return t.value

    def poll(self) -> List[int]:
        return [t for t, _ in self.poll_status()]

    def poll_status(self):
        """Finished tickets with their device status (OK, ETIMEOUT, EFAULT)."""
        out = []
        while True:
            n = ctypes.c_int()
            _check(lib.eithot_server_poll_status(self._h, self._done, self._status, len(self._done),
                                                 ctypes.byref(n)))
            out += list(zip(self._done[: n.value], self._status[: n.value]))
            if n.value < len(self._done):
                return out

    def memory(self):
        """(resident tensor bytes, pool bytes, scratch held in free HBM)."""
        r, p, h = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        _check(lib.eithot_server_memory(self._h, ctypes.byref(r), ctypes.byref(p), ctypes.byref(h)))
        return r.value, p.value, h.value

    def pending(self):
        q, r = ctypes.c_int(), ctypes.c_int()
        _check(lib.eithot_server_pending(self._h, ctypes.byref(q), ctypes.byref(r)))
        return q.value, r.value

    @property
    def launches(self) -> int:
        v = ctypes.c_int()
        _check(lib.eithot_server_launches(self._h, ctypes.byref(v)))
        return v.value

    def close(self):
        if self._h:
            lib.eithot_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sync_timeouts() -> int:
    """Bounded group-barrier waits that gave up since the last call (their
    transposes' outputs are invalid); synchronises the device."""
    v = ctypes.c_uint()
    _check(lib.eithot_sync_timeouts(ctypes.byref(v)))
    return v.value


def selftest_wait() -> int:
    """Runs one bounded wait that nothing releases; returns the timeouts it
    counted (1 when the bound holds)."""
    v = ctypes.c_uint()
    _check(lib.eithot_selftest_wait(ctypes.byref(v)))
    return v.value


def tune_set(key: str, value: float) -> None:
    """Process-wide lowering knob ("dbuf", "max_cluster", "variant", "col_batch", "col_chunk",
    "col_owner", "col_form", "row_prefetch", "row_block", "slab_pack", "slab_cluster", "factor", "sync_sleep_ns",
    "sync_spin_limit", "sync_relaxed",
    "group_per_sm", "l2_prefetch", "batch_graph")."""
    _check(lib.eithot_tune_set(key.encode(), float(value)))


def tune_shape_set(dims, perm, elem_size: int, key: str, value: float) -> None:
    """Knob for one exact (dims, perm, element size) request (autotuner)."""
    r, d, p = _arrays(dims, perm)
    _check(lib.eithot_tune_shape_set(r, d, p, elem_size, key.encode(), float(value)))


def tune_shape_clear() -> None:
    _check(lib.eithot_tune_shape_clear())


def tune_shape_count() -> int:
    v = ctypes.c_int()
    _check(lib.eithot_tune_shape_count(ctypes.byref(v)))
    return v.value


def tune_get(key: str) -> float:
    v = ctypes.c_double()
    _check(lib.eithot_tune_get(key.encode(), ctypes.byref(v)))
    return v.value

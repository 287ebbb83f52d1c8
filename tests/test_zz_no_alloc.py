"""eithot_transpose_noalloc: the entry point for callers that may not
allocate device memory during the call (for instance because another
allocator owns the device's memory).  Its scratch is a fixed 32 MiB array
inside the library.  Checked through the C ABI against the allocating entry
point (eithot_transpose_ex) on the same inputs, for two calls in a row, on
transposes that do use scratch.  Collected last so that a failure here comes
after every other test has run."""
import ctypes
import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NOALLOC_SCRATCH = 32 << 20


def _fn(E):
    f = E.lib.eithot_transpose_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                  ctypes.POINTER(ctypes.c_int), ctypes.c_size_t, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    return f


def _noalloc(E, t, cap, dims, perm, elem, nb, alpha, stream):
    r = len(dims)
    rc = _fn(E)(ctypes.c_void_p(t.data_ptr()), cap, r, (ctypes.c_int64 * r)(*dims), (ctypes.c_int * r)(*perm),
                elem, nb, alpha, ctypes.c_void_p(stream.cuda_stream))
    return rc


@pytest.mark.parametrize("dims,perm,elem,nb,alpha", [
    ([4, 20011, 819, 2], [1, 3, 2, 4], 4, 1, 0.01),  # group column passes: barrier counters in scratch
    ([4, 20011, 819, 2], [1, 3, 2, 4], 4, 2, 0.01),  # and padded blocks moved through scratch in pieces
    ([3301, 70, 5], [3, 1, 2], 4, 4, 0.01),          # padded sub-tensors: block moves through scratch
    ([3, 1000003], [2, 1], 4, 1, 0.01),              # prime sides: a column tile staged in global scratch
])
def test_noalloc_matches_allocating_entry_point(E, dims, perm, elem, nb, alpha):
    assert E.workspace_size(dims, perm, elem, nb, alpha) > 0  # the case does use scratch
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    n = math.prod(dims)
    plan = E.plan(dims, perm, nb, alpha)
    cap = plan.padded_volume * elem
    host = oracle.fill_hash(n, elem, 1234)
    a = torch.zeros(cap, dtype=torch.uint8, device=dev)
    b = torch.zeros(cap, dtype=torch.uint8, device=dev)
    a[:n * elem] = torch.from_numpy(host).to(dev)
    b[:n * elem] = a[:n * elem]
    for _ in range(2):  # two calls in a row, each on the previous call's output
        E.transpose_ptr(a.data_ptr(), cap, dims, perm, elem, nb, alpha, E.ORDER_MIXED, stream.cuda_stream)
        rc = _noalloc(E, b, cap, dims, perm, elem, nb, alpha, stream)
        assert rc == E.OK, E.lib.eithot_last_error().decode()
        stream.synchronize()
        assert E.index_faults() == 0
        assert E.sync_timeouts() == 0
        assert torch.equal(a[:n * elem], b[:n * elem])
    # and the first call alone matches the oracle
    c = torch.zeros(cap, dtype=torch.uint8, device=dev)
    c[:n * elem] = torch.from_numpy(host).to(dev)
    assert _noalloc(E, c, cap, dims, perm, elem, nb, alpha, stream) == E.OK
    stream.synchronize()
    assert np.array_equal(c[:n * elem].cpu().numpy(), oracle.permute(host, dims, perm, elem))


def test_noalloc_rejects_scratch_beyond_its_limit(E):
    """A transpose whose staged column tile exceeds the fixed array (two
    prime sides: nothing to split it along) is refused with EITHOT_EINVAL
    before any device work."""
    dims, perm, elem = [3, 9000011], [2, 1], 4
    assert E.workspace_size(dims, perm, elem) > NOALLOC_SCRATCH
    dev = torch.device("cuda:0")
    n = math.prod(dims)
    t = torch.arange(n, dtype=torch.int32, device=dev)
    before = t.clone()
    rc = _noalloc(E, t, n * elem, dims, perm, elem, 1, 0.01, torch.cuda.current_stream(dev))
    assert rc == E.EINVAL
    assert "scratch" in E.lib.eithot_last_error().decode()
    torch.cuda.synchronize()
    assert torch.equal(t, before)


def test_noalloc_without_scratch_and_on_two_streams(E):
    """A transpose that needs no scratch at all (the array is not touched),
    then scratch-using calls on two different streams one after the other:
    each matches the allocating entry point and the oracle."""
    dev = torch.device("cuda:0")
    cases = [([37, 64, 5, 3], [3, 1, 4, 2], 4, 1, 0.01), ([4, 20011, 819, 2], [1, 3, 2, 4], 4, 1, 0.01)]
    assert E.workspace_size(*cases[0][:3]) == 0
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    for k, (dims, perm, elem, nb, alpha) in enumerate(cases):
        for s in streams:
            n = math.prod(dims)
            host = oracle.fill_hash(n, elem, 77 + k)
            a = torch.from_numpy(host.copy()).to(dev)
            b = a.clone()
            torch.cuda.synchronize()
            E.transpose_ptr(a.data_ptr(), a.numel(), dims, perm, elem, nb, alpha, E.ORDER_MIXED, s.cuda_stream)
            assert _noalloc(E, b, b.numel(), dims, perm, elem, nb, alpha, s) == E.OK, E.lib.eithot_last_error().decode()
            s.synchronize()
            assert torch.equal(a, b)
            assert np.array_equal(b.cpu().numpy(), oracle.permute(host, dims, perm, elem))
    assert E.index_faults() == 0 and E.sync_timeouts() == 0

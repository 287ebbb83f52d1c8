"""Per-call device status and the ordering of group-synchronised passes.

A group column pass waits at a bounded barrier; when the wait gives up, the
launch skips its remaining writes and the call's own status word says so
(EITHOT_ETIMEOUT through eithot_call_status).  The tests make the wait run
out by setting its poll limit to zero through a tuning knob: nothing faults
or hangs, the CTAs simply stop waiting.  Group passes issued on different
streams, or by the served form's executor streams, are ordered one after
another on the device and come back bit-exact."""
import math
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GROUP_DIMS, GROUP_PERM = [4, 20011, 819, 2], [1, 3, 2, 4]  # a 20011-row column shuffle of 16-byte elements


@pytest.fixture
def knobs(E):
    keys = ("col_form", "variant", "sync_spin_limit")
    saved = {k: E.tune_get(k) for k in keys}

    def set_(**kw):
        for k, v in kw.items():
            E.tune_set(k, v)
    yield set_
    for k, v in saved.items():
        E.tune_set(k, v)


def fresh(E, dims, elem, seed):
    n = math.prod(dims)
    host = oracle.fill_hash(n, elem, seed)
    return host, torch.from_numpy(host.copy()).cuda()


def test_status_of_a_good_call_is_ok(E):
    host, t = fresh(E, [301, 4096], 4, 3)
    s = torch.cuda.current_stream()
    E.transpose_ptr(t.data_ptr(), t.numel(), [301, 4096], [2, 1], 4, stream=s.cuda_stream)
    cid = E.last_call()
    assert E.call_status(cid, s.cuda_stream) == E.OK
    assert np.array_equal(t.cpu().numpy(), oracle.permute(host, [301, 4096], [2, 1], 4))
    with pytest.raises(E.EithotError) as ei:
        E.call_status(cid + 10 ** 9)
    assert ei.value.code == E.EINVAL


def test_group_wait_that_runs_out_is_reported_for_that_call(E, knobs):
    """A real group-pass transpose whose barrier waits are limited to zero
    polls: the call reports EITHOT_ETIMEOUT; the next call on the same
    context, with the default limit, is correct and reports OK."""
    knobs(col_form=2, variant=2, sync_spin_limit=0)
    s = torch.cuda.current_stream()
    host, t = fresh(E, GROUP_DIMS, 4, 5)
    E.transpose_ptr(t.data_ptr(), t.numel(), GROUP_DIMS, GROUP_PERM, 4, stream=s.cuda_stream)
    bad = E.last_call()
    assert E.call_status(bad, s.cuda_stream) == E.ETIMEOUT
    assert E.sync_timeouts() > 0  # the process-wide count saw it too (and is cleared)
    knobs(sync_spin_limit=1 << 20)
    host, t = fresh(E, GROUP_DIMS, 4, 6)
    E.transpose_ptr(t.data_ptr(), t.numel(), GROUP_DIMS, GROUP_PERM, 4, stream=s.cuda_stream)
    good = E.last_call()
    assert E.call_status(good, s.cuda_stream) == E.OK
    assert E.call_status(bad, s.cuda_stream) == E.ETIMEOUT  # each call keeps its own word
    assert np.array_equal(t.cpu().numpy(), oracle.permute(host, GROUP_DIMS, GROUP_PERM, 4))
    assert E.sync_timeouts() == 0


def test_group_passes_on_two_streams(E, knobs):
    """Two group-pass transposes issued back to back on two streams (no host
    synchronisation between them) are ordered on the device and both come
    back bit-exact with status OK."""
    knobs(col_form=2)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    cases = []
    for k, s in enumerate(streams):
        host, t = fresh(E, GROUP_DIMS, 4, 20 + k)
        torch.cuda.synchronize()
        E.transpose_ptr(t.data_ptr(), t.numel(), GROUP_DIMS, GROUP_PERM, 4, stream=s.cuda_stream)
        cases.append((host, t, E.last_call(), s))
    for host, t, cid, s in cases:
        assert E.call_status(cid, s.cuda_stream) == E.OK
        assert np.array_equal(t.cpu().numpy(), oracle.permute(host, GROUP_DIMS, GROUP_PERM, 4))
    assert E.sync_timeouts() == 0


def _serve(E, srv, bufs, reqs, timeout=120, nb=1):
    tickets = {srv.submit(b.data_ptr(), b.numel(), d, p, e, nb): i for i, (b, (d, p, e)) in enumerate(zip(bufs, reqs))}
    got = {}
    t0 = time.time()
    while len(got) < len(tickets):
        for t, st in srv.poll_status():
            got[tickets[t]] = st
        assert time.time() - t0 < timeout
    return got


def test_server_runs_two_large_group_requests_at_once(E, knobs):
    """Two requests whose column passes are group-synchronised, in flight on
    two executor streams at once: both bit-exact, both status OK."""
    knobs(col_form=2)
    reqs = [(GROUP_DIMS, GROUP_PERM, 4), ([4, 20011, 700, 2], GROUP_PERM, 4)]
    hosts, bufs = zip(*[fresh(E, d, e, 40 + i) for i, (d, p, e) in enumerate(reqs)])
    torch.cuda.synchronize()
    srv = E.Server(64 << 20, streams=2)
    got = _serve(E, srv, bufs, reqs)
    srv.close()
    assert got == {0: E.OK, 1: E.OK}
    for h, b, (d, p, e) in zip(hosts, bufs, reqs):
        assert np.array_equal(b.cpu().numpy(), oracle.permute(h, d, p, e))
    assert E.sync_timeouts() == 0


def test_server_result_is_the_same_alone_and_in_the_mix(E):
    """One request served alone and the same request (same input) served in
    a mix of large and small requests leave identical buffers."""
    probe = ([4, 20011, 300, 2], [1, 3, 2, 4], 4)
    rng = np.random.default_rng(3)
    mix = [probe]
    for i in range(40):
        r = int(rng.integers(2, 6))
        elem = int(rng.choice([1, 2, 4, 8]))
        n = max(1, int(math.exp(rng.uniform(math.log(1 << 16), math.log(24 << 20))) / elem))
        w = rng.uniform(0.1, 1.0, size=r)
        dims = [max(1, int(round(math.exp(x)))) for x in w / w.sum() * math.log(n)]
        mix.append((dims, [int(x) + 1 for x in rng.permutation(r)], elem))
    mix.append(([3001, 4096], [2, 1], 4))
    host_probe, alone = fresh(E, probe[0], 4, 77)
    srv = E.Server(128 << 20, streams=4)
    got = _serve(E, srv, [alone], [probe])
    assert got == {0: E.OK}
    bufs = [torch.from_numpy(host_probe.copy()).cuda()]
    hosts = [host_probe]
    for i, (d, p, e) in enumerate(mix[1:]):
        h, b = fresh(E, d, e, 100 + i)
        hosts.append(h)
        bufs.append(b)
    torch.cuda.synchronize()
    got = _serve(E, srv, bufs, mix)
    srv.close()
    assert all(st == E.OK for st in got.values())
    assert torch.equal(alone, bufs[0])
    assert np.array_equal(bufs[0].cpu().numpy(), oracle.permute(host_probe, *probe))
    for h, b, (d, p, e) in zip(hosts[1:], bufs[1:], mix[1:]):
        assert np.array_equal(b.cpu().numpy(), oracle.permute(h, d, p, e)), (d, p, e)


def test_server_pool_sized_for_one_request_serves_many_small_ones(E):
    """A pool that holds one request's scratch and sixteen small requests
    that each need scratch (padding moves of 4 sub-tensors): a batch of them
    would need sixteen lanes' scratch, so the batches shrink until their
    workspace fits and every request finishes bit-exact (the queue never
    stalls)."""
    dims, perm, elem, nb = [5001, 20, 30], [2, 3, 1], 4, 4
    need = E.workspace_size(dims, perm, elem, num_sub_tensors=nb)
    assert need > 0
    reqs = [(dims, perm, elem)] * 16
    pairs = [fresh(E, dims, elem, 200 + i) for i in range(16)]
    hosts = [h for h, _ in pairs]
    # each buffer with the padding slack the sub-tensor plan needs
    bufs = []
    for h in hosts:
        b = torch.zeros(h.size * 103 // 100 + 256, dtype=torch.uint8, device="cuda")
        b[:h.size] = torch.from_numpy(h).cuda()
        bufs.append(b)
    torch.cuda.synchronize()
    srv = E.Server(need, streams=4)
    got = _serve(E, srv, bufs, reqs, timeout=60, nb=nb)
    srv.close()
    assert all(st == E.OK for st in got.values()) and len(got) == 16
    for h, b in zip(hosts, bufs):
        assert np.array_equal(b[:h.size].cpu().numpy(), oracle.permute(h, dims, perm, elem))


def test_server_admits_beyond_its_pool_against_free_hbm(E):
    """A request whose scratch exceeds the server's pool is admitted against
    the device's free memory, runs alone and comes back bit-exact; the
    server's memory accounting returns to zero."""
    dims, perm, elem = [60000, 300], [2, 1], 4
    need = E.workspace_size(dims, perm, elem)
    host, buf = fresh(E, dims, elem, 300)
    torch.cuda.synchronize()
    srv = E.Server(0, streams=1)
    got = _serve(E, srv, [buf], [(dims, perm, elem)], timeout=60)
    assert got == {0: E.OK}
    assert srv.memory() == (0, 0, 0)
    srv.close()
    assert need > 0
    assert np.array_equal(buf.cpu().numpy(), oracle.permute(host, dims, perm, elem))

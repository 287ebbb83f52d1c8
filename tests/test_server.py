"""The served form (eithot_server_*): requests resident on the device are
admitted against the server's workspace pool, batched when small, and all
come back bit-exact."""
import math
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_server_mixed_requests(E):
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(120):
        r = int(rng.integers(2, 6))
        elem = int(rng.choice([1, 2, 4, 8]))
        big = i % 30 == 7
        total = math.exp(rng.uniform(math.log(1 << 20), math.log((96 if big else 8) << 20)))
        n = max(1, int(total / elem))
        w = rng.uniform(0.1, 1.0, size=r)
        w = w / w.sum() * math.log(n)
        dims = [max(1, int(round(math.exp(x)))) for x in w]
        perm = [int(x) + 1 for x in rng.permutation(r)]
        reqs.append((dims, perm, elem))
    sizes = [math.prod(d) * e for d, p, e in reqs]
    offs = np.cumsum([0] + [(s + 511) // 256 * 256 for s in sizes])
    buf = torch.empty(int(offs[-1]), dtype=torch.uint8, device=dev)
    for t, ((d, p, e), o) in enumerate(zip(reqs, offs)):
        E.fill_hash_ptr(buf.data_ptr() + int(o), math.prod(d), e, 100 + t)
    torch.cuda.synchronize()
    srv = E.Server(256 << 20, streams=4)
    tickets = {}
    for t, ((d, p, e), o, s) in enumerate(zip(reqs, offs, sizes)):
        tickets[srv.submit(buf.data_ptr() + int(o), s + 256, d, p, e)] = t
    done = set()
    t0 = time.time()
    while len(done) < len(reqs):
        done.update(srv.poll())
        assert time.time() - t0 < 120
    assert set(tickets) == done
    assert srv.pending() == (0, 0)
    assert srv.launches > 0
    srv.close()
    torch.cuda.synchronize()
    assert E.index_faults() == 0 and E.sync_timeouts() == 0
    for t, ((d, p, e), o) in enumerate(zip(reqs, offs)):
        assert E.check_hash_ptr(buf.data_ptr() + int(o), d, p, e, 100 + t) == (0, -1), (t, d, p, e)


def test_server_refuses_what_neither_pool_nor_free_hbm_can_hold(E):
    """A request whose scratch exceeds both the pool and the device's free
    memory is refused at submission (no device work is issued for it)."""
    dev = torch.device("cuda:0")
    dims, perm, alpha = [2097152, 1048576], [2, 1], 0.05  # an 8 TiB int32 matrix, described only
    need = E.workspace_size(dims, perm, 4, alpha=alpha)
    free, _ = torch.cuda.mem_get_info(dev)
    assert need > free
    buf = torch.zeros(256, dtype=torch.uint8, device=dev)
    srv = E.Server(1 << 20, streams=1)
    with pytest.raises(E.EithotError) as ei:
        srv.submit(buf.data_ptr(), 4 * math.prod(dims), dims, perm, 4, alpha=alpha)
    assert ei.value.code == E.EBUSY
    assert srv.pending() == (0, 0)
    srv.close()


def test_server_small_requests_match_oracle(E):
    dev = torch.device("cuda:0")
    reqs = [([37, 64, 5, 3], [3, 1, 4, 2], 4), ([301, 4096], [2, 1], 4), ([6, 7, 8], [2, 3, 1], 1),
            ([5, 70000], [2, 1], 8), ([3, 5, 1000], [2, 1, 3], 2)]
    hosts = [oracle.fill_hash(math.prod(d), e, 7 + t) for t, (d, p, e) in enumerate(reqs)]
    bufs = [torch.from_numpy(h.copy()).to(dev) for h in hosts]
    srv = E.Server(64 << 20, streams=2)
    ids = [srv.submit(b.data_ptr(), b.numel(), d, p, e) for b, (d, p, e) in zip(bufs, reqs)]
    got = set()
    t0 = time.time()
    while len(got) < len(ids):
        got.update(srv.poll())
        assert time.time() - t0 < 60
    srv.close()
    for b, h, (d, p, e) in zip(bufs, hosts, reqs):
        assert np.array_equal(b.cpu().numpy(), oracle.permute(h, d, p, e))

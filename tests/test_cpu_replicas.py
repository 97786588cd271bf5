"""Multi-process helpers of the replica runs, with the gloo backend on CPU
(world size 2): barrier, max/sum over ranks and ensemble sharding."""
import os
import socket

import pytest

from solaris_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    r, w, _ = replicas.init(backend="gloo")
    replicas.barrier()
    mx = replicas.max_over_ranks(10.0 + r)
    sm = replicas.sum_over_ranks(1.5 * (r + 1))
    lo, hi = replicas.shard(4096, r, w)
    out.put((r, mx, sm, lo, hi))
    replicas.finalize()


def test_gloo_world_size_2():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]
    assert [r[2] for r in res] == [4.5, 4.5]
    assert (res[0][3], res[0][4], res[1][3], res[1][4]) == (0, 2048, 2048, 4096)


def test_shard_covers_everything():
    for n in (0, 1, 7, 4096, 4097):
        for w in (1, 2, 3, 8):
            parts = [replicas.shard(n, r, w) for r in range(w)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[k][1] == parts[k + 1][0] for k in range(w - 1))
            assert max(h - l for l, h in parts) - min(h - l for l, h in parts) <= 1


def test_single_process_is_identity(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert replicas.init() == (0, 1, 0)
    assert replicas.max_over_ranks(3.0) == 3.0

"""A system's sinks partitioned over two gloo ranks on the CPU
(solaris_gb300.sharded): each rank evaluates GravityAC for its own block of
sinks against every source (the oracle restatement of Acceleration.cpp:
248-329 restricted to the block), the blocks' positions are all-gathered at
every stage, and after several RungeKutta4 driver calls the concatenated
state equals the single-process RK4 driver's bit for bit.  The ensemble's
systems, sharded the same way, are covered exactly once."""
import os
import socket

import numpy as np
import pytest

from solaris_gb300 import abi, replicas, scenarios


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleSinks:
    """The sinks [lo, hi) of a system evaluated by the oracle on the host
    (the CPU stand-in of DeviceSinks)."""

    def __init__(self, system, lo, hi):
        import oracle
        self.o = oracle.Oracle(system)
        self.lo, self.hi = lo, hi

    def zeros(self, n):
        return np.zeros(n)

    def accel(self, t, y_all):
        d, _ = self.o.gravity_sample(y_all, self.lo, self.hi)
        return d.reshape(-1, 6)[self.lo:self.hi]


def _system():
    # 1 star + giants + protoplanets + planetesimals: sources and sink-only
    # bodies on both ranks
    s = scenarios.mixed_gas_system(seed=3101, n_spl=0, n_pl=60, n_tp=20, n_proto=40)
    s.gas = None
    return s


def _worker(rank, world, port, n_steps, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from solaris_gb300 import sharded
    replicas.init(backend="gloo")
    s = _system()
    sh = sharded.ShardedRK4(s, backend_factory=OracleSinks)
    sh.set_state(s.y0)
    t = sh.step(0.0, s.h0 * 200, n_steps)
    y = sh.get_state()
    lo, hi = replicas.shard(4096, rank, world)
    out.put((rank, t, y, (sh.lo, sh.hi), (lo, hi)))
    replicas.finalize()


@pytest.mark.parametrize("world", [2, 4])
def test_ranks_equal_the_single_process_driver(world):
    """Two ranks, and four with sink blocks of uneven size (123 bodies: 31,
    31, 31, 30; the all-gather pads them to the largest block)."""
    torch = pytest.importorskip("torch")
    import oracle
    s = _system()
    n_steps = 6
    ref = oracle.Oracle(s).driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0 * 200, n_steps)
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    ps = [mp.Process(target=_worker, args=(r, world, port, n_steps, q)) for r in range(world)]
    for p in ps:
        p.start()
    res = sorted((q.get(timeout=300) for _ in ps), key=lambda r: r[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    blocks = [r[3] for r in res]
    assert blocks[0][0] == 0 and blocks[-1][1] == s.n
    assert all(blocks[k][1] == blocks[k + 1][0] for k in range(world - 1))
    if world == 4:
        assert len({hi - lo for lo, hi in blocks}) > 1
    for _, t, y, _, _ in res:
        assert t == ref["tl"][0]
        assert np.array_equal(y.view(np.uint64), ref["y0"].view(np.uint64))
    systems = [r[4] for r in res]
    covered = np.zeros(4096, int)
    for lo, hi in systems:
        covered[lo:hi] += 1
    assert (covered == 1).all()


def test_single_process_sharded_driver_is_the_plain_driver():
    import oracle
    from solaris_gb300 import sharded
    s = _system()
    sh = sharded.ShardedRK4(s, backend_factory=OracleSinks)
    sh.set_state(s.y0)
    sh.step(0.0, s.h0 * 200, 3)
    ref = oracle.Oracle(s).driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0 * 200, 3)
    assert np.array_equal(sh.get_state().view(np.uint64), ref["y0"].view(np.uint64))

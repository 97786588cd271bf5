"""The device side of a sink-partitioned system, on one GPU.

sol_accel_sinks_device evaluates the sinks of a block against every
source: the blocks of a partition, evaluated one after the other into one
buffer, give the whole evaluation's rows bit for bit (FP64, SPLIT and
SPLIT_FF; the split forms sum each sink's sources in the same order
whatever the block).  solaris_gb300.sharded's RK4 driver with the device
backend, in one process, equals the context's own RungeKutta4 driver bit for
bit.  The exchange between ranks is covered with gloo on the CPU
(tests/test_cpu_sharded.py)."""
import numpy as np
import pytest

from solaris_gb300 import abi, engine, replicas, scenarios

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [3001, 20000])
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_SPLIT, abi.PRECISION_SPLIT_FF])
def test_sink_blocks_equal_the_whole_evaluation(n, precision):
    torch = pytest.importorskip("torch")
    s = scenarios.config3(seed=515, n=n)
    with engine.Context(s, precision=precision) as ctx:
        whole, rm3, nn, nd = ctx.accel(0.0, s.y0)
        dev = torch.device("cuda", 0)
        y = torch.from_numpy(s.y0.copy()).to(dev)
        out = torch.full((6 * s.n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        for r in range(3):
            lo, hi = replicas.shard(s.n, r, 3)
            abi.check(ctx.lib, ctx.lib.sol_accel_sinks_device(ctx.h, 0.0, y.data_ptr(), lo, hi, out.data_ptr()))
            rm3_b, nn_b, nd_b = ctx.last_eval()
            assert np.array_equal(nn_b[lo:hi], nn[lo:hi])
            assert np.array_equal(nd_b[lo:hi].view(np.uint64), nd[lo:hi].view(np.uint64))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
    assert np.array_equal(got.view(np.uint64), whole.view(np.uint64))


def test_sharded_rk4_on_one_gpu_is_the_rk4_driver():
    pytest.importorskip("torch")
    from solaris_gb300 import sharded
    s = scenarios.config3(seed=516, n=5000)
    h = s.h0 * 100
    sh = sharded.ShardedRK4(s)
    try:
        sh.set_state(s.y0)
        sh.step(0.0, h, 4)
        y = sh.get_state()
    finally:
        sh.close()
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        ctx.driver(abi.RUNGE_KUTTA4, 0.0, h, 4)
        ref = ctx.get_state()
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64))

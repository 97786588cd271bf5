"""sol_gravity_noalloc: the force evaluation for callers that cannot allocate
device memory (a host framework that owns all device memory, a fixed-budget
plugin, a real-time loop).  It must give the same results as the context
entry point, sol_accel_compute, call after call, although its scratch array
is shared between calls and keeps the previous call's contents.  This file is
collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

from solaris_gb300 import abi, build, engine, scenarios

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_SPLIT])
def test_noalloc_matches_context_on_two_calls(precision):
    torch = pytest.importorskip("torch")
    build.build()
    lib = abi.load_library()
    s = scenarios.config3(seed=9001, n=3001)
    states = [s.y0, s.y0 * (1.0 + 1.0e-3)]
    with engine.Context(s, precision=precision) as ctx:
        refs = [ctx.accel(0.0, y) for y in states]
    dev = torch.device("cuda", 0)
    n = s.n
    d_type = torch.from_numpy(s.type.astype(np.int32)).to(dev)
    d_mass = torch.from_numpy(s.mass.copy()).to(dev)
    d_y = torch.empty(6 * n, dtype=torch.float64, device=dev)
    d_dydt = torch.empty(6 * n, dtype=torch.float64, device=dev)
    d_rm3 = torch.empty(n, dtype=torch.float64, device=dev)
    d_nn = torch.empty(n, dtype=torch.int32, device=dev)
    d_nd = torch.empty(n, dtype=torch.float64, device=dev)
    counts = abi.SolNBodies(*s.counts)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for y, (dydt, rm3, nn, nd) in zip(states, refs):
        d_y.copy_(torch.from_numpy(y))
        for t in (d_dydt, d_rm3, d_nd):
            t.fill_(float("nan"))  # anything left unwritten shows up
        d_nn.fill_(-7)
        rc = lib.sol_gravity_noalloc(C.byref(counts), d_type.data_ptr(), d_mass.data_ptr(), d_y.data_ptr(),
                                     d_dydt.data_ptr(), d_rm3.data_ptr(), d_nn.data_ptr(), d_nd.data_ptr(),
                                     int(precision), stream)
        assert rc == abi.SOL_OK, lib.sol_last_error()
        torch.cuda.synchronize(dev)
        got = d_dydt.cpu().numpy()
        if precision == abi.PRECISION_FP64:
            # the reference arithmetic in the same order as the context path: identical bits
            assert np.array_equal(_bits(got), _bits(dydt))
        else:
            # the split form sums in a different order than the context's
            # chunked kernel: the split bound of the other tests, 1e-12
            a, b = got.reshape(-1, 6)[1:, 3:], dydt.reshape(-1, 6)[1:, 3:]
            rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
            assert rel.max() <= 1e-12
            assert np.array_equal(_bits(got.reshape(-1, 6)[:, :3]), _bits(dydt.reshape(-1, 6)[:, :3]))
        assert np.array_equal(_bits(d_rm3.cpu().numpy()), _bits(rm3))
        assert np.array_equal(d_nn.cpu().numpy(), nn)
        assert np.array_equal(_bits(d_nd.cpu().numpy()), _bits(nd))


def test_noalloc_rejects_more_bodies_than_its_scratch_holds():
    build.build()
    lib = abi.load_library()
    counts = abi.SolNBodies(1, 0, 0, 16384, 0, 0, 0)  # 16,385 bodies
    rc = lib.sol_gravity_noalloc(C.byref(counts), 1, 1, 1, 1, 1, 1, 1, abi.PRECISION_FP64, None)
    assert rc == abi.SOL_ERR_ARG
    assert b"16384" in lib.sol_last_error()

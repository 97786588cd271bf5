"""sol_gravity_noalloc: the force evaluation for callers that cannot allocate
device memory (a host framework that owns all device memory, a fixed-budget
plugin, a real-time loop).  It must give the same results as the context
entry point, sol_accel_compute, call after call, although its scratch array
is shared between calls and keeps the previous call's contents: at its full
capacity of 16,384 bodies, and after calls of another size or precision.
sol_gravity_noalloc_status reports each call's device status.  This file is
collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

from solaris_gb300 import abi, build, engine, scenarios

pytestmark = pytest.mark.gpu

CAPACITY = 16384


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


class NoAlloc:
    """Caller-owned device buffers (torch) for systems of up to CAPACITY
    bodies, and one sol_gravity_noalloc call on a given state."""

    def __init__(self):
        self.torch = pytest.importorskip("torch")
        build.build()
        self.lib = abi.load_library()
        torch, dev = self.torch, self.torch.device("cuda", 0)
        self.dev = dev
        self.d_type = torch.empty(CAPACITY, dtype=torch.int32, device=dev)
        self.d_mass = torch.empty(CAPACITY, dtype=torch.float64, device=dev)
        self.d_y = torch.empty(6 * CAPACITY, dtype=torch.float64, device=dev)
        self.d_dydt = torch.empty(6 * CAPACITY, dtype=torch.float64, device=dev)
        self.d_rm3 = torch.empty(CAPACITY, dtype=torch.float64, device=dev)
        self.d_nn = torch.empty(CAPACITY, dtype=torch.int32, device=dev)
        self.d_nd = torch.empty(CAPACITY, dtype=torch.float64, device=dev)
        self.stream = torch.cuda.current_stream(dev).cuda_stream

    def call(self, s, y, precision):
        torch, n = self.torch, s.n
        self.d_type[:n].copy_(torch.from_numpy(s.type.astype(np.int32)))
        self.d_mass[:n].copy_(torch.from_numpy(s.mass.copy()))
        self.d_y[: 6 * n].copy_(torch.from_numpy(np.ascontiguousarray(y)))
        for t in (self.d_dydt, self.d_rm3, self.d_nd):
            t.fill_(float("nan"))  # anything left unwritten shows up
        self.d_nn.fill_(-7)
        counts = abi.SolNBodies(*s.counts)
        rc = self.lib.sol_gravity_noalloc(C.byref(counts), self.d_type.data_ptr(), self.d_mass.data_ptr(),
                                          self.d_y.data_ptr(), self.d_dydt.data_ptr(), self.d_rm3.data_ptr(),
                                          self.d_nn.data_ptr(), self.d_nd.data_ptr(), int(precision), self.stream)
        assert rc == abi.SOL_OK, self.lib.sol_last_error()
        word = C.c_int32(-1)
        status = self.lib.sol_gravity_noalloc_status(self.stream, C.byref(word))
        return status, word.value, (self.d_dydt[: 6 * n].cpu().numpy(), self.d_rm3[:n].cpu().numpy(),
                                    self.d_nn[:n].cpu().numpy(), self.d_nd[:n].cpu().numpy())


def _context_eval(s, y, precision):
    with engine.Context(s, precision=precision) as ctx:
        return ctx.accel(0.0, y)


def _assert_matches(got, ref, precision):
    dydt, rm3, nn, nd = got
    r_dydt, r_rm3, r_nn, r_nd = ref
    if precision == abi.PRECISION_FP64:
        # the reference arithmetic in the same order as the context path: identical bits
        assert np.array_equal(_bits(dydt), _bits(r_dydt))
    else:
        # the split form sums in a different order than the context's kernels:
        # the split bound of the other tests, 1e-12 relative
        a, b = dydt.reshape(-1, 6)[1:, 3:], r_dydt.reshape(-1, 6)[1:, 3:]
        rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
        assert rel.max() <= 1e-12
        assert np.array_equal(_bits(dydt.reshape(-1, 6)[:, :3]), _bits(r_dydt.reshape(-1, 6)[:, :3]))
    assert np.array_equal(_bits(rm3), _bits(r_rm3))
    assert np.array_equal(nn, r_nn)
    assert np.array_equal(_bits(nd), _bits(r_nd))


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_SPLIT])
def test_noalloc_matches_context_on_two_calls(precision):
    na = NoAlloc()
    s = scenarios.config3(seed=9001, n=3001)
    for y in (s.y0, s.y0 * (1.0 + 1.0e-3)):
        status, word, got = na.call(s, y, precision)
        assert status == abi.SOL_OK and word == 0, na.lib.sol_last_error()
        _assert_matches(got, _context_eval(s, y, precision), precision)


def test_noalloc_at_capacity_then_smaller_then_other_precision():
    """Full scratch (16,384 bodies: every source-table row and prepass
    partial slot in use), then a smaller system whose padded size is
    different, then the other precision: stale contents never leak in."""
    na = NoAlloc()
    big = scenarios.config3(seed=9002, n=CAPACITY)
    small = scenarios.config3(seed=9003, n=1000)
    for s, prec in ((big, abi.PRECISION_FP64), (small, abi.PRECISION_FP64), (big, abi.PRECISION_SPLIT),
                    (small, abi.PRECISION_SPLIT), (big, abi.PRECISION_FP64)):
        status, word, got = na.call(s, s.y0, prec)
        assert status == abi.SOL_OK and word == 0, na.lib.sol_last_error()
        _assert_matches(got, _context_eval(s, s.y0, prec), prec)


def test_noalloc_status_reports_a_wait_that_ran_out():
    """A source tile withheld (sol_set_wait_test) makes the bulk-copy wait of
    every CTA run out after 4,096 polls: the kernel returns, the status query
    says SOL_ERR_TIMEOUT, and the next call is correct again."""
    na = NoAlloc()
    s = scenarios.config3(seed=9004, n=2000)
    assert na.lib.sol_set_wait_test(None, 4096, 1) == abi.SOL_OK
    try:
        status, word, _ = na.call(s, s.y0, abi.PRECISION_FP64)
    finally:
        assert na.lib.sol_set_wait_test(None, 0, -1) == abi.SOL_OK
    assert status == abi.SOL_ERR_TIMEOUT and word != 0
    assert b"ran out" in na.lib.sol_last_error()
    status, word, got = na.call(s, s.y0, abi.PRECISION_FP64)
    assert status == abi.SOL_OK and word == 0
    _assert_matches(got, _context_eval(s, s.y0, abi.PRECISION_FP64), abi.PRECISION_FP64)


def test_noalloc_rejects_more_bodies_than_its_scratch_holds():
    build.build()
    lib = abi.load_library()
    counts = abi.SolNBodies(1, 0, 0, CAPACITY, 0, 0, 0)  # 16,385 bodies
    rc = lib.sol_gravity_noalloc(C.byref(counts), 1, 1, 1, 1, 1, 1, 1, abi.PRECISION_FP64, None)
    assert rc == abi.SOL_ERR_ARG
    assert b"16384" in lib.sol_last_error()

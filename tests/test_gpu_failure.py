"""Failure paths, reached without faulting or hanging the GPU.

* A bounded device wait that runs out: one CTA of the group driver is kept
  from arriving at the group barrier (sol_set_wait_test) and the others give
  up after a short spin limit.  The launch returns, sol_driver reports
  SOL_ERR_TIMEOUT, and the same context then integrates bit for bit like a
  fresh one.
* Non-finite values injected into the host state before sol_set_state: the
  device drivers follow RungeKuttaFehlberg78::GetErrorMax, whose comparison
  `err > errorMax` never takes a NaN (RungeKuttaFehlberg78.cpp:252-262).
* The Driver's retry loop ending in the step-size underflow error
  (RungeKuttaFehlberg78.cpp:108-122).
Each is checked against the oracle.
"""
import ctypes as C
import time

import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu

RKF78 = abi.RUNGE_KUTTA_FEHLBERG78


def _same(a, b):
    """Bit-identical where finite; NaN where the other is NaN (NaN payloads
    differ between the CPU and the GPU)."""
    a, b = np.asarray(a), np.asarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint64), b[~nb].view(np.uint64))


def test_group_barrier_timeout_is_reported_and_the_context_recovers():
    s = scenarios.config1()  # 253 test particles: 16 CTAs in the group driver
    with engine.Context(s) as ctx, engine.Context(s) as fresh:
        ctx.set_state(s.y0)
        ctx.set_wait_test(4096, 0)  # CTA 0 never arrives; the others give up after 4,096 polls
        t0 = time.perf_counter()
        with pytest.raises(abi.SolError) as err:
            ctx.driver(RKF78, 0.0, s.h0, 5)
        assert err.value.code == abi.SOL_ERR_TIMEOUT
        assert "ran out" in str(err.value)
        assert time.perf_counter() - t0 < 60.0
        ctx.set_wait_test(0, -1)
        ctx.set_state(s.y0)
        fresh.set_state(s.y0)
        r1 = ctx.driver(RKF78, 0.0, s.h0, 20)
        r2 = fresh.driver(RKF78, 0.0, s.h0, 20)
        assert r1["stats"] == r2["stats"]
        assert (r1["time"], r1["h_next"]) == (r2["time"], r2["h_next"])
        assert np.array_equal(ctx.get_state().view(np.uint64), fresh.get_state().view(np.uint64))


def _inject(s, case):
    """Host state with a non-finite entry planted: NaN position and velocity
    of a test particle (it attracts nobody), NaN position of a giant (every
    body's acceleration turns NaN), an infinite velocity of a test particle."""
    y0 = s.y0.copy()
    if case == "nan_test_particle":
        k = s.n - 5
        y0[6 * k + 0] = np.nan
        y0[6 * k + 4] = np.nan
    elif case == "nan_giant":
        y0[6 * 1 + 1] = np.nan
    elif case == "inf_velocity":
        y0[6 * (s.n - 3) + 3] = np.inf
    return y0


@pytest.mark.parametrize("device_loop", [True, False])
@pytest.mark.parametrize("case", ["nan_test_particle", "nan_giant", "inf_velocity"])
def test_non_finite_state_follows_the_error_norm_comparison(case, device_loop):
    """NaN error entries never become errorMax: a NaN test particle leaves
    every other body stepping exactly as without it; a NaN giant makes every
    entry NaN, errorMax 0 and every step 5 h (ERRCON branch); an infinite
    velocity turns that body NaN at the first stage.  Step counts, time line
    and state (NaN where the oracle has NaN) equal the oracle's, in the group
    driver and in the host-driven attempt loop."""
    s = scenarios.config1()
    y0 = _inject(s, case)
    ro = oracle.Oracle(s).driver(RKF78, y0, 0.0, s.h0, 12)
    assert ro["status"] == abi.SOL_OK
    with engine.Context(s) as ctx:
        ctx.set_device_loop(device_loop)
        ctx.set_state(y0)
        r = ctx.driver(RKF78, 0.0, s.h0, 12)
        y = ctx.get_state()
    assert r["stats"][:2] == ro["stats"][:2]
    assert (r["time"], r["h_next"]) == ro["tl"][:2]
    assert _same(y, ro["y0"])
    if case == "nan_test_particle":
        clean = oracle.Oracle(s).driver(RKF78, s.y0, 0.0, s.h0, 12)
        assert clean["stats"] == ro["stats"] and clean["tl"] == ro["tl"]


def test_step_size_underflow_at_a_time_beyond_the_step_resolution():
    """At t = 1e19 days a double resolves 2,048 days: a first step of 1e5
    days is rejected, the shrunken step no longer changes t (t + h == t) and
    the driver stops with the reference's 'Stepsize-underflow' error
    (RungeKuttaFehlberg78.cpp:116-122) after the oracle's number of
    rejections, leaving the time where it was."""
    s = scenarios.config1()
    t, h = 1.0e19, 1.0e5
    ro = oracle.Oracle(s).driver(RKF78, s.y0, t, h, 1)
    assert ro["status"] == abi.SOL_ERR_UNDERFLOW
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(t, h, 0.0)
        st = abi.SolStepStats()
        rc = ctx.lib.sol_driver(ctx.h, RKF78, C.byref(tl), 1, C.byref(st))
        assert rc == abi.SOL_ERR_UNDERFLOW
        assert b"underflow" in ctx.lib.sol_last_error()
    assert (st.accepted, st.rejected) == ro["stats"][:2]
    assert tl.time == t

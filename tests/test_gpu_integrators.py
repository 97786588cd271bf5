"""Integrator drivers on the GPU against fixtures produced by the reference.

With the FP64 force the stage sums, final sums and error estimates follow
the reference's operation order and are bit-identical per attempt.  The step
controls' powers (pow(errorMax, -0.2 / -0.25), pow(eps / errorMax, 1/7)) are
correctly rounded on the device; libm's pow is too but for ~8e-4 of its
calls, so driver calls agree bit for bit and long adaptive runs until the
reference's pow first misrounds.  Gas drag and migration use CUDA's pow /
exp / log10, whose last bit may differ from glibc: those systems are
compared to a tolerance."""
import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

from golden_io import load, system_from

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def body_rel(a, b):
    """Per body, the larger of |dr|/|r| and |dv|/|v| (components near zero make
    per-component relative errors meaningless).  Bodies that are non-finite
    must be non-finite in both (explicit steps through stiff Epstein drag blow
    up in the reference too); they count as 0."""
    a, b = np.asarray(a).reshape(-1, 6), np.asarray(b).reshape(-1, 6)
    fa, fb = np.isfinite(a).all(1), np.isfinite(b).all(1)
    assert np.array_equal(fa, fb), "non-finite bodies differ"
    a, b = np.where(fa[:, None], a, 0.0), np.where(fb[:, None], b, 0.0)
    out = np.zeros(len(a))
    for sl in (slice(0, 3), slice(3, 6)):
        num = np.linalg.norm(a[:, sl] - b[:, sl], axis=1)
        den = np.linalg.norm(b[:, sl], axis=1)
        out = np.maximum(out, np.where(den > 0, num / np.where(den > 0, den, 1), num))
    return out


def test_rkf78_attempt_bit_exact_config1():
    d = load("rkf78_step_config1")
    s = system_from(d)
    with engine.Context(s) as ctx:
        y, err, em = ctx.rkf78_step(float(d["meta_t"]), float(d["meta_h"]), s.y0)
    assert np.array_equal(bits(y), bits(d["out_y"]))
    assert np.array_equal(bits(err), bits(d["out_error"]))
    assert np.array_equal(bits([em]), bits(d["out_error_max"]))


def test_rkf78_attempt_mixed_gas():
    """With gas drag the forces carry CUDA-vs-glibc pow/exp rounding (1e-16
    relative); the error estimate h |f0 + f10 - f11 - f12| 41/840 is a
    cancellation that amplifies it, so errorMax is compared loosely."""
    d = load("rkf78_step_mixed_gas")
    s = system_from(d)
    with engine.Context(s) as ctx:
        y, err, em = ctx.rkf78_step(float(d["meta_t"]), float(d["meta_h"]), s.y0)
    assert body_rel(y, d["out_y"]).max() <= 1e-12
    ref_em = float(d["out_error_max"][0])
    assert abs(em - ref_em) <= 1e-3 * ref_em


def test_rk4_driver_bit_exact_against_reference():
    """30 RungeKutta4 driver calls reproduce the reference build bit for bit."""
    d = load("rk4_driver_selfgrav64")
    s = system_from(d)
    n = int(d["meta_nsteps"])
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(float(d["meta_t"]), float(d["meta_h"]), 0.0)
        times = []
        for _ in range(n):
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
            times.append(tl.time)
        y0 = ctx.get_state()
        rm3, nn, nd = ctx.last_eval()
    assert np.array_equal(bits(times), bits(d["out_time"]))
    assert np.array_equal(bits(y0), bits(d["out_y0"]))
    assert np.array_equal(nn, d["out_nn_idx"])


def _per_step(system, integrator, n_steps, h0, exact):
    """Each GPU driver call starts from the oracle's state and time line; the
    oracle is pinned bit-exactly to the reference build (test_oracle_golden)."""
    o = oracle.Oracle(system)
    y, t, h = system.y0.copy(), 0.0, h0
    with engine.Context(system) as ctx:
        for k in range(n_steps):
            ro = o.driver(integrator, y, t, h, 1)
            ctx.set_state(y)
            tl = abi.SolTimeLine(t, h, 0.0)
            r = ctx.driver(integrator, 0, 0, 1, time_line=tl)
            yg = ctx.get_state()
            assert r["stats"][:2] == ro["stats"][:2], f"step {k}: accepted/rejected differ"
            if exact:  # accepted, rejected and retried attempts alike
                assert np.array_equal(bits(yg), bits(ro["y0"])), f"step {k}"
                assert tl.time == ro["tl"][0] and tl.h_did == ro["tl"][2], f"step {k}"
                assert tl.h_next == ro["tl"][1], f"step {k}"
            else:
                # with gas drag the error norm carries pow/exp rounding amplified
                # by the cancellation in the error estimate: a retried step's h
                # (and so the time) agrees to the 1e-3 of that amplification
                assert body_rel(yg, ro["y0"]).max() <= (1e-12 if r["stats"][1] == 0 else 1e-6), f"step {k}"
                np.testing.assert_allclose(tl.time, ro["tl"][0], rtol=1e-14 if r["stats"][1] == 0 else 1e-3)
                np.testing.assert_allclose(tl.h_next, ro["tl"][1], rtol=1e-3)
            y, t, h = ro["y0"], ro["tl"][0], ro["tl"][1]
        assert np.array_equal(ctx.mig_type(), o.mig_type())


def test_rkf78_driver_per_step_config1():
    s = scenarios.config1(seed=1501)
    _per_step(s, abi.RUNGE_KUTTA_FEHLBERG78, 40, s.h0, exact=True)


def test_rkf78_driver_per_step_mixed_gas():
    s = scenarios.mixed_gas_system(seed=3300)
    _per_step(s, abi.RUNGE_KUTTA_FEHLBERG78, 25, s.h0, exact=False)


def test_rk4_driver_per_step_config1():
    """RK4 driver calls of a few-source system run in the group kernel."""
    s = scenarios.config1(seed=1503)
    _per_step(s, abi.RUNGE_KUTTA4, 20, s.h0 * 100, exact=True)


def test_rk4_driver_per_step_mixed_gas():
    """RK4 in the group kernel with drag and type I / II migration (stage times
    t + c h for the gas factor)."""
    s = scenarios.mixed_gas_system(seed=3301)
    _per_step(s, abi.RUNGE_KUTTA4, 15, s.h0 * 100, exact=False)


def test_dormand_prince_driver_per_step_config1():
    s = scenarios.config1(seed=1502)
    _per_step(s, abi.DORMAND_PRINCE, 20, s.h0 * 50, exact=True)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_SPLIT])
def test_rkf78_long_run_statistics(precision):
    """500 device-driven RKF78 steps (device-side accept/reject).  Adaptive
    control is chaotic at the last bit and libm's pow, which the oracle and
    the reference call, is not quite correctly rounded (measured: 8e-4 of
    pow(errorMax, -0.2) calls land on the other neighbour of a near-midpoint
    value), so over ~800 calls the device's correctly rounded power parts
    from it once or so: the comparison is statistical, step counts and
    reached time agree to a few per cent.  (The heliocentric energy of
    Calculate::Integrals is not a conserved quantity, the frame being
    non-inertial.)"""
    s = scenarios.config1(seed=1501)
    o = oracle.Oracle(s)
    ref = o.driver(abi.RUNGE_KUTTA_FEHLBERG78, s.y0, 0.0, s.h0, 500)
    with engine.Context(s, precision=precision) as ctx:
        ctx.set_state(s.y0)
        r = ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, s.h0, 500)
        y = ctx.get_state()
    assert r["stats"][0] == 500
    assert abs(r["stats"][1] - ref["stats"][1]) <= max(3, 0.1 * ref["stats"][1])
    assert abs(r["time"] - ref["tl"][0]) <= 0.05 * ref["tl"][0]
    assert np.isfinite(y).all()


def test_rk4_full_size_bit_exact_two_steps():
    """Two RK4 steps of 8,192 self-gravitating bodies: FP64 stays bit-identical
    to the oracle (no pow in RK4)."""
    s = scenarios.config3(n=8192)
    o = oracle.Oracle(s)
    ref = o.driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0, 2)
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        ctx.driver(abi.RUNGE_KUTTA4, 0.0, s.h0, 2)
        y = ctx.get_state()
    assert np.array_equal(bits(y), bits(ref["y0"]))


def test_underflow_is_reported():
    """A tolerance no step can meet shrinks h until t + h == t and the driver
    returns SOL_ERR_UNDERFLOW (RungeKuttaFehlberg78.cpp:116-122)."""
    s = scenarios.config3(seed=77, n=17)
    with engine.Context(s) as ctx:
        ctx.set_tolerance(1e-300)
        ctx.set_state(s.y0)
        with pytest.raises(abi.SolError) as ei:
            ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 1.0e6, 1.0, 1)
        assert ei.value.code == abi.SOL_ERR_UNDERFLOW


@pytest.mark.parametrize("integrator", [abi.RUNGE_KUTTA_FEHLBERG78, abi.DORMAND_PRINCE])
def test_device_loop_matches_host_loop(integrator):
    """The CUDA-graph driver (attempt loop in a conditional WHILE node on the
    device) runs the same kernels in the same order as the host-driven loop:
    identical bits, identical step counts."""
    s = scenarios.config1(seed=1601)
    h0 = s.h0 if integrator == abi.RUNGE_KUTTA_FEHLBERG78 else s.h0 * 50
    out = {}
    for loop in (1, 0):
        with engine.Context(s) as ctx:
            ctx.set_device_loop(loop)
            ctx.set_state(s.y0)
            r = ctx.driver(integrator, 0.0, h0, 120)
            out[loop] = (ctx.get_state(), r["time"], r["h_next"], r["stats"])
    assert np.array_equal(bits(out[1][0]), bits(out[0][0]))
    assert out[1][1:] == out[0][1:]
    assert out[1][3][1] > 0  # the run exercised rejected attempts


@pytest.mark.parametrize("case", ["mixed_gas", "config2", "many_sources"])
def test_persistent_and_graph_drivers_match_host_loop(case):
    """Few-source systems run their RKF78 driver calls in one cooperative
    launch (one thread per body, a grid barrier per stage); systems with more
    sources run the CUDA-graph driver.  Either way: the bits, step counts,
    time line, last evaluation (rm3, nearest neighbours) and migType of the
    host-driven loop."""
    if case == "mixed_gas":
        s, n = scenarios.mixed_gas_system(seed=3300), 30
    elif case == "config2":
        s, n = scenarios.config2(n_pl=3000), 12
    else:
        s, n = scenarios.config3(seed=1602, n=300), 10
        s.integrator = abi.RUNGE_KUTTA_FEHLBERG78
    out = {}
    for loop in (1, 0):
        with engine.Context(s) as ctx:
            ctx.set_tolerance(s.epsilon)
            ctx.set_device_loop(loop)
            ctx.set_state(s.y0)
            r = ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, s.h0, n)
            out[loop] = (ctx.get_state(), (r["time"], r["h_next"], r["h_did"]), r["stats"], ctx.last_eval(),
                         ctx.mig_type())
    g, hst = out[1], out[0]
    assert np.array_equal(bits(g[0]), bits(hst[0]))
    assert g[1] == hst[1] and g[2] == hst[2]
    for a, b in zip(g[3], hst[3]):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))
    assert np.array_equal(g[4], hst[4])


def test_device_loop_reports_underflow():
    s = scenarios.config3(seed=78, n=17)
    with engine.Context(s) as ctx:
        ctx.set_device_loop(1)
        ctx.set_tolerance(1e-300)
        ctx.set_state(s.y0)
        with pytest.raises(abi.SolError) as ei:
            ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 1.0e6, 1.0, 3)
        assert ei.value.code == abi.SOL_ERR_UNDERFLOW

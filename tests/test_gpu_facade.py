"""The C++ class facade (Acceleration, RungeKuttaFehlberg78, RungeKutta4,
DormandPrince with the reference's interface) driven from C++ as the
reference's Simulator drives its classes: against the oracle (pinned to the
reference build) and against the C-ABI engine."""
import numpy as np
import pytest

import oracle
from facade_io import compile_program, run
from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu


def bits(a):
    return np.asarray(a, np.float64).view(np.uint64)


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return compile_program(str(tmp_path_factory.mktemp("facade")))


def test_compute_terms_and_step_match_the_oracle(exe, tmp_path):
    s = scenarios.config1(n_tp=61)
    out = run(exe, str(tmp_path), s, abi.RUNGE_KUTTA4, 0, 0.0, s.h0)
    assert out["compute_status"][0] == 0, out.get("compute_status_msg")
    o = oracle.Oracle(s)
    d = o.compute(0.0, s.y0)
    rm3, nn, nd = o.last_eval()
    assert np.array_equal(bits(out["compute_dydt"]), bits(d))
    assert np.array_equal(bits(out["compute_rm3"]), bits(rm3))
    assert np.array_equal(out["compute_nn_idx"], nn)
    assert np.array_equal(bits(out["compute_nn_dist"]), bits(nd))
    # GravityAC alone equals Compute without a nebula
    assert np.array_equal(bits(out["gravity"]), bits(d))
    # RungeKuttaFehlberg78::Step from BodyData's y0 and accel, and GetErrorMax
    y, err, _ = o.rkf78_step(0.0, s.h0, s.y0)
    assert np.array_equal(bits(out["step_y"]), bits(y))
    assert np.array_equal(bits(out["step_error"]), bits(err))
    yscale = np.abs(s.y0) + np.abs(s.h0 * d) + 1.0e-30
    assert out["step_error_max"][0] == np.max(np.abs(err / yscale)) / 1.0e-10
    assert out["dp_error_max"][0] == np.max(np.abs(err))


def test_rk4_driver_matches_the_oracle_bit_for_bit(exe, tmp_path):
    s = scenarios.config1(n_tp=61)
    out = run(exe, str(tmp_path), s, abi.RUNGE_KUTTA4, 12, 0.0, s.h0)
    assert out["drv_status"][0] == 0, out.get("drv_status_msg")
    o = oracle.Oracle(s)
    ro = o.driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0, 12)
    assert np.array_equal(bits(out["drv_y0"]), bits(ro["y0"]))
    assert np.array_equal(bits(out["drv_time"]), bits(ro["time"]))
    assert np.array_equal(bits(out["drv_h_did"]), bits(ro["h_did"]))
    # rm3 and nearest neighbours of the last evaluation (stage 4 of the last step)
    rm3, nn, nd = o.last_eval()
    assert np.array_equal(bits(out["drv_rm3"]), bits(rm3))
    assert np.array_equal(out["drv_nn_idx"], nn)
    # BodyData and Acceleration as the reference's Driver leaves them
    assert out["drv_bd_time_h"][0] == ro["time"][-1] and out["drv_bd_time_h"][1] == s.h0
    assert list(out["drv_flags"]) == [1, 0, 0]
    # y holds the state before the last step (y0 / y swapped)
    prev = o.driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0, 11)["y0"]
    assert np.array_equal(bits(out["drv_y"]), bits(prev))


@pytest.mark.parametrize("integrator", [abi.RUNGE_KUTTA_FEHLBERG78, abi.DORMAND_PRINCE])
def test_adaptive_driver_matches_the_engine(exe, tmp_path, integrator):
    """The facade's Driver calls are the engine's driver calls and the
    oracle's: the same bits step after step, retried attempts included (the
    step controls' powers are correctly rounded on the device)."""
    s = scenarios.config1(n_tp=61)
    h0 = s.h0 * (50 if integrator == abi.DORMAND_PRINCE else 1)
    n = 15
    out = run(exe, str(tmp_path), s, integrator, n, 0.0, h0)
    assert out["drv_status"][0] == 0, out.get("drv_status_msg")
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, h0, 0.0)
        times = []
        for _ in range(n):
            ctx.driver(integrator, 0, 0, 1, time_line=tl)
            times.append(tl.time)
        y = ctx.get_state()
    assert np.array_equal(bits(out["drv_y0"]), bits(y))
    assert np.array_equal(bits(out["drv_time"]), bits(times))
    ro = oracle.Oracle(s).driver(integrator, s.y0, 0.0, h0, n)
    assert np.array_equal(bits(out["drv_y0"]), bits(ro["y0"]))
    assert out["drv_time"][-1] == ro["tl"][0]


def test_body_removal_between_driver_calls(exe, tmp_path):
    """Simulator::RemoveBody compacts BodyData between Driver calls; the facade
    notices and rebuilds its context."""
    s = scenarios.config1(n_tp=40)
    k, n1, n2 = 17, 4, 4
    out = run(exe, str(tmp_path), s, abi.RUNGE_KUTTA4, n1, 0.0, s.h0, remove=k, n_steps2=n2)
    assert out["drv2_status"][0] == 0, out.get("drv2_status_msg")
    o = oracle.Oracle(s)
    y = o.driver(abi.RUNGE_KUTTA4, s.y0, 0.0, s.h0, n1)["y0"]
    keep = np.arange(s.n) != k
    counts = list(s.counts)
    counts[int(s.type[k]) - 1] -= 1
    r = scenarios.System(name="removed", counts=tuple(counts), id=s.id[keep], type=s.type[keep],
                         mig_type=s.mig_type[keep], mig_stop_at=s.mig_stop_at[keep], mass=s.mass[keep],
                         radius=s.radius[keep], density=s.density[keep], cd=s.cd[keep],
                         gamma_stokes=s.gamma_stokes[keep], gamma_epstein=s.gamma_epstein[keep],
                         y0=y.reshape(-1, 6)[keep].reshape(-1), h0=s.h0)
    ro = oracle.Oracle(r).driver(abi.RUNGE_KUTTA4, r.y0, n1 * s.h0, s.h0, n2)
    assert np.array_equal(bits(out["drv2_y0"]), bits(ro["y0"]))
    assert out["drv2_y0"].size == 6 * (s.n - 1)


def test_nebula_terms_and_migration(exe, tmp_path):
    s = scenarios.mixed_gas_system()
    out = run(exe, str(tmp_path), s, abi.RUNGE_KUTTA_FEHLBERG78, 3, 0.0, s.h0)
    assert out["compute_status"][0] == 0, out.get("compute_status_msg")
    o = oracle.Oracle(s)
    d = o.compute(0.0, s.y0)
    # pow / exp / log10 in the gas terms may round differently in the last bit
    np.testing.assert_allclose(out["compute_dydt"], d, rtol=1e-12, atol=1e-300)
    assert np.array_equal(out["compute_mig_type"], o.mig_type())
    # GasDragAC alone equals the side buffer Compute left in accelGasDrag
    assert np.array_equal(bits(out["drag"]), bits(out["compute_drag"]))
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        for _ in range(3):
            ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0, 0, 1, time_line=tl)
        assert np.array_equal(bits(out["drv_y0"]), bits(ctx.get_state()))
        assert np.array_equal(out["drv_mig_type"], ctx.mig_type())


def test_split_precision_through_the_environment(exe, tmp_path):
    import os
    s = scenarios.config1(n_tp=61)
    env = dict(os.environ, SOLARIS_GB300_PRECISION="split_ff")
    out = run(exe, str(tmp_path), s, abi.RUNGE_KUTTA4, 2, 0.0, s.h0, env=env)
    d = oracle.Oracle(s).compute(0.0, s.y0)
    a, b = out["compute_dydt"].reshape(-1, 6)[1:, 3:], d.reshape(-1, 6)[1:, 3:]
    rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
    assert rel.max() <= 1e-12

"""Two configurations at their stated lengths on the device.

* 1 star + 2 giants + 8,190 planetesimals with gas drag, adaptive RKF78 at
  epsilon 1e-11, 10^4 accepted steps.  Every 1,000 steps the device state is
  handed to the oracle for one driver call (RungeKuttaFehlberg78::Driver,
  RungeKuttaFehlberg78.cpp:66-140, with Acceleration::ComputeAstroCentric's
  drag, Acceleration.cpp:166-246), which the device repeats from the same
  state: the same accept / reject sequence, the step size and the state
  within 1e-10 relative (the drag's exp / log10 / pow are CUDA's and may
  differ from glibc's in the last bit; the gravity-only arithmetic is the
  reference's bit for bit).
* The discrete adjoint of fixed-step RKF78 on 1 star + 8 planets + 1,024
  planetesimals, 10^4 steps of a tenth of the shortest period / 500 with a
  checkpoint every 100: backward within 4x the forward time, and
  directional derivatives along two random directions and two single
  coordinates against central differences of the device forward at eps =
  1e-7, within 1e-6.  The random directions move every body and their
  differences carry large truncation terms (8e-3 relative at eps, 2e-5
  after removing the eps^2 term), so they are extrapolated from eps, 2 eps
  and 4 eps, which removes the eps^2 and eps^4 terms; the single
  coordinates, whose derivatives are ~400 times smaller, are limited by
  rounding instead and take the two-point extrapolation.  With steps of the
  shortest period / 500 a planetesimal is scattered out to 49 AU during the
  10^4 steps, and finite differences of the computed map no longer track
  its exact derivative: at 7,000 such steps the oracle's FP64
  tangent-linear integration agrees with the adjoint to 3e-8 and 1.6e-6
  along a planetesimal's velocity and a planet's position while central
  differences differ by 1e-3 and 7% (tests/check_adjoint_tlm.py repeats
  that comparison).
"""
import time

import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu

RKF78 = abi.RUNGE_KUTTA_FEHLBERG78
GRAD_RTOL = 1e-6


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_config2_ten_thousand_steps_with_sampled_oracle_checks():
    s = scenarios.config2()
    o = oracle.Oracle(s)
    with engine.Context(s) as ctx, engine.Context(s) as probe:
        ctx.set_tolerance(s.epsilon)
        probe.set_tolerance(s.epsilon)
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        accepted = 0
        for chunk in range(10):
            r = ctx.driver(RKF78, 0, 0, 1000, time_line=tl)
            accepted += r["stats"][0]
            y = ctx.get_state()
            assert np.isfinite(y).all()
            # one driver call from this state on the device and in the oracle
            probe.set_state(y)
            rp = probe.driver(RKF78, tl.time, tl.h_next, 1)
            ro = o.driver(RKF78, y, tl.time, tl.h_next, 1)
            assert ro["status"] == abi.SOL_OK
            assert rp["stats"][:2] == ro["stats"][:2], chunk
            assert abs(rp["h_next"] / ro["tl"][1] - 1.0) < 1e-10, chunk
            assert _rel(probe.get_state(), ro["y0"]) < 1e-10, chunk
    assert accepted == 10000
    assert tl.time > 0.0


def _loss_grad(y, target):
    r = y.reshape(-1, 6)[:, :3] - target
    g = np.zeros_like(y).reshape(-1, 6)
    g[:, :3] = 2.0 * r
    return float((r * r).sum()), g.reshape(-1)


def test_adjoint_ten_thousand_steps():
    s = scenarios.config5()
    h, n_steps, every = s.h0 * 10, 10000, 100  # shortest period / 5,000
    rng = np.random.default_rng(1005)
    with engine.Context(s) as ctx:
        ctx.adjoint_forward(s.y0, h, 20, 10)  # warm-up
        t0 = time.perf_counter()
        y_final = ctx.adjoint_forward(s.y0, h, n_steps, every)
        tf = time.perf_counter() - t0
        target = y_final.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
        _, g = _loss_grad(y_final, target)
        t0 = time.perf_counter()
        dy0, dmass = ctx.adjoint_backward(g)
        tb = time.perf_counter() - t0
        assert tb <= 4.0 * tf, (tb, tf)

        def loss(y0, mass):
            ctx.set_masses(mass)
            yf = ctx.adjoint_forward(y0, h, n_steps, every)
            return _loss_grad(yf, target)[0]

        def central(e, dy, dm):
            return (loss(s.y0 + e * dy, s.mass + e * dm) - loss(s.y0 - e * dy, s.mass - e * dm)) / (2 * e)

        scale = np.tile([1.0, 1.0, 1.0, 1e-2, 1e-2, 1e-2], s.n)
        dirs = []
        for _ in range(2):
            v = rng.standard_normal(7 * s.n)
            v[:6] = 0.0  # the central body's state is fixed
            dirs.append((v[:6 * s.n] * scale, v[6 * s.n:] * s.mass, 3))
        for k in (6 * 3 + 1, 6 * 500 + 3):  # a planet's y, a planetesimal's vx
            dy = np.zeros(6 * s.n)
            dy[k] = scale[k]
            dirs.append((dy, np.zeros(s.n), 2))
        eps, rel = 1e-7, []
        for dy, dm, points in dirs:
            d1, d2 = central(eps, dy, dm), central(2 * eps, dy, dm)
            if points == 2:
                fd = (4.0 * d1 - d2) / 3.0
            else:
                fd = (64.0 * d1 - 20.0 * d2 + central(4 * eps, dy, dm)) / 45.0
            adj = float(dy0 @ dy + dmass @ dm)
            rel.append(abs(adj - fd) / max(abs(fd), 1e-30))
        ctx.set_masses(s.mass)
    print(f"10^4 steps: forward {tf:.1f} s, backward {tb:.1f} s; relative differences",
          " ".join(f"{r:.1e}" for r in rel))
    assert max(rel) <= GRAD_RTOL, rel

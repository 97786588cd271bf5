"""Discrete adjoint of fixed-step RKF78 (sol_adjoint_forward/backward):
gradients of L = sum |r_final - r_target|^2 with respect to the initial
positions, velocities and masses, against the oracle's FP64 tangent-linear
(variational) integration and against central finite differences."""
import time

import numpy as np
import pytest

import oracle
from solaris_gb300 import engine, scenarios

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-6  # bound on the gradient's relative error


def _system(n_pl=24, seed=1005):
    return scenarios.config5(seed=seed, n_pl=n_pl)


def _loss_grad(y, target):
    r = y.reshape(-1, 6)[:, :3] - target
    g = np.zeros_like(y).reshape(-1, 6)
    g[:, :3] = 2.0 * r
    return float((r * r).sum()), g.reshape(-1)


def _directions(s, k, rng):
    out = []
    for _ in range(k):
        dy = rng.standard_normal(6 * s.n)
        dy.reshape(-1, 6)[0] = 0.0  # the central body's state is fixed
        dy.reshape(-1, 6)[:, 3:] *= 1e-2  # velocities are ~1e-2 AU/day
        dm = rng.standard_normal(s.n) * s.mass
        out.append((dy, dm))
    return out


def test_adjoint_matches_tangent_linear_model():
    """<dL/dy0, dy> + <dL/dm, dm> equals dL/dy_final . TLM(dy, dm) for random
    directions (the TLM is the oracle's FP64 variational integration)."""
    s = _system()
    h, n_steps, every = s.h0 * 2000, 40, 7
    rng = np.random.default_rng(11)
    with engine.Context(s) as ctx:
        y_final = ctx.adjoint_forward(s.y0, h, n_steps, every)
        target = y_final.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
        L, g = _loss_grad(y_final, target)
        dy0, dmass = ctx.adjoint_backward(g)
    o = oracle.Oracle(s)
    dirs = _directions(s, 4, rng)
    for k in (0, int(np.argmax(s.mass[1:])) + 1):  # the central mass, the heaviest planet
        dm = np.zeros(s.n)
        dm[k] = s.mass[k]
        dirs.append((np.zeros(6 * s.n), dm))
    for dy, dm in dirs:
        y_o, dy_final = o.rkf78_fixed(s.y0, h, n_steps, dy, dm)
        # z coordinates near zero: the floor is relative to the orbit scale
        np.testing.assert_allclose(y_o, y_final, rtol=1e-12, atol=1e-12 * np.abs(y_o).max())
        tlm = float(g @ dy_final)
        adj = float(dy0 @ dy + dmass @ dm)
        assert abs(adj - tlm) <= GRAD_RTOL * abs(tlm), (adj, tlm)


def test_adjoint_matches_central_differences():
    """Directional derivatives along random directions and single coordinates
    (positions, velocities, masses) against central differences h = 1e-7 of
    the GPU forward itself."""
    s = _system(n_pl=40, seed=1006)
    h, n_steps, every = s.h0 * 2000, 30, 10
    rng = np.random.default_rng(12)
    with engine.Context(s) as ctx:
        y_final = ctx.adjoint_forward(s.y0, h, n_steps, every)
        target = y_final.reshape(-1, 6)[:, :3] + 1e-4 * rng.standard_normal((s.n, 3))
        _, g = _loss_grad(y_final, target)
        dy0, dmass = ctx.adjoint_backward(g)

        def loss(y0, mass):
            ctx.set_masses(mass)
            yf = ctx.adjoint_forward(y0, h, n_steps, every)
            return _loss_grad(yf, target)[0]

        eps = 1e-7
        dirs = _directions(s, 3, rng)
        # a planet position, a planetesimal position and velocity (velocities
        # scaled to their ~1e-2 AU/day magnitude so that eps stays relative)
        for idx, scale in ((6, 1.0), (6 * 9 + 1, 1.0), (6 * 20 + 4, 1e-2)):
            dy = np.zeros(6 * s.n)
            dy[idx] = scale
            dirs.append((dy, np.zeros(s.n)))
        # the central mass; a single planet's mass derivative is below the
        # differencing noise of the final positions' last bits and is checked
        # against the tangent-linear model instead
        dm = np.zeros(s.n)
        dm[0] = s.mass[0]
        dirs.append((np.zeros(6 * s.n), dm))
        for dy, dm in dirs:
            fd = (loss(s.y0 + eps * dy, s.mass + eps * dm) - loss(s.y0 - eps * dy, s.mass - eps * dm)) / (2 * eps)
            adj = float(dy0 @ dy + dmass @ dm)
            assert abs(adj - fd) <= max(GRAD_RTOL * abs(fd), 1e-12), (adj, fd)
        ctx.set_masses(s.mass)


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from solaris_gb300 import adjoint
    s = _system(n_pl=16, seed=1007)
    h, n_steps = s.h0 * 2000, 12
    with engine.Context(s) as ctx:
        y0 = torch.tensor(s.y0, dtype=torch.float64, requires_grad=True)
        m = torch.tensor(s.mass, dtype=torch.float64, requires_grad=True)
        yf = adjoint.integrate(ctx, y0, m, h, n_steps, checkpoint_every=5)
        target = yf.detach().reshape(-1, 6)[:, :3] + 1e-5
        loss = ((yf.reshape(-1, 6)[:, :3] - target) ** 2).sum()
        loss.backward()
        _, g = _loss_grad(yf.detach().numpy(), target.numpy())
        ctx.set_masses(s.mass)
        ctx.adjoint_forward(s.y0, h, n_steps, 5)
        dy0, dm = ctx.adjoint_backward(g)
    np.testing.assert_allclose(y0.grad.numpy(), dy0, rtol=1e-12, atol=0)
    np.testing.assert_allclose(m.grad.numpy(), dm, rtol=1e-12, atol=0)


def test_backward_cost_within_four_forwards():
    """Config-5 size (1 star + 8 planets + 1024 planetesimals): backward time
    with checkpoint/recompute stays within 4x the forward time."""
    s = scenarios.config5()
    h, n_steps, every = s.h0 * 100, 60, 20
    with engine.Context(s) as ctx:
        ctx.adjoint_forward(s.y0, h, 4, 2)  # warm-up
        t0 = time.perf_counter()
        yf = ctx.adjoint_forward(s.y0, h, n_steps, every)
        tf = time.perf_counter() - t0
        _, g = _loss_grad(yf, yf.reshape(-1, 6)[:, :3] + 1e-6)
        t0 = time.perf_counter()
        ctx.adjoint_backward(g)
        tb = time.perf_counter() - t0
    assert tb <= 4.0 * tf, (tb, tf)


def test_adjoint_full_size_directions():
    """The full adjoint workload (1 star + 8 planets + 1,024 planetesimals,
    h = shortest period / 500, 200 steps, target = final state + 1e-6 AU
    noise): 16 random directions and 32 single coordinates against central
    differences of the GPU forward at h = 1e-7, within 1e-6.

    Directions are in units of each coordinate's scale (positions 1 AU,
    velocities 1e-2 AU/day, masses the body's mass) with a standard normal
    component per coordinate; a direction normalised over all 7,231
    parameters moves each by ~1/85 of its scale and its derivative sinks to
    the rounding noise of the loss difference.  Along directions that move
    every body of this system the plain h = 1e-7 difference carries an h^2
    truncation error of ~1e-5 (measured: 0.137, 1.4e-3, 1.3e-5 at h = 1e-5,
    1e-6, 1e-7, while the oracle's tangent-linear model agrees with the
    adjoint to 1.3e-14), so the h = 1e-7 difference is Richardson-extrapolated
    with the 2h difference, (4 D(h) - D(2h)) / 3, which removes that term."""
    s = scenarios.config5()
    h, n_steps, every = s.h0 * 100, 200, 20
    rng = np.random.default_rng(1005)
    with engine.Context(s) as ctx:
        y_final = ctx.adjoint_forward(s.y0, h, n_steps, every)
        target = y_final.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
        _, g = _loss_grad(y_final, target)
        dy0, dmass = ctx.adjoint_backward(g)

        def loss(y0, mass):
            ctx.set_masses(mass)
            yf = ctx.adjoint_forward(y0, h, n_steps, every)
            return _loss_grad(yf, target)[0]

        scale = np.tile([1.0, 1.0, 1.0, 1e-2, 1e-2, 1e-2], s.n)
        dirs = []
        for _ in range(16):
            v = rng.standard_normal(7 * s.n)
            v[:6] = 0.0  # the central body's state is fixed
            dirs.append((v[:6 * s.n] * scale, v[6 * s.n:] * s.mass))
        for k in rng.choice(np.arange(6, 6 * s.n), 32, replace=False):
            dy = np.zeros(6 * s.n)
            dy[k] = scale[k]
            dirs.append((dy, np.zeros(s.n)))
        eps, rel = 1e-7, []

        def central(e, dy, dm):
            return (loss(s.y0 + e * dy, s.mass + e * dm) - loss(s.y0 - e * dy, s.mass - e * dm)) / (2 * e)

        for dy, dm in dirs:
            fd = (4.0 * central(eps, dy, dm) - central(2 * eps, dy, dm)) / 3.0
            adj = float(dy0 @ dy + dmass @ dm)
            rel.append((abs(adj - fd) / max(abs(fd), 1e-30), adj, fd))
        ctx.set_masses(s.mass)
    print("relative differences to central differences:", " ".join(f"{r[0]:.1e}" for r in rel))
    bad = [r for r in rel if r[0] > GRAD_RTOL]
    assert not bad, bad


def test_adjoint_full_size_against_tangent_linear_model():
    """Two random directions of the full adjoint workload (20 steps) against
    the oracle's FP64 tangent-linear integration."""
    s = scenarios.config5()
    h, n_steps, every = s.h0 * 100, 20, 5
    rng = np.random.default_rng(77)
    with engine.Context(s) as ctx:
        y_final = ctx.adjoint_forward(s.y0, h, n_steps, every)
        target = y_final.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
        _, g = _loss_grad(y_final, target)
        dy0, dmass = ctx.adjoint_backward(g)
    o = oracle.Oracle(s)
    for dy, dm in _directions(s, 2, rng):
        _, dy_final = o.rkf78_fixed(s.y0, h, n_steps, dy, dm)
        tlm = float(g @ dy_final)
        adj = float(dy0 @ dy + dmass @ dm)
        assert abs(adj - tlm) <= GRAD_RTOL * abs(tlm), (adj, tlm)

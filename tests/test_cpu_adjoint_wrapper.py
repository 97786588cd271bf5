"""solaris_gb300.adjoint (the torch.autograd.Function over the discrete
adjoint of fixed-step RKF78) on the CPU: the engine context is replaced by a
stand-in built on the oracle (the forward is the oracle's fixed-step RKF78,
RungeKuttaFehlberg78.cpp:147-250; the backward J^T w is assembled from the
oracle's tangent-linear integration, one direction per input, on a system
small enough for that).  Checked: the gradients reach the initial state and
the masses in body order, as float64 tensors, and a loss's gradient agrees
with central differences of the oracle's forward."""
import numpy as np
import pytest

from solaris_gb300 import abi, scenarios

torch = pytest.importorskip("torch")


class OracleAdjointContext:
    """The three calls adjoint.integrate makes of an engine context."""

    def __init__(self, system):
        import oracle
        self.o = oracle.Oracle(system)
        self.n = system.n

    def set_masses(self, mass):
        self.mass = np.array(mass, dtype=np.float64)
        self.o.set_masses(self.mass)

    def adjoint_forward(self, y0, h, n_steps, checkpoint_every):
        self.y0, self.h, self.n_steps = np.array(y0, dtype=np.float64), h, n_steps
        return self.o.rkf78_fixed(self.y0, h, n_steps)

    def _tangent(self, dy0, dm):
        return self.o.rkf78_fixed(self.y0, self.h, self.n_steps, dy0=dy0, dm=dm)[1]

    def adjoint_backward(self, w):
        nv = 6 * self.n
        zero_m, zero_y = np.zeros(self.n), np.zeros(nv)
        dy0 = np.array([self._tangent(np.eye(nv)[k], zero_m) @ w for k in range(nv)])
        dm = np.array([self._tangent(zero_y, np.eye(self.n)[k]) @ w for k in range(self.n)])
        return dy0, dm


def _system():
    rng = np.random.default_rng(808)
    mu = abi.GAUSS2 * 1.001

    def phase(a):
        return scenarios.elements_to_phase(np.array([mu]), np.array([a]), np.array([0.05]),
                                           np.array([0.02]), *rng.uniform(0, 2 * np.pi, (3, 1)))
    groups = [scenarios._star(),
              (abi.GIANT_PLANET, dict(mass=np.array([1e-3]), phase=phase(5.2))),
              (abi.PROTO_PLANET, dict(mass=np.array([3e-6]), phase=phase(1.0)))]
    return scenarios._assemble("adjoint_wrapper", groups)


def test_gradients_reach_state_and_masses_and_match_differences():
    from solaris_gb300 import adjoint
    s = _system()
    h, n_steps = 2.0, 20
    ctx = OracleAdjointContext(s)
    y0 = torch.tensor(s.y0, dtype=torch.float64, requires_grad=True)
    mass = torch.tensor(s.mass, dtype=torch.float64, requires_grad=True)
    y = adjoint.integrate(ctx, y0, mass, h, n_steps, checkpoint_every=5)
    assert y.dtype == torch.float64 and y.shape == (6 * s.n,)
    target = torch.tensor(s.y0, dtype=torch.float64)
    loss = ((y - target) ** 2).sum()
    loss.backward()
    assert y0.grad is not None and mass.grad is not None
    assert y0.grad.dtype == torch.float64 and mass.grad.shape == (s.n,)

    def f(yy, mm):
        ctx.set_masses(mm)
        return float(((ctx.adjoint_forward(yy, h, n_steps, 5) - s.y0) ** 2).sum())

    eps = 1e-7
    rng = np.random.default_rng(3)
    for _ in range(3):
        dy = rng.standard_normal(6 * s.n)
        dy[:6] = 0.0
        dy *= np.tile([1.0, 1.0, 1.0, 1e-2, 1e-2, 1e-2], s.n)
        fd = (f(s.y0 + eps * dy, s.mass) - f(s.y0 - eps * dy, s.mass)) / (2 * eps)
        ad = float(y0.grad.numpy() @ dy)
        assert abs(ad - fd) <= 1e-6 * abs(fd)
    # a mass change moves every body's path, so its differences need a larger
    # step to rise above rounding: 1% of the mass (truncation < 1e-6 here)
    eps_m = 1e-2
    for k in (1, 2):  # a planet's mass, by its index in the body order
        dm = np.zeros(s.n)
        dm[k] = s.mass[k]
        fd = (f(s.y0, s.mass + eps_m * dm) - f(s.y0, s.mass - eps_m * dm)) / (2 * eps_m)
        ad = float(mass.grad.numpy() @ dm)
        assert abs(ad - fd) <= 1e-6 * abs(fd)

"""The discrete adjoint against the oracle's FP64 tangent-linear integration
over a long, chaotic stretch (a check script, not part of the test suite:
the tangent-linear run takes minutes on the host cores).

    python tests/check_adjoint_tlm.py [n_steps] [threads]

The adjoint workload (1 star + 8 planets + 1,024 planetesimals, fixed-step
RKF78 at the shortest period / 500, a checkpoint every 100 steps) for
n_steps (default 7,000; a planetesimal is scattered out from step ~7,500):
the device's adjoint gradient of L = sum |r_final - r_target|^2 along a
planetesimal's velocity and a planet's position, against the same
directional derivatives from the oracle's tangent-linear integration
(orc_rkf78_fixed, RungeKuttaFehlberg78.cpp:147-250 and Acceleration.cpp:
248-329 restated, its sink loops on `threads` host threads) and against
central differences of the device forward (eps = 1e-9).  Needs a GPU.
"""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from solaris_gb300 import engine, scenarios  # noqa: E402


def main(n_steps=7000, threads=None):
    s = scenarios.config5()
    h, every, eps = s.h0 * 100, 100, 1e-9
    rng = np.random.default_rng(1005)
    dirs = {"planetesimal_vx": np.zeros(6 * s.n), "planet_y": np.zeros(6 * s.n)}
    dirs["planetesimal_vx"][6 * 500 + 3] = 1e-2
    dirs["planet_y"][6 * 3 + 1] = 1.0

    def loss_grad(y, target):
        r = y.reshape(-1, 6)[:, :3] - target
        g = np.zeros_like(y).reshape(-1, 6)
        g[:, :3] = 2.0 * r
        return float((r * r).sum()), g.reshape(-1)

    with engine.Context(s) as ctx:
        yf = ctx.adjoint_forward(s.y0, h, n_steps, every)
        target = yf.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
        _, g = loss_grad(yf, target)
        dy0, _ = ctx.adjoint_backward(g)
        fd = {k: (loss_grad(ctx.adjoint_forward(s.y0 + eps * v, h, n_steps, every), target)[0] -
                  loss_grad(ctx.adjoint_forward(s.y0 - eps * v, h, n_steps, every), target)[0]) / (2 * eps)
              for k, v in dirs.items()}
    o = oracle.Oracle(s)
    o.set_threads(threads or os.cpu_count() or 1)
    out = {}
    for k, v in dirs.items():
        _, dyf = o.rkf78_fixed(s.y0, h, n_steps, v, None)
        tlm = float(g @ dyf)
        adj = float(dy0 @ v)
        out[k] = {"adjoint": adj, "tangent_linear": tlm, "central_difference": fd[k],
                  "adjoint_vs_tlm": abs(adj - tlm) / abs(tlm), "difference_vs_tlm": abs(fd[k] - tlm) / abs(tlm)}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main(*(int(a) for a in sys.argv[1:]))

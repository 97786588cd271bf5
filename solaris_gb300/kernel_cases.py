"""One small, representative launch of each kernel family, for profilers.

    python -m solaris_gb300.kernel_cases <case>

Cases (each sized to a few hundred MB of device memory at most):
  fp64_few       k_gravity_ac_few: FP64 force, 2,048 self-gravitating bodies
  fp64_wide      k_gravity_ac_wide: FP64 force, 16,384 self-gravitating bodies
  split_ff_warp  k_pairs_few<SPLIT_FF>: float-float force, 4,096 bodies
  split_ff_2d    k_pairs<SPLIT_FF> + k_combine: float-float force, 32,768 bodies
  persistent     k_group_rkf78: 20 RKF78 driver calls of 1 star + 2 giants +
                 253 test particles in one cooperative launch
  ensemble       k_ensemble_rkf78: 2 driver calls of 512 small systems
  adjoint        k_vjp: forward and backward of 20 fixed RKF78 steps,
                 1 star + 8 planets + 1,024 planetesimals
  stages         k_stage / k_rkf78_final: the elementwise kernels of 2 RKF78
                 attempts over 1,048,576 bodies
"""
from __future__ import annotations

import sys

import numpy as np

from solaris_gb300 import abi, engine, scenarios


def run(case: str) -> None:
    if case in ("fp64_few", "fp64_wide", "split_ff_warp", "split_ff_2d"):
        n = {"split_ff_2d": 32768, "fp64_wide": 16384, "fp64_few": 2048}.get(case, 4096)
        prec = abi.PRECISION_FP64 if case.startswith("fp64") else abi.PRECISION_SPLIT_FF
        s = scenarios.config3(n=n)
        with engine.Context(s, precision=prec) as ctx:
            ctx.accel(0.0, s.y0)
    elif case == "persistent":
        s = scenarios.config1()
        with engine.Context(s) as ctx:
            ctx.set_state(s.y0)
            ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, s.h0, 20)
    elif case == "ensemble":
        systems = scenarios.config4()[:512]
        with engine.Ensemble(systems, precision=abi.PRECISION_FP64) as ens:
            ens.set_state([x.y0 for x in systems], [0.0] * len(systems), [x.h0 for x in systems])
            ens.advance(2)
    elif case == "adjoint":
        s = scenarios.config5()
        with engine.Context(s) as ctx:
            yf = ctx.adjoint_forward(s.y0, s.h0 * 100, 20, 10)
            g = np.zeros_like(yf)
            g[0::6] = 1.0
            ctx.adjoint_backward(g)
    elif case == "stages":
        s = scenarios.config3(n=1048576)
        with engine.Context(s) as ctx:
            ctx.set_state(s.y0)
            ctx.bench_stages(2)
    else:
        raise SystemExit(f"unknown case {case!r}; see the module docstring")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    run(sys.argv[1])
    print("ok", sys.argv[1])

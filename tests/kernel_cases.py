"""One representative launch of each kernel family, for profilers.

    python tests/kernel_cases.py <case>

Cases (each holds a few hundred MB of device memory at most):
  fp64_few        k_gravity_ac_few: FP64 force, 2,048 self-gravitating bodies
  fp64_wide       k_gravity_ac_wide: FP64 force, 16,384 self-gravitating bodies
  fp64_wide_65536 k_gravity_ac_wide: FP64 force at the bench size, 65,536 bodies
  split_65536     k_pairs<SPLIT> + k_combine: 65,536 bodies (bench size)
  split_ff_65536  k_split_table + k_pairs_ff + k_combine: 65,536 bodies (bench size)
  split_ff_warp   k_pairs_few<SPLIT_FF>: float-float force, one warp per sink,
                  2,048 bodies (below the 4,096 where k_pairs_ff takes over)
  split_ff_2d     k_pairs_ff + k_combine: float-float force, 32,768 bodies
  potential       k_potential_pairs: the integrals' potential energy, 65,536
                  bodies
  fp64_rate       k_fp64_rate<0,1,2>: the FP64 pipe throughput probe (DFMA,
                  DADD, DMUL chains), prints the rates and the SM clock
  fp32_rate       k_fp32_rate<0,1>: the FP32 pipe throughput probe (FFMA,
                  FFMA2 chains)
  persistent      k_group_rkf78: 20 RKF78 driver calls of 1 star + 2 giants +
                  253 test particles in one cooperative launch
  ensemble        k_ensemble_rkf78: 2 driver calls of 512 small systems
  adjoint         k_vjp: forward and backward of 20 fixed RKF78 steps,
                  1 star + 8 planets + 1,024 planetesimals
  stages          k_stage / k_rkf78_final: the elementwise kernels of 2 RKF78
                  attempts over 1,048,576 bodies
"""
from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

from solaris_gb300 import abi, engine, scenarios  # noqa: E402

FORCE_CASES = {
    "fp64_few": (2048, abi.PRECISION_FP64),
    "fp64_wide": (16384, abi.PRECISION_FP64),
    "fp64_wide_65536": (65536, abi.PRECISION_FP64),
    "split_65536": (65536, abi.PRECISION_SPLIT),
    "split_ff_65536": (65536, abi.PRECISION_SPLIT_FF),
    "split_ff_warp": (2048, abi.PRECISION_SPLIT_FF),
    "split_ff_2d": (32768, abi.PRECISION_SPLIT_FF),
}


def run(case: str) -> None:
    if case in FORCE_CASES:
        n, prec = FORCE_CASES[case]
        s = scenarios.config3(n=n)
        with engine.Context(s, precision=prec) as ctx:
            ctx.accel(0.0, s.y0)
    elif case == "potential":
        s = scenarios.config3(n=65536)
        with engine.Context(s) as ctx:
            ctx.integrals(s.y0)
    elif case == "fp64_rate":
        print(engine.fp64_pipe_rates(0))
    elif case == "fp32_rate":
        print(engine.fp32_pipe_rates(0))
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

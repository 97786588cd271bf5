"""Batched ensembles (sol_ensemble_*): many systems of uneven size, each with
its own adaptive RKF78 driver calls, in one persistent launch."""
import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _systems(k, seed=1004):
    rng = np.random.default_rng(seed)
    return [scenarios.config4_system(rng, i) for i in range(k)]


def test_fp64_ensemble_matches_single_system_path_bit_for_bit():
    """In FP64 mode a system in the ensemble evolves exactly as it does through
    the single-system context (same reference-order arithmetic, same device
    pow): identical state, time line and step counts after 12 driver calls."""
    systems = _systems(24)
    with engine.Ensemble(systems) as ens:
        ens.set_state([s.y0 for s in systems], [0.0] * len(systems), [s.h0 for s in systems])
        acc, rej, _ = ens.advance(12)
        ys, tls, st = ens.get_state()
    assert acc == 12 * len(systems) and not st.any()
    assert rej > 0  # some systems needed retries
    for k, s in enumerate(systems):
        with engine.Context(s) as ctx:
            ctx.set_state(s.y0)
            r = ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, s.h0, 12)
            y = ctx.get_state()
        assert np.array_equal(bits(ys[k]), bits(y)), f"system {k}"
        assert tls[k][0] == r["time"] and tls[k][1] == r["h_next"], f"system {k}"


def test_fp64_ensemble_first_step_against_oracle():
    """One driver call per system against the oracle (pinned to the reference
    build): bit-identical unless the call retried an attempt, where the CUDA
    pow of the shrink rule may round differently in the last bit."""
    systems = _systems(16, seed=77)
    with engine.Ensemble(systems) as ens:
        ens.set_state([s.y0 for s in systems], [0.0] * len(systems), [s.h0 for s in systems])
        ens.advance(1)
        ys, tls, _ = ens.get_state()
    for k, s in enumerate(systems):
        r = oracle.Oracle(s).driver(abi.RUNGE_KUTTA_FEHLBERG78, s.y0, 0.0, s.h0, 1)
        if r["stats"][1] == 0:
            assert np.array_equal(bits(ys[k]), bits(r["y0"])), f"system {k}"
            assert tls[k][0] == r["tl"][0]
        else:
            np.testing.assert_allclose(ys[k], r["y0"], rtol=1e-13, atol=1e-300)


def test_split_ff_ensemble_close_to_fp64():
    systems = _systems(32, seed=5)
    out = {}
    for p in (abi.PRECISION_FP64, abi.PRECISION_SPLIT_FF):
        with engine.Ensemble(systems, precision=p) as ens:
            ens.set_state([s.y0 for s in systems], [0.0] * len(systems), [s.h0 for s in systems])
            ens.advance(1)
            out[p] = ens.get_state()
    for k in range(len(systems)):
        a, b = out[abi.PRECISION_SPLIT_FF][0][k], out[abi.PRECISION_FP64][0][k]
        assert np.allclose(a, b, rtol=1e-12, atol=1e-15), f"system {k}"


def test_autotune_keeps_state_and_picks_a_shape():
    systems = _systems(64, seed=9)
    with engine.Ensemble(systems) as ens:
        ens.set_state([s.y0 for s in systems], [0.0] * len(systems), [s.h0 for s in systems])
        before = ens.get_state()
        threads, per_sm, ms = ens.autotune(steps=1)
        after = ens.get_state()
        assert threads in (64, 128, 256) and per_sm in (2, 4, 8, 16) and ms > 0
        for a, b in zip(before[0], after[0]):
            assert np.array_equal(bits(a), bits(b))
        assert before[1] == after[1]
        ens.advance(2)

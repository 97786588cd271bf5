"""The float-float pair kernel of large systems (k_pairs_ff: the SPLIT_FF form
beyond 16,384 bodies), against the reference (FP64) form on the device.

Its displacements come from each coordinate's grid triple a + b + c
(f2_grid_disp): exact for every pair at least one grid step G1 apart, which
for coordinates up to 8 AU is 2^-20 AU; closer pairs take FP64 arithmetic.
The system mixes every body class, so tiles cross the source ranges of
GravityAC (NOfMassive with or without super-planetesimals,
Acceleration.cpp:285-289) and the central body, and it plants pairs closer
than, near and farther than the grid step.  Bound: 1e-12 relative
acceleration error per body; the nearest neighbours and the velocity rows
are the reference's."""
import numpy as np
import pytest

from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu

SPLIT_RTOL = 1e-12


def _mixed_system(seed=4242, n_giant=3, n_proto=9000, n_spl=7, n_pl=6000, n_tp=5000):
    rng = np.random.default_rng(seed)
    G = abi.GAUSS2

    def phases(n, mu, a_lo, a_hi, e_max, i_max_deg):
        a = rng.uniform(a_lo, a_hi, n)
        e = rng.uniform(0, e_max, n)
        inc = rng.uniform(0, i_max_deg, n) * np.pi / 180
        ang = rng.uniform(0, 2 * np.pi, (3, n))
        return scenarios.elements_to_phase(mu * np.ones(n), a, e, inc, ang[0], ang[1], ang[2])

    pg = phases(n_giant, G * 1.001, 4.0, 7.0, 0.05, 1.0)
    pp = phases(n_proto, G, 0.5, 5.0, 0.05, 2.0)
    # close pairs among the protoplanets: 1e-9 and 3e-7 AU (FP64 branch),
    # 1.2e-6 and 5e-6 AU (float-float, just beyond the grid step 2^-20 AU)
    for k, sep in enumerate((1.0e-9, 3.0e-7, 1.2e-6, 5.0e-6)):
        a, b = 100 + 2 * k, 101 + 2 * k
        pp[b] = pp[a]
        pp[b, :3] += sep * np.array([0.6, -0.48, 0.64])
    ps = phases(n_spl, G, 1.0, 4.0, 0.05, 2.0)
    pl = phases(n_pl, G, 0.5, 5.0, 0.1, 3.0)
    pt = phases(n_tp, G, 0.5, 6.0, 0.1, 3.0)
    rho = 2.0 * scenarios.GRAM_PER_CM3_TO_SOLAR_PER_AU3
    groups = [scenarios._star(),
              (abi.GIANT_PLANET, dict(mass=np.full(n_giant, 1e-3), phase=pg)),
              (abi.PROTO_PLANET, dict(mass=rng.uniform(0.5e-9, 2e-9, n_proto), phase=pp)),
              (abi.SUPER_PLANETESIMAL, dict(mass=np.full(n_spl, 1e-8), radius=np.full(n_spl, 1e-7),
                                            density=np.full(n_spl, rho), phase=ps)),
              (abi.PLANETESIMAL, dict(mass=np.full(n_pl, 1e-11), radius=np.full(n_pl, 1e-8),
                                      density=np.full(n_pl, rho), phase=pl)),
              (abi.TEST_PARTICLE, dict(mass=np.zeros(n_tp), phase=pt))]
    return scenarios._assemble("split_ff_mix", groups)


def _rel(a, ref):
    a, ref = a.reshape(-1, 6)[1:, 3:], ref.reshape(-1, 6)[1:, 3:]
    return np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)


def test_split_ff_large_kernel_mixed_classes_and_close_pairs():
    s = _mixed_system()
    assert s.n > 16384  # the 2-D kernel, not the warp-per-sink one
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        d64, rm3_64, nn64, nd64 = ctx.accel(0.0, s.y0)
        ctx.set_precision(abi.PRECISION_SPLIT_FF)
        dff, rm3_ff, nnff, ndff = ctx.accel(0.0, s.y0)
        ctx.set_precision(abi.PRECISION_SPLIT)
        dsp, *_ = ctx.accel(0.0, s.y0)
    err = _rel(dff, d64)
    assert err.max() <= SPLIT_RTOL, f"max rel err {err.max():.3e} at body {int(err.argmax()) + 1}"
    assert _rel(dsp, d64).max() <= SPLIT_RTOL
    assert np.array_equal(dff.reshape(-1, 6)[:, :3].view(np.uint64), d64.reshape(-1, 6)[:, :3].view(np.uint64))
    assert np.array_equal(rm3_ff.view(np.uint64), rm3_64.view(np.uint64))
    assert np.array_equal(nnff, nn64)
    assert np.array_equal(ndff.view(np.uint64), nd64.view(np.uint64))
    # the planted pairs are each other's nearest neighbours
    first = 1 + 3  # star, giants
    for k in range(4):
        a, b = first + 100 + 2 * k, first + 101 + 2 * k
        assert nnff[a] == b and nnff[b] == a


def test_split_ff_large_kernel_far_from_the_origin():
    """Coordinates up to ~40 AU (a coarser grid, G1 = 2^-17 AU) and a system
    shifted off the central body's axis: still within the bound."""
    s = scenarios.config3(seed=77, n=20000)
    y = s.y0.reshape(-1, 6)
    y[1:, :3] *= 8.0
    y[1:, 3:] /= np.sqrt(8.0)
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        d64, *_ = ctx.accel(0.0, s.y0)
        nn64 = ctx.last_eval()[1]
        ctx.set_precision(abi.PRECISION_SPLIT_FF)
        dff, *_ = ctx.accel(0.0, s.y0)
        nnff = ctx.last_eval()[1]
    assert _rel(dff, d64).max() <= SPLIT_RTOL
    assert np.array_equal(nnff, nn64)


@pytest.mark.parametrize("n", [4096, 9000])
def test_split_ff_small_systems_use_short_chunks(n):
    """From 4,096 bodies SPLIT_FF runs k_pairs_ff with source chunks of 1 to 16
    tiles, chosen so that the grid fills the GPU (one or two tiles at these
    sizes): still within the bound, same nearest neighbours."""
    s = scenarios.config3(seed=78, n=n)
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        d64, *_ = ctx.accel(0.0, s.y0)
        nn64 = ctx.last_eval()[1]
        ctx.set_precision(abi.PRECISION_SPLIT_FF)
        dff, *_ = ctx.accel(0.0, s.y0)
        nnff = ctx.last_eval()[1]
    assert _rel(dff, d64).max() <= SPLIT_RTOL
    assert np.array_equal(nnff, nn64)

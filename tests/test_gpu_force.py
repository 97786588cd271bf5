"""Force evaluation on the GPU against fixtures produced by the reference
build (tests/golden) and against the oracle.

FP64 is the reference's arithmetic and must be bit-identical for every body
whose acceleration has no transcendental gas term.  Bodies with gas drag or
migration use CUDA's pow/exp/log10, which may differ from glibc in the last
bit: they are held to 1e-12 relative.  SPLIT is held to the 1e-12 relative
acceleration bound of the split-precision form."""
import hashlib

import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

from golden_io import ACCEL_CASES, GOLDEN, load, system_from

pytestmark = pytest.mark.gpu

SPLIT_RTOL = 1e-12  # relative acceleration error bound of the split form
GAS_RTOL = 1e-12    # bodies whose acceleration includes pow/exp gas terms


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def gas_bodies(s):
    """Indices whose acceleration includes a transcendental gas term."""
    if s.gas is None:
        return np.zeros(s.n, bool)
    c = s.counts
    nm = c[0] + c[1] + c[2] + c[3]
    m = np.zeros(s.n, bool)
    m[nm:nm + c[4] + c[5]] = True                       # drag
    m[1:nm] |= s.mig_type[1:nm] != abi.MIGRATION_NO     # migration
    return m


def rel_accel_err(a, ref):
    a = a.reshape(-1, 6)[:, 3:]
    ref = ref.reshape(-1, 6)[:, 3:]
    num = np.linalg.norm(a - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    out = np.zeros_like(num)
    nz = den > 0
    out[nz] = num[nz] / den[nz]
    out[~nz] = num[~nz]
    return out


@pytest.mark.parametrize("case", ACCEL_CASES)
def test_fp64_matches_reference_bits(case):
    d = load(case)
    s = system_from(d)
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        dydt, rm3, nn, nd = ctx.accel(float(d["meta_t"]), s.y0, int(d["meta_flags"]))
        mig = ctx.mig_type()
    ref = d["out_dydt"]
    g = gas_bodies(s)
    got6, ref6 = dydt.reshape(-1, 6), ref.reshape(-1, 6)
    assert np.array_equal(bits(got6[~g]), bits(ref6[~g])), "gravity-only bodies must be bit-identical"
    assert np.array_equal(bits(got6[:, :3]), bits(ref6[:, :3]))
    if g.any():
        assert rel_accel_err(dydt, ref)[g].max() <= GAS_RTOL
    if "out_rm3" in d:
        assert np.array_equal(bits(rm3), bits(d["out_rm3"]))
    assert np.array_equal(nn, d["out_nn_idx"])
    assert np.array_equal(bits(nd), bits(d["out_nn_dist"]))
    assert np.array_equal(mig, d["out_mig_type"])


SPLITS = [abi.PRECISION_SPLIT, abi.PRECISION_SPLIT_FF]


@pytest.mark.parametrize("precision", SPLITS)
@pytest.mark.parametrize("case", [c for c in ACCEL_CASES if "_bc" not in c])
def test_split_within_bound(case, precision):
    d = load(case)
    s = system_from(d)
    with engine.Context(s, precision=precision) as ctx:
        dydt, rm3, nn, nd = ctx.accel(float(d["meta_t"]), s.y0, int(d["meta_flags"]))
    ref = d["out_dydt"]
    err = rel_accel_err(dydt, ref)
    assert err.max() <= SPLIT_RTOL, f"max rel err {err.max():.3e}"
    assert np.array_equal(bits(dydt.reshape(-1, 6)[:, :3]), bits(ref.reshape(-1, 6)[:, :3]))
    assert np.array_equal(bits(rm3), bits(d["out_rm3"]))
    assert np.array_equal(nn, d["out_nn_idx"])
    np.testing.assert_allclose(nd, d["out_nn_dist"], rtol=1e-15, atol=0)


def test_full_size_fp64_checksum_and_split_bound():
    """65,536 self-gravitating bodies: the FP64 path reproduces the reference
    build's dydt, rm3 and nearest-neighbour arrays byte for byte (sha256 of the
    reference's outputs); both split forms stay within 1e-12 of it."""
    fx = dict(np.load(f"{GOLDEN}/full_disk_exact_checksums.npz"))
    s = scenarios.disk_exact()
    assert hashlib.sha256(s.y0.tobytes()).hexdigest() == str(fx["y0_sha256"]), "input generator not reproducible"
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        dydt, rm3, nn, nd = ctx.accel(0.0, s.y0)
        splits = {}
        for p in SPLITS:
            ctx.set_precision(p)
            splits[p] = ctx.accel(0.0, s.y0)
    assert hashlib.sha256(dydt.tobytes()).hexdigest() == str(fx["dydt_sha256"])
    assert hashlib.sha256(rm3.tobytes()).hexdigest() == str(fx["rm3_sha256"])
    assert hashlib.sha256(nn.tobytes()).hexdigest() == str(fx["nn_idx_sha256"])
    assert hashlib.sha256(nd.tobytes()).hexdigest() == str(fx["nn_dist_sha256"])
    for p, (dsp, rm3s, nns, nds) in splits.items():
        err = rel_accel_err(dsp, dydt)
        assert err.max() <= SPLIT_RTOL, f"precision {p}: split max rel err {err.max():.3e}"
        # nearest neighbours agree except where two candidates tie within rounding
        mism = np.nonzero(nns != nn)[0]
        assert len(mism) <= 2
        for i in mism:
            assert abs(nds[i] - nd[i]) <= 1e-13 * nd[i]


@pytest.mark.parametrize("n", [2, 3, 17, 255, 256, 257, 1000, 4097, 9727, 9728, 9729, 16384, 16385])
def test_tails_against_oracle(n):
    """Tile tails, tiny systems and the sizes where the kernel choice changes
    (one thread per sink below one tile of sources; the 32-sink FP64 kernel
    from two CTAs per SM, 9,728 bodies on 152 SMs; the few-sinks kernels up
    to 16,384 bodies for the split forms), every precision, against the
    oracle."""
    s = scenarios.config3(seed=5000 + n, n=n)
    o = oracle.Oracle(s)
    ref = o.compute(0.0, s.y0)
    rm3_o, nn_o, nd_o = o.last_eval()
    with engine.Context(s) as ctx:
        d64, rm3, nn, nd = ctx.accel(0.0, s.y0)
        outs = {}
        for p in SPLITS:
            ctx.set_precision(p)
            outs[p] = ctx.accel(0.0, s.y0)
    assert np.array_equal(bits(d64), bits(ref))
    assert np.array_equal(nn, nn_o) and np.array_equal(bits(nd), bits(nd_o))
    for p, (dsp, _, nns, nds) in outs.items():
        assert rel_accel_err(dsp, ref).max() <= SPLIT_RTOL, p
        assert np.array_equal(nns, nn_o), p
        assert np.array_equal(bits(nds), bits(nd_o)), p


def test_mixed_classes_against_oracle_split():
    """Every body class with gas drag in all three regimes, both precisions."""
    s = scenarios.mixed_gas_system(seed=3100, n_spl=40, n_pl=300, n_tp=50, n_proto=20)
    o = oracle.Oracle(s)
    ref = o.compute(3.0, s.y0)
    with engine.Context(s) as ctx:
        d64, *_ = ctx.accel(3.0, s.y0)
        outs = {}
        for p in SPLITS:
            ctx.set_precision(p)
            outs[p] = ctx.accel(3.0, s.y0)[0]
    g = gas_bodies(s)
    assert np.array_equal(bits(d64.reshape(-1, 6)[~g]), bits(ref.reshape(-1, 6)[~g]))
    assert rel_accel_err(d64, ref).max() <= GAS_RTOL
    for p, dsp in outs.items():
        assert rel_accel_err(dsp, ref).max() <= SPLIT_RTOL, p


def test_mixed_classes_wide_fp64():
    """The 32-sink FP64 kernel with sinks of both source ranges side by side
    (massive sinks see the super-planetesimals, planetesimals do not), gas
    drag and migration, against the oracle bit for bit away from the gas
    bodies."""
    s = scenarios.mixed_gas_system(seed=3200, n_spl=260, n_pl=9600, n_tp=300, n_proto=200)
    assert s.n >= 2 * 152 * 32
    o = oracle.Oracle(s)
    ref = o.compute(3.0, s.y0)
    rm3_o, nn_o, nd_o = o.last_eval()
    with engine.Context(s) as ctx:
        d64, rm3, nn, nd = ctx.accel(3.0, s.y0)
    g = gas_bodies(s)
    assert np.array_equal(bits(d64.reshape(-1, 6)[~g]), bits(ref.reshape(-1, 6)[~g]))
    assert rel_accel_err(d64, ref).max() <= GAS_RTOL
    assert np.array_equal(bits(rm3), bits(rm3_o))
    assert np.array_equal(nn, nn_o) and np.array_equal(bits(nd), bits(nd_o))


def test_eval_flags_and_stale_buffers():
    """Acceleration::evaluate* switches: a disabled term reuses the buffer of
    the last evaluation that computed it (Acceleration.cpp:182-242)."""
    s = scenarios.mixed_gas_system(seed=3200)
    o = oracle.Oracle(s)
    y1 = s.y0.copy()
    y2 = s.y0 * (1.0 + 1e-6)
    with engine.Context(s) as ctx:
        for y, flags in ((y1, abi.EVAL_ALL), (y2, abi.EVAL_GAS_DRAG), (y1, 0)):
            ref = o.compute(1.0, y, flags)
            got, *_ = ctx.accel(1.0, y, flags)
            assert rel_accel_err(got, ref).max() <= GAS_RTOL
        assert np.array_equal(ctx.mig_type(), o.mig_type())


@pytest.mark.parametrize("n", [64, 600])
def test_split_ff_close_pairs_and_coincident_sink(n):
    """Float-float branch limits: a pair closer than 1e-12 AU is evaluated in
    FP64 by the fall-back branch; the sink itself contributes exactly 0 (in
    the 2-D kernel and in the few-sinks kernel)."""
    s = scenarios.config3(seed=6001, n=n)
    y = s.y0.reshape(-1, 6).copy()
    y[10, :3] = y[9, :3] + np.array([3e-13, -2e-13, 1e-13])  # 3.7e-13 AU apart
    y[20, :3] = y[19, :3] + np.array([1e-9, 0.0, 0.0])
    s.y0 = np.ascontiguousarray(y.reshape(-1))
    o = oracle.Oracle(s)
    ref = o.compute(0.0, s.y0)
    with engine.Context(s, precision=abi.PRECISION_SPLIT_FF) as ctx:
        dff, _, nn, _ = ctx.accel(0.0, s.y0)
    assert np.isfinite(dff).all()
    assert rel_accel_err(dff, ref).max() <= SPLIT_RTOL
    assert nn[10] == 9 and nn[9] == 10 and nn[20] == 19


@pytest.mark.parametrize("n", [400, 4000])
def test_fp64_fallback_paths_bit_identical(n):
    """The FP64 kernels' rare fallbacks against the oracle, bit for bit: two
    bodies 1e-93 and 2e-93 AU from the star (their rm3 and their pair have
    squared distances below 2^-600: IEEE sqrt and division instead of the
    FMA-remainder rounding) and a source of subnormal mass (its term
    multiplies leave the integer pipe for the FP64 instruction).  400 bodies
    run the 4-sink kernel, 4,000 the 32-sink kernel."""
    s = scenarios.config3(seed=7000 + n, n=n)
    y = s.y0.reshape(-1, 6)
    y[5, :3] = (1.0e-93, 0.0, 0.0)
    y[7, :3] = (2.0e-93, 0.0, 0.0)
    s.mass[9] = 1.0e-310
    o = oracle.Oracle(s)
    ref = o.compute(0.0, s.y0)
    rm3_o, nn_o, nd_o = o.last_eval()
    with engine.Context(s) as ctx:
        d64, rm3, nn, nd = ctx.accel(0.0, s.y0)
    assert np.array_equal(bits(d64), bits(ref))
    assert np.array_equal(bits(rm3), bits(rm3_o))
    assert np.array_equal(nn, nn_o) and np.array_equal(bits(nd), bits(nd_o))
    assert nn[5] == 7 and nn[7] == 5


def test_barycentric_context_rejects_the_split_forms():
    """GravityBC_* has only the reference (FP64) form here: a barycentric
    context refuses SPLIT and SPLIT_FF with SOL_ERR_ARG instead of silently
    computing in FP64, and keeps evaluating bit for bit afterwards."""
    d = load("accel_mixed_gas_bc")
    s = system_from(d)
    with engine.Context(s, precision=abi.PRECISION_FP64) as ctx:
        for p in SPLITS:
            with pytest.raises(abi.SolError) as err:
                ctx.set_precision(p)
            assert err.value.code == abi.SOL_ERR_ARG
            assert "barycentric" in str(err.value)
        dydt, *_ = ctx.accel(float(d["meta_t"]), s.y0, int(d["meta_flags"]))
    g = gas_bodies(s)
    assert np.array_equal(bits(dydt.reshape(-1, 6)[~g]), bits(d["out_dydt"].reshape(-1, 6)[~g]))

"""The correctly rounded square root and reciprocal of the FP64 pair
(sol_crmath.cuh: remainders by FMA, rounding decided from the measured
distance to the neighbouring doubles) against IEEE sqrt and division, and
the integer-pipe multiply of the pair terms against the FP64 instruction,
bit for bit, and the step-size control's inverse roots for correct
rounding, on seeded sample families (sol_check_pair_math)."""
import pytest

from solaris_gb300 import engine

pytestmark = pytest.mark.gpu

N = 1 << 28


@pytest.mark.parametrize("mode,max_slow", [
    (0, 2e-4),   # log-uniform a: the slow path is the 2^-16 band (and powers of two)
    (1, 0.25),   # square roots 2^-27 .. 2^-13.4 ulp from a midpoint: ~15% inside the band
    (2, 2e-4),   # squared distances in a 100 AU box
    (3, 0.3),    # reciprocals x^2 2^-54 ulp from a midpoint (x < 2^19: inside the band), approximations 300 ulps off
    (4, 2e-4),   # log-uniform reciprocals, approximations 300 ulps off
    (5, 0.4),    # square roots and reciprocals next to powers of two (results on a power of two go the IEEE way)
    (6, 0.0),    # integer-pipe multiply, random operands
    (7, 0.0),    # integer-pipe multiply next to the normalisation boundaries, zeros, squares
    (8, 0.0),    # step-size control pow(errorMax, -0.2): correctly rounded
    (9, 0.0),    # step-size control pow(errorMax, -0.25): correctly rounded
])
def test_pair_math_matches_ieee(mode, max_slow):
    r = engine.check_pair_math(mode, N, seed=1000 + mode)
    # pow(em, -0.2): ln em from FP32 in the exponent's own-rounding correction
    # leaves results within ~1e-7 ulp of a midpoint undecided (~5e-8 of samples)
    assert r["mismatches"] <= (1e-6 * N if mode == 8 else 0), r
    assert r["slow"] <= max_slow * N, r

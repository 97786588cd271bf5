"""Calculate::Integrals (Solaris/Calculate.cpp:43-172) on the device above the
exact-order size: the potential energy from k_potential_pairs (each
unordered pair once, 1/r by an FP32 seed and an FP64 Newton step).  The O(N)
integrals are the oracle's (the reference's sums), bit for bit.  The
potential energy is held to 1e-13 relative against an accurately summed
value (numpy pairwise row sums, math.fsum over the rows): the reference's
own sequential sum of N^2 terms strays from it by ~sqrt(N^2) 2^-53 (2e-12
at 20,000 bodies), so it is compared within 1e-11.  Block counts odd and
even, zero-mass bodies, and a coincident pair (the reference's division
gives +inf)."""
import math

import numpy as np
import pytest

from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu


def _accurate_potential(s, y):
    """Gauss2 / 2 * sum over ordered pairs of m_i m_j / r_ij, summed
    accurately (each unordered pair's row sums pairwise, the rows by fsum)."""
    p = y.reshape(-1, 6)[:, :3]
    m = s.mass
    rows = []
    for i in range(s.n - 1):
        d = p[i + 1:] - p[i]
        r = np.sqrt(np.einsum("ij,ij->i", d, d))
        rows.append(m[i] * np.sum(m[i + 1:] / r))
    return math.fsum(rows) * abi.GAUSS2  # 2 x unordered x Gauss2 / 2


@pytest.mark.parametrize("n", [1025, 3001, 4096, 20000])
def test_potential_energy_against_oracle(n):
    import oracle
    s = scenarios.config3(seed=700 + n, n=n)
    s.mass[n // 2:n // 2 + 50] = 0.0  # massless bodies in the middle of a block
    ref = oracle.Oracle(s).integrals(s.y0)
    with engine.Context(s) as ctx:
        got = ctx.integrals(s.y0)
    assert np.array_equal(got[:14].view(np.uint64), ref[:14].view(np.uint64))
    exact = _accurate_potential(s, s.y0)
    assert abs(got[14] - exact) <= 1e-13 * abs(exact)
    assert abs(ref[14] - exact) <= 1e-11 * abs(exact)
    assert got[15] == got[13] - got[14]


def test_coincident_bodies_give_infinite_potential_energy():
    """m_i m_j / 0: +inf for two massive bodies, NaN when one is massless."""
    s = scenarios.config3(seed=799, n=2000)
    y = s.y0.copy().reshape(-1, 6)
    y[1500, :3] = y[700, :3]
    with engine.Context(s) as ctx:
        got = ctx.integrals(y.ravel())
    assert np.isinf(got[14]) and got[14] > 0
    s.mass[1500] = 0.0
    with engine.Context(s) as ctx:
        got = ctx.integrals(y.ravel())
    assert np.isnan(got[14])


def test_potential_energy_is_deterministic():
    s = scenarios.config3(seed=798, n=9000)
    with engine.Context(s) as ctx:
        a = ctx.integrals(s.y0)
        b = ctx.integrals(s.y0)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))

"""The oracle's Calculate::Integrals (restated from Solaris/Calculate.cpp:
43-172), the checker of sol_integrals: its potential energy (the reference's
single running sum over ordered pairs, Calculate.cpp:139-159) against an
accurately summed value, its kinetic energy and total mass against plain
sums, on a small mixed system (massive and massless bodies)."""
import math

import numpy as np

from solaris_gb300 import abi, scenarios


def test_oracle_integrals_against_accurate_sums():
    import oracle
    s = scenarios.config3(seed=611, n=300)
    s.mass[100:120] = 0.0
    out = oracle.Oracle(s).integrals(s.y0)
    p = s.y0.reshape(-1, 6)
    m = s.mass
    rows = []
    for i in range(s.n - 1):
        d = p[i + 1:, :3] - p[i, :3]
        rows.append(m[i] * np.sum(m[i + 1:] / np.sqrt(np.einsum("ij,ij->i", d, d))))
    pe = math.fsum(rows) * abi.GAUSS2  # twice the unordered sum, times Gauss2 / 2
    ke = math.fsum(0.5 * m * np.einsum("ij,ij->i", p[:, 3:], p[:, 3:]))
    assert abs(out[14] - pe) <= 1e-13 * abs(pe)
    assert abs(out[13] - ke) <= 1e-13 * abs(ke)
    assert out[15] == out[13] - out[14]
    total = 0.0  # Calculate::TotalMass: a sequential sum over the massive bodies
    for x in m[:sum(s.counts[:4])]:
        total += float(x)
    assert out[0] == total

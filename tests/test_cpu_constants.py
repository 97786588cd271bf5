"""Constants of the device arithmetic that stands in for the reference's
libm calls, checked by exact rational arithmetic: the step-size controls
raise to the doubles nearest 1/5 (PGROW = -0.2, RungeKuttaFehlberg78.cpp:61)
and 1/7 (DormandPrince.cpp:156), and a merge to the double nearest 1/3; the
device's correctly rounded powers carry each exponent's own rounding,
delta = double(1/N) - 1/N, written in sol_internal.cuh as 1 / integer."""
import os
import re
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "solaris_gb300", "csrc", "sol_internal.cuh")


def _deltas():
    text = open(SRC).read()
    five = re.search(r"kDelta = \(N == 5\) \? 1\.0 / (\d+)\.0 : 0\.0", text)
    three_seven = re.search(r"kDelta = N == 3 \? -1\.0 / (\d+)\.0 : -1\.0 / (\d+)\.0", text)
    assert five and three_seven, "constants not found"
    return {5: Fraction(1, int(five.group(1))), 3: Fraction(-1, int(three_seven.group(1))),
            7: Fraction(-1, int(three_seven.group(2)))}


def test_exponent_offsets_are_exact():
    for n, d in _deltas().items():
        assert Fraction(1.0 / n) - Fraction(1, n) == d, n


def test_quarter_exponent_is_exact():
    assert Fraction(0.25) == Fraction(1, 4)  # PSHRNK = -0.25 needs no offset

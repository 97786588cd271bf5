"""Known answers of the reference's test programs on the device: the phase of
a known orbit from sol_phases_from_elements with a converged Kepler solution
(unit_test.cpp:812-865, 1e-14), and total mass and barycentre of an
equilateral triangle from sol_integrals (Test/Test.cpp:130-190)."""
import math

import numpy as np
import pytest

from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu
TORAD = math.pi / 180.0


def test_phase_of_a_known_orbit():
    mu = np.array([abi.GAUSS2 * 1.0])
    el = np.array([[1.944132, 0.0737774, 22.50914 * TORAD, 124.04003 * TORAD, 175.33712 * TORAD, 217.31447 * TORAD]])
    want = np.array([-1.824214307389804, 0.9081741252311457, -0.3136484471795240, -4.959970348405931e-03,
                     -9.644216216654788e-03, 4.150430491295794e-03])
    ph, st = engine.phases_from_elements(mu, el, quirks=0)
    assert st[0] == abi.SOL_OK
    assert np.max(np.abs(ph[0] - want)) <= 1e-14


def test_total_mass_and_barycentre_of_a_triangle():
    y = np.zeros(18)
    y[6] = 1.0
    y[12], y[13] = 0.5, math.sqrt(3.0) / 2.0
    s = scenarios.System(name="triangle", counts=(1, 2, 0, 0, 0, 0, 0), id=np.arange(1, 4, dtype=np.int32),
                         type=np.array([abi.CENTRAL_BODY, abi.GIANT_PLANET, abi.GIANT_PLANET], np.int32),
                         mig_type=np.zeros(3, np.int32), mig_stop_at=np.zeros(3), mass=np.full(3, 1.0 / 3.0),
                         radius=np.zeros(3), density=np.zeros(3), cd=np.zeros(3), gamma_stokes=np.zeros(3),
                         gamma_epstein=np.zeros(3), y0=y)
    with engine.Context(s) as ctx:
        out = ctx.integrals(y)
    assert abs(out[0] - 1.0) <= 1e-10
    assert np.all(np.abs(out[1:7] - [0.5, 1.0 / (2.0 * math.sqrt(3.0)), 0.0, 0.0, 0.0, 0.0]) <= 1e-14)

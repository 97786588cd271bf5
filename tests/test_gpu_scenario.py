"""Scenario files run on the device (solaris_gb300.simulator with the device
context) against the reference program's own output files for the same
scenario files (tests/golden/make_scenarios.py).

The initial record and the property files are the reference's bytes; the
trajectory records agree to a tolerance: on the device the step-size
control's pow() (and the gas terms' pow / exp) may round differently in the
last bit; the error estimate's cancellation amplifies that into the
accepted step sizes (~1e-9 relative), so records at fixed output times agree
to PHASE_RTOL and an event's time (the end of its step) to 1e-7."""
import os

import numpy as np
import pytest

from solaris_gb300 import engine
from solaris_gb300 import scenario_xml as sx
from solaris_gb300 import simulator as sim
from scenario_files import (NAMES, golden_dir, read_affairs, read_integrals, read_phases,
                            read_variable_properties, xml_path)

pytestmark = pytest.mark.gpu

PHASE_RTOL = 1e-7  # per body, relative to |r| and |v| (measured: 3.4e-8 after the collision, which lands
#                    a rounding-sized time apart and so merges slightly different states)
INTEGRALS_RTOL = 1e-8


def _rel_body(a, b):
    ra = np.linalg.norm(a[:, :3], axis=1)
    va = np.linalg.norm(a[:, 3:], axis=1)
    dr = np.linalg.norm(a[:, :3] - b[:, :3], axis=1) / np.maximum(ra, 1e-300)
    dv = np.linalg.norm(a[:, 3:] - b[:, 3:], axis=1) / np.maximum(va, 1e-300)
    return float(max(dr.max(), dv.max()))


def _collapse(records):
    out = []
    for r in records:
        if out and abs(r[0] - out[-1][0]) <= 1e-9 * max(1.0, abs(r[0])):
            out[-1] = r
        else:
            out.append(r)
    return out


@pytest.mark.parametrize("name", NAMES)
def test_scenario_on_the_device(tmp_path, name):
    sc = sx.load(xml_path(name))
    st = sc.settings
    out = str(tmp_path)
    k0 = engine.kernel_launches()
    r = sim.Simulator(sc, directory=out).run()
    assert engine.kernel_launches() - k0 >= r["phases"]  # the steps ran on the device (many per launch)
    gold = golden_dir(name)
    assert sorted(f for f in os.listdir(out) if f != st.log) == sorted(os.listdir(gold))

    for fn in (st.constant_properties, st.composition_properties):
        path = os.path.join(gold, fn)
        if os.path.exists(path):
            with open(path, "rb") as f, open(os.path.join(out, fn), "rb") as g:
                assert g.read() == f.read(), fn
    vw, vg = read_variable_properties(os.path.join(gold, st.variable_properties)), \
        read_variable_properties(os.path.join(out, st.variable_properties))
    assert len(vw) == len(vg)
    for a, b in zip(vw, vg):  # a merge's record carries the event's time
        assert a[:2] == b[:2] and a[3:] == b[3:] and abs(a[2] - b[2]) <= 1e-7 * abs(a[2])

    want, got = read_phases(os.path.join(gold, st.phases)), read_phases(os.path.join(out, st.phases))
    # Whether the last output step lands exactly on the end of the run depends
    # on the last bit of the accumulated time: one run may write its last
    # output record and then a final one a rounding-sized step later.
    want, got = _collapse(want), _collapse(got)
    assert len(got) == len(want)
    assert np.array_equal(got[0][2], want[0][2]) and got[0][0] == want[0][0]
    worst = 0.0
    for (tw, iw, yw), (tg, ig, yg) in zip(want, got):
        assert np.array_equal(iw, ig)
        assert abs(tg - tw) <= 1e-12 * max(1.0, abs(tw))
        worst = max(worst, _rel_body(yw, yg))
    assert worst <= PHASE_RTOL, f"worst body deviation {worst:.3e}"

    hw, iw = read_integrals(os.path.join(gold, st.integrals))
    hg, ig = read_integrals(os.path.join(out, st.integrals))
    iw, ig = _collapse(iw), _collapse(ig)
    assert hg == hw and len(ig) == len(iw)
    for (tw, vw), (tg, vg) in zip(iw, ig):
        # the barycentre's coordinates of a barycentric run are rounding noise around 0
        assert np.all(np.abs(vg - vw) <= INTEGRALS_RTOL * np.abs(vw) + 1e-15), (tw, np.abs(vg - vw).max())

    aw = read_affairs(os.path.join(gold, st.two_body_affair))
    ag = read_affairs(os.path.join(out, st.two_body_affair))
    assert len(ag) == len(aw)
    for a, b in zip(aw, ag):
        assert (a["id"], a["type"], a["id1"], a["id2"]) == (b["id"], b["type"], b["id1"], b["id2"])
        # an event's time is the end of its step: the sum of the accepted steps,
        # whose sizes follow the error estimate's cancellation-amplified rounding
        assert abs(a["time"] - b["time"]) <= 1e-7 * abs(a["time"])
        # the recorded phases are taken at the event's step, whose end moved by
        # |dt| above: positions move by |v| |dt| (~3e-7 AU for the collision)
        dt = abs(a["time"] - b["time"])
        for k in ("phase1", "phase2"):
            r, v = np.linalg.norm(a[k][:3]), np.linalg.norm(a[k][3:])
            assert np.linalg.norm(a[k][:3] - b[k][:3]) <= 4.0 * v * dt + PHASE_RTOL * r, k
            assert np.linalg.norm(a[k][3:] - b[k][3:]) <= 1e-6 * v, k


class _OneStepAtATime:
    """The device context driven one host call per step (the reference loop's shape)."""

    def __init__(self, system, st, directory):
        self.b = sim.EngineBackend(system, st, directory)

    def __getattr__(self, k):
        if k in ("run_until", "step_start"):
            raise AttributeError(k)
        return getattr(self.b, k)


@pytest.mark.parametrize("name", ["collision_rkf78", "epochs_rkf78", "gas_rk4"])
def test_device_step_loop_matches_host_step_loop(tmp_path, name):
    """sol_run_until (DecisionMaking's clamps, the event predicates and the
    smallest-number flush on the device) writes the same bytes as the same
    device driver called once per step from the host."""
    outs = []
    for k, backend in enumerate((None, _OneStepAtATime)):
        sc = sx.load(xml_path(name))
        d = tmp_path / f"run{k}"
        kw = {} if backend is None else {"backend": backend}
        r = sim.Simulator(sc, directory=str(d), **kw).run()
        files = {f: (d / f).read_bytes() for f in sorted(os.listdir(d)) if f != sc.settings.log}
        outs.append((r["steps"], len(r["affairs"]), files))
    assert outs[0][0] == outs[1][0] and outs[0][1] == outs[1][1]
    assert outs[0][2].keys() == outs[1][2].keys()
    for f in outs[0][2]:
        assert outs[0][2][f] == outs[1][2][f], f

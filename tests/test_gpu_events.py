"""Events on the device (sol_handle_events) against the oracle's restatement
of Simulator::CheckEvent / RemoveBody / HandleCollision (Simulator.cpp:
621-935): planted ejections, hit-centrum bodies and collisions (a pair, an
equal-mass pair, a super-planetesimal into a giant, a test particle that
does not merge, a collision that only a previous merge's larger radius
makes), the affairs, the compacted bodies and state, and an evaluation of
the compacted system."""
import struct

import numpy as np
import pytest

import oracle
from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu
EJECTION, HIT_CENTRUM, FACTOR = 40.0, 0.05, 1.0


def bits(a):
    return np.asarray(a, np.float64).view(np.uint64)


def _planted():
    s = scenarios.mixed_gas_system(seed=3500)
    y = s.y0.reshape(-1, 6).copy()
    mass, radius = s.mass.copy(), s.radius.copy()

    def place(i, j, d):  # body i at distance d from body j along x
        y[i, :3] = y[j, :3] + np.array([d, 0.0, 0.0])

    y[55, :3] *= 50.0 / np.linalg.norm(y[55, :3])  # ejections: a test particle, a planetesimal
    y[20, :3] *= 50.0 / np.linalg.norm(y[20, :3])
    y[30, :3] *= 0.02 / np.linalg.norm(y[30, :3])  # hit centrum: a planetesimal, a test particle
    y[60, :3] *= 0.02 / np.linalg.norm(y[60, :3])
    mass[4] = 0.5 * mass[3]
    place(4, 3, 1.0e-5)                           # protoplanets 3 and 4 collide, 3 survives
    mass[6] = mass[5]
    place(6, 5, 2.0e-5)                           # equal masses: 5 survives
    place(8, 1, 1.0e-4)                           # a super-planetesimal into giant 1
    place(58, 2, 1.0e-4)                          # a test particle at giant 2: no merge
    # planetesimal 40 touches protoplanet 3 only once 3 has grown by merging 4
    r3_new = (radius[3] ** 3 + radius[4] ** 3) ** (1.0 / 3.0)
    y[40, :3] = y[3, :3] + np.array([0.0, -(radius[40] + 0.5 * (radius[3] + r3_new)), 0.0])
    s.y0 = np.ascontiguousarray(y.reshape(-1))
    s.mass = mass
    return s


def test_planted_events_match_the_oracle(tmp_path):
    s = _planted()
    o = oracle.Oracle(s)
    o.compute(0.0, s.y0)
    y_o, aff_o = o.handle_events(5.0, s.y0, EJECTION, HIT_CENTRUM, FACTOR)
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        ctx.accel(0.0, s.y0)
        aff = ctx.handle_events(5.0, EJECTION, HIT_CENTRUM, FACTOR)
        y = ctx.get_state()
        b = ctx.bodies()
        # the compacted system evaluates as the oracle's does
        d, rm3, nn, nd = ctx.accel(1.0, y)
        path = str(tmp_path / "TwoBodyAffair.dat")
        arr = (abi.SolAffair * len(aff))()
        for k, a in enumerate(aff):
            for f in ("type", "idx1", "idx2", "id1", "id2", "time"):
                setattr(arr[k], f, a[f])
            arr[k].phase1[:] = list(a["phase1"])
            arr[k].phase2[:] = list(a["phase2"])
        abi.check(ctx.lib, ctx.lib.sol_write_affairs(path.encode(), arr, len(aff), 100))
    bo = o.bodies()
    kinds = [a["type"] for a in aff_o]
    assert kinds.count(0) == 2 and kinds.count(1) == 2 and kinds.count(3) == 4, kinds
    assert len(aff) == len(aff_o)
    for a, e in zip(aff, aff_o):
        for f in ("type", "idx1", "idx2", "id1", "id2", "time"):
            assert a[f] == e[f], (f, a, e)
        assert np.array_equal(bits(a["phase1"]), bits(e["phase1"]))
        assert np.array_equal(bits(a["phase2"]), bits(e["phase2"]))
    assert b["counts"] == bo["counts"] and sum(b["counts"]) == s.n - 8
    assert np.array_equal(b["id"], bo["id"]) and np.array_equal(b["type"], bo["type"])
    assert np.array_equal(bits(b["mass"]), bits(bo["mass"]))
    # a merge's radius: pow(x, 1/3) correctly rounded on the device, as libm's is for these
    assert np.array_equal(bits(b["radius"]), bits(bo["radius"]))
    assert np.array_equal(bits(b["density"]), bits(bo["density"]))
    assert np.array_equal(bits(y), bits(y_o))
    ref = o.compute(1.0, y_o)
    np.testing.assert_allclose(d, ref, rtol=1e-12, atol=1e-300)
    # SaveTwoBodyAffair records
    raw = open(path, "rb").read()
    rec = struct.calcsize("<4i13d")
    assert len(raw) == rec * len(aff)
    for k, a in enumerate(aff):
        v = struct.unpack_from("<4i13d", raw, k * rec)
        assert v[:4] == (100 + k, a["type"], a["id1"], a["id2"])
        assert v[4:10] == tuple(a["phase1"]) and v[10:16] == tuple(a["phase2"]) and v[16] == a["time"]


def test_no_events_leave_the_system_alone():
    s = scenarios.config1(n_tp=40)
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, s.h0, 3)
        y = ctx.get_state()
        assert ctx.handle_events(1.0, 1000.0, 1e-4, 1.0) == []
        assert np.array_equal(bits(ctx.get_state()), bits(y)) and ctx.n == s.n


def test_driver_continues_after_removals():
    """Ejected test particles leave; the compacted context keeps integrating
    (graph and persistent paths rebuilt for the new body count) like a fresh
    context of the remaining bodies."""
    s = scenarios.config1(n_tp=60)
    y = s.y0.reshape(-1, 6).copy()
    for i in (10, 11, 30, 59):
        y[i, :3] *= 60.0 / np.linalg.norm(y[i, :3])
    s.y0 = np.ascontiguousarray(y.reshape(-1))
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0, 0, 2, time_line=tl)
        aff = ctx.handle_events(tl.time, 50.0, 0.0, 0.0)
        assert [a["id2"] for a in aff] == [int(s.id[i]) for i in (10, 11, 30, 59)]
        y_after = ctx.get_state()
        tl_after = (tl.time, tl.h_next, tl.h_did)
        ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0, 0, 5, time_line=tl)
        y_end = ctx.get_state()
    keep = np.ones(s.n, bool)
    keep[[10, 11, 30, 59]] = False
    counts = list(s.counts)
    counts[6] -= 4
    r = scenarios.System(name="kept", counts=tuple(counts), id=s.id[keep], type=s.type[keep],
                         mig_type=s.mig_type[keep], mig_stop_at=s.mig_stop_at[keep], mass=s.mass[keep],
                         radius=s.radius[keep], density=s.density[keep], cd=s.cd[keep],
                         gamma_stokes=s.gamma_stokes[keep], gamma_epstein=s.gamma_epstein[keep], y0=y_after, h0=s.h0)
    with engine.Context(r) as ctx2:
        ctx2.set_state(y_after)
        ctx2.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0, 0, 5, time_line=abi.SolTimeLine(*tl_after))
        assert np.array_equal(bits(ctx2.get_state()), bits(y_end))

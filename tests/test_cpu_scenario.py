"""The scenario-file surface on the CPU: the XML reader and the preparation
(XmlFileAdapter.cpp, Simulation.cpp, Simulator.cpp:449-593) and the main
loop of solaris_gb300.simulator driven by the oracle, against output files
written by the reference's own program on the same scenario files
(tests/golden/make_scenarios.py): every file byte for byte."""
import os

import numpy as np
import pytest

import oracle
from solaris_gb300 import abi
from solaris_gb300 import scenario_xml as sx
from solaris_gb300 import simulator as sim
from scenario_files import NAMES, golden_dir, read_phases, xml_path

HEAD = """<Simulation><Settings{sattr}><Integrator name="{integ}"/><TimeLine length="{length}" output="1" unit="day"/>
{extra}</Settings><BodyGroupList>{groups}</BodyGroupList>{nebula}</Simulation>"""
STAR = '<Body type="centralbody" name="S"><Characteristics><Mass value="1"/></Characteristics></Body>'


def planet(kind="giantplanet", name="P", a=5.0, M=0.5, chars='<Mass value="1" unit="jupiter"/>', extra=""):
    body_chars = "" if kind == "testparticle" else f"<Characteristics>{chars}</Characteristics>"
    return (f'<Body type="{kind}" name="{name}"><OrbitalElement a="{a}" e="0.05" incl="0.01" peri="0.2" node="0.3" '
            f'M="{M}"/>{body_chars}{extra}</Body>')


def write(tmp_path, groups, integ="rungekutta78", length="10", sattr="", extra="", nebula="", name="s.xml"):
    g = "".join(f"<BodyGroup><Items>{''.join(bs)}</Items></BodyGroup>" for bs in groups)
    p = tmp_path / name
    p.write_text(HEAD.format(sattr=sattr, integ=integ, length=length, extra=extra, groups=g, nebula=nebula))
    return str(p)


@pytest.mark.parametrize("name", NAMES)
def test_scenario_files_match_the_reference_program(tmp_path, name):
    """Phases, integrals, affairs and the constant / variable / composition
    property files of the oracle-driven run are the reference program's bytes."""
    sc = sx.load(xml_path(name))
    out = str(tmp_path)
    r = sim.Simulator(sc, directory=out, backend=oracle.ScenarioBackend).run()
    assert r["steps"] > 40
    gold = golden_dir(name)
    expected = sorted(os.listdir(gold))
    produced = sorted(f for f in os.listdir(out) if f != sc.settings.log)
    assert produced == expected
    for fn in expected:
        with open(os.path.join(gold, fn), "rb") as f:
            want = f.read()
        with open(os.path.join(out, fn), "rb") as f:
            got = f.read()
        assert got == want, fn
    if name in ("ejection_rkf78", "gas_rk4", "collision_rkf78"):
        assert len(r["affairs"]) == 1
    assert r["phases"] == {"epochs_rkf78": 3, "pre_dopri": 3}.get(name, 1)


def test_initial_state_is_the_reference_programs():
    """The first phases record (t = 0) of every golden run is the prepared
    state: ids, insertion order, units, Kepler phases, barycentric shift."""
    for name in NAMES:
        sc = sx.load(xml_path(name))
        if sc.n_distinct_start_times > 1 or sc.settings.start_defined:
            continue  # the first record is the first synchronisation phase's
        ph = [f for f in os.listdir(golden_dir(name)) if f.endswith("Phases.dat")][0]
        t, ids, y = read_phases(os.path.join(golden_dir(name), ph))[0]
        assert t == 0.0
        assert np.array_equal(ids, sc.system.id)
        assert np.array_equal(y.reshape(-1).view(np.uint64), sc.system.y0.view(np.uint64)), name


def test_units_and_defaults(tmp_path):
    p = write(tmp_path, [[STAR, planet(chars='<Mass value="2" unit="earth"/><Radius value="6000" unit="km"/>'),
                          '<Body type="rockyplanet"><Phase><Position x="1.5e8" unit="km"/>'
                          '<Velocity y="30" unit="kmsec"/></Phase><Characteristics><Mass value="5.9722e24" '
                          'unit="kg"/><Density value="5.5" unit="gcm3"/></Characteristics></Body>']],
              length="2", extra='<Ejection value="1.5e9" unit="km"/><HitCentrum value="2" unit="solarradius"/>')
    sc = sx.load(p)
    st = sc.settings
    assert st.length == 2.0 and st.output == 1.0 and st.integrator == abi.RUNGE_KUTTA_FEHLBERG78
    assert st.ejection == 1.5e9 * sx.KILOMETER_TO_AU and st.hit_centrum == 2.0 * sx.SOLAR_RADIUS_TO_AU
    giant, rocky = sc.bodies[1], sc.bodies[2]
    assert giant.mass == 2.0 * (1.0 / 3.3294605e5) and giant.radius == 6000.0 * sx.KILOMETER_TO_AU
    assert giant.density == giant.mass / (4.0 / 3.0 * sx.PI * giant.radius ** 3)
    assert rocky.phase[0] == 1.5e8 * sx.KILOMETER_TO_AU and rocky.phase[4] == 30 * (sx.KILOMETER_TO_AU / sx.SECOND_TO_DAY)
    assert rocky.mass == 5.9722e24 * sx.KILOGRAM_TO_SOLAR
    assert rocky.density == 5.5 * sx.GRAM_PER_CM3_TO_SOLAR_PER_AU3
    assert rocky.radius == (3.0 / (4.0 * sx.PI) * rocky.mass / rocky.density) ** (1.0 / 3.0)
    assert sc.system.gas is None and not st.barycentric


def test_quantities_inherit_unit_and_value(tmp_path):
    """Sibling quantities share the reader's value and unit variables: a
    Radius without unit takes the Mass's unit, which is no distance unit, so
    the value stays as written; a Radius without value takes the Mass's value."""
    p = write(tmp_path, [[STAR, planet(chars='<Mass value="3" unit="earth"/><Radius value="0.01"/>'),
                          planet(name="Q", a=7.0, chars='<Mass value="2" unit="jupiter"/><Radius unit="km"/>')]])
    b1, b2 = sx.load(p).bodies[1:3]
    assert b1.radius == 0.01
    assert b2.radius == 2.0 * sx.KILOMETER_TO_AU
    p = write(tmp_path, [[STAR, planet()]], extra='<Ejection value="3" unit="km"/><HitCentrum value="2"/>')
    st = sx.load(p).settings
    assert st.hit_centrum == 2.0 * sx.KILOMETER_TO_AU


def test_elements_and_gas(tmp_path):
    neb = ('<Nebula><GasComponent alpha="0.004" type="exponential" timeScale="2" t0="1" t1="3" unit="year">'
           '<Eta c="0.002" index="0.6"/><Tau c="0.7"/><ScaleHeight index="1.3"/><DensityFunction index="-2.5">'
           '<Density value="1e-9" unit="gcm3"/></DensityFunction></GasComponent></Nebula>')
    body = ('<Body type="protoplanet"><OrbitalElement a="1" e="0.1" incl="10" peri="400" node="-30" M="725" '
            'angleUnit="degree"/><Characteristics><Mass value="0.1" unit="earth"/></Characteristics>'
            '<Migration type="I" stopAt="0.5"/></Body>')
    sc = sx.load(write(tmp_path, [[STAR, body]], nebula=neb))
    el = sc.bodies[1].elements
    assert el[2] == 10 * sx.DEGREE_TO_RADIAN
    assert 0.0 <= el[3] < 2 * sx.PI and 0.0 <= el[4] < 2 * sx.PI and 0.0 <= el[5] < 2 * sx.PI
    assert sc.bodies[1].mig_type == abi.MIGRATION_TYPE_I and sc.bodies[1].mig_stop_at == 0.5
    g = sc.system.gas
    assert g["alpha"] == 0.004 and g["decrease_type"] == abi.GAS_EXPONENTIAL
    assert g["time_scale"] == 2 * sx.YEAR_TO_DAY and g["t0"] == sx.YEAR_TO_DAY and g["t1"] == 3 * sx.YEAR_TO_DAY
    assert g["eta"] == (0.002, 0.6) and g["tau"][0] == 0.7 and g["scale_height"][1] == 1.3
    assert g["density"] == (1e-9 * sx.GRAM_PER_CM3_TO_SOLAR_PER_AU3, -2.5)
    from solaris_gb300 import scenarios
    assert g["mean_free_path"] == scenarios.default_gas()["mean_free_path"]  # built from the default density
    ref = oracle.calculate_phase(abi.GAUSS2 * 1.0 + abi.GAUSS2 * sc.bodies[1].mass, el)[1]
    assert np.array_equal(np.array(sc.bodies[1].phase), ref)  # the reference build's CalculatePhase


def test_insertion_order_and_ids(tmp_path):
    """Bodies are numbered in reading order; Simulator::Insert orders each
    group by type and inserts it after the bodies of the same type."""
    rocky = planet(kind="rockyplanet", name="R", a=1.0, chars='<Mass value="1" unit="earth"/>')
    g1 = [planet(kind="testparticle", name="T1"), STAR, rocky, planet(name="G1")]
    g2 = [planet(kind="testparticle", name="T2", a=2.0), planet(name="G2", a=8.0)]
    sc = sx.load(write(tmp_path, [g1, g2]))
    assert [b.name for b in sc.bodies] == ["S", "G1", "G2", "R", "T1", "T2"]
    assert [b.id for b in sc.bodies] == [1, 3, 5, 2, 0, 4]
    assert sc.insertion == [1, 3, 2, 0, 5, 4]
    assert sc.system.counts == (1, 2, 1, 0, 0, 0, 2)
    # a backward run inserts the groups in reverse order
    g2 = [planet(name="G2", a=8.0), planet(kind="testparticle", name="T2", a=2.0)]
    sc = sx.load(write(tmp_path, [g2, [STAR, planet(name="G1"), rocky]], length="-10"))
    assert [b.id for b in sc.bodies] == [2, 3, 0, 4, 1]
    assert sc.insertion == [2, 3, 4, 0, 1]
    assert sc.settings.h0 < 0
    with pytest.raises(sx.ScenarioError, match="type order"):  # forward, the same groups break the order
        sx.load(write(tmp_path, [g2, [STAR, planet(name="G1"), rocky]]))


def test_first_step(tmp_path):
    sc = sx.load(write(tmp_path, [[STAR, planet(a=1.0)]], length="1e9"))
    b = sc.bodies[1]
    mu = abi.GAUSS2 * 1.0 + abi.GAUSS2 * b.mass
    a = 1.0 / (2.0 / np.linalg.norm(b.phase[:3]) - np.dot(b.phase[3:], b.phase[3:]) / mu)
    assert abs(sc.settings.h0 - 2 * np.pi * np.sqrt(a ** 3 / mu) / 50000.0) <= 1e-14 * sc.settings.h0
    assert sx.load(write(tmp_path, [[STAR, planet(a=1.0)]], length="1e-4")).settings.h0 == 1e-4


def test_barycentric_shift(tmp_path):
    sc = sx.load(write(tmp_path, [[STAR, planet(), planet(name="Q", a=9.0)]], sattr=' barycentric="True"'))
    y = sc.system.y0.reshape(-1, 6)
    m = sc.system.mass
    assert np.allclose((m[:, None] * y).sum(0), 0.0, atol=1e-15)
    assert sc.settings.barycentric and sc.system.barycentric


@pytest.mark.parametrize("groups, kw, message", [
    ([[planet()]], {}, "only one body"),
    ([[STAR, STAR.replace('"S"', '"S2"'), planet()]], {}, "more than 1 central"),
    ([[planet(), planet(name="Q")]], {}, "central body is not defined"),
    ([[STAR, planet(kind="testparticle")]], {}, "massive bodies"),
    ([[STAR, planet()]], {"integ": "euler"}, "Unknown integrator"),
    ([[STAR, planet()]], {"length": "0"}, "length"),
    ([[STAR, planet()]], {"sattr": ' color="red"'}, "Unknown attribute"),
    ([[STAR, planet()]], {"extra": '<Collision factor="0.5"/>'}, "factor"),
    ([[STAR, planet(chars='<Mass value="1"/><Radius value="1"/><Density value="1"/>')]], {}, "radius and the density"),
    ([[STAR, planet(chars='<Radius value="1"/>')]], {}, "Missing Mass"),
    ([[STAR, planet(chars='<Mass value="-1"/>')]], {}, "out of range"),
    ([[STAR, planet(chars='<Mass value="1" unit="parsec"/>')]], {}, "Undefined unit"),
    ([[STAR, planet(extra='<Migration type="III"/>')]], {}, "migration type"),
    ([[STAR, planet(chars='<Mass value="1"/><ComponentList><Component name="a" ratio="40"/></ComponentList>')]],
     {}, "component ratios"),
    ([[STAR, planet(kind="testparticle"), planet()],
      [planet(kind="rockyplanet", name="R", a=1.0, chars='<Mass value="1" unit="earth"/>')]], {}, "type order"),
])
def test_reader_errors(tmp_path, groups, kw, message):
    with pytest.raises(sx.ScenarioError, match=message):
        sx.load(write(tmp_path, groups, **kw))


def test_julian_dates():
    """Ephemeris::GetJulianDate: Julian dates, dates and packed dates at 0h UT."""
    assert sx.julian_date("JD2451545.0") == 2451545.0 and sx.julian_date("jd10") == 10.0
    assert sx.julian_date("20000101") == 2451544.5
    assert sx.julian_date("19991231") == 2451543.5
    assert sx.julian_date("K0111") == 2451910.5      # 2001-01-01
    assert sx.julian_date("J961A") == sx.julian_date("19960110")
    assert sx.julian_date("15821004") - sx.julian_date("15821015") == -1.0  # the Gregorian reform
    for bad in ("JD24x", "123456789", "L0101", "K01D1", "K01", "x"):
        with pytest.raises(sx.ScenarioError, match="format"):
            sx.julian_date(bad)


def _epoch_xml(tmp_path, epochs, extra_settings="", timeline='length="2" output="0.5" unit="year"', name="ep.xml"):
    groups = [[STAR, planet(name="G", a=5.0), planet(kind="rockyplanet", name="R", a=1.0,
                                                     chars='<Mass value="1" unit="earth"/>')],
              [planet(kind="testparticle", name="T", a=2.0), planet(kind="testparticle", name="U", a=3.0, M=2.0)]]
    g = "".join(f'<BodyGroup epoch="{e}"><Items>{"".join(bs)}</Items></BodyGroup>' if e else
                f'<BodyGroup><Items>{"".join(bs)}</Items></BodyGroup>' for e, bs in zip(epochs, groups))
    p = tmp_path / name
    p.write_text(f'<Simulation><Settings{extra_settings}><Integrator/><TimeLine {timeline}/></Settings>'
                 f'<BodyGroupList>{g}</BodyGroupList></Simulation>')
    return str(p)


def test_start_times(tmp_path):
    sc = sx.load(_epoch_xml(tmp_path, ["JD100", "JD40"]))
    assert sc.time0 == 100.0 and sc.n_distinct_start_times == 2 and sc.settings.start == 100.0
    assert [g.start_time for g in sc.groups] == [40.0, 100.0]
    assert sx.sync_start_times(sc.settings, sc.groups, sc.time0) == [100.0, 40.0, 100.0]
    sc = sx.load(_epoch_xml(tmp_path, ["JD100", ""]))  # a group without epoch starts at the last epoch
    assert sc.n_distinct_start_times == 1 and sc.time0 == 100.0
    with pytest.raises(sx.ScenarioError, match="different start times"):
        p = tmp_path / "two.xml"
        p.write_text('<Simulation><Settings><Integrator/><TimeLine length="1"/></Settings><BodyGroupList>'
                     f'<BodyGroup epoch="JD1"><Items>{STAR}{planet()}</Items></BodyGroup>'
                     f'<BodyGroup epoch="JD2"><Items>{planet(name="Q", a=7.0)}</Items></BodyGroup>'
                     '</BodyGroupList></Simulation>')
        sx.load(str(p))


def test_relative_end_test_shifts_a_run_in_time(tmp_path):
    """With the phase-relative end test, a run whose groups share an epoch is
    the run without epochs moved in time: the same steps and phases."""
    out = []
    for k, epochs in enumerate((["", ""], ["JD2451545.0", "JD2451545.0"])):
        sc = sx.load(_epoch_xml(tmp_path, epochs, name=f"e{k}.xml"))
        d = tmp_path / f"o{k}"
        r = sim.Simulator(sc, directory=str(d), backend=oracle.ScenarioBackend, relative_end_test=True).run()
        out.append((r, read_phases(str(d / "Phases.dat"))))
    (r0, p0), (r1, p1) = out
    assert r0["steps"] == r1["steps"] > 50 and len(p0) == len(p1) == 5
    for (t0, i0, y0), (t1, i1, y1) in zip(p0, p1):
        assert np.array_equal(i0, i1) and np.array_equal(y0, y1)
        assert abs((t1 - 2451545.0) - t0) <= 1e-6
    # the reference's end test compares the absolute time: the same epoch run stops after one step
    sc = sx.load(_epoch_xml(tmp_path, ["JD2451545.0", "JD2451545.0"], name="e2.xml"))
    r = sim.Simulator(sc, directory=str(tmp_path / "o2"), backend=oracle.ScenarioBackend).run()
    assert r["steps"] == 1


def test_synchronisation_integrates_the_groups_to_a_common_time(tmp_path):
    """relative_end_test: the planets are integrated back from their epoch to
    the test particles' epoch, the particles join, and both go forward."""
    sc = sx.load(_epoch_xml(tmp_path, ["JD100", "JD40"]))
    r = sim.Simulator(sc, directory=str(tmp_path / "o"), backend=oracle.ScenarioBackend,
                      relative_end_test=True).run()
    recs = read_phases(str(tmp_path / "o" / "Phases.dat"))
    times = [t for t, _, _ in recs]
    assert r["phases"] == 3
    assert times[0] == 100.0 and abs(times[1] - 40.0) <= 1e-9       # back to the particles' epoch
    assert abs(times[3] - 100.0) <= 1e-9 and len(recs[3][1]) == 5  # forward to the planets' epoch, all bodies
    assert abs(times[-1] - (100.0 + 2 * 365.25)) <= 1e-9


def test_pre_integration_without_synchronisation(tmp_path):
    """The reference reads the front of an empty body list here (it crashes);
    the body list is populated first, then pre-integrated to the start."""
    sc = sx.load(_epoch_xml(tmp_path, ["JD10", "JD10"], timeline='start="30" length="100" output="50" unit="day"'))
    assert sc.settings.start_defined and sc.n_distinct_start_times == 1
    r = sim.Simulator(sc, directory=str(tmp_path / "o"), backend=oracle.ScenarioBackend,
                      relative_end_test=True).run()
    recs = read_phases(str(tmp_path / "o" / "Phases.dat"))
    assert r["phases"] == 2 and recs[0][0] == 10.0 and abs(recs[1][0] - 30.0) <= 1e-9


def test_legacy_gas_tags(tmp_path):
    neb = ('<Nebula><GasComponent><GasDensityFunction index="-2.75"><VolumeDensity value="2.8e-9" unit="gcm3"/>'
           '</GasDensityFunction></GasComponent></Nebula>')
    p = write(tmp_path, [[STAR, planet()]], nebula=neb)
    from solaris_gb300 import scenarios
    assert sx.load(p).system.gas["density"] == scenarios.default_gas()["density"]  # the reference's reader
    assert sx.load(p, legacy_gas_tags=True).system.gas["density"] == (2.8e-9 * sx.GRAM_PER_CM3_TO_SOLAR_PER_AU3,
                                                                      -2.75)


def test_zero_length_writes_nothing(tmp_path):
    p = tmp_path / "z.xml"
    p.write_text('<Simulation><Settings><Integrator/><TimeLine output="1"/></Settings>'
                 f'<BodyGroupList><BodyGroup><Items>{STAR}{planet()}</Items></BodyGroup></BodyGroupList></Simulation>')
    sc = sx.load(str(p))
    out = tmp_path / "out"
    r = sim.Simulator(sc, directory=str(out), backend=oracle.ScenarioBackend).run()
    assert r["steps"] == 0 and os.listdir(out) == []


def test_guid_layout():
    g = sim._guid_bytes("00112233-4455-6677-8899-aabbccddeeff")
    assert g == bytes([0x33, 0x22, 0x11, 0x00, 0x55, 0x44, 0x77, 0x66, 0x88, 0x99, 0xaa, 0xbb, 0xcc, 0xdd, 0xee, 0xff])
    assert sim._guid_bytes("") == bytes(16)


def test_config1_full_length_matches_the_reference_program(tmp_path):
    """The 256-body RKF78 configuration over its full 1,000 years
    (tests/golden/make_config1.py): the oracle-driven simulator writes the
    reference program's integrals and ejection records byte for byte, with
    its number of accepted steps (driver calls) and rejected attempts (from
    the program's force-evaluation count)."""
    import json
    name = "config1_1000yr"
    summary = json.load(open(os.path.join(golden_dir(name), "summary.json")))
    sc = sx.load(xml_path(name))
    r = sim.Simulator(sc, directory=str(tmp_path), backend=oracle.ScenarioBackend).run()
    assert (r["steps"], r["rejected"]) == (summary["accepted"], summary["rejected"])
    assert len(r["affairs"]) == len(summary["events"])
    for fn in ("Integrals.dat", "TwoBodyAffair.dat"):
        with open(os.path.join(golden_dir(name), fn), "rb") as f:
            want = f.read()
        with open(os.path.join(str(tmp_path), fn), "rb") as f:
            assert f.read() == want, fn

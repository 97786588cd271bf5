"""Solaris scenario files: the reference's Simulation XML
(Solaris/XmlFileAdapter.cpp) read into the body set, gas disk and run
settings of one simulation, prepared the way Solaris/Simulation.cpp and
Solaris/Simulator.cpp prepare it.

Read as the reference reads it: Settings (Output file names, Integrator by
name or xsi:type, Accuracy, TimeLine length / output and unit, Ejection,
HitCentrum, Collision, the barycentric attribute), BodyGroupList /
BodyGroup / Items / Body (type, name, guid, designations, Lagrange point,
MPC orbit type) with a Phase or an OrbitalElement, Characteristics (Mass,
Radius, Density, cd, absVisMag, ComponentList) and Migration, Nebula /
GasComponent (alpha, decrease type, time scale, t0, t1, Eta, Tau,
ScaleHeight, DensityFunction / Density) with every unit of Solaris/Units.cpp
and the same defaults, validations and error cases.  Two of the reference's
parsing habits are kept because they change values: a dimensional quantity
without a unit (or value) attribute inherits the unit (and value) of the one
read before it in the same Settings or Characteristics element
(XmlFileAdapter.cpp:204-235, :1374-1421), and a carried-over unit that does
not belong to the quantity leaves the value unconverted (UnitTool returns an
error nobody reads).

Refused with ScenarioError (the reference's synchronisation and
pre-integration phases are not built): body groups with an epoch or an
offset, distinct start times, a TimeLine start.  Also refused: a central body
given by orbital elements (the reference leaves its phase unset) and a body
list the reference's insertion would leave out of type order (its
Acceleration would integrate it with the wrong index ranges).

Preparation (Simulation::SetPhasesRadiiDensity, Simulator::PopulateBodyList,
Simulator::BodyListToBodyData, Simulator::MainIntegration) runs once on the
host in the reference's operation order, so a scenario's initial state is
the reference's bit for bit: body ids in reading order from 0 (Body.cpp:8-12),
phases from orbital elements with mu = G m_central + G m (0 for test
particles) by Ephemeris::CalculatePhase and the reference build's Kepler
stopping rule, radius or density completed from the mass, the insertion order
of Simulator::Insert, the Epstein and Stokes coefficients, and the first step,
the shortest orbital period / 50,000.
"""
from __future__ import annotations

import math
import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import abi, scenarios

# ---- constants and unit factors (Solaris/Constants.h) ---------------------------
PI = 3.14159265358979323846
GAUSS2 = 2.959122082855911025e-4
DEGREE_TO_RADIAN = 1.745329251994329509e-2
SOLAR_TO_KILOGRAM = 1.98911e30
SOLAR_TO_GRAM = 1.0e3 * SOLAR_TO_KILOGRAM
AU_TO_METER = 1.495978707e11
AU_TO_KILOMETER = AU_TO_METER / 1.0e3
YEAR_TO_DAY = 365.25
DAY_TO_SECOND = 86400.0
METER_TO_AU = 1.0 / AU_TO_METER
KILOMETER_TO_AU = 1.0 / AU_TO_KILOMETER
SOLAR_RADIUS_TO_AU = 1.0 / 215.094
SECOND_TO_DAY = 1.0 / DAY_TO_SECOND
GRAM_TO_SOLAR = 1.0 / SOLAR_TO_GRAM
KILOGRAM_TO_SOLAR = 1.0 / SOLAR_TO_KILOGRAM
_CM = 1.0e-2 * METER_TO_AU
GRAM_PER_CM3_TO_SOLAR_PER_AU3 = GRAM_TO_SOLAR / (_CM * _CM * _CM)

# UnitTool (Solaris/Units.cpp): value *= factor
MASS_UNITS = {"solar": 1.0, "mercury": 1.0 / 6.023600e6, "venus": 1.0 / 4.0852371e5, "earth": 1.0 / 3.3294605e5,
              "earthmoon": 1.0 / 3.2890056e5, "mars": 1.0 / 3.098708e6, "jupiter": 1.0 / 1.0473486e3,
              "saturn": 1.0 / 3.497898e3, "uranus": 1.0 / 2.290298e4, "neptune": 1.0 / 1.941224e4,
              "kilogram": KILOGRAM_TO_SOLAR, "kg": KILOGRAM_TO_SOLAR, "gram": GRAM_TO_SOLAR, "g": GRAM_TO_SOLAR}
TIME_UNITS = {"day": 1.0, "year": YEAR_TO_DAY, "second": SECOND_TO_DAY}
DISTANCE_UNITS = {"au": 1.0, "m": METER_TO_AU, "meter": METER_TO_AU, "km": KILOMETER_TO_AU,
                  "kilometer": KILOMETER_TO_AU, "solarradius": SOLAR_RADIUS_TO_AU}
ANGLE_UNITS = {"radian": 1.0, "degree": DEGREE_TO_RADIAN}
VELOCITY_UNITS = {"auday": 1.0, "kmsec": KILOMETER_TO_AU / SECOND_TO_DAY, "msec": METER_TO_AU / SECOND_TO_DAY}
VOLUME_DENSITY_UNITS = {"solarau3": 1.0, "gcm3": GRAM_PER_CM3_TO_SOLAR_PER_AU3}

BODY_TYPES = {"centralbody": abi.CENTRAL_BODY, "giantplanet": abi.GIANT_PLANET, "rockyplanet": abi.ROCKY_PLANET,
              "protoplanet": abi.PROTO_PLANET, "superplanetesimal": abi.SUPER_PLANETESIMAL,
              "planetesimal": abi.PLANETESIMAL, "testparticle": abi.TEST_PARTICLE}
INTEGRATORS = {"rungekutta78": abi.RUNGE_KUTTA_FEHLBERG78, "rungekuttafehlberg78": abi.RUNGE_KUTTA_FEHLBERG78,
               "rungekutta4": abi.RUNGE_KUTTA4, "dormandprince": abi.DORMAND_PRINCE}
GAS_DECREASE = {"constant": abi.GAS_CONSTANT, "linear": abi.GAS_LINEAR, "exponential": abi.GAS_EXPONENTIAL}
LAGRANGE_POINTS = {"l1": 1, "l2": 2, "l3": 3, "l4": 4, "l5": 5}
# SetMPCOrbitType compares the lower-cased value, so only these names can match
MPC_ORBIT_TYPES = {"aten": 2, "apollo": 3, "amor": 4, "objectwithqlt1_665": 5, "hungaria": 6, "phocaea": 7,
                   "hilda": 8}
MIGRATION_TYPES = {"i": abi.MIGRATION_TYPE_I, "ii": abi.MIGRATION_TYPE_II}
_XSI = "{http://www.w3.org/2001/XMLSchema-instance}"


class ScenarioError(ValueError):
    pass


@dataclass
class Settings:
    phases: str = "Phases.dat"
    integrals: str = "Integrals.dat"
    constant_properties: str = "ConstantProperties.dat"
    variable_properties: str = "VariableProperties.dat"
    composition_properties: str = "CompositionProperties.dat"
    two_body_affair: str = "TwoBodyAffair.dat"
    log: str = "Log.txt"
    integrator_name: str = "rungekutta78"
    integrator: int = abi.RUNGE_KUTTA_FEHLBERG78
    accuracy: float = -10.0   # read and validated; the integrators use epsilon = 1e-10 regardless
    barycentric: bool = False
    length: float = 0.0       # days
    output: float = 0.0       # days
    ejection: float = 0.0     # AU, 0: off
    hit_centrum: float = 0.0  # AU, 0: off
    collision: float | None = None  # factor; None: no Collision element
    h0: float = 0.0           # first step of the main integration
    start: float = 0.0        # TimeLine start (days), else the last (forward) or first epoch
    start_defined: bool = False
    enable_distinct_start_times: bool = False


@dataclass
class Component:
    name: str
    ratio: float


@dataclass
class BodySpec:
    """One Body element after preparation (Body + Characteristics)."""
    id: int
    type: int
    group: int
    name: str = ""
    guid: str = ""
    designation: str = ""
    provisional_designation: str = ""
    reference: str = ""
    opposition: str = ""
    ln: int = 0
    mpc_orbit_type: int = 0
    mig_type: int = abi.MIGRATION_NO
    mig_stop_at: float = 0.0
    has_characteristics: bool = False
    mass: float = 0.0
    radius: float = 0.0
    density: float = 0.0
    cd: float = 0.0
    abs_vis_mag: float = 0.0
    components: list = field(default_factory=list)
    phase: list | None = None
    elements: list | None = None


@dataclass
class Scenario:
    name: str
    description: str
    directory: str
    settings: Settings
    bodies: list            # BodySpec, in integration order
    system: scenarios.System
    insertion: list         # body ids in the order Simulator::Insert writes their properties
    groups: list            # BodyGroup, ordered by start time (reversed for a backward run)
    time0: float            # the time line's time: the start time of the first group with massive bodies
    n_distinct_start_times: int
    gas: dict | None


# ---- attribute handling ------------------------------------------------------------
def _attrs(el, allowed: tuple) -> dict:
    out = {}
    for k, v in el.attrib.items():
        key = ("xsi:" + k[len(_XSI):]) if k.startswith(_XSI) else k
        key = key.lower()
        if key not in allowed:
            raise ScenarioError(f"Unknown attribute: '{k}' in <{el.tag}>")
        out[key] = v
    return out


def _double(a: dict, key: str, el) -> float:
    try:
        return float(a[key].strip())
    except ValueError:
        raise ScenarioError(f"Invalid value: {key}={a[key]!r} in <{el.tag}>") from None


def _unit_attr(a: dict, name: str, table: dict, carried: str, default: str, el) -> str:
    """Valid*UnitAttribute: the element's own unit (validated), else the carried one, else the default."""
    if name in a:
        u = a[name].lower()
        if u not in table:
            raise ScenarioError(f"Undefined unit {a[name]!r} in <{el.tag}>")
        return u
    return carried or default


def _convert(value: float, unit: str, table: dict) -> float:
    f = table.get(unit.lower())
    return value if f is None else value * f  # an unknown carried unit: the reference leaves the value as is


class _Quantity:
    """DeserializeDimensionalQuantity with the value and unit variables its
    callers share between sibling elements."""

    def __init__(self):
        self.value = 0.0
        self.unit = ""

    def read(self, el, table: dict, default: str) -> float:
        a = _attrs(el, ("value", "unit"))
        if "value" in a:
            v = _double(a, "value", el)
            if not v >= 0.0:
                raise ScenarioError(f"Value out of range: value={a['value']!r} in <{el.tag}>")
            self.value = v
        self.unit = _unit_attr(a, "unit", table, self.unit.lower(), default, el)
        return _convert(self.value, self.unit, table)


def _shift_into_range(lower: float, upper: float, value: float) -> float:
    """Ephemeris::ShiftIntoRange (Ephemeris.cpp:228-239)."""
    rng = upper - lower
    while value >= upper:
        value -= rng
    while value < lower:
        value += rng
    return value


def _text(el) -> str:
    return (el.text or "").strip()


# ---- Settings --------------------------------------------------------------------------
def _read_settings(se) -> Settings:
    st = Settings()
    a = _attrs(se, ("enabledistinctstarttimes", "barycentric"))
    for key in a:
        v = a[key].strip().lower()
        if v not in ("true", "false"):
            raise ScenarioError(f"Invalid value: {key}={a[key]!r}")
        if key == "barycentric":
            st.barycentric = v == "true"
        else:
            st.enable_distinct_start_times = v == "true"
    out = se.find("Output")
    if out is not None:
        for tag, key in (("Phases", "phases"), ("ConstantProperties", "constant_properties"),
                         ("Integrals", "integrals"), ("VariableProperties", "variable_properties"),
                         ("CompositionProperties", "composition_properties"),
                         ("TwoBodyAffair", "two_body_affair"), ("Log", "log")):
            e = out.find(tag)
            if e is not None and _text(e):
                setattr(st, key, _text(e))
    integ = se.find("Integrator")
    if integ is None:
        raise ScenarioError("Missing Integrator tag")
    ia = _attrs(integ, ("name", "xsi:type", "xmlns:xsi", "xmlns:xsd"))
    for key in ("name", "xsi:type"):
        if key in ia:
            st.integrator_name = ia[key].strip().lower()
    if st.integrator_name not in INTEGRATORS:
        raise ScenarioError("Unknown integrator type!")
    st.integrator = INTEGRATORS[st.integrator_name]
    acc = integ.find("Accuracy")
    if acc is not None:
        aa = _attrs(acc, ("value",))
        if "value" in aa:
            st.accuracy = _double(aa, "value", acc)
            if not -16.0 <= st.accuracy <= 0.0:
                raise ScenarioError(f"Value out of range: value={aa['value']!r} in <Accuracy>")
    tl = se.find("TimeLine")
    if tl is None:
        raise ScenarioError("Missing TimeLine tag")
    ta = _attrs(tl, ("start", "length", "output", "unit"))
    tu = _unit_attr(ta, "unit", TIME_UNITS, "", "day", tl)
    if "start" in ta:
        st.start = _convert(_double(ta, "start", tl), tu, TIME_UNITS)
        st.start_defined = True
    if "length" in ta:
        length = _double(ta, "length", tl)
        if length == 0.0:
            raise ScenarioError(f"Invalid value: length={ta['length']!r}")
        st.length = _convert(length, tu, TIME_UNITS)
    if "output" in ta:
        output = _double(ta, "output", tl)
        if not output > 0.0:
            raise ScenarioError(f"Value out of range: output={ta['output']!r}")
        st.output = _convert(output, tu, TIME_UNITS)
    q = _Quantity()
    e = se.find("Ejection")
    if e is not None:
        st.ejection = q.read(e, DISTANCE_UNITS, "au")
    e = se.find("HitCentrum")
    if e is not None:
        st.hit_centrum = q.read(e, DISTANCE_UNITS, "au")
    col = se.find("Collision")
    if col is not None:
        factor = _event_condition(col)
        if factor < 1.0:
            raise ScenarioError("Invalid value for 'factor' in <Collision>")
        st.collision = factor
    for tag in ("CloseEncounter", "WeakCapture"):  # read and validated; no event uses them
        e = se.find(tag)
        if e is not None:
            _event_condition(e)
    return st


def _event_condition(el) -> float:
    a = _attrs(el, ("factor", "stop"))
    factor = 0.0
    if "factor" in a:
        factor = _double(a, "factor", el)
        if not factor >= 0.0:
            raise ScenarioError(f"Value out of range: factor={a['factor']!r}")
    if "stop" in a and a["stop"].strip().lower() not in ("true", "false"):
        raise ScenarioError(f"Invalid value: stop={a['stop']!r}")
    return factor


# ---- gas -----------------------------------------------------------------------------------
def _power_law(el, current: tuple) -> tuple:
    a = _attrs(el, ("c", "index"))
    c, idx = current
    if "c" in a:
        c = _double(a, "c", el)
    if "index" in a:
        idx = _double(a, "index", el)
    return (c, idx)


def _read_gas(gc, legacy_gas_tags: bool = False) -> dict:
    """DeserializeGasComponent (:1900-2170) over GasComponent's defaults; the
    mean free path keeps the default density's value."""
    gas = scenarios.default_gas()
    a = _attrs(gc, ("alpha", "type", "timescale", "t0", "t1", "unit"))
    tu = _unit_attr(a, "unit", TIME_UNITS, "", "day", gc)
    for key in a:
        if key == "alpha":
            v = _double(a, key, gc)
            if not v > 0.0:
                raise ScenarioError(f"Value out of range: alpha={a[key]!r}")
            gas["alpha"] = v
        elif key == "type":
            t = a[key].strip().lower()
            if t not in GAS_DECREASE:
                raise ScenarioError(f"Invalid gas decrease type {a[key]!r}")
            gas["decrease_type"] = GAS_DECREASE[t]
        elif key == "timescale":
            v = _double(a, key, gc)
            if not v >= 0.0:
                raise ScenarioError(f"Value out of range: timeScale={a[key]!r}")
            gas["time_scale"] = _convert(v, tu, TIME_UNITS)
        elif key in ("t0", "t1"):
            gas[key] = _convert(_double(a, key, gc), tu, TIME_UNITS)
    for tag, key in (("Eta", "eta"), ("Tau", "tau"), ("ScaleHeight", "scale_height")):
        e = gc.find(tag)
        if e is not None:
            gas[key] = _power_law(e, gas[key])
    for tag, child in (("DensityFunction", "Density"),) + ((("GasDensityFunction", "VolumeDensity"),)
                                                             if legacy_gas_tags else ()):
        df = gc.find(tag)
        if df is None:
            continue
        c, idx = gas["density"]
        da = _attrs(df, ("index",))
        if "index" in da:
            idx = _double(da, "index", df)
        d = df.find(child)
        if d is not None:
            c = _Quantity().read(d, VOLUME_DENSITY_UNITS, "solarau3")
        gas["density"] = (c, idx)
    return gas


# ---- bodies -----------------------------------------------------------------------------------
def _read_vector(el, table: dict, default: str) -> list:
    a = _attrs(el, ("x", "y", "z", "unit"))
    u = _unit_attr(a, "unit", table, "", default, el)
    return [_convert(_double(a, k, el) if k in a else 0.0, u, table) for k in "xyz"]


_OE_NAMES = {"semimajoraxis": 0, "a": 0, "eccentricity": 1, "e": 1, "inclination": 2, "incl": 2,
             "argumentofpericenter": 3, "peri": 3, "longitudeofnode": 4, "node": 4, "meananomaly": 5, "m": 5}


def _read_elements(el) -> list:
    """DeserializeOrbitalElement (:1241-1365): angles to radians, the
    argument of pericentre, the node and the mean anomaly shifted into [0, 2 pi)."""
    a = _attrs(el, tuple(_OE_NAMES) + ("angleunit", "distanceunit"))
    du = _unit_attr(a, "distanceunit", DISTANCE_UNITS, "", "au", el)
    au = _unit_attr(a, "angleunit", ANGLE_UNITS, "", "radian", el)
    oe = [-1.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    for key in a:
        if key not in _OE_NAMES:
            continue
        k = _OE_NAMES[key]
        v = _double(a, key, el)
        if k == 0:
            if not v > 0:
                raise ScenarioError(f"Value out of range: {key}={a[key]!r}")
            v = _convert(v, du, DISTANCE_UNITS)
        elif k == 1:
            if not 0.0 <= v < 1.0:
                raise ScenarioError(f"Value out of range: {key}={a[key]!r}")
        elif k == 2:
            v = _convert(v, au, ANGLE_UNITS)
            if not 0.0 <= v <= PI:
                raise ScenarioError(f"Value out of range: {key}={a[key]!r}")
        else:
            v = _shift_into_range(0.0, 2.0 * PI, _convert(v, au, ANGLE_UNITS))
        oe[k] = v
    if oe[0] < 0.0:
        raise ScenarioError("the semi-major axis of an OrbitalElement is not defined")
    return oe


def _read_characteristics(ch, b: BodySpec):
    a = _attrs(ch, ("absvismag", "cd"))
    if "absvismag" in a:
        b.abs_vis_mag = _double(a, "absvismag", ch)
    if "cd" in a:
        v = _double(a, "cd", ch)
        if not v >= 0.0:
            raise ScenarioError(f"Value out of range: cd={a['cd']!r}")
        b.cd = v
    q = _Quantity()
    m = ch.find("Mass")
    if m is None:
        raise ScenarioError("Missing Mass tag")
    b.mass = q.read(m, MASS_UNITS, "solar")
    r = ch.find("Radius")
    if r is not None:
        b.radius = q.read(r, DISTANCE_UNITS, "au")
    d = ch.find("Density")
    if b.type != abi.SUPER_PLANETESIMAL and d is not None and b.radius > 0:
        raise ScenarioError("Both the radius and the density are defined")
    if d is not None:
        b.density = q.read(d, VOLUME_DENSITY_UNITS, "solarau3")
    cl = ch.find("ComponentList")
    if cl is not None:
        for c in cl.findall("Component"):
            ca = _attrs(c, ("name", "ratio"))
            ratio = 0.0
            if "ratio" in ca:
                ratio = _double(ca, "ratio", c)
                if not 0.0 <= ratio <= 100.0:
                    raise ScenarioError(f"Value out of range: ratio={ca['ratio']!r}")
            b.components.append(Component(ca.get("name", ""), ratio))
        if not b.components:
            raise ScenarioError("The ComponentList is empty")
        total = 100.0
        for c in b.components:
            total -= c.ratio
        if abs(total) > 1.0e-4:
            raise ScenarioError("The sum of the component ratios is not 100")
    b.has_characteristics = True


def _read_body(el, bid: int, group: int) -> BodySpec:
    a = _attrs(el, ("name", "type", "mpcorbittype", "designation", "des", "provisionaldesignation", "provdes",
                    "reference", "ref", "opposition", "opp", "ln", "guid"))
    b = BodySpec(id=bid, type=0, group=group)
    for key, v in a.items():
        v = v.strip()
        if key == "type":
            t = v.lower()
            if t not in BODY_TYPES:
                raise ScenarioError(f"Invalid body type {v!r}")
            b.type = BODY_TYPES[t]
        elif key == "name":
            b.name = v
        elif key == "guid":
            b.guid = v
        elif key in ("designation", "des"):
            b.designation = v
        elif key in ("provisionaldesignation", "provdes"):
            b.provisional_designation = v
        elif key in ("reference", "ref"):
            b.reference = v
        elif key in ("opposition", "opp"):
            b.opposition = v
        elif key == "ln":
            if v.lower() not in LAGRANGE_POINTS:
                raise ScenarioError(f"Invalid ln {v!r}")
            b.ln = LAGRANGE_POINTS[v.lower()]
        elif key == "mpcorbittype":
            if v.lower() not in MPC_ORBIT_TYPES:
                raise ScenarioError(f"Invalid mpcOrbitType {v!r}")
            b.mpc_orbit_type = MPC_ORBIT_TYPES[v.lower()]
    if b.type == 0:
        raise ScenarioError(f"The type of body {b.name or bid} is not defined")
    ph, oe = el.find("Phase"), el.find("OrbitalElement")
    if b.type == abi.CENTRAL_BODY and ph is None and oe is None:
        b.phase = [0.0] * 6
    elif ph is not None and oe is not None:
        raise ScenarioError(f"body {b.name or bid}: both Phase and OrbitalElement are defined")
    elif ph is None and oe is None:
        raise ScenarioError(f"body {b.name or bid}: neither Phase nor OrbitalElement is defined")
    elif ph is not None:
        pos, vel = ph.find("Position"), ph.find("Velocity")
        if pos is None:
            raise ScenarioError("Missing Position tag")
        if vel is None:
            raise ScenarioError("Missing Velocity tag")
        b.phase = _read_vector(pos, DISTANCE_UNITS, "au") + _read_vector(vel, VELOCITY_UNITS, "auday")
    else:
        if b.type == abi.CENTRAL_BODY:
            raise ScenarioError("a central body given by orbital elements is not supported")
        b.elements = _read_elements(oe)
    if b.type != abi.TEST_PARTICLE:
        ch = el.find("Characteristics")
        if ch is None:
            raise ScenarioError("Missing Characteristics tag")
        _read_characteristics(ch, b)
        mg = el.find("Migration")
        if mg is not None:
            ma = _attrs(mg, ("type", "stopat"))
            if "type" in ma:
                t = ma["type"].strip().lower()
                if t not in MIGRATION_TYPES:
                    raise ScenarioError(f"Invalid migration type {ma['type']!r}")
                b.mig_type = MIGRATION_TYPES[t]
            if "stopat" in ma:
                v = _double(ma, "stopat", mg)
                if not v > 0.0:
                    raise ScenarioError(f"Value out of range: stopAt={ma['stopat']!r}")
                b.mig_stop_at = v
    return b


# ---- epochs (Ephemeris::GetJulianDate and friends, Ephemeris.cpp:247-462) -----------------
def _atof(text: str) -> float:
    k = 0
    while k < len(text) and (text[k].isdigit() or text[k] == "."):
        k += 1
    head = text[:k]
    while head:
        try:
            return float(head)
        except ValueError:
            head = head[:-1]
    return 0.0


def _atoi(text: str) -> int:
    k = 0
    while k < len(text) and text[k].isdigit():
        k += 1
    return int(text[:k]) if k else 0


def _to_julian_date(year: int, month: int, day: int) -> float:
    """Ephemeris::ToJulianDate (Ephemeris.cpp:394-424) at 0h UT."""
    y = year - 1 if month <= 2 else year
    m = month + 12 if month <= 2 else month
    if year < 1582 or (year == 1582 and month < 10) or (year == 1582 and month == 10 and day <= 4):
        b = -2
    else:
        b = math.floor(y / 400.0) - math.floor(y / 100.0)
    universal_time = 0 / 3600000.0 + 0 / 3600.0 + 0 / 60.0 + 0
    return (math.floor(365.25 * y) + math.floor(30.6001 * (m + 1)) + b) + 1720996.5 + day + universal_time / 24.0


def julian_date(epoch: str) -> float:
    """An epoch as the reference reads it: 'JD2451545.0' (a Julian date),
    'YYYYMMDD' (a date, at most 8 digits) or a 5-character packed date
    ('K0101': century letter I-K, two digits of the year, month 1-9 / A-C,
    day 1-9 / A-V)."""
    if epoch[:2].lower() == "jd":
        if not all(c.isdigit() or c == "." for c in epoch[2:]):
            raise ScenarioError(f"Bad JulianDate format: {epoch}")
        return _atof(epoch[2:])
    if epoch[:1].isdigit():
        if len(epoch) > 8 or not epoch.isdigit():
            raise ScenarioError(f"Bad Date format: {epoch}")
        return _to_julian_date(_atoi(epoch[0:4]), _atoi(epoch[4:6]), _atoi(epoch[6:8]))
    if (len(epoch) != 5 or not "I" <= epoch[0] <= "K" or not epoch[1:3].isdigit()
            or not (epoch[3].isdigit() or "A" <= epoch[3] <= "C")
            or not (epoch[4].isdigit() or "A" <= epoch[4] <= "V")):
        raise ScenarioError(f"Bad PackedDate format: {epoch}")
    year = (ord(epoch[0]) - ord("I") + 18) * 100 + _atoi(epoch[1:3])
    month = int(epoch[3]) if epoch[3].isdigit() else ord(epoch[3]) - ord("A") + 10
    day = int(epoch[4]) if epoch[4].isdigit() else ord(epoch[4]) - ord("A") + 10
    return _to_julian_date(year, month, day)


# ---- the simulation -------------------------------------------------------------------------
@dataclass
class BodyGroup:
    description: str
    epoch: str
    offset: float
    reference_frame: str
    bodies: list
    start_time: float = 0.0


def load(path: str, legacy_gas_tags: bool = False) -> Scenario:
    """Read and prepare a scenario file; raises ScenarioError where the
    reference reports an error.  legacy_gas_tags also reads the gas density
    written as <GasDensityFunction index=..><VolumeDensity value unit/>
    (the form the reference's own scenario files use, which its reader
    ignores) as the DensityFunction."""
    try:
        root = ET.parse(path).getroot()
    except ET.ParseError as e:
        raise ScenarioError(f"{path}: {e}") from None
    if root.tag != "Simulation":
        raise ScenarioError("Missing Simulation tag")
    sa = _attrs(root, ("name", "description"))
    se = root.find("Settings")
    if se is None:
        raise ScenarioError("Missing Settings tag")
    st = _read_settings(se)
    bgl = root.find("BodyGroupList")
    if bgl is None:
        raise ScenarioError("Missing BodyGroupList tag")
    groups = []
    next_id = 0
    for g, bg in enumerate(bgl.findall("BodyGroup")):
        ga = _attrs(bg, ("description", "epoch", "offset", "referenceframe", "guid"))
        offset = _double(ga, "offset", bg) if "offset" in ga else 0.0
        items = bg.find("Items")
        if items is None:
            raise ScenarioError("Missing Items tag")
        bodies = []
        for be in items.findall("Body"):
            bodies.append(_read_body(be, next_id, g))
            next_id += 1
        if not bodies:
            raise ScenarioError("Missing Body tag")
        groups.append(BodyGroup(ga.get("description", "").strip(), ga.get("epoch", "").strip(), offset,
                                ga.get("referenceframe", "").strip(), bodies))
    if not groups:
        raise ScenarioError("Missing BodyGroup tag")
    gas = None
    neb = root.find("Nebula")
    if neb is not None:
        na = _attrs(neb, ("name", "description", "fargopath"))
        if na.get("fargopath"):
            raise ScenarioError("FARGO coupling is not supported")
        gc = neb.find("GasComponent")
        gas = _read_gas(gc, legacy_gas_tags) if gc is not None else scenarios.default_gas()
    _check_body_group_list(groups)
    groups, time0, n_distinct = _initialize(st, groups)
    body_list, insertion = [], []
    for g in insertion_order(st, groups, time0, n_distinct):
        body_list, written = insert_group(body_list, g.bodies)
        insertion += [b.id for b in written]
    check_type_order(body_list)
    system = build_system(st, body_list, gas)
    st.h0 = first_step(body_list, st.length)
    system.h0 = st.h0
    return Scenario(name=sa.get("name", ""), description=sa.get("description", ""),
                    directory=os.path.dirname(os.path.abspath(path)), settings=st, bodies=body_list, system=system,
                    insertion=insertion, groups=groups, time0=time0, n_distinct_start_times=n_distinct, gas=gas)


def _calculate_phase(mu: float, el: list) -> list:
    """Ephemeris::CalculatePhase (Ephemeris.cpp:141-176) with the reference
    build's KeplerEquationSolver (:187-211): the change of each Newton step is
    measured through int abs(), so the iteration ends once it is below 1."""
    a, e, inc, peri, node, m = el
    if e == 0.0 or m == 0.0 or m == PI:
        E = m
    else:
        E = m + e * (math.sin(m)) / (1.0 - math.sin(m + e) + math.sin(m))
        step = 0
        while True:
            E1 = E - (E - e * math.sin(E) - m) / (1.0 - e * math.cos(E))
            err = float(abs(int(E1 - E)))
            E = E1
            step += 1
            if not (err > 1.0e-14 and step <= 25):
                break
        if step > 25:
            raise ScenarioError("The phase could not be computed (Kepler's equation)")
    v = 2.0 * math.atan(math.sqrt((1.0 + e) / (1.0 - e)) * math.tan(E / 2.0))
    p = a * (1.0 - e * e)
    r = p / (1.0 + e * math.cos(v))
    kszi = r * math.cos(v)
    eta = r * math.sin(v)
    vk = -math.sqrt(mu / p) * math.sin(v)
    ve = math.sqrt(mu / p) * (e + math.cos(v))
    cw, sw = math.cos(peri), math.sin(peri)
    cO, sO = math.cos(node), math.sin(node)
    ci, si = math.cos(inc), math.sin(inc)
    P = (cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si)
    Q = (-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si)
    return [kszi * P[k] + eta * Q[k] for k in range(3)] + [vk * P[k] + ve * Q[k] for k in range(3)]


def _check_body_group_list(groups: list):
    """Simulation::CheckBodyGroupList (Simulation.cpp:174-220)."""
    if len(groups) == 1 and len(groups[0].bodies) <= 1:
        raise ScenarioError("There is only one body defined in the Simulation!")
    all_bodies = [b for g in groups for b in g.bodies]
    n_cb = sum(1 for b in all_bodies if b.type == abi.CENTRAL_BODY)
    if n_cb > 1:
        raise ScenarioError("There are more than 1 central body defined!")
    if n_cb == 0:
        raise ScenarioError("The central body is not defined!")
    if len({g.reference_frame for g in groups if g.reference_frame}) > 1:
        raise ScenarioError("The BodyGroups have different reference frames!")


def _initialize(st: Settings, groups: list):
    """Simulation::Initialize (Simulation.cpp:28-172): start times from the
    epochs, the groups ordered by start time, the time line's time, phases
    and radii.  Returns the ordered groups, the time line's time and the
    number of distinct start times."""
    forward = st.length >= 0
    if not st.start_defined:  # SetStartTimeOfMainPhase: the last (forward) or first epoch, else 0
        jds = sorted({julian_date(g.epoch) for g in groups if g.epoch})
        st.start = (jds[-1] if forward else jds[0]) if jds else 0.0
    for g in groups:  # BodyGroup::SetStartTime
        g.start_time = (julian_date(g.epoch) if g.epoch else st.start) + g.offset
    distinct = sorted({g.start_time for g in groups})
    count = 0  # BodyGroupList::DistinctStartTimesOfMassiveBodies: non-central bodies with characteristics
    for t in distinct:
        count += sum(1 for g in groups if g.start_time == t for b in g.bodies
                     if b.type not in (abi.TEST_PARTICLE, abi.CENTRAL_BODY)) > 0
    if not st.enable_distinct_start_times and count > 1:
        raise ScenarioError("More than 1 BodyGroup contain massive bodies with different start times!")
    groups = sorted(groups, key=lambda g: g.start_time)  # std::list::sort is stable
    if not forward:
        groups.reverse()
    if not st.enable_distinct_start_times:  # SetTimeAndSaveOfTimeLine
        massive = [g for g in groups
                   if any(b.type not in (abi.CENTRAL_BODY, abi.TEST_PARTICLE) and b.mass > 0 for b in g.bodies)]
        if not massive:
            raise ScenarioError("None of the BodyGroups contains massive bodies!")
        time0 = massive[0].start_time
    else:
        time0 = groups[0].start_time
    central = next(b for g in groups for b in g.bodies if b.type == abi.CENTRAL_BODY)
    central_gm = GAUSS2 * central.mass
    for g in groups:  # Simulation::SetPhasesRadiiDensity (:131-172)
        for b in g.bodies:
            if b.type != abi.CENTRAL_BODY and b.phase is None:
                mu = central_gm + (GAUSS2 * b.mass if b.type != abi.TEST_PARTICLE else 0.0)
                b.phase = _calculate_phase(mu, b.elements)
            if b.type in (abi.SUPER_PLANETESIMAL, abi.TEST_PARTICLE):
                continue
            if b.radius == 0.0 and b.density == 0.0:
                continue
            if b.radius == 0.0:  # Characteristics::CalculateRadius
                b.radius = math.pow(3.0 / (4.0 * PI) * b.mass / b.density, 1.0 / 3.0)
            else:                # Characteristics::CalculateDensity / CalculateVolume
                b.density = b.mass / (4.0 / 3.0 * PI * math.pow(b.radius, 3))
    return groups, time0, len(distinct)


def sync_start_times(st: Settings, groups: list, time0: float) -> list:
    """The start times Simulator::Synchronization (Simulator.cpp:322-390) walks:
    the distinct start times in the run's direction, preceded by the time
    line's time unless distinct start times are enabled."""
    times = sorted({g.start_time for g in groups})
    if st.length < 0:
        times.reverse()
    if not st.enable_distinct_start_times:
        times.insert(0, time0)
    return times


def insertion_order(st: Settings, groups: list, time0: float, n_distinct: int) -> list:
    """The groups in the order the run inserts them: by the synchronisation's
    start times when there are several, else in the list's order
    (Simulator::PopulateBodyList)."""
    if n_distinct <= 1:
        return list(groups)
    out = []
    for t in sync_start_times(st, groups, time0):
        out += [g for g in groups if g.start_time == t and g not in out]
    return out


def insert_group(body_list: list, group_bodies: list):
    """Simulator::Insert / SetIteratorAfter (Simulator.cpp:449-495): each type
    of the group, in type order, goes after the bodies of that type found from
    the position the previous type left.  Returns the new list and the
    group's bodies in the order their properties are written."""
    body_list = list(body_list)
    written = []
    it = 0
    for t in range(1, 8):
        of_type = [b for b in group_bodies if b.type == t]
        if not of_type:
            continue
        written += of_type
        while it < len(body_list) and body_list[it].type != t:
            it += 1
        while it < len(body_list) and body_list[it].type == t:
            it += 1
        body_list[it:it] = of_type
        it += len(of_type)  # std::list::insert leaves the iterator after the inserted range
    return body_list, written


def check_type_order(body_list: list):
    if (not body_list or body_list[0].type != abi.CENTRAL_BODY
            or any(body_list[k].type > body_list[k + 1].type for k in range(len(body_list) - 1))):
        raise ScenarioError("the body groups would be integrated out of type order (central body first, then "
                            "giant, rocky and proto-planets, super-planetesimals, planetesimals, test particles)")


def build_system(st: Settings, bodies: list, gas: dict | None) -> scenarios.System:
    """Simulator::BodyListToBodyData (Simulator.cpp:525-593): the body data of
    the current body list, moved to the barycentre in a barycentric run."""
    n = len(bodies)
    counts = tuple(sum(1 for b in bodies if b.type == t) for t in range(1, 8))
    ge, gs = np.zeros(n), np.zeros(n)
    mass, radius, density, cd = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
    for i, b in enumerate(bodies):
        if b.type == abi.TEST_PARTICLE:
            continue
        mass[i], radius[i], density[i], cd[i] = b.mass, b.radius, b.density, b.cd
        if b.radius > 0:  # Characteristics::GammaEpstein / GammaStokes
            ge[i] = 1.0 / (b.density * b.radius)
            gs[i] = (3.0 / 8.0) * b.cd / (b.density * b.radius) if b.cd > 0 else 0.0
    y0 = np.array([v for b in bodies for v in b.phase], np.float64)
    if st.barycentric:  # Calculate::PhaseOfBC / PhaseWithRespectToBC (Calculate.cpp:65-105)
        n_massive = counts[0] + counts[1] + counts[2] + counts[3]
        total = 0.0
        for i in range(n_massive):
            total += mass[i]
        bc = [0.0] * 6
        for i in range(n):
            for j in range(6):
                bc[j] += mass[i] * y0[6 * i + j]
        bc = [c / total for c in bc]
        for i in range(n):
            for j in range(6):
                y0[6 * i + j] -= bc[j]
    return scenarios.System(
        name="scenario", counts=counts, id=np.array([b.id for b in bodies], np.int32),
        type=np.array([b.type for b in bodies], np.int32),
        mig_type=np.array([b.mig_type for b in bodies], np.int32),
        mig_stop_at=np.array([b.mig_stop_at for b in bodies]), mass=mass, radius=radius, density=density, cd=cd,
        gamma_stokes=gs, gamma_epstein=ge, y0=y0, gas=gas, barycentric=st.barycentric, integrator=st.integrator,
        length=st.length)


def first_step(bodies: list, length: float, divisor: float = 50000.0) -> float:
    """Simulator::ShortestPeriod (Simulator.cpp:510-523) with
    Body::CalculateOrbitalPeriod (Body.cpp:89-98) over the body list's phases,
    / 50,000 (the main integration; 50 for synchronisation and
    pre-integration), signed by the direction and clamped to the length."""
    central_gm = GAUSS2 * bodies[0].mass
    period = 1.0e10
    for b in bodies:
        if b.type == abi.CENTRAL_BODY:
            continue
        mu = central_gm + (0.0 if b.type == abi.TEST_PARTICLE else GAUSS2 * b.mass)
        x, y, z, vx, vy, vz = b.phase
        h = (vx * vx + vy * vy + vz * vz) / 2.0 + (-mu / math.sqrt(x * x + y * y + z * z))
        if h > 0.0:
            p = -1.0
        else:
            a = -mu / (2.0 * h)
            p = 2.0 * PI * math.sqrt((a * a * a) / mu)
        if 0 < p < period:
            period = p
    h0 = period / divisor if length >= 0 else -period / divisor
    if abs(h0) > abs(length):
        h0 = length
    return h0

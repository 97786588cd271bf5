"""Seeded synthetic scenarios with the shapes and distributions of the five
workloads the engine is measured on (no dataset is involved).

Bodies are sorted by BodyType with the central body at index 0, as
Simulator::BodyListToBodyData lays them out (Solaris/Simulator.cpp:525-593).
Initial phases come from Keplerian elements with mu = G (m0 + m_i) (test
particles: G m0), following Ephemeris::CalculatePhase
(Solaris/Ephemeris.cpp:141-176) with a converged Kepler solver.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import abi

# Solaris/Constants.h
SOLAR_TO_KILOGRAM = 1.98911e30
AU_TO_METER = 1.495978707e11
METER_TO_AU = 1.0 / AU_TO_METER
GRAM_TO_SOLAR = 1.0 / (1.0e3 * SOLAR_TO_KILOGRAM)
GRAM_PER_CM3_TO_SOLAR_PER_AU3 = GRAM_TO_SOLAR / (1.0e-2 * METER_TO_AU) ** 3
SOLAR_RADIUS_TO_AU = 1.0 / 215.094
DEG = 1.745329251994329509e-2
YEAR_TO_DAY = 365.25
PROTON_MASS_CMU = 1.672621777e-27 * (1.0 / SOLAR_TO_KILOGRAM)


@dataclasses.dataclass
class System:
    """BodyData contents of one system plus its run settings."""
    name: str
    counts: tuple
    id: np.ndarray
    type: np.ndarray
    mig_type: np.ndarray
    mig_stop_at: np.ndarray
    mass: np.ndarray
    radius: np.ndarray
    density: np.ndarray
    cd: np.ndarray
    gamma_stokes: np.ndarray
    gamma_epstein: np.ndarray
    y0: np.ndarray
    gas: dict | None = None
    barycentric: bool = False
    integrator: int = abi.RUNGE_KUTTA_FEHLBERG78
    epsilon: float = 1.0e-10
    h0: float = 0.0
    length: float = 0.0

    @property
    def n(self) -> int:
        return int(sum(self.counts))

    def pair_count(self) -> int:
        """Pair interactions per force evaluation: one Kepler term per body
        i >= 1 plus the direct terms of GravityAC (Acceleration.cpp:268-317)."""
        c = self.counts
        nm = c[0] + c[1] + c[2] + c[3]
        nspl = c[4]
        n = self.n
        t = self.type
        total = 0
        for lo, hi, ns in _sink_ranges(t, nm, nspl):
            cnt = hi - lo
            total += cnt * (ns - 1)
            total -= max(0, min(hi, ns) - max(lo, 1))  # j == i excluded
        return int(total + (n - 1))


def _sink_ranges(t, nm, nspl):
    n = len(t)
    out = []
    lo = 1
    while lo < n:
        massive_src = t[lo] <= abi.PROTO_PLANET
        hi = lo
        while hi < n and (t[hi] <= abi.PROTO_PLANET) == massive_src:
            hi += 1
        out.append((lo, hi, nm + nspl if massive_src else nm))
        lo = hi
    return out


def default_gas() -> dict:
    """GasComponent::GasComponent() defaults (Solaris/GasComponent.cpp:9-34).
    The mean free path is built from the default density and, as in the
    reference, is not rebuilt when the density is changed later."""
    density_c = 1.4e-9 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    density_idx = -2.75
    mmw = 2.3
    pdiam = 3.0e-10
    clambda = mmw * PROTON_MASS_CMU / (math.sqrt(2.0) * math.pi * (pdiam * METER_TO_AU) ** 2 * density_c)
    return dict(alpha=2.0e-3, decrease_type=abi.GAS_CONSTANT, quirks=abi.QUIRKS_REFERENCE, time_scale=0.0,
                t0=0.0, t1=0.0, inner_edge=10.0 * SOLAR_RADIUS_TO_AU, mean_molecular_weight=mmw,
                particle_diameter=pdiam, eta=(0.0019, 0.5), tau=(2.0 / 3.0, 2.0), scale_height=(0.02, 1.25),
                density=(density_c, density_idx), mean_free_path=(clambda, -density_idx))


def kepler_E(e, M):
    E = np.where(e < 0.8, M, np.pi * np.ones_like(M))
    for _ in range(60):
        f = E - e * np.sin(E) - M
        E = E - f / (1.0 - e * np.cos(E))
    return E


def elements_to_phase(mu, a, e, inc, peri, node, M):
    """Vectorised Keplerian elements -> heliocentric phase (x, y, z, vx, vy, vz)."""
    mu = np.broadcast_to(np.asarray(mu, dtype=np.float64), np.shape(a))
    E = kepler_E(e, M)
    v = 2.0 * np.arctan(np.sqrt((1.0 + e) / (1.0 - e)) * np.tan(E / 2.0))
    p = a * (1.0 - e * e)
    r = p / (1.0 + e * np.cos(v))
    kszi, eta = r * np.cos(v), r * np.sin(v)
    vk = -np.sqrt(mu / p) * np.sin(v)
    ve = np.sqrt(mu / p) * (e + np.cos(v))
    cw, sw, cO, sO, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    P = np.stack([cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si], axis=-1)
    Q = np.stack([-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si], axis=-1)
    pos = kszi[:, None] * P + eta[:, None] * Q
    vel = vk[:, None] * P + ve[:, None] * Q
    return np.concatenate([pos, vel], axis=1)


def orbital_period(mu, a):
    return 2.0 * math.pi * math.sqrt(a ** 3 / mu)


def _assemble(name, groups, gas=None, **kw) -> System:
    """groups: list of (type, dict of per-body arrays incl. 'phase')."""
    order = sorted(groups, key=lambda g: g[0])
    counts = [0] * 7
    cols = {k: [] for k in ("type", "mig_type", "mig_stop_at", "mass", "radius", "density", "cd", "phase")}
    for t, d in order:
        m = len(d["mass"])
        counts[t - 1] += m
        cols["type"].append(np.full(m, t, np.int32))
        cols["mig_type"].append(np.asarray(d.get("mig_type", np.zeros(m)), np.int32))
        cols["mig_stop_at"].append(np.asarray(d.get("mig_stop_at", np.zeros(m)), np.float64))
        for k in ("mass", "radius", "density", "cd"):
            cols[k].append(np.asarray(d.get(k, np.zeros(m)), np.float64))
        cols["phase"].append(np.asarray(d["phase"], np.float64).reshape(m, 6))
    arr = {k: np.concatenate(v) for k, v in cols.items()}
    n = len(arr["mass"])
    radius, density, cd = arr["radius"], arr["density"], arr["cd"]
    # Simulator::BodyListToBodyData (Solaris/Simulator.cpp:542-568) and
    # Characteristics::GammaEpstein/GammaStokes (Characteristics.cpp:75-87)
    with np.errstate(divide="ignore", invalid="ignore"):
        ge = np.where(radius > 0, 1.0 / (density * radius), 0.0)
        gs = np.where((radius > 0) & (cd > 0), (3.0 / 8.0) * cd / (density * radius), 0.0)
    tp = arr["type"] == abi.TEST_PARTICLE
    for a in (arr["mass"], radius, density, cd, ge, gs):
        a[tp] = 0.0
    return System(name=name, counts=tuple(counts), id=np.arange(1, n + 1, dtype=np.int32), type=arr["type"],
                  mig_type=arr["mig_type"], mig_stop_at=arr["mig_stop_at"], mass=arr["mass"], radius=radius,
                  density=density, cd=cd, gamma_stokes=gs, gamma_epstein=ge,
                  y0=np.ascontiguousarray(arr["phase"].reshape(-1)), gas=gas, **kw)


def _star(mass=1.0):
    rho = 1.408 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    return (abi.CENTRAL_BODY, dict(mass=[mass], radius=[SOLAR_RADIUS_TO_AU], density=[rho], phase=np.zeros((1, 6))))


def _shortest_period(sysm: System) -> float:
    """Simulator::ShortestPeriod (Solaris/Simulator.cpp:510-523) from the phases."""
    m0 = sysm.mass[0]
    y = sysm.y0.reshape(-1, 6)
    best = 1.0e10
    for i in range(1, sysm.n):
        mu = abi.GAUSS2 * (m0 + (0.0 if sysm.type[i] == abi.TEST_PARTICLE else sysm.mass[i]))
        r = np.linalg.norm(y[i, :3])
        v2 = float(np.dot(y[i, 3:], y[i, 3:]))
        en = 0.5 * v2 - mu / r
        if en >= 0:
            continue
        a = -mu / (2 * en)
        p = orbital_period(mu, a)
        if 0 < p < best:
            best = p
    return best


def config1(seed: int = 1001, n_tp: int = 253) -> System:
    """1 star + 2 giants (1e-3, 3e-4 Msun at 5.2, 9.5 AU) + 253 test particles;
    RKF78 eps 1e-10, 1000 yr, heliocentric."""
    rng = np.random.default_rng(seed)
    m0 = 1.0
    mg = np.array([1.0e-3, 3.0e-4])
    ag = np.array([5.2, 9.5])
    eg = rng.uniform(0, 0.05, 2)
    ig = rng.uniform(0, 1.0, 2) * DEG
    ang = rng.uniform(0, 2 * np.pi, (3, 2))
    pg = elements_to_phase(abi.GAUSS2 * (m0 + mg), ag, eg, ig, ang[0], ang[1], ang[2])
    at = rng.uniform(3, 12, n_tp)
    et = rng.uniform(0, 0.1, n_tp)
    it = rng.uniform(0, 2.0, n_tp) * DEG
    angt = rng.uniform(0, 2 * np.pi, (3, n_tp))
    pt = elements_to_phase(abi.GAUSS2 * m0, at, et, it, angt[0], angt[1], angt[2])
    rho_g = 1.33 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    rg = (3.0 * mg / (4.0 * np.pi * rho_g)) ** (1.0 / 3.0)
    s = _assemble("config1", [_star(m0), (abi.GIANT_PLANET, dict(mass=mg, radius=rg, density=np.full(2, rho_g), phase=pg)),
                              (abi.TEST_PARTICLE, dict(mass=np.zeros(n_tp), phase=pt))],
                  integrator=abi.RUNGE_KUTTA_FEHLBERG78, epsilon=1.0e-10, length=1000.0 * YEAR_TO_DAY)
    s.h0 = _shortest_period(s) / 50000.0
    return s


def config2(seed: int = 1002, n_pl: int = 8190) -> System:
    """1 star + 2 giants + 8190 planetesimals (lognormal mass, median 1e-9,
    sigma 1; density 2 g/cm^3); power-law gas h/r = 0.05, rho ~ r^-2.5, cd = 1;
    RKF78 eps 1e-11."""
    rng = np.random.default_rng(seed)
    m0 = 1.0
    mg = np.array([1.0e-3, 3.0e-4])
    ag = np.array([5.2, 9.5])
    eg = rng.uniform(0, 0.05, 2)
    ig = rng.uniform(0, 1.0, 2) * DEG
    ang = rng.uniform(0, 2 * np.pi, (3, 2))
    pg = elements_to_phase(abi.GAUSS2 * (m0 + mg), ag, eg, ig, ang[0], ang[1], ang[2])
    rho_g = 1.33 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    rg = (3.0 * mg / (4.0 * np.pi * rho_g)) ** (1.0 / 3.0)
    mp = np.exp(np.log(1.0e-9) + rng.standard_normal(n_pl))
    rho_p = 2.0 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    rp = (3.0 * mp / (4.0 * np.pi * rho_p)) ** (1.0 / 3.0)
    ap = rng.uniform(1, 10, n_pl)
    ep = np.minimum(rng.rayleigh(0.01, n_pl), 0.5)
    ip = rng.rayleigh(0.01, n_pl)
    angp = rng.uniform(0, 2 * np.pi, (3, n_pl))
    pp = elements_to_phase(abi.GAUSS2 * (m0 + mp), ap, ep, ip, angp[0], angp[1], angp[2])
    gas = default_gas()
    gas["scale_height"] = (0.05, 1.0)
    gas["density"] = (gas["density"][0], -2.5)
    s = _assemble("config2", [_star(m0), (abi.GIANT_PLANET, dict(mass=mg, radius=rg, density=np.full(2, rho_g), phase=pg)),
                              (abi.PLANETESIMAL, dict(mass=mp, radius=rp, density=np.full(n_pl, rho_p),
                                                      cd=np.ones(n_pl), phase=pp))],
                  gas=gas, integrator=abi.RUNGE_KUTTA_FEHLBERG78, epsilon=1.0e-11)
    s.h0 = _shortest_period(s) / 50000.0
    return s


def config3(seed: int = 1003, n: int = 65536) -> System:
    """1 star + (n-1) equal-mass (1e-10) self-gravitating bodies typed
    ProtoPlanet, a ~ U(0.5, 5) AU, e, i Rayleigh 0.02; RK4."""
    rng = np.random.default_rng(seed)
    m0 = 1.0
    k = n - 1
    mp = np.full(k, 1.0e-10)
    a = rng.uniform(0.5, 5.0, k)
    e = np.minimum(rng.rayleigh(0.02, k), 0.5)
    inc = rng.rayleigh(0.02, k)
    ang = rng.uniform(0, 2 * np.pi, (3, k))
    ph = elements_to_phase(abi.GAUSS2 * (m0 + mp), a, e, inc, ang[0], ang[1], ang[2])
    rho = 2.0 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    rp = (3.0 * mp / (4.0 * np.pi * rho)) ** (1.0 / 3.0)
    s = _assemble("config3", [_star(m0), (abi.PROTO_PLANET, dict(mass=mp, radius=rp, density=np.full(k, rho), phase=ph))],
                  integrator=abi.RUNGE_KUTTA4)
    s.h0 = _shortest_period(s) / 50000.0
    return s


def disk_exact(seed: int = 2003, n: int = 65536) -> System:
    """A config-3-shaped disk built with +, -, *, / and sqrt only, so that it is
    bit-identical on every IEEE-754 machine (used for full-size checksum
    fixtures).  Bodies on near-circular orbits in an annulus 0.5-5 AU."""
    rng = np.random.default_rng(seed)
    k = n - 1
    out = np.empty((0, 2))
    while out.shape[0] < k:
        u = rng.random((2 * k, 2)) * 10.0 - 5.0
        r2 = u[:, 0] * u[:, 0] + u[:, 1] * u[:, 1]
        out = np.concatenate([out, u[(r2 >= 0.25) & (r2 <= 25.0)]])
    xy = out[:k]
    z = (rng.random(k) - 0.5) * 0.02
    r = np.sqrt(xy[:, 0] * xy[:, 0] + xy[:, 1] * xy[:, 1])
    mp = np.full(k, 1.0e-10)
    vc = np.sqrt(abi.GAUSS2 * (1.0 + mp) / r)
    ph = np.stack([xy[:, 0], xy[:, 1], z, -vc * xy[:, 1] / r, vc * xy[:, 0] / r, (rng.random(k) - 0.5) * 1e-4],
                  axis=1)
    rho = 2.0 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    s = _assemble("disk_exact", [(abi.CENTRAL_BODY, dict(mass=[1.0], radius=[SOLAR_RADIUS_TO_AU], density=[rho],
                                                        phase=np.zeros((1, 6)))),
                                 (abi.PROTO_PLANET, dict(mass=mp, radius=np.full(k, 1e-7), density=np.full(k, rho),
                                                         phase=ph))], integrator=abi.RUNGE_KUTTA4)
    return s


def config4_system(rng: np.random.Generator, idx: int) -> System:
    """One ensemble member: 1 star + U{2..12} planets (log-U mass 1e-6..1e-3,
    log-U a 0.1..30 AU, e ~ U(0, 0.2), i = 0) + U{0..512} test particles."""
    m0 = 1.0
    npl = int(rng.integers(2, 13))
    ntp = int(rng.integers(0, 513))
    mp = np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), npl))
    ap = np.exp(rng.uniform(np.log(0.1), np.log(30.0), npl))
    ep = rng.uniform(0, 0.2, npl)
    angp = rng.uniform(0, 2 * np.pi, (3, npl))
    pp = elements_to_phase(abi.GAUSS2 * (m0 + mp), ap, ep, np.zeros(npl), angp[0], angp[1], angp[2])
    at = np.exp(rng.uniform(np.log(0.1), np.log(30.0), ntp))
    et = rng.uniform(0, 0.2, ntp)
    angt = rng.uniform(0, 2 * np.pi, (3, ntp))
    pt = elements_to_phase(abi.GAUSS2 * m0, at, et, np.zeros(ntp), angt[0], angt[1], angt[2]) if ntp else np.zeros((0, 6))
    groups = [_star(m0), (abi.GIANT_PLANET, dict(mass=mp, phase=pp))]
    if ntp:
        groups.append((abi.TEST_PARTICLE, dict(mass=np.zeros(ntp), phase=pt)))
    s = _assemble(f"config4[{idx}]", groups, integrator=abi.RUNGE_KUTTA_FEHLBERG78, epsilon=1e-10)
    s.h0 = _shortest_period(s) / 50000.0
    return s


def config4(seed: int = 1004, n_systems: int = 4096) -> list:
    rng = np.random.default_rng(seed)
    return [config4_system(rng, k) for k in range(n_systems)]


def config5(seed: int = 1005, n_pl: int = 1024) -> System:
    """1 star + 8 planets (log-U 1e-7..1e-3 Msun, log-U a 0.3..30 AU,
    e ~ U(0, 0.1)) + 1024 massive planetesimals (1e-10 Msun) typed
    ProtoPlanet so that they attract each other; fixed-step RKF78."""
    rng = np.random.default_rng(seed)
    m0 = 1.0
    mpl = np.exp(rng.uniform(np.log(1e-7), np.log(1e-3), 8))
    apl = np.exp(rng.uniform(np.log(0.3), np.log(30.0), 8))
    epl = rng.uniform(0, 0.1, 8)
    ang = rng.uniform(0, 2 * np.pi, (3, 8))
    ppl = elements_to_phase(abi.GAUSS2 * (m0 + mpl), apl, epl, np.zeros(8), ang[0], ang[1], ang[2])
    mp = np.full(n_pl, 1.0e-10)
    a = rng.uniform(0.5, 5.0, n_pl)
    e = np.minimum(rng.rayleigh(0.02, n_pl), 0.5)
    inc = rng.rayleigh(0.02, n_pl)
    angp = rng.uniform(0, 2 * np.pi, (3, n_pl))
    pp = elements_to_phase(abi.GAUSS2 * (m0 + mp), a, e, inc, angp[0], angp[1], angp[2])
    s = _assemble("config5", [_star(m0), (abi.GIANT_PLANET, dict(mass=mpl, phase=ppl)),
                              (abi.PROTO_PLANET, dict(mass=mp, phase=pp))], integrator=abi.RUNGE_KUTTA_FEHLBERG78)
    s.h0 = _shortest_period(s) / 50000.0
    return s


def mixed_gas_system(seed: int = 3001, n_spl: int = 6, n_pl: int = 40, n_tp: int = 10, n_proto: int = 4,
                     barycentric: bool = False) -> System:
    """Small system with every class the force model distinguishes: giants
    with type-II migration, protoplanets with type-I migration,
    super-planetesimals and planetesimals whose radii span the Epstein,
    transition and Stokes drag regimes, and test particles."""
    rng = np.random.default_rng(seed)
    m0 = 1.0
    gas = default_gas()
    gas["scale_height"] = (0.05, 1.0)
    gas["density"] = (gas["density"][0], -2.5)
    mg = np.array([1.0e-3, 3.0e-4])
    ag = np.array([5.2, 9.5])
    pg = elements_to_phase(abi.GAUSS2 * (m0 + mg), ag, rng.uniform(0, 0.05, 2), rng.uniform(0, 0.02, 2),
                           *rng.uniform(0, 2 * np.pi, (3, 2)))
    mpp = np.exp(rng.uniform(np.log(1e-8), np.log(1e-6), n_proto))
    app = rng.uniform(1.0, 4.0, n_proto)
    ppp = elements_to_phase(abi.GAUSS2 * (m0 + mpp), app, rng.uniform(0, 0.05, n_proto),
                            rng.uniform(0, 0.02, n_proto), *rng.uniform(0, 2 * np.pi, (3, n_proto)))
    rho = 2.0 * GRAM_PER_CM3_TO_SOLAR_PER_AU3
    rpp = (3.0 * mpp / (4.0 * np.pi * rho)) ** (1.0 / 3.0)

    def small(k, lo, hi):
        a = rng.uniform(0.3, 8.0, k)
        ph = elements_to_phase(abi.GAUSS2 * m0, a, rng.uniform(0, 0.1, k), rng.uniform(0, 0.05, k),
                               *rng.uniform(0, 2 * np.pi, (3, k)))
        # mean free path ~ 4.6e-14 AU * r^2.75: radii from 1e-17 to 1e-8 AU
        # cover Epstein (R <= 0.1 lambda), transition and Stokes (R >= 10 lambda).
        rad = np.exp(rng.uniform(np.log(lo), np.log(hi), k))
        m = 4.0 / 3.0 * np.pi * rad ** 3 * rho
        return ph, rad, m

    pspl, rspl, mspl = small(n_spl, 1e-12, 1e-8)
    ppl, rpl, mpl = small(n_pl, 1e-17, 1e-9)
    ptp = elements_to_phase(abi.GAUSS2 * m0, rng.uniform(2, 12, n_tp), rng.uniform(0, 0.1, n_tp),
                            rng.uniform(0, 0.05, n_tp), *rng.uniform(0, 2 * np.pi, (3, n_tp)))
    groups = [_star(m0),
              (abi.GIANT_PLANET, dict(mass=mg, radius=[4.8e-4, 4.0e-4], density=[rho, rho], phase=pg,
                                      mig_type=[abi.MIGRATION_TYPE_II, abi.MIGRATION_TYPE_II], mig_stop_at=[0.5, 0.5])),
              (abi.PROTO_PLANET, dict(mass=mpp, radius=rpp, density=np.full(n_proto, rho), phase=ppp,
                                      mig_type=np.full(n_proto, abi.MIGRATION_TYPE_I),
                                      mig_stop_at=np.full(n_proto, 0.2))),
              (abi.SUPER_PLANETESIMAL, dict(mass=mspl, radius=rspl, density=np.full(n_spl, rho), cd=np.ones(n_spl),
                                            phase=pspl)),
              (abi.PLANETESIMAL, dict(mass=mpl, radius=rpl, density=np.full(n_pl, rho), cd=np.ones(n_pl), phase=ppl)),
              (abi.TEST_PARTICLE, dict(mass=np.zeros(n_tp), phase=ptp))]
    s = _assemble("mixed_gas", groups, gas=gas, barycentric=barycentric)
    s.h0 = _shortest_period(s) / 50000.0
    return s

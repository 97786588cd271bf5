"""Python binding of the CPU oracle (test infrastructure only).

The oracle is the checker for the GB300 kernels: tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg may load it; the solaris_gb300 package never
does.  ``build()`` compiles solaris_oracle.c with -ffp-contract=off so that its
arithmetic is the reference's on x86-64 and aarch64 alike.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from solaris_gb300 import abi

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
SRC = os.path.join(ORACLE_DIR, "solaris_oracle.c")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
REF_HARNESS = os.path.join(REF_DIR, "ref_harness")
# Where the reference sources lie (read only by the build recipes and fixture
# generators, never by the GPU tests or the bench).
REFERENCE_SRC = os.environ.get("SOLARIS_REFERENCE_SRC", "/root/reference")


def build(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(ORACLE_DIR, "solaris_oracle.h"))):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fopenmp", SRC, "-o",
               LIB + ".tmp", "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_reference(ref_root: str = REFERENCE_SRC) -> bool:
    """Compile the reference CPU build into oracle/_ref (only where the
    reference sources exist)."""
    if not os.path.isdir(os.path.join(ref_root, "Solaris")):
        return False
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, f"REF={ref_root}", "-j8"], check=True)
    return os.path.exists(REF_HARNESS)


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        F, I = abi._PF64, abi._PI32
        lib.orc_create.restype = P
        lib.orc_create.argtypes = [C.POINTER(abi.SolBodyData), C.POINTER(abi.SolGasComponent), C.c_int32]
        lib.orc_destroy.argtypes = [P]
        lib.orc_n_total.restype = C.c_int32
        lib.orc_n_total.argtypes = [P]
        lib.orc_set_eval_flags.argtypes = [P, C.c_uint32]
        lib.orc_set_epsilon.argtypes = [P, C.c_double]
        lib.orc_set_threads.argtypes = [P, C.c_int32]
        lib.orc_compute.argtypes = [P, C.c_double, F, F]
        lib.orc_get_last_eval.argtypes = [P, F, I, F]
        lib.orc_get_mig_type.argtypes = [P, I]
        lib.orc_rkf78_step.argtypes = [P, C.c_double, C.c_double, F, F, F, F]
        lib.orc_driver.argtypes = [P, C.c_int32, F, C.POINTER(abi.SolTimeLine), C.c_int32,
                                   C.POINTER(abi.SolStepStats), F, F, F]
        lib.orc_check_events.argtypes = [P, F, C.c_double, C.c_double, C.c_double, C.POINTER(abi.SolEvent),
                                         C.c_int32, C.POINTER(C.c_int32)]
        lib.orc_integrals.argtypes = [P, F, F]
        lib.orc_kepler_equation_solver.argtypes = [C.c_double, C.c_double, C.c_double, F]
        lib.orc_calculate_phase.argtypes = [C.c_double, F, F]
        lib.orc_calculate_orbital_element.argtypes = [C.c_double, F, F, F, C.c_int32]
        lib.orc_jvp.argtypes = [P, F, F, F, F]
        lib.orc_rkf78_fixed.argtypes = [P, F, C.c_double, C.c_int32, F, F, F, F]
        lib.orc_set_masses.argtypes = [P, F]
        lib.orc_gas_probe.restype = C.c_double
        lib.orc_gas_probe.argtypes = [C.POINTER(abi.SolGasComponent), C.c_int32, F, F]
        lib.orc_kepler_solve.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int32, F]
        lib.orc_get_bodies.argtypes = [P, C.POINTER(abi.SolNBodies), I, I, F, F, F]
        lib.orc_handle_events.argtypes = [P, C.c_double, C.c_double, C.c_double, C.c_double, F,
                                          C.POINTER(abi.SolAffair), C.c_int32, C.POINTER(C.c_int32)]
        lib.orc_gravity_ac_sample.restype = C.c_int64
        lib.orc_gravity_ac_sample.argtypes = [P, F, C.c_int32, C.c_int32, F, C.c_int32]
        _lib = lib
    return _lib


class Oracle:
    """One reference-semantics system (Acceleration + BodyData + integrators)."""

    def __init__(self, system, barycentric=None):
        self.lib = load()
        self.system = system
        self.view = abi.BodyDataView(system)
        self.gas = abi.gas_struct(system.gas) if system.gas is not None else None
        bary = system.barycentric if barycentric is None else barycentric
        self.h = self.lib.orc_create(C.byref(self.view.struct), C.byref(self.gas) if self.gas else None, int(bary))
        self.n = system.n
        self.lib.orc_set_epsilon(self.h, system.epsilon)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_threads(self, n_threads):
        """Host threads of the force and tangent-linear sink loops (default 1;
        the results do not depend on it)."""
        self.lib.orc_set_threads(self.h, int(n_threads))

    def set_eval_flags(self, flags):
        self.lib.orc_set_eval_flags(self.h, flags)

    def compute(self, t, y, flags=abi.EVAL_ALL):
        self.set_eval_flags(flags)
        y = np.ascontiguousarray(y, dtype=np.float64)
        d = np.zeros(6 * self.n)
        self.lib.orc_compute(self.h, t, abi.f64p(y), abi.f64p(d))
        return d

    def last_eval(self):
        rm3, nd = np.zeros(self.n), np.zeros(self.n)
        nn = np.zeros(self.n, np.int32)
        self.lib.orc_get_last_eval(self.h, abi.f64p(rm3), abi.i32p(nn), abi.f64p(nd))
        return rm3, nn, nd

    def mig_type(self):
        m = np.zeros(self.n, np.int32)
        self.lib.orc_get_mig_type(self.h, abi.i32p(m))
        return m

    def rkf78_step(self, t, h, y0):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        y, err, em = np.zeros(6 * self.n), np.zeros(6 * self.n), np.zeros(1)
        self.lib.orc_rkf78_step(self.h, t, h, abi.f64p(y0), abi.f64p(y), abi.f64p(err), abi.f64p(em))
        return y, err, float(em[0])

    def driver(self, integrator, y0, t, h, n_steps):
        y = np.array(y0, dtype=np.float64, copy=True)
        tl = abi.SolTimeLine(t, h, 0.0)
        st = abi.SolStepStats()
        times, hd, hn = np.zeros(n_steps), np.zeros(n_steps), np.zeros(n_steps)
        rc = self.lib.orc_driver(self.h, integrator, abi.f64p(y), C.byref(tl), n_steps, C.byref(st), abi.f64p(times),
                                 abi.f64p(hd), abi.f64p(hn))
        return dict(status=rc, y0=y, time=times, h_did=hd, h_next=hn, tl=(tl.time, tl.h_next, tl.h_did),
                    stats=(st.accepted, st.rejected, st.evaluations))

    def check_events(self, y0, ejection, hit_centrum, collision_factor, capacity=4096):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        ev = (abi.SolEvent * capacity)()
        n = C.c_int32(0)
        self.lib.orc_check_events(self.h, abi.f64p(y0), ejection, hit_centrum, collision_factor, ev, capacity,
                                  C.byref(n))
        return [(e.kind, e.idx1, e.idx2, e.distance) for e in ev[: min(n.value, capacity)]], n.value

    def integrals(self, y0):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        out = np.zeros(16)
        self.lib.orc_integrals(self.h, abi.f64p(y0), abi.f64p(out))
        return out

    def jvp(self, y, dy, dm=None):
        y, dy = np.ascontiguousarray(y, np.float64), np.ascontiguousarray(dy, np.float64)
        out = np.zeros(6 * self.n)
        dmp = abi.f64p(np.ascontiguousarray(dm, np.float64)) if dm is not None else None
        self.lib.orc_jvp(self.h, abi.f64p(y), abi.f64p(dy), dmp, abi.f64p(out))
        return out

    def set_masses(self, m):
        m = np.ascontiguousarray(m, np.float64)
        self.lib.orc_set_masses(self.h, abi.f64p(m))

    def rkf78_fixed(self, y0, h, n_steps, dy0=None, dm=None):
        y0 = np.ascontiguousarray(y0, np.float64)
        y = np.zeros(6 * self.n)
        dyo = np.zeros(6 * self.n)
        dyp = abi.f64p(np.ascontiguousarray(dy0, np.float64)) if dy0 is not None else None
        dmp = abi.f64p(np.ascontiguousarray(dm, np.float64)) if dm is not None else None
        self.lib.orc_rkf78_fixed(self.h, abi.f64p(y0), h, n_steps, abi.f64p(y), dyp, dmp, abi.f64p(dyo))
        return (y, dyo) if dy0 is not None else y

    def handle_events(self, time, y0, ejection=0.0, hit_centrum=0.0, collision_factor=0.0):
        """Events on the last evaluation; returns the compacted y0 and the affairs."""
        y = np.array(y0, dtype=np.float64, copy=True)
        arr = (abi.SolAffair * max(self.n, 1))()
        k = C.c_int32(0)
        self.lib.orc_handle_events(self.h, float(time), float(ejection), float(hit_centrum), float(collision_factor),
                                   abi.f64p(y), arr, self.n, C.byref(k))
        self.n = int(self.lib.orc_n_total(self.h))
        return y[:6 * self.n].copy(), abi.affairs_to_list(arr, k.value)

    def bodies(self):
        n = self.n
        counts = abi.SolNBodies()
        ids, types = np.empty(n, np.int32), np.empty(n, np.int32)
        mass, radius, density = np.empty(n), np.empty(n), np.empty(n)
        self.lib.orc_get_bodies(self.h, C.byref(counts), abi.i32p(ids), abi.i32p(types), abi.f64p(mass),
                                abi.f64p(radius), abi.f64p(density))
        return dict(counts=tuple(getattr(counts, f) for f, _ in abi.SolNBodies._fields_), id=ids, type=types,
                    mass=mass, radius=radius, density=density)

    def gravity_sample(self, y, i_begin, i_end, n_threads=1):
        y = np.ascontiguousarray(y, dtype=np.float64)
        d = np.zeros(6 * self.n)
        pairs = self.lib.orc_gravity_ac_sample(self.h, abi.f64p(y), i_begin, i_end, abi.f64p(d), n_threads)
        return d, pairs


def kepler(e, m, eps=1e-14):
    lib = load()
    E = np.zeros(1)
    rc = lib.orc_kepler_equation_solver(e, m, eps, abi.f64p(E))
    return rc, float(E[0])


def calculate_phase(mu, elements):
    lib = load()
    el = np.ascontiguousarray(elements, dtype=np.float64)
    ph = np.zeros(6)
    rc = lib.orc_calculate_phase(mu, abi.f64p(el), abi.f64p(ph))
    return rc, ph


def orbital_element(mu, phase, quirks=abi.QUIRKS_REFERENCE):
    lib = load()
    ph = np.ascontiguousarray(phase, dtype=np.float64)
    a, e = np.zeros(1), np.zeros(1)
    rc = lib.orc_calculate_orbital_element(mu, abi.f64p(ph), abi.f64p(a), abi.f64p(e), quirks)
    return rc, float(a[0]), float(e[0])


def gas_probe(gas: dict, which: int, *args):
    """GasComponent helpers of the oracle: (value, vector)."""
    lib = load()
    g = abi.gas_struct(gas)
    a = np.ascontiguousarray(args, dtype=np.float64)
    out = np.zeros(3)
    v = lib.orc_gas_probe(C.byref(g), int(which), abi.f64p(a), abi.f64p(out))
    return float(v), out


def kepler_solve(e, m, eps=1e-14, quirks=0):
    lib = load()
    E = np.zeros(1)
    rc = lib.orc_kepler_solve(e, m, eps, int(quirks), abi.f64p(E))
    return rc, float(E[0])


class ScenarioBackend:
    """The oracle behind solaris_gb300.simulator.Simulator: one Driver call per
    step on the host, events by orc_handle_events, records formatted by the
    library's BinaryFileAdapter layouts (test infrastructure: the checker of
    the device run of a scenario file)."""

    def __init__(self, system, st, directory):
        from solaris_gb300 import engine
        self.fmt_phases, self.fmt_integrals = engine.format_phases_record, engine.format_integrals_record
        self.o = Oracle(system)
        self.y0 = np.array(system.y0, dtype=np.float64, copy=True)
        self.integrator = st.integrator
        self.phases = os.path.join(directory, st.phases)
        self.integrals_path = os.path.join(directory, st.integrals)
        self.rejected = 0

    def step(self, time, h_next):
        r = self.o.driver(self.integrator, self.y0, time, h_next, 1)
        if r["status"] != 0:
            raise RuntimeError(f"oracle driver status {r['status']}")
        self.rejected += r["stats"][1]
        self.y0 = r["y0"]
        t, hn, hd = r["tl"]
        return t, hd, hn

    def events(self, time, ejection, hit_centrum, collision_factor):
        self.y0, affairs = self.o.handle_events(time, self.y0, ejection, hit_centrum, collision_factor)
        return affairs

    def n_total(self):
        return self.o.n

    def state(self):
        return self.y0.copy()

    def zero_below_smallest(self):
        self.y0[np.abs(self.y0) < 1.0e-50] = 0.0

    def save_phases(self, time):
        ids = self.o.bodies()["id"]
        with open(self.phases, "ab") as f:
            f.write(self.fmt_phases(time, self.y0, ids))

    def save_integrals(self, time):
        first = not os.path.exists(self.integrals_path) or os.path.getsize(self.integrals_path) == 0
        rec = self.fmt_integrals(time, self.o.integrals(self.y0), header=first)
        with open(self.integrals_path, "ab") as f:
            f.write(rec)

    def close(self):
        pass

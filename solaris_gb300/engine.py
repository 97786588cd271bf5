"""Python handle on one engine context (ctypes over the C-ABI).

:class:`Context` mirrors the reference's C++ surface for the hot path:
``accel`` is ``Acceleration::Compute`` (Solaris/Acceleration.cpp:60-80),
``driver`` runs ``RungeKuttaFehlberg78::Driver`` / ``RungeKutta4::Driver`` /
``DormandPrince::Driver`` calls (Solaris/Simulator.cpp:133-153), ``events``
evaluates the predicates of ``Simulator::CheckEvent`` and ``integrals`` is
``Calculate::Integrals``.  Errors raise :class:`abi.SolError` carrying the
reference-style status code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class Context:
    def __init__(self, system, device: int = 0, precision: int = abi.PRECISION_FP64, barycentric=None):
        self.lib = abi.load_library()
        self.system = system
        self.n = system.n
        self._view = abi.BodyDataView(system)
        self._gas = abi.gas_struct(system.gas) if system.gas is not None else None
        bary = system.barycentric if barycentric is None else barycentric
        h = C.c_void_p()
        abi.check(self.lib, self.lib.sol_create(C.byref(self._view.struct),
                                                C.byref(self._gas) if self._gas is not None else None,
                                                int(bool(bary)), int(device), C.byref(h)))
        self.h = h
        self.set_precision(precision)
        abi.check(self.lib, self.lib.sol_set_tolerance(self.h, float(system.epsilon)))

    # -- lifetime ---------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.sol_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- settings -----------------------------------------------------------------
    def set_precision(self, precision: int):
        abi.check(self.lib, self.lib.sol_set_precision(self.h, int(precision)))

    def set_eval_flags(self, flags: int):
        abi.check(self.lib, self.lib.sol_set_eval_flags(self.h, int(flags)))

    def set_device_loop(self, enable: bool):
        abi.check(self.lib, self.lib.sol_set_device_loop(self.h, int(bool(enable))))

    def set_tolerance(self, eps: float):
        abi.check(self.lib, self.lib.sol_set_tolerance(self.h, float(eps)))

    def set_wait_test(self, spin_limit: int, withhold: int):
        """Failure-path test hook (sol_set_wait_test): the group driver's
        barrier gives up after spin_limit polls (0: default) and CTA
        `withhold` never arrives (-1: none)."""
        abi.check(self.lib, self.lib.sol_set_wait_test(self.h, int(spin_limit), int(withhold)))

    # -- force ----------------------------------------------------------------
    def accel(self, t, y, flags=abi.EVAL_ALL):
        self.set_eval_flags(flags)
        y = np.ascontiguousarray(y, dtype=np.float64)
        d = np.empty(6 * self.n)
        rm3, nd = np.empty(self.n), np.empty(self.n)
        nn = np.empty(self.n, np.int32)
        abi.check(self.lib, self.lib.sol_accel_compute(self.h, float(t), abi.f64p(y), abi.f64p(d), abi.f64p(rm3),
                                                       abi.i32p(nn), abi.f64p(nd)))
        return d, rm3, nn, nd

    def mig_type(self):
        m = np.empty(self.n, np.int32)
        abi.check(self.lib, self.lib.sol_get_mig_type(self.h, abi.i32p(m)))
        return m

    def last_eval(self):
        rm3, nd = np.empty(self.n), np.empty(self.n)
        nn = np.empty(self.n, np.int32)
        abi.check(self.lib, self.lib.sol_get_last_eval(self.h, abi.f64p(rm3), abi.i32p(nn), abi.f64p(nd)))
        return rm3, nn, nd

    # -- integrators ------------------------------------------------------------
    def set_state(self, y0):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        abi.check(self.lib, self.lib.sol_set_state(self.h, abi.f64p(y0)))

    def get_state(self):
        y = np.empty(6 * self.n)
        abi.check(self.lib, self.lib.sol_get_state(self.h, abi.f64p(y)))
        return y

    def driver(self, integrator, t, h, n_steps, time_line=None):
        tl = time_line or abi.SolTimeLine(float(t), float(h), 0.0)
        st = abi.SolStepStats()
        abi.check(self.lib, self.lib.sol_driver(self.h, int(integrator), C.byref(tl), int(n_steps), C.byref(st)))
        return dict(time=tl.time, h_next=tl.h_next, h_did=tl.h_did,
                    stats=(st.accepted, st.rejected, st.evaluations), time_line=tl)

    def run_until(self, integrator, line, max_steps, ejection=0.0, hit_centrum=0.0, collision_factor=0.0):
        """The Simulator's step loop until the host has work (sol_run_until):
        updates line (abi.SolSimLine) and returns the stop reason and the
        (accepted, rejected, evaluations) counters."""
        reason = C.c_int32(0)
        st = abi.SolStepStats()
        abi.check(self.lib, self.lib.sol_run_until(self.h, int(integrator), C.byref(line), int(max_steps),
                                                   float(ejection), float(hit_centrum), float(collision_factor),
                                                   C.byref(reason), C.byref(st)))
        return reason.value, (st.accepted, st.rejected, st.evaluations)

    def flush_smallest(self):
        abi.check(self.lib, self.lib.sol_flush_smallest(self.h))

    def step_start(self):
        y = np.empty(6 * self.n)
        abi.check(self.lib, self.lib.sol_get_step_start(self.h, abi.f64p(y)))
        return y

    def rkf78_step(self, t, h, y0):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        y, err, em = np.empty(6 * self.n), np.empty(6 * self.n), np.zeros(1)
        abi.check(self.lib, self.lib.sol_rkf78_step(self.h, float(t), float(h), abi.f64p(y0), abi.f64p(y),
                                                    abi.f64p(err), abi.f64p(em)))
        return y, err, float(em[0])

    # -- measurement ----------------------------------------------------------
    def stream_handle(self) -> int:
        v = C.c_void_p()
        abi.check(self.lib, self.lib.sol_get_stream(self.h, C.byref(v)))
        return int(v.value or 0)

    def bench_stages(self, reps) -> float:
        ms = C.c_double(0)
        abi.check(self.lib, self.lib.sol_bench_stages(self.h, int(reps), C.byref(ms)))
        return float(ms.value)

    def bench_force(self, precision, reps) -> float:
        ms = C.c_double(0)
        abi.check(self.lib, self.lib.sol_bench_force(self.h, int(precision), int(reps), C.byref(ms)))
        return float(ms.value)

    # -- events ---------------------------------------------------------------
    def handle_events(self, time, ejection=0.0, hit_centrum=0.0, collision_factor=0.0):
        """Simulator::CheckEvent on the device: removals and merges compact the
        context's bodies.  Returns the affairs (TwoBodyAffair) in order."""
        cap = self.n
        arr = (abi.SolAffair * max(cap, 1))()
        k = C.c_int32(0)
        abi.check(self.lib, self.lib.sol_handle_events(self.h, float(time), float(ejection), float(hit_centrum),
                                                       float(collision_factor), arr, cap, C.byref(k)))
        counts = abi.SolNBodies()
        self.lib.sol_get_bodies(self.h, C.byref(counts), None, None, None, None, None)
        self.n = int(sum(getattr(counts, f) for f, _ in abi.SolNBodies._fields_))
        return abi.affairs_to_list(arr, k.value)

    def bodies(self):
        n = self.n
        counts = abi.SolNBodies()
        ids, types = np.empty(n, np.int32), np.empty(n, np.int32)
        mass, radius, density = np.empty(n), np.empty(n), np.empty(n)
        abi.check(self.lib, self.lib.sol_get_bodies(self.h, C.byref(counts), abi.i32p(ids), abi.i32p(types),
                                                    abi.f64p(mass), abi.f64p(radius), abi.f64p(density)))
        return dict(counts=tuple(getattr(counts, f) for f, _ in abi.SolNBodies._fields_), id=ids, type=types,
                    mass=mass, radius=radius, density=density)

    # -- discrete adjoint ---------------------------------------------------------
    def set_masses(self, mass):
        m = np.ascontiguousarray(mass, dtype=np.float64)
        abi.check(self.lib, self.lib.sol_set_masses(self.h, abi.f64p(m)))

    def adjoint_forward(self, y0, h, n_steps, checkpoint_every=100):
        y0 = np.ascontiguousarray(y0, dtype=np.float64)
        y = np.empty(6 * self.n)
        abi.check(self.lib, self.lib.sol_adjoint_forward(self.h, float(h), int(n_steps), int(checkpoint_every),
                                                         abi.f64p(y0), abi.f64p(y)))
        return y

    def adjoint_backward(self, dl_dy_final):
        g = np.ascontiguousarray(dl_dy_final, dtype=np.float64)
        dy0, dm = np.empty(6 * self.n), np.empty(self.n)
        abi.check(self.lib, self.lib.sol_adjoint_backward(self.h, abi.f64p(g), abi.f64p(dy0), abi.f64p(dm)))
        return dy0, dm

    # -- events and integrals ----------------------------------------------------
    def events(self, ejection, hit_centrum, collision_factor, capacity=4096):
        ev = (abi.SolEvent * max(capacity, 1))()
        n = C.c_int32(0)
        abi.check(self.lib, self.lib.sol_check_events(self.h, float(ejection), float(hit_centrum),
                                                      float(collision_factor), ev, int(capacity), C.byref(n)))
        return [(e.kind, e.idx1, e.idx2, e.distance) for e in ev[: min(n.value, capacity)]], n.value

    def integrals(self, y0=None):
        out = np.zeros(16)
        yp = None
        if y0 is not None:
            y0 = np.ascontiguousarray(y0, dtype=np.float64)
            yp = abi.f64p(y0)
        abi.check(self.lib, self.lib.sol_integrals(self.h, yp, abi.f64p(out)))
        return out


class Ensemble:
    """Many independent systems advanced in one persistent launch
    (sol_ensemble_*): each system runs its own adaptive RKF78 driver calls."""

    def __init__(self, systems, device: int = 0, precision: int = abi.PRECISION_FP64, epsilon: float = 1e-10):
        self.lib = abi.load_library()
        self.systems = systems
        self._views = [abi.BodyDataView(s) for s in systems]
        arr = (abi.SolBodyData * len(systems))(*[v.struct for v in self._views])
        self._arr = arr
        h = C.c_void_p()
        abi.check(self.lib, self.lib.sol_ensemble_create(arr, len(systems), int(device), C.byref(h)))
        self.h = h
        self.offsets = np.cumsum([0] + [s.n for s in systems])
        abi.check(self.lib, self.lib.sol_ensemble_set_precision(self.h, int(precision)))
        abi.check(self.lib, self.lib.sol_ensemble_set_tolerance(self.h, float(epsilon)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.sol_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_precision(self, p):
        abi.check(self.lib, self.lib.sol_ensemble_set_precision(self.h, int(p)))

    def set_state(self, y0s, times, h_next):
        y = np.ascontiguousarray(np.concatenate([np.asarray(v, np.float64) for v in y0s]))
        tls = (abi.SolTimeLine * len(self.systems))(*[abi.SolTimeLine(float(t), float(h), 0.0)
                                                     for t, h in zip(times, h_next)])
        abi.check(self.lib, self.lib.sol_ensemble_set_state(self.h, abi.f64p(y), tls))

    def get_state(self):
        y = np.empty(6 * int(self.offsets[-1]))
        tls = (abi.SolTimeLine * len(self.systems))()
        st = np.zeros(len(self.systems), np.int32)
        abi.check(self.lib, self.lib.sol_ensemble_get_state(self.h, abi.f64p(y), tls, abi.i32p(st)))
        ys = [y[6 * self.offsets[k]:6 * self.offsets[k + 1]] for k in range(len(self.systems))]
        return ys, [(t.time, t.h_next, t.h_did) for t in tls], st

    def advance(self, n_steps):
        st = abi.SolStepStats()
        abi.check(self.lib, self.lib.sol_ensemble_advance(self.h, int(n_steps), C.byref(st)))
        return st.accepted, st.rejected, st.evaluations

    def configure(self, threads, per_sm):
        abi.check(self.lib, self.lib.sol_ensemble_configure(self.h, int(threads), int(per_sm)))

    def autotune(self, steps=1):
        b, p, ms = C.c_int32(0), C.c_int32(0), C.c_double(0)
        abi.check(self.lib, self.lib.sol_ensemble_autotune(self.h, int(steps), C.byref(b), C.byref(p), C.byref(ms)))
        return b.value, p.value, ms.value


def kernel_launches() -> int:
    lib = abi.load_library()
    v = C.c_int64(0)
    lib.sol_kernel_launch_count(C.byref(v))
    return int(v.value)


def fp64_peak_flops(device: int = 0) -> float:
    lib = abi.load_library()
    v = C.c_double(0)
    abi.check(lib, lib.sol_measure_fp64_peak(int(device), C.byref(v)))
    return float(v.value)


def fp64_pipe_rates(device: int = 0) -> dict:
    """FP64 pipe throughput of this GPU (sol_measure_fp64_pipe): thread
    instructions per second of DFMA, DADD and DMUL chains, and the SM clock
    (MHz) the DFMA rate was measured at."""
    lib = abi.load_library()
    r = (C.c_double * 3)()
    mhz = C.c_double(0)
    abi.check(lib, lib.sol_measure_fp64_pipe(int(device), r, C.byref(mhz)))
    return {"dfma": float(r[0]), "dadd": float(r[1]), "dmul": float(r[2]), "sm_mhz": float(mhz.value)}


def fp32_pipe_rates(device: int = 0) -> dict:
    """FP32 pipe throughput of this GPU (sol_measure_fp32_pipe): FP32 lane
    operations per second of scalar FFMA and paired FFMA2 chains, and the SM
    clock (MHz) of the FFMA2 measurement."""
    lib = abi.load_library()
    r = (C.c_double * 2)()
    mhz = C.c_double(0)
    abi.check(lib, lib.sol_measure_fp32_pipe(int(device), r, C.byref(mhz)))
    return {"ffma": float(r[0]), "ffma2": float(r[1]), "sm_mhz": float(mhz.value)}


def check_pair_math(mode: int, n: int, seed: int = 1, device: int = 0) -> dict:
    """Self-check of the correctly rounded sqrt / reciprocal of the FP64 pair
    against IEEE sqrt and division (sol_check_pair_math): mismatches (0 when
    correct), samples handed to IEEE arithmetic, first mismatching index."""
    lib = abi.load_library()
    r = (C.c_int64 * 3)()
    abi.check(lib, lib.sol_check_pair_math(int(device), int(mode), int(n), int(seed) & (2**64 - 1), r))
    return {"mismatches": int(r[0]), "slow": int(r[1]), "first": int(r[2])}


# -- output files (BinaryFileAdapter record layouts) -------------------------------
class Output:
    """Phases / integrals files of a context: records appended in the
    reference's layout; phases snapshots are written by a background thread
    while the integration continues."""

    def __init__(self, ctx: "Context", phases: str | None = None, integrals: str | None = None,
                 text: bool = False):
        self.lib = ctx.lib
        self.ctx = ctx
        h = C.c_void_p()
        abi.check(self.lib, self.lib.sol_output_open(ctx.h, phases.encode() if phases else None,
                                                     integrals.encode() if integrals else None, int(text),
                                                     C.byref(h)))
        self.h = h

    def save_phases(self, time: float):
        abi.check(self.lib, self.lib.sol_output_save_phases(self.h, float(time)))

    def save_integrals(self, time: float):
        abi.check(self.lib, self.lib.sol_output_save_integrals(self.h, float(time)))

    def flush(self):
        abi.check(self.lib, self.lib.sol_output_flush(self.h))

    def close(self):
        if getattr(self, "h", None):
            h, self.h = self.h, None
            abi.check(self.lib, self.lib.sol_output_close(h))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def format_phases_record(time: float, y, ids, text: bool = False) -> bytes:
    lib = abi.load_library()
    y = np.ascontiguousarray(y, np.float64)
    ids = np.ascontiguousarray(ids, np.int32)
    n = C.c_int64(0)
    abi.check(lib, lib.sol_format_phases_record(float(time), len(ids), abi.f64p(y), abi.i32p(ids), int(text), None,
                                                0, C.byref(n)))
    buf = C.create_string_buffer(n.value)
    abi.check(lib, lib.sol_format_phases_record(float(time), len(ids), abi.f64p(y), abi.i32p(ids), int(text), buf,
                                                n.value, C.byref(n)))
    return buf.raw[:n.value]


def format_integrals_record(time: float, values, header: bool = False) -> bytes:
    lib = abi.load_library()
    v = np.ascontiguousarray(values, np.float64)
    n = C.c_int64(0)
    abi.check(lib, lib.sol_format_integrals_record(float(time), len(v), abi.f64p(v), int(header), None, 0,
                                                   C.byref(n)))
    buf = C.create_string_buffer(n.value)
    abi.check(lib, lib.sol_format_integrals_record(float(time), len(v), abi.f64p(v), int(header), buf, n.value,
                                                   C.byref(n)))
    return buf.raw[:n.value]


def phases_from_elements(mu, elements, quirks: int = abi.QUIRKS_REFERENCE, device: int = 0):
    """Ephemeris::CalculatePhase for many bodies on the device: elements (n, 6)
    = a, e, i, argument of pericentre, longitude of node, mean anomaly; mu (n,)
    = G (m0 + m).  Returns phases (n, 6) and the per-body status."""
    lib = abi.load_library()
    mu = np.ascontiguousarray(mu, np.float64)
    el = np.ascontiguousarray(elements, np.float64).reshape(-1, 6)
    n = len(mu)
    ph = np.empty((n, 6))
    st = np.empty(n, np.int32)
    rc = lib.sol_phases_from_elements(int(device), n, abi.f64p(mu), abi.f64p(el), int(quirks), abi.f64p(ph),
                                      abi.i32p(st))
    if rc not in (abi.SOL_OK, abi.SOL_ERR_ORBIT):
        abi.check(lib, rc)
    return ph, st

"""ctypes mirror of include/solaris_gb300.h and the loader of the CUDA library.

The library is the in-tree ``solaris_gb300/libsolaris_gb300.so`` built by
``solaris_gb300.build``.  Loading it never falls back to anything else: if it
is missing, :func:`load_library` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libsolaris_gb300.so")

# status codes (enum sol_status)
SOL_OK = 0
SOL_ERR_ARG = 1
SOL_ERR_CUDA = 2
SOL_ERR_NAN = 3
SOL_ERR_UNDERFLOW = 4
SOL_ERR_TIMEOUT = 5
SOL_ERR_MAXITER = 6
SOL_ERR_NOMEM = 7
SOL_ERR_STATE = 8
SOL_ERR_ORBIT = 9

# BodyType (Solaris/Body.h:231-241)
CENTRAL_BODY, GIANT_PLANET, ROCKY_PLANET, PROTO_PLANET = 1, 2, 3, 4
SUPER_PLANETESIMAL, PLANETESIMAL, TEST_PARTICLE = 5, 6, 7
# MigrationType (Solaris/Body.h:252-256)
MIGRATION_NO, MIGRATION_TYPE_I, MIGRATION_TYPE_II = 0, 1, 2
# GasDecreaseType
GAS_CONSTANT, GAS_LINEAR, GAS_EXPONENTIAL = 0, 1, 2
# IntegratorType (Solaris/IntegratorType.h)
DORMAND_PRINCE, RUNGE_KUTTA4, RUNGE_KUTTA56, RUNGE_KUTTA_FEHLBERG78 = 0, 1, 2, 3
# sol_precision
PRECISION_FP64, PRECISION_SPLIT, PRECISION_SPLIT_FF = 0, 1, 2
# evaluate flags
EVAL_GAS_DRAG, EVAL_TYPE_I, EVAL_TYPE_II, EVAL_ALL = 1, 2, 4, 7
TERM_GRAVITY, TERM_GAS_DRAG, TERM_TYPE_I, TERM_TYPE_II = 0, 1, 2, 3
HELPER_TYPE_I_MIGRATION_TIME, HELPER_TYPE_I_ECC_DAMPING_TIME, HELPER_TAU_NU = 0, 1, 2
# quirks
QUIRK_INT_ABS, QUIRK_BC_TAU_NU = 1, 2
QUIRKS_REFERENCE = QUIRK_INT_ABS | QUIRK_BC_TAU_NU
# events
EVENT_EJECTION, EVENT_HIT_CENTRUM, EVENT_COLLISION = 1, 2, 3

GAUSS = 1.720209895e-2
GAUSS2 = 2.959122082855911025e-4


class SolNBodies(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("central_body", "giant_planet", "rocky_planet", "proto_planet",
                                         "super_planetesimal", "planetesimal", "test_particle")]


_PI32 = C.POINTER(C.c_int32)
_PF64 = C.POINTER(C.c_double)


class SolBodyData(C.Structure):
    _fields_ = [("n", SolNBodies), ("id", _PI32), ("type", _PI32), ("mig_type", _PI32),
                ("mig_stop_at", _PF64), ("mass", _PF64), ("radius", _PF64), ("density", _PF64),
                ("cd", _PF64), ("gamma_stokes", _PF64), ("gamma_epstein", _PF64)]


class SolPowerLaw(C.Structure):
    _fields_ = [("c", C.c_double), ("index", C.c_double)]


class SolGasComponent(C.Structure):
    _fields_ = [("alpha", C.c_double), ("decrease_type", C.c_int32), ("quirks", C.c_int32),
                ("time_scale", C.c_double), ("t0", C.c_double), ("t1", C.c_double),
                ("inner_edge", C.c_double), ("mean_molecular_weight", C.c_double),
                ("particle_diameter", C.c_double), ("eta", SolPowerLaw), ("tau", SolPowerLaw),
                ("scale_height", SolPowerLaw), ("density", SolPowerLaw), ("mean_free_path", SolPowerLaw)]


class SolAffair(C.Structure):
    _fields_ = [("type", C.c_int32), ("idx1", C.c_int32), ("idx2", C.c_int32), ("id1", C.c_int32),
                ("id2", C.c_int32), ("pad", C.c_int32), ("time", C.c_double), ("phase1", C.c_double * 6),
                ("phase2", C.c_double * 6)]


class SolTimeLine(C.Structure):
    _fields_ = [("time", C.c_double), ("h_next", C.c_double), ("h_did", C.c_double)]


class SolSimLine(C.Structure):
    _fields_ = [("time", C.c_double), ("length", C.c_double), ("output", C.c_double), ("h_next", C.c_double),
                ("h_did", C.c_double), ("elapsed", C.c_double), ("last_save", C.c_double), ("steps", C.c_int64),
                ("relative_end", C.c_int32), ("pad", C.c_int32)]


STOP_STEPS, STOP_EVENT, STOP_LENGTH, STOP_OUTPUT = 0, 1, 2, 3


class SolStepStats(C.Structure):
    _fields_ = [("accepted", C.c_int64), ("rejected", C.c_int64), ("evaluations", C.c_int64)]


class SolEvent(C.Structure):
    _fields_ = [("kind", C.c_int32), ("idx1", C.c_int32), ("idx2", C.c_int32), ("pad", C.c_int32),
                ("distance", C.c_double)]


def f64p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_PF64)


def i32p(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_PI32)


def opt_f64p(a):
    return f64p(a) if a is not None else None


def opt_i32p(a):
    return i32p(a) if a is not None else None


class BodyDataView:
    """Keeps the numpy arrays alive behind a SolBodyData."""

    FIELDS_I = ("id", "type", "mig_type")
    FIELDS_F = ("mig_stop_at", "mass", "radius", "density", "cd", "gamma_stokes", "gamma_epstein")

    def __init__(self, system):
        self.arrays = {}
        sd = SolBodyData()
        c = system.counts
        sd.n = SolNBodies(*[int(x) for x in c])
        for k in self.FIELDS_I:
            a = np.ascontiguousarray(getattr(system, k), dtype=np.int32)
            self.arrays[k] = a
            setattr(sd, k, i32p(a))
        for k in self.FIELDS_F:
            a = np.ascontiguousarray(getattr(system, k), dtype=np.float64)
            self.arrays[k] = a
            setattr(sd, k, f64p(a))
        self.struct = sd


def gas_struct(gas: dict) -> SolGasComponent:
    g = SolGasComponent()
    g.alpha = gas["alpha"]
    g.decrease_type = int(gas["decrease_type"])
    g.quirks = int(gas.get("quirks", QUIRKS_REFERENCE))
    g.time_scale = gas["time_scale"]
    g.t0 = gas["t0"]
    g.t1 = gas["t1"]
    g.inner_edge = gas["inner_edge"]
    g.mean_molecular_weight = gas["mean_molecular_weight"]
    g.particle_diameter = gas["particle_diameter"]
    for k in ("eta", "tau", "scale_height", "density", "mean_free_path"):
        c, idx = gas[k]
        setattr(g, k, SolPowerLaw(c, idx))
    return g


_lib = None


def _declare(lib):
    P = C.c_void_p
    sig = {
        "sol_last_error": (C.c_char_p, []),
        "sol_version": (C.c_int, []),
        "sol_gas_component_init": (C.c_int, [C.POINTER(SolGasComponent)]),
        "sol_create": (C.c_int, [C.POINTER(SolBodyData), C.POINTER(SolGasComponent), C.c_int32, C.c_int32,
                                 C.POINTER(P)]),
        "sol_destroy": (C.c_int, [P]),
        "sol_set_precision": (C.c_int, [P, C.c_int32]),
        "sol_set_eval_flags": (C.c_int, [P, C.c_uint32]),
        "sol_get_n_total": (C.c_int, [P, C.POINTER(C.c_int32)]),
        "sol_accel_compute": (C.c_int, [P, C.c_double, _PF64, _PF64, _PF64, _PI32, _PF64]),
        "sol_get_mig_type": (C.c_int, [P, _PI32]),
        "sol_set_state": (C.c_int, [P, _PF64]),
        "sol_get_state": (C.c_int, [P, _PF64]),
        "sol_set_tolerance": (C.c_int, [P, C.c_double]),
        "sol_set_device_loop": (C.c_int, [P, C.c_int32]),
        "sol_driver": (C.c_int, [P, C.c_int32, C.POINTER(SolTimeLine), C.c_int32, C.POINTER(SolStepStats)]),
        "sol_driver_host": (C.c_int, [P, C.c_int32, _PF64, C.POINTER(SolTimeLine), C.c_int32,
                                      C.POINTER(SolStepStats)]),
        "sol_rkf78_step": (C.c_int, [P, C.c_double, C.c_double, _PF64, _PF64, _PF64, _PF64]),
        "sol_get_last_eval": (C.c_int, [P, _PF64, _PI32, _PF64]),
        "sol_check_events": (C.c_int, [P, C.c_double, C.c_double, C.c_double, C.POINTER(SolEvent), C.c_int32,
                                       C.POINTER(C.c_int32)]),
        "sol_integrals": (C.c_int, [P, _PF64, _PF64]),
        "sol_measure_fp64_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
        "sol_measure_fp64_pipe": (C.c_int, [C.c_int32, _PF64, C.POINTER(C.c_double)]),
        "sol_measure_fp32_pipe": (C.c_int, [C.c_int32, _PF64, C.POINTER(C.c_double)]),
        "sol_check_pair_math": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, C.c_uint64, C.POINTER(C.c_int64)]),
        "sol_kernel_launch_count": (C.c_int, [C.POINTER(C.c_int64)]),
        "sol_get_stream": (C.c_int, [P, C.POINTER(C.c_void_p)]),
        "sol_bench_force": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
        "sol_bench_stages": (C.c_int, [P, C.c_int32, C.POINTER(C.c_double)]),
        "sol_adjoint_forward": (C.c_int, [P, C.c_double, C.c_int32, C.c_int32, _PF64, _PF64]),
        "sol_adjoint_backward": (C.c_int, [P, _PF64, _PF64, _PF64]),
        "sol_set_masses": (C.c_int, [P, _PF64]),
        "sol_ensemble_create": (C.c_int, [C.POINTER(SolBodyData), C.c_int32, C.c_int32, C.POINTER(P)]),
        "sol_ensemble_destroy": (C.c_int, [P]),
        "sol_ensemble_set_precision": (C.c_int, [P, C.c_int32]),
        "sol_ensemble_set_tolerance": (C.c_int, [P, C.c_double]),
        "sol_ensemble_set_state": (C.c_int, [P, _PF64, C.POINTER(SolTimeLine)]),
        "sol_ensemble_get_state": (C.c_int, [P, _PF64, C.POINTER(SolTimeLine), _PI32]),
        "sol_ensemble_advance": (C.c_int, [P, C.c_int32, C.POINTER(SolStepStats)]),
        "sol_ensemble_configure": (C.c_int, [P, C.c_int32, C.c_int32]),
        "sol_ensemble_autotune": (C.c_int, [P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_double)]),
        "sol_accel_term": (C.c_int, [P, C.c_int32, C.c_double, _PF64, _PF64]),
        "sol_migration_helper": (C.c_int, [P, C.c_int32, _PF64, _PF64]),
        "sol_error_max": (C.c_int, [P, C.c_int32, C.c_int32, _PF64, _PF64, C.c_double, _PF64]),
        "sol_integrator_attempt": (C.c_int, [P, C.c_int32, C.c_double, C.c_double, _PF64, _PF64, _PF64, _PF64,
                                             _PF64, _PF64]),
        "sol_get_driver_vectors": (C.c_int, [P, _PF64, _PF64, _PF64]),
        "sol_get_side_buffers": (C.c_int, [P, _PF64, _PF64, _PF64]),
        "sol_output_open": (C.c_int, [P, C.c_char_p, C.c_char_p, C.c_int32, C.POINTER(P)]),
        "sol_output_save_phases": (C.c_int, [P, C.c_double]),
        "sol_output_save_integrals": (C.c_int, [P, C.c_double]),
        "sol_output_flush": (C.c_int, [P]),
        "sol_output_close": (C.c_int, [P]),
        "sol_format_phases_record": (C.c_int, [C.c_double, C.c_int32, _PF64, _PI32, C.c_int32, C.c_char_p,
                                               C.c_int64, C.POINTER(C.c_int64)]),
        "sol_format_integrals_record": (C.c_int, [C.c_double, C.c_int32, _PF64, C.c_int32, C.c_char_p, C.c_int64,
                                                  C.POINTER(C.c_int64)]),
        "sol_phases_from_elements": (C.c_int, [C.c_int32, C.c_int32, _PF64, _PF64, C.c_int32, _PF64, _PI32]),
        "sol_handle_events": (C.c_int, [P, C.c_double, C.c_double, C.c_double, C.c_double, C.POINTER(SolAffair),
                                        C.c_int32, C.POINTER(C.c_int32)]),
        "sol_get_bodies": (C.c_int, [P, C.POINTER(SolNBodies), _PI32, _PI32, _PF64, _PF64, _PF64]),
        "sol_write_affairs": (C.c_int, [C.c_char_p, C.POINTER(SolAffair), C.c_int32, C.c_int32]),
        "sol_run_until": (C.c_int, [P, C.c_int32, C.POINTER(SolSimLine), C.c_int32, C.c_double, C.c_double,
                                    C.c_double, C.POINTER(C.c_int32), C.POINTER(SolStepStats)]),
        "sol_flush_smallest": (C.c_int, [P]),
        "sol_get_step_start": (C.c_int, [P, _PF64]),
        "sol_gravity_noalloc": (C.c_int, [C.POINTER(SolNBodies), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
        "sol_gravity_noalloc_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
        "sol_set_wait_test": (C.c_int, [P, C.c_uint32, C.c_int32]),
        "sol_accel_sinks_device": (C.c_int, [P, C.c_double, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return sig


# Every symbol include/solaris_gb300.h declares; checked by the CPU test suite.
def exported_names():
    return [
        "sol_last_error", "sol_version", "sol_gas_component_init", "sol_create", "sol_destroy",
        "sol_set_precision", "sol_set_eval_flags", "sol_get_n_total", "sol_accel_compute", "sol_get_mig_type",
        "sol_set_state", "sol_get_state", "sol_set_tolerance", "sol_set_device_loop", "sol_driver", "sol_driver_host",
        "sol_rkf78_step", "sol_get_last_eval", "sol_check_events", "sol_integrals", "sol_measure_fp64_peak",
        "sol_measure_fp64_pipe", "sol_measure_fp32_pipe", "sol_kernel_launch_count", "sol_get_stream", "sol_bench_force", "sol_gravity_noalloc",
        "sol_gravity_noalloc_status", "sol_set_wait_test", "sol_accel_sinks_device",
        "sol_ensemble_create", "sol_ensemble_destroy", "sol_ensemble_set_precision", "sol_ensemble_set_tolerance",
        "sol_ensemble_set_state", "sol_ensemble_get_state", "sol_ensemble_advance", "sol_ensemble_configure",
        "sol_ensemble_autotune", "sol_adjoint_forward", "sol_adjoint_backward", "sol_set_masses",
        "sol_accel_term", "sol_migration_helper", "sol_error_max", "sol_integrator_attempt",
        "sol_get_driver_vectors", "sol_get_side_buffers", "sol_bench_stages", "sol_output_open",
        "sol_output_save_phases", "sol_output_save_integrals", "sol_output_flush", "sol_output_close",
        "sol_format_phases_record", "sol_format_integrals_record", "sol_phases_from_elements",
        "sol_handle_events", "sol_get_bodies", "sol_write_affairs", "sol_run_until", "sol_flush_smallest", "sol_get_step_start",
        "sol_check_pair_math"]


def load_library(path: str | None = None):
    """Load the in-tree CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"solaris_gb300: CUDA library not built ({p}); run solaris_gb300.build.build()")
    lib = C.CDLL(p)
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


class SolError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"solaris_gb300 status {code}: {msg}")
        self.code = code


def check(lib, rc):
    if rc != SOL_OK:
        msg = lib.sol_last_error()
        raise SolError(rc, msg.decode() if msg else "")
    return rc


def affairs_to_list(arr, n):
    return [dict(type=a.type, idx1=a.idx1, idx2=a.idx2, id1=a.id1, id2=a.id2, time=a.time,
                 phase1=np.array(a.phase1[:]), phase2=np.array(a.phase2[:])) for a in arr[:n]]

"""Load the golden fixtures (tests/golden/*.npz) back into scenario objects."""
from __future__ import annotations

import os

import numpy as np

from solaris_gb300 import scenarios

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

GAS_KEYS = ["alpha", "decrease_type", "quirks", "time_scale", "t0", "t1", "inner_edge", "mean_molecular_weight",
            "particle_diameter"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def system_from(d, name="golden"):
    gas = None
    if "in_gas" in d:
        v = d["in_gas"]
        gas = {k: float(v[i]) for i, k in enumerate(GAS_KEYS)}
        gas["decrease_type"] = int(gas["decrease_type"])
        gas["quirks"] = int(gas["quirks"])
        p = 9
        for k in ("eta", "tau", "scale_height", "density", "mean_free_path"):
            gas[k] = (float(v[p]), float(v[p + 1]))
            p += 2
    return scenarios.System(
        name=name, counts=tuple(int(x) for x in d["in_counts"]), id=d["in_id"].astype(np.int32),
        type=d["in_type"].astype(np.int32), mig_type=d["in_mig_type"].astype(np.int32),
        mig_stop_at=d["in_mig_stop_at"], mass=d["in_mass"], radius=d["in_radius"], density=d["in_density"],
        cd=d["in_cd"], gamma_stokes=d["in_gamma_stokes"], gamma_epstein=d["in_gamma_epstein"],
        y0=np.ascontiguousarray(d["in_y0"]), gas=gas, barycentric=bool(int(d["in_barycentric"])),
        epsilon=float(d["in_epsilon"]))


ACCEL_CASES = ["accel_config1", "accel_mixed_gas", "accel_mixed_gas_bc", "accel_mixed_gas_linear",
               "accel_selfgrav1024", "accel_selfgrav2", "accel_selfgrav3", "accel_selfgrav17", "accel_selfgrav255",
               "accel_selfgrav257", "accel_lattice28"]

"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs only where the reference sources are available: it builds the reference
CPU code into oracle/_ref/ (oracle/Makefile), drives it through
oracle/ref_harness.cpp on seeded synthetic inputs and stores inputs and
outputs as .npz files.  The committed fixtures are what the test suite checks
the oracle and the GPU kernels against; this script is how they were made.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from solaris_gb300 import abi, scenarios  # noqa: E402

CMD_ACCEL, CMD_RKF78_STEP, CMD_RKF78_DRIVER, CMD_RK4_DRIVER = 1, 2, 3, 4
CMD_DP_DRIVER, CMD_INTEGRALS, CMD_EPHEMERIS, CMD_KEPLER = 5, 6, 7, 8
CMD_TIME_ACCEL, CMD_ORBITAL_ELEMENT = 9, 10


def write_case(path, cmd, s, t=0.0, h=0.0, nsteps=0, flags=0, extra=None):
    neb = np.zeros(16)
    g = s.gas
    if g is not None:
        neb[:13] = [g["alpha"], g["decrease_type"], g["time_scale"], g["t0"], g["t1"], g["eta"][0], g["eta"][1],
                    g["tau"][0], g["tau"][1], g["scale_height"][0], g["scale_height"][1], g["density"][0],
                    g["density"][1]]
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", 0x534F4C31, cmd))
        f.write(struct.pack("<7i", *s.counts))
        f.write(struct.pack("<ii", int(s.barycentric), int(g is not None)))
        f.write(neb.astype("<f8").tobytes())
        f.write(struct.pack("<ddii", t, h, nsteps, flags))
        for k in ("id", "type", "mig_type"):
            f.write(np.ascontiguousarray(getattr(s, k), "<i4").tobytes())
        for k in ("mig_stop_at", "mass", "radius", "density", "cd", "gamma_stokes", "gamma_epstein", "y0"):
            f.write(np.ascontiguousarray(getattr(s, k), "<f8").tobytes())
        ex = np.zeros(0) if extra is None else np.asarray(extra, "<f8").reshape(-1)
        f.write(struct.pack("<i", len(ex)))
        f.write(ex.tobytes())


def read_out(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        (ln,) = struct.unpack_from("<i", data, p); p += 4
        name = data[p:p + ln].decode(); p += ln
        kind, cnt = struct.unpack_from("<iq", data, p); p += 12
        dt = "<f8" if kind == 0 else "<i4"
        sz = 8 if kind == 0 else 4
        out[name] = np.frombuffer(data[p:p + cnt * sz], dtype=dt).copy(); p += cnt * sz
    return out


def run_ref(cmd, s, **kw):
    with tempfile.TemporaryDirectory() as td:
        ci, co = os.path.join(td, "case.bin"), os.path.join(td, "out.bin")
        write_case(ci, cmd, s, **kw)
        subprocess.run([oracle.REF_HARNESS, ci, co], check=True, stdout=subprocess.DEVNULL)
        return read_out(co)


def system_arrays(s):
    d = {f"in_{k}": np.asarray(getattr(s, k)) for k in ("id", "type", "mig_type", "mig_stop_at", "mass", "radius",
                                                      "density", "cd", "gamma_stokes", "gamma_epstein", "y0")}
    d["in_counts"] = np.asarray(s.counts, np.int32)
    d["in_barycentric"] = np.asarray(int(s.barycentric))
    d["in_epsilon"] = np.asarray(s.epsilon)
    if s.gas is not None:
        g = s.gas
        d["in_gas"] = np.asarray([g["alpha"], g["decrease_type"], g["quirks"], g["time_scale"], g["t0"], g["t1"],
                                  g["inner_edge"], g["mean_molecular_weight"], g["particle_diameter"], *g["eta"],
                                  *g["tau"], *g["scale_height"], *g["density"], *g["mean_free_path"]])
    return d


def save(name, s, res, **meta):
    d = system_arrays(s)
    for k, v in res.items():
        d[f"out_{k}"] = v
    for k, v in meta.items():
        d[f"meta_{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"  {name}: N={s.n} keys={sorted(res)}")


def small_self_gravitating(seed, n):
    s = scenarios.config3(seed=seed, n=n)
    s.name = f"selfgrav{n}"
    return s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.REFERENCE_SRC)
    ap.add_argument("--skip-full", action="store_true", help="skip the full-size (65,536 body) checksum fixture")
    args = ap.parse_args()
    if not oracle.build_reference(args.ref):
        sys.exit("reference sources not found: nothing generated")

    # --- force evaluations -------------------------------------------------
    s1 = scenarios.config1()
    save("accel_config1", s1, run_ref(CMD_ACCEL, s1, t=0.0, flags=7), t=0.0, flags=7)
    mg = scenarios.mixed_gas_system()
    save("accel_mixed_gas", mg, run_ref(CMD_ACCEL, mg, t=10.0, flags=7), t=10.0, flags=7)
    mgb = scenarios.mixed_gas_system(seed=3002, barycentric=True)
    save("accel_mixed_gas_bc", mgb, run_ref(CMD_ACCEL, mgb, t=10.0, flags=7), t=10.0, flags=7)
    # gas decreasing linearly: t between t0 and t1
    mgl = scenarios.mixed_gas_system(seed=3003)
    mgl.gas["decrease_type"] = abi.GAS_LINEAR
    mgl.gas["t0"], mgl.gas["t1"] = 0.0, 1000.0
    save("accel_mixed_gas_linear", mgl, run_ref(CMD_ACCEL, mgl, t=250.0, flags=7), t=250.0, flags=7)
    sg = small_self_gravitating(1013, 1024)
    save("accel_selfgrav1024", sg, run_ref(CMD_ACCEL, sg, t=0.0, flags=7), t=0.0, flags=7)
    for n in (2, 3, 17, 255, 257):
        s = small_self_gravitating(1100 + n, n)
        save(f"accel_selfgrav{n}", s, run_ref(CMD_ACCEL, s, t=0.0, flags=7), t=0.0, flags=7)
    # nearest-neighbour ties: bodies on a lattice so many distances coincide
    lt = small_self_gravitating(1200, 28)
    y = lt.y0.reshape(-1, 6)
    g = np.stack(np.meshgrid(np.arange(3), np.arange(3), np.arange(3), indexing="ij"), -1).reshape(-1, 3)
    y[1:, :3] = 1.0 + 0.125 * g
    lt.y0 = np.ascontiguousarray(y.reshape(-1))
    lt.name = "lattice28"
    save("accel_lattice28", lt, run_ref(CMD_ACCEL, lt, t=0.0, flags=7), t=0.0, flags=7)

    # --- integrators ----------------------------------------------------------
    save("rkf78_step_config1", s1, run_ref(CMD_RKF78_STEP, s1, t=0.0, h=s1.h0 * 200.0), t=0.0, h=s1.h0 * 200.0)
    save("rkf78_step_mixed_gas", mg, run_ref(CMD_RKF78_STEP, mg, t=5.0, h=0.5), t=5.0, h=0.5)
    save("rkf78_driver_config1", s1, run_ref(CMD_RKF78_DRIVER, s1, t=0.0, h=s1.h0, nsteps=40),
         t=0.0, h=s1.h0, nsteps=40)
    save("rkf78_driver_mixed_gas", mg, run_ref(CMD_RKF78_DRIVER, mg, t=0.0, h=mg.h0, nsteps=25), t=0.0, h=mg.h0,
         nsteps=25)
    sg64 = small_self_gravitating(1300, 64)
    save("rk4_driver_selfgrav64", sg64, run_ref(CMD_RK4_DRIVER, sg64, t=0.0, h=sg64.h0 * 100, nsteps=30),
         t=0.0, h=sg64.h0 * 100, nsteps=30)
    save("dp_driver_config1", s1, run_ref(CMD_DP_DRIVER, s1, t=0.0, h=s1.h0 * 50, nsteps=15),
         t=0.0, h=s1.h0 * 50, nsteps=15)
    save("integrals_mixed_gas", mg, run_ref(CMD_INTEGRALS, mg))

    # --- ephemeris helpers ---------------------------------------------------
    rng = np.random.default_rng(4001)
    M = 64
    el = np.stack([np.full(M, abi.GAUSS2 * 1.001), rng.uniform(0.3, 30, M), rng.uniform(0, 0.9, M),
                   rng.uniform(0, 0.5, M), rng.uniform(0, 6.28, M), rng.uniform(0, 6.28, M),
                   rng.uniform(0, 6.28, M)], 1)
    res = run_ref(CMD_EPHEMERIS, mg, extra=el)
    kep = np.stack([el[:, 2], el[:, 6]], 1)
    res.update({f"kepler_{k}": v for k, v in run_ref(CMD_KEPLER, mg, extra=kep).items()})
    ph = res["phase"].reshape(M, 6)
    oe_in = np.concatenate([el[:, :1], ph], 1)
    res.update({f"oe_{k}": v for k, v in run_ref(CMD_ORBITAL_ELEMENT, mg, extra=oe_in).items()})
    d = {"in_elements": el, **{f"out_{k}": v for k, v in res.items()}}
    np.savez_compressed(os.path.join(HERE, "ephemeris.npz"), **d)
    print("  ephemeris")

    # --- full size: checksum of the reference's dydt on a trig-free disk -----
    if not args.skip_full:
        de = scenarios.disk_exact()
        r = run_ref(CMD_ACCEL, de, t=0.0, flags=7)
        digest = {k: hashlib.sha256(np.ascontiguousarray(r[k]).tobytes()).hexdigest() for k in
                  ("dydt", "rm3", "nn_idx", "nn_dist")}
        y_digest = hashlib.sha256(de.y0.tobytes()).hexdigest()
        sample = np.arange(0, de.n, 4099)
        np.savez_compressed(os.path.join(HERE, "full_disk_exact_checksums.npz"),
                            y0_sha256=np.asarray(y_digest), n=np.asarray(de.n),
                            sample_index=sample, sample_dydt=r["dydt"].reshape(-1, 6)[sample],
                            **{f"{k}_sha256": np.asarray(v) for k, v in digest.items()},
                            dydt_abs_sum=np.abs(r["dydt"].reshape(-1, 6)).sum(0))
        print("  full_disk_exact_checksums", digest)


if __name__ == "__main__":
    main()

"""Build and drive tests/facade_program.cpp (the C++ class facade used the
way the reference's Simulator uses its classes)."""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

from solaris_gb300 import abi, build

HERE = os.path.dirname(os.path.abspath(__file__))
PROGRAM_SRC = os.path.join(HERE, "facade_program.cpp")


def compile_program(out_dir: str) -> str:
    """g++ the test program against the standalone class headers and
    libsolaris_facade.so."""
    build.build_facade()
    exe = os.path.join(out_dir, "facade_program")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, *build.facade_compile_flags(), PROGRAM_SRC, "-o", exe, f"-L{build.PKG}", "-lsolaris_facade",
           "-lsolaris_gb300", f"-Wl,-rpath,{build.PKG}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def write_input(path, system, integrator, n_steps, t0, h0, remove=-1, n_steps2=0):
    hdr = np.array(list(system.counts) + [integrator, n_steps, 1 if system.gas else 0, remove, n_steps2], np.int32)
    gas = abi.gas_struct(system.gas) if system.gas else abi.SolGasComponent()
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(bytes(memoryview(gas)))
        f.write(np.array([t0, h0], np.float64).tobytes())
        for k in ("id", "type", "mig_type"):
            f.write(np.ascontiguousarray(getattr(system, k), np.int32).tobytes())
        for k in ("mig_stop_at", "mass", "radius", "density", "cd", "gamma_stokes", "gamma_epstein"):
            f.write(np.ascontiguousarray(getattr(system, k), np.float64).tobytes())
        f.write(np.ascontiguousarray(system.y0, np.float64).tobytes())


def read_output(path) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        (ln,) = np.frombuffer(data, np.int32, 1, p)
        p += 4
        name = data[p:p + ln].decode()
        p += ln
        (kind,) = np.frombuffer(data, np.int32, 1, p)
        p += 4
        (cnt,) = np.frombuffer(data, np.int64, 1, p)
        p += 8
        dt = np.float64 if kind == 0 else np.int32
        out[name] = np.frombuffer(data, dt, int(cnt), p).copy()
        p += int(cnt) * np.dtype(dt).itemsize
    for k in list(out):
        if k.endswith("_msg"):
            out[k] = "".join(chr(int(c)) for c in out[k])
    return out


def run(exe, tmp, system, integrator, n_steps, t0, h0, remove=-1, n_steps2=0, env=None) -> dict:
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    write_input(fin, system, integrator, n_steps, t0, h0, remove, n_steps2)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    return read_output(fout)


assert C.sizeof(abi.SolGasComponent) == 144

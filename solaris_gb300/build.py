"""Build libsolaris_gb300.so in-tree with nvcc for sm_103a.

    python -m solaris_gb300.build [--force]

Translation units are compiled in parallel, then linked into
solaris_gb300/libsolaris_gb300.so (the CUDA runtime is linked statically).
The whole library is compiled with --fmad=false so that unfused arithmetic
rounds like the reference CPU build; kernels write fused multiply-adds out
explicitly where they want them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsolaris_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

SOURCES = ["sol_api.cu", "sol_force.cu", "sol_integrate.cu", "sol_diag.cu", "sol_ensemble.cu", "sol_adjoint.cu",
           "sol_terms.cu", "sol_persist.cu",
           "sol_output.cu", "sol_ephem.cu",
           "sol_events.cu", "sol_group.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     f"-I{INCLUDE}"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "solaris_gb300.h")]
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc(), *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


# ---- the C++ class facade (Acceleration, RungeKuttaFehlberg78, RungeKutta4,
# DormandPrince with the reference's interface) over the C-ABI -----------------
FACADE = os.path.join(PKG, "facade")
FACADE_INCLUDE = os.path.join(FACADE, "include")
FACADE_LIB = os.path.join(PKG, "libsolaris_facade.so")
# the classes the facade implements, and (standalone builds only) the data
# classes they read
FACADE_CLASSES = ["Acceleration.cpp", "RungeKuttaFehlberg78.cpp", "RungeKutta4.cpp", "DormandPrince.cpp",
                  "facade_state.cpp"]
FACADE_SUPPORT = ["BodyData.cpp", "NBodies.cpp", "TimeLine.cpp", "PowerLaw.cpp", "GasComponent.cpp", "Error.cpp"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function"]


def facade_sources(standalone: bool = True) -> list[str]:
    src = [os.path.join(FACADE, f) for f in FACADE_CLASSES]
    if standalone:
        src += [os.path.join(FACADE, "support", f) for f in FACADE_SUPPORT]
    return src


def facade_compile_flags(class_headers: str = FACADE_INCLUDE) -> list[str]:
    """g++ flags for the facade sources.  class_headers is the directory of the
    Solaris class headers to compile against: the standalone set here, or a
    Solaris source tree for a drop-in build of the reference program."""
    return [*CXX_FLAGS, f"-I{class_headers}", f"-I{FACADE}", f"-I{INCLUDE}"]


def build_facade(force: bool = False) -> str:
    """libsolaris_facade.so: the facade classes plus the standalone data
    classes, linked against libsolaris_gb300.so (rpath $ORIGIN)."""
    build(force=force)
    srcs = facade_sources()
    hdrs = [os.path.join(FACADE_INCLUDE, f) for f in os.listdir(FACADE_INCLUDE)]
    newest = max(os.path.getmtime(f) for f in srcs + hdrs + [LIB, os.path.join(FACADE, "facade_state.h")])
    if not force and os.path.exists(FACADE_LIB) and os.path.getmtime(FACADE_LIB) >= newest:
        return FACADE_LIB
    cxx = shutil.which("g++") or "g++"
    tmp = FACADE_LIB + ".tmp"
    cmd = [cxx, *facade_compile_flags(), "-shared", "-o", tmp, *srcs, f"-L{PKG}", "-lsolaris_gb300",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"facade build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, FACADE_LIB)
    return FACADE_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_facade(force="--force" in sys.argv))

"""The C++ class facade without a GPU: it builds, exports the reference's class
members, the test program links against it, and the reference's own program
links with its Acceleration and integrator classes replaced by the facade."""
import os
import shutil
import subprocess

import pytest

import oracle
from facade_io import compile_program
from solaris_gb300 import build

REF = oracle.REFERENCE_SRC


def _defined_symbols(path):
    r = subprocess.run(["nm", "-DC", "--defined-only", path], capture_output=True, text=True, check=True)
    return r.stdout


def test_facade_library_exports_the_reference_classes():
    lib = build.build_facade()
    syms = _defined_symbols(lib)
    for s in ("Acceleration::Acceleration(IntegratorType, bool, BodyData*, Nebula*)",
              "Acceleration::Compute(double, double*, double*)", "Acceleration::GravityAC(double, double*, double*)",
              "Acceleration::GasDragAC(double, double*, double*)", "Acceleration::TauNu(double, double)",
              "Acceleration::GravityBC_NonSelfInteracting(double, double*, double*)",
              "RungeKuttaFehlberg78::Driver(BodyData*, Acceleration*, TimeLine*)",
              "RungeKuttaFehlberg78::Step(BodyData*, Acceleration*)",
              "RungeKuttaFehlberg78::GetErrorMax(int, double const*, double const*)",
              "RungeKutta4::Driver(BodyData*, Acceleration*, TimeLine*)",
              "DormandPrince::Driver(BodyData*, Acceleration*, TimeLine*)",
              "DormandPrince::Step2(BodyData*, Acceleration*)", "BodyData::Allocate()"):
        assert s in syms, s


def test_test_program_links(tmp_path):
    exe = compile_program(str(tmp_path))
    assert os.access(exe, os.X_OK)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "Solaris")), reason="reference sources not present")
def test_reference_program_links_with_the_facade(tmp_path):
    """oracle/Makefile's dropin target: the reference's Solaris.cpp, Simulator
    and the rest of its objects, with Acceleration.o, RungeKuttaFehlberg78.o,
    RungeKutta4.o and DormandPrince.o replaced by the facade compiled against
    the reference's own headers."""
    if shutil.which("make") is None:
        pytest.skip("make not available")
    build.build()
    oracle_dir = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
    subprocess.run(["make", "-s", "-C", oracle_dir, f"REF={REF}", "dropin"], check=True, capture_output=True)
    exe = os.path.join(oracle_dir, "_ref", "solaris_gb300_dropin")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True, check=True).stdout
    assert " T RungeKuttaFehlberg78::Driver(BodyData*, Acceleration*, TimeLine*)" in syms
    assert " U sol_driver_host" in syms
    import torch
    if torch.cuda.is_available():
        return
    # without a GPU the reference's Simulator reaches the facade, which reports
    # the CUDA failure through the reference's own Error::_errMsg
    case = os.path.join(REF, "TestCases", "EjectionTest")
    for f in os.listdir(case):
        shutil.copy(os.path.join(case, f), tmp_path)
    r = subprocess.run([exe, "-i", str(tmp_path / "EjectionTest.xml")], capture_output=True, text=True, cwd=tmp_path,
                       env=dict(os.environ, OSTYPE="linux"), timeout=60)
    assert r.returncode != 0
    assert "CUDA error" in r.stderr and "Simulator.cpp" in r.stderr

"""C-ABI checks that need no GPU: the library builds, loads and exports every
symbol include/solaris_gb300.h declares; host-side argument validation runs
before any CUDA call."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from solaris_gb300 import abi, build, scenarios

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.load_library()


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(sol_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    decl = declared_symbols()
    assert len(decl) >= 20
    missing = [n for n in decl if not hasattr(lib, n)]
    assert not missing, missing
    assert set(abi.exported_names()) <= set(decl)


def test_gas_defaults_match_scenarios(lib):
    g = abi.SolGasComponent()
    assert lib.sol_gas_component_init(C.byref(g)) == abi.SOL_OK
    d = scenarios.default_gas()
    assert g.inner_edge == d["inner_edge"] and g.alpha == d["alpha"]
    assert (g.density.c, g.density.index) == d["density"]
    assert g.mean_free_path.index == d["mean_free_path"][1]
    assert abs(g.mean_free_path.c - d["mean_free_path"][0]) <= 1e-15 * d["mean_free_path"][0]
    assert g.quirks == abi.QUIRKS_REFERENCE


def _create(lib, s, gas=None):
    view = abi.BodyDataView(s)
    h = C.c_void_p()
    rc = lib.sol_create(C.byref(view.struct), C.byref(gas) if gas else None, 0, 0, C.byref(h))
    return rc, h


def test_unsorted_bodies_rejected(lib):
    s = scenarios.config3(n=17)
    s.type = s.type.copy()
    s.type[5] = abi.TEST_PARTICLE
    rc, h = _create(lib, s)
    assert rc == abi.SOL_ERR_ARG
    assert b"sorted" in lib.sol_last_error()


def test_missing_central_body_rejected(lib):
    s = scenarios.config3(n=17)
    s.counts = (0,) + tuple(s.counts[1:4]) + (s.counts[4], s.counts[5], s.counts[6] + 1)
    rc, _ = _create(lib, s)
    assert rc == abi.SOL_ERR_ARG


def test_bad_gas_type_rejected(lib):
    s = scenarios.config3(n=17)
    g = abi.SolGasComponent()
    lib.sol_gas_component_init(C.byref(g))
    g.decrease_type = 7
    rc, _ = _create(lib, s, g)
    assert rc == abi.SOL_ERR_ARG


def test_null_arguments(lib):
    assert lib.sol_create(None, None, 0, 0, None) == abi.SOL_ERR_ARG
    assert lib.sol_set_precision(None, 0) == abi.SOL_ERR_ARG
    assert lib.sol_accel_compute(None, 0.0, None, None, None, None, None) == abi.SOL_ERR_ARG
    assert lib.sol_destroy(None) == abi.SOL_OK
    r = (C.c_int64 * 3)()
    assert lib.sol_check_pair_math(0, 10, 16, 1, r) == abi.SOL_ERR_ARG   # no such sample family
    assert lib.sol_check_pair_math(0, -1, 16, 1, r) == abi.SOL_ERR_ARG
    assert lib.sol_check_pair_math(0, 0, -1, 1, r) == abi.SOL_ERR_ARG
    assert lib.sol_check_pair_math(0, 0, 16, 1, None) == abi.SOL_ERR_ARG


def test_pair_count_matches_oracle_sample():
    """Pair counting convention: one Kepler term per body plus the direct terms
    GravityAC evaluates."""
    import oracle
    s = scenarios.config1()
    assert s.pair_count() == 255 + 2 + 253 * 2
    o = oracle.Oracle(s)
    _, pairs = o.gravity_sample(s.y0, 1, s.n)
    assert pairs == s.pair_count()
    s3 = scenarios.config3(n=300)
    assert s3.pair_count() == 299 + 299 * 298
    o3 = oracle.Oracle(s3)
    assert o3.gravity_sample(s3.y0, 1, s3.n)[1] == s3.pair_count()


def test_ensemble_rejects_unsorted_system(lib):
    s = scenarios.config3(n=17)
    t = scenarios.config3(n=9)
    t.type = t.type.copy()
    t.type[3] = abi.TEST_PARTICLE
    views = [abi.BodyDataView(x) for x in (s, t)]
    arr = (abi.SolBodyData * 2)(*[v.struct for v in views])
    h = C.c_void_p()
    assert lib.sol_ensemble_create(arr, 2, 0, C.byref(h)) == abi.SOL_ERR_ARG
    assert b"system 1" in lib.sol_last_error()

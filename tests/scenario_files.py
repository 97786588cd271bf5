"""Readers of the reference's binary output files (BinaryFileAdapter.cpp
record layouts) for the scenario tests."""
from __future__ import annotations

import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SCENARIOS = os.path.join(HERE, "golden", "scenarios")
NAMES = ("ejection_rkf78", "gas_rk4", "bary_dopri", "collision_rkf78", "epochs_rkf78", "pre_dopri")


def xml_path(name: str) -> str:
    return os.path.join(SCENARIOS, name + ".xml")


def golden_dir(name: str) -> str:
    return os.path.join(SCENARIOS, name)


def read_phases(path):
    """[(time, ids (n,), phases (n, 6))] of SavePhases records."""
    b = open(path, "rb").read()
    out, o = [], 0
    while o < len(b):
        t, n = struct.unpack_from("<di", b, o)
        o += 12
        ids, ys = np.empty(n, np.int32), np.empty((n, 6))
        for i in range(n):
            ids[i] = struct.unpack_from("<i", b, o)[0]
            ys[i] = struct.unpack_from("<6d", b, o + 4)
            o += 52
        out.append((t, ids, ys))
    return out


def read_integrals(path):
    """(header, [(time, 16 values)]) of SaveIntegrals records."""
    b = open(path, "rb").read()
    (ln,) = struct.unpack_from("<i", b, 0)
    header, o, out = b[4:4 + ln], 4 + ln, []
    while o < len(b):
        (ne,) = struct.unpack_from("<i", b, o)
        vals = struct.unpack_from(f"<{ne}d", b, o + 4)
        out.append((vals[0], np.array(vals[1:])))
        o += 4 + 8 * ne
    return header, out


def read_affairs(path):
    """SaveTwoBodyAffair records: dicts of id, type, id1, id2, phase1, phase2, time."""
    b = open(path, "rb").read() if os.path.exists(path) else b""
    out = []
    for o in range(0, len(b), 120):
        i, t, b1, b2 = struct.unpack_from("<4i", b, o)
        p = struct.unpack_from("<13d", b, o + 16)
        out.append(dict(id=i, type=t, id1=b1, id2=b2, phase1=np.array(p[:6]), phase2=np.array(p[6:12]), time=p[12]))
    return out


def read_variable_properties(path):
    """SaveVariableProperty records: (property id, body id, time, mass, radius, density)."""
    b = open(path, "rb").read()
    return [struct.unpack_from("<iid3d", b, o) for o in range(0, len(b), 40)]

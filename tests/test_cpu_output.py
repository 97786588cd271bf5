"""Record layouts of the output files against a plain restatement of the
reference's BinaryFileAdapter (Solaris/BinaryFileAdapter.cpp:107-219):
binary phases, text phases and integrals with and without the header."""
import struct

import numpy as np

from solaris_gb300 import engine

HEADER = ("time [day], mass [Solar], bary center position r: x [AU], y [AU], z [AU], bary center velocity v: "
          "x [AU/day], y [AU/day], z [AU/day], length of r [AU], length of v [AU/day], angular momentum vector c: "
          "x, y, z, length of c, kinetic energy, potential energy, total energy")


def test_binary_phases_record():
    rng = np.random.default_rng(5)
    y = rng.standard_normal(6 * 5)
    ids = np.array([7, 3, 11, 2, 40], np.int32)
    rec = engine.format_phases_record(123.25, y, ids)
    want = struct.pack("<di", 123.25, 5) + b"".join(struct.pack("<i6d", int(ids[i]), *y[6 * i:6 * i + 6])
                                                     for i in range(5))
    assert rec == want


def test_text_phases_record():
    y = np.array([1.0, -2.5e-3, 3.14159265358979, 1e-10, -7.0, 123456.789] * 2)
    ids = np.array([1, 22], np.int32)
    rec = engine.format_phases_record(3652.5, y, ids, text=True).decode()
    want = "%15.10g" % 3652.5 + "%8d" % 2
    for i in range(2):
        want += "%8d" % ids[i] + "".join("%15.6g" % v for v in y[6 * i:6 * i + 6])
    assert rec == want + "\n"


def test_integrals_record_and_header():
    v = np.arange(16, dtype=np.float64) * 0.5 - 3.0
    rec = engine.format_integrals_record(10.0, v)
    assert rec == struct.pack("<id", 17, 10.0) + v.tobytes()
    first = engine.format_integrals_record(0.0, v, header=True)
    assert first == struct.pack("<i", len(HEADER)) + HEADER.encode() + struct.pack("<id", 17, 0.0) + v.tobytes()

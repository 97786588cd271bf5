"""Output files written during an integration: the phases and integrals
records of every save, byte for byte, against states stepped separately and
formatted by the record functions; snapshots taken just before the next
driver calls keep the state of the save."""
import os

import numpy as np
import pytest

from solaris_gb300 import abi, engine, scenarios

pytestmark = pytest.mark.gpu


def _reference_records(s, n_steps, every_integrals, text=False):
    phases, integrals = b"", b""
    with engine.Context(s) as ctx:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        first = True
        for k in range(n_steps):
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
            phases += engine.format_phases_record(tl.time, ctx.get_state(), s.id, text=text)
            if k % every_integrals == 0:
                integrals += engine.format_integrals_record(tl.time, ctx.integrals(), header=first)
                first = False
    return phases, integrals


@pytest.mark.parametrize("text", [False, True])
def test_phases_and_integrals_files(tmp_path, text):
    s = scenarios.config3(seed=91, n=300)
    n_steps = 6
    ph, it = str(tmp_path / "Phases.dat"), str(tmp_path / "Integrals.dat")
    with engine.Context(s) as ctx, engine.Output(ctx, ph, it, text=text) as out:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        for k in range(n_steps):
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
            out.save_phases(tl.time)
            if k % 2 == 0:
                out.save_integrals(tl.time)
    want_ph, want_it = _reference_records(s, n_steps, 2, text)
    assert open(ph, "rb").read() == want_ph
    assert open(it, "rb").read() == want_it


def test_snapshots_overlap_the_next_driver_calls(tmp_path):
    """65,536 bodies: each snapshot is followed at once by the next driver
    call; the file still holds the state of each save."""
    s = scenarios.config3(seed=92, n=65536)
    ph = str(tmp_path / "Phases.dat")
    states = []
    with engine.Context(s, precision=abi.PRECISION_SPLIT_FF) as ctx, engine.Output(ctx, ph) as out:
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        times = []
        for _ in range(3):
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
            out.save_phases(tl.time)
            times.append(tl.time)
            states.append(ctx.get_state())  # waits for the stream; the next call starts after
        out.flush()
    data = open(ph, "rb").read()
    want = b"".join(engine.format_phases_record(t, y, s.id) for t, y in zip(times, states))
    assert data == want
    # an integrals file that already has records gets no second header
    it = str(tmp_path / "Integrals.dat")
    for _ in range(2):
        with engine.Context(s) as ctx, engine.Output(ctx, None, it) as out:
            ctx.set_state(s.y0)
            out.save_integrals(0.0)
    raw = open(it, "rb").read()
    hlen = int(np.frombuffer(raw[:4], np.int32)[0])
    assert raw.count(raw[4:4 + hlen]) == 1
    assert len(raw) == 4 + hlen + 2 * (4 + 8 + 16 * 8)

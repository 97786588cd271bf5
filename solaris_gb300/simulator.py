"""The reference's simulation of a scenario file on the device:
Simulator::Run with its synchronisation of body groups that start at
different epochs, the pre-integration to a TimeLine start and the main
integration (Solaris/Simulator.cpp:62-447), each an Integrate /
DecisionMaking / CheckEvent loop (:121-250, :621-735), with the output files
of Solaris/BinaryFileAdapter.cpp.

Per accepted step, as the reference does it: one integrator Driver call on
the device, then the events (ejection, hit-centrum, collisions) applied on
the device, the stop test, the step clamped to the end of the phase, a
phases + integrals record when the output interval is full, the step clamped
to the next output time; every 100 steps (counted over the whole run)
coordinates below 1e-50 are set to zero (Tools::CheckAgainstSmallestNumber).
Phases and integrals records are written in the reference's binary layouts
by the output writer thread; TwoBodyAffair records, the constant / variable
/ composition property records of body insertion and of every merge, and the
log lines are written here on the host, which keeps the reference's body
list (the characteristics it replays with the reference's arithmetic, the
phases it takes back from the device after every phase).

The end test: the reference compares the absolute time with the phase's
length (DecisionMaking, :197-219), so a run that starts at an epoch's Julian
date stops as soon as |time| >= |length|, after one step for dates beyond the
length; relative_end_test=True measures the time integrated in the phase
instead, as the reference's unused second DecisionMaking (:252-320) does.

A collision's TwoBodyAffair record carries, as the reference writes it
(Simulator.cpp:709), the phases of the step's starting state at the
survivor's and the merger's current indices (bodyData.y after the swap);
that state is read back before each step of a run with collisions.

A backend does the numerical work of one Integrate call: EngineBackend is a
device context; any factory (system, settings, directory) -> object with
the same methods (step, events, n_total, state, zero_below_smallest,
save_phases, save_integrals, close) can stand in for it.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct
import time as _time

import numpy as np

from . import abi, engine
from . import scenario_xml as sx
from .scenario_xml import BodySpec, Component, Scenario, ScenarioError, YEAR_TO_DAY, PI

SMALLEST_NUMBER = 1.0e-50
CHECK_FOR_SMALLEST = 100
EJECTION, HIT_CENTRUM, COLLISION = 0, 1, 3


class EngineBackend:
    """A device context driven one accepted step at a time."""

    def __init__(self, system, st, directory: str, device: int = 0, precision: int = abi.PRECISION_FP64):
        # barycentric frames (GravityBC_*) have the FP64 form only
        prec = abi.PRECISION_FP64 if system.barycentric else precision
        self.ctx = engine.Context(system, device=device, precision=prec)
        self.ctx.set_state(system.y0)
        self.integrator = st.integrator
        self.out = engine.Output(self.ctx, os.path.join(directory, st.phases), os.path.join(directory, st.integrals))
        self.tl = abi.SolTimeLine(0.0, 0.0, 0.0)
        self.rejected = 0  # attempts the step-size control rejected

    def step(self, time: float, h_next: float):
        """One Driver call: returns (time, h_did, h_next)."""
        self.tl.time, self.tl.h_next, self.tl.h_did = time, h_next, 0.0
        r = self.ctx.driver(self.integrator, time, h_next, 1, time_line=self.tl)
        self.rejected += r["stats"][1]
        return r["time"], r["h_did"], r["h_next"]

    def events(self, time, ejection, hit_centrum, collision_factor):
        return self.ctx.handle_events(time, ejection, hit_centrum, collision_factor)

    def run_until(self, sim, tl, clock, max_steps: int = 1 << 20) -> int:
        """Steps on the device until the host has work (sol_run_until)."""
        st = sim.sc.settings
        rel = sim.relative_end_test
        line = abi.SolSimLine(time=tl.time, length=tl.length, output=tl.output, h_next=tl.h_next, h_did=tl.h_did,
                              elapsed=clock.all if rel else tl.elapsed,
                              last_save=clock.save if rel else tl.last_save, steps=sim.steps,
                              relative_end=1 if rel else 0)
        factor = st.collision if st.collision is not None else 0.0
        reason, stats = self.ctx.run_until(self.integrator, line, max_steps, st.ejection, st.hit_centrum, factor)
        self.rejected += stats[1]
        tl.time, tl.h_next, tl.h_did = line.time, line.h_next, line.h_did
        if rel:
            clock.all, clock.save = line.elapsed, line.last_save
        else:
            tl.elapsed, tl.last_save = line.elapsed, line.last_save
        sim.steps = int(line.steps)
        return reason

    def step_start(self):
        return self.ctx.step_start()

    def n_total(self) -> int:
        return self.ctx.n

    def state(self):
        return self.ctx.get_state()

    def zero_below_smallest(self):
        y = self.ctx.get_state()
        small = np.abs(y) < SMALLEST_NUMBER
        if np.any(small & (y != 0.0)):
            y[small] = 0.0
            self.ctx.set_state(y)

    def save_phases(self, time: float):
        self.out.save_phases(time)

    def save_integrals(self, time: float):
        self.out.save_integrals(time)

    def close(self):
        self.out.close()
        self.ctx.close()


# ---- property records (BinaryFileAdapter.cpp:263-475) -------------------------------------
def _guid_bytes(guid: str) -> bytes:
    """Tools::GuidToCharArray, reordered for .NET's Guid(int, short, short, 8 bytes)."""
    hexs = guid.replace("-", "")
    raw = bytearray(16)
    for k in range(min(16, len(hexs) // 2)):
        try:
            raw[k] = int(hexs[2 * k:2 * k + 2], 16)
        except ValueError:
            raise ScenarioError(f"invalid guid {guid!r}") from None
    return bytes(raw[3::-1] + raw[5:3:-1] + raw[7:5:-1] + raw[8:16])


def _short_string(s: str) -> bytes:
    b = s.encode("utf-8")
    if len(b) > 127:
        raise ScenarioError(f"the name {s[:20]!r}... is longer than 127 bytes")
    return bytes([len(b)]) + b


class _Body:
    """The host's copy of a body (the reference's Body list entry): its
    characteristics, replayed through merges, and its phase, taken back from
    the device after every phase."""

    def __init__(self, spec: BodySpec):
        self.spec = spec
        self.id = spec.id
        self.type = spec.type
        self.mig_type = spec.mig_type
        self.mig_stop_at = spec.mig_stop_at
        self.cd = spec.cd
        self.mass = spec.mass if spec.type != abi.TEST_PARTICLE else 0.0
        self.radius = spec.radius if spec.type != abi.TEST_PARTICLE else 0.0
        self.density = spec.density if spec.type != abi.TEST_PARTICLE else 0.0
        self.components = [Component(c.name, c.ratio) for c in spec.components]
        self.phase = list(spec.phase)


@dataclasses.dataclass
class _Clock:
    """Time integrated in the current phase (all) and since its last record (save)."""
    all: float = 0.0
    save: float = 0.0


@dataclasses.dataclass
class TimeLine:
    """Solaris/TimeLine.h: one phase's time line."""
    time: float
    length: float
    output: float
    h_next: float = 0.0
    h_did: float = 0.0
    elapsed: float = 0.0
    last_save: float = 0.0
    save: float = 0.0

    def forward(self) -> bool:
        return self.length >= 0


class _Properties:
    def __init__(self, directory: str, st):
        self.const_path = os.path.join(directory, st.constant_properties)
        self.var_path = os.path.join(directory, st.variable_properties)
        self.comp_path = os.path.join(directory, st.composition_properties)
        self.property_id = 0
        self.composition_id = 0

    def constant(self, b: _Body) -> bytes:
        s = b.spec
        rec = struct.pack("<i", s.id) + _guid_bytes(s.guid)
        for text in (s.name, s.designation, s.provisional_designation, s.reference, s.opposition):
            rec += _short_string(text)
        rec += struct.pack("<iiii", s.ln, s.type, s.mpc_orbit_type, s.mig_type)
        rec += struct.pack("<dd", s.abs_vis_mag, s.cd) if s.has_characteristics else bytes(16)
        return rec

    def variable(self, b: _Body, time: float, comp_out: list) -> bytes:
        pid = self.property_id
        self.property_id += 1
        rec = struct.pack("<iid", pid, b.spec.id, time)
        if b.spec.has_characteristics:
            rec += struct.pack("<ddd", b.mass, b.radius, b.density)
            for c in b.components:
                comp_out.append(struct.pack("<ii", self.composition_id, pid) + _short_string(c.name) +
                                struct.pack("<d", c.ratio))
                self.composition_id += 1
        else:
            rec += bytes(24)
        return rec

    def append(self, const: list, var: list, comp: list):
        for path, recs in ((self.const_path, const), (self.var_path, var), (self.comp_path, comp)):
            if recs or path != self.comp_path:
                with open(path, "ab") as f:
                    f.write(b"".join(recs))


def _merge_characteristics(s: _Body, m: _Body, m_type: int):
    """Simulator::CalculateCharacteristicsAfterCollision (Simulator.cpp:827-898)
    and CalculateComponentListUnion (:901-935) on the host's copies."""
    surviv_mass = s.mass
    if m_type == abi.SUPER_PLANETESIMAL:
        merger_mass = m.density * (4.0 / 3.0 * PI * (m.radius * m.radius * m.radius))
    else:
        merger_mass = m.mass
    total = surviv_mass + merger_mass
    if s.components or m.components:
        if not s.components:
            s.components.append(Component("Unknown", 100.0))
        if not m.components:
            m.components.append(Component("Unknown", 100.0))
        union = [Component(c.name, c.ratio) for c in s.components]  # Tools::MergeComponentList
        for c in m.components:
            if not any(u.name.lower() == c.name.lower() for u in union):
                union.append(Component(c.name, c.ratio))
        for u in union:
            cs = next((c for c in s.components if c.name.lower() == u.name.lower()), None)
            cm = next((c for c in m.components if c.name.lower() == u.name.lower()), None)
            if cs is not None and cm is not None:
                u.ratio = 1.0 / total * (surviv_mass * cs.ratio + merger_mass * cm.ratio)
            elif cs is None and cm is not None:
                u.ratio = 1.0 / total * merger_mass * cm.ratio
            else:
                u.ratio = 1.0 / total * surviv_mass * cs.ratio
        s.components = union
    s.mass = total
    if s.radius == 0:
        return
    if m.radius == 0:
        m.density = s.density
        m.radius = math.pow(3.0 / (4.0 * PI) * m.mass / m.density, 1.0 / 3.0)
    rs, rm = s.radius, m.radius
    volume = 4.0 / 3.0 * PI * (rs * rs * rs + rm * rm * rm)
    s.radius = math.pow(3.0 / (4.0 * PI) * volume, 1.0 / 3.0)
    s.density = total / volume


def _yr(days: float) -> str:
    return "%g" % (days * (1.0 / YEAR_TO_DAY))


class Simulator:
    """Runs a scenario (synchronisation, pre-integration, main integration)
    and writes the reference's output files into `directory` (the scenario
    file's directory by default)."""

    def __init__(self, scenario: Scenario, directory: str | None = None, backend=None, device: int = 0,
                 precision: int = abi.PRECISION_FP64, relative_end_test: bool = False):
        self.sc = scenario
        self.dir = directory or scenario.directory
        os.makedirs(self.dir, exist_ok=True)
        self.factory = backend if backend is not None else (
            lambda system, st, d: EngineBackend(system, st, d, device, precision))
        self.relative_end_test = relative_end_test
        self.bodies = {b.id: _Body(b) for g in scenario.groups for b in g.bodies}
        self.body_list = []  # the bodies being integrated, in the device's order
        self.props = _Properties(self.dir, scenario.settings)
        self.event_id = 0
        self.steps = 0      # Counter::succededStep, over the whole run
        self.rejected = 0   # attempts rejected by the step-size control (the reference does not count them)
        self.phases = 0
        self.affairs = []
        self.be = None

    # -- log (BinaryFileAdapter::Log) ----------------------------------------------------
    def _log(self, msg: str):
        stamp = _time.strftime("%Y-%m-%d %H:%M:%S", _time.localtime())
        with open(os.path.join(self.dir, self.sc.settings.log), "a") as f:
            f.write(f"{stamp} {msg}\n")

    # -- Simulator::Insert: a group joins the body list; its properties are written ----------
    def _insert(self, group, time: float):
        self.body_list, written = sx.insert_group(self.body_list, [self.bodies[b.id] for b in group.bodies])
        const, var, comp = [], [], []
        for b in written:
            const.append(self.props.constant(b))
            var.append(self.props.variable(b, time, comp))
        self.props.append(const, var, comp)

    def _populate(self, time: float):
        for g in self.sc.groups:
            self._insert(g, time)

    # -- CheckEvent ------------------------------------------------------------------------
    def _check_event(self, time: float, y_start):
        st = self.sc.settings
        factor = st.collision if st.collision is not None else 0.0
        if st.ejection <= 0.0 and st.hit_centrum <= 0.0 and factor <= 0.0:
            return
        affairs = self.be.events(time, st.ejection, st.hit_centrum, factor)
        if not affairs:
            return
        # TwoBodyAffair ids: ejections and hit-centrum bodies are numbered in body
        # order as they are found, collisions after them; the records are written
        # ejections first, then hit-centrum bodies, then collisions
        found = sorted((a["idx2"], a["type"], k) for k, a in enumerate(affairs) if a["type"] != COLLISION)
        ids = {k: self.event_id + r for r, (_, _, k) in enumerate(found)}
        next_id = self.event_id + len(found)
        for k, a in enumerate(affairs):
            if a["type"] == COLLISION:
                ids[k] = next_id
                next_id += 1
        self.event_id = next_id
        lib = abi.load_library()
        path = os.path.join(self.dir, st.two_body_affair).encode()
        var, comp = [], []
        for k, a in enumerate(affairs):
            rec = (abi.SolAffair * 1)()
            rec[0].type, rec[0].idx1, rec[0].idx2 = a["type"], a["idx1"], a["idx2"]
            rec[0].id1, rec[0].id2, rec[0].time = a["id1"], a["id2"], a["time"]
            if a["type"] == COLLISION and y_start is not None:
                a = dict(a, phase1=y_start[6 * a["idx1"]:6 * a["idx1"] + 6],
                         phase2=y_start[6 * a["idx2"]:6 * a["idx2"] + 6])
            rec[0].phase1[:] = list(a["phase1"])
            rec[0].phase2[:] = list(a["phase2"])
            abi.check(lib, lib.sol_write_affairs(path, rec, 1, ids[k]))
            self.affairs.append(dict(a, id=ids[k]))
            if a["type"] == EJECTION:
                self._log(f"Ejection: At {_yr(a['time'])} [yr] body with id: {a['id2']}")
                self._remove(a["id2"])
                continue
            if a["type"] == HIT_CENTRUM:
                c, b = self.bodies[a["id1"]], self.bodies[a["id2"]]
                s, m = (c, b) if c.mass >= b.mass else (b, c)  # HandleCollision: the central body has index 0
            else:
                s, m = self.bodies[a["id1"]], self.bodies[a["id2"]]
            if m.type != abi.TEST_PARTICLE:
                _merge_characteristics(s, m, m.type)
                var.append(self.props.variable(s, a["time"], comp))
            if a["type"] == HIT_CENTRUM:
                self._log(f"HitCentrum: At {_yr(a['time'])} [yr] body with id: {a['id2']}")
            else:
                self._log(f"Collision: At {_yr(a['time'])} [yr] between body with id: {a['id1']} "
                          f"and id: {a['id2']}")
            self._remove(a["id2"] if a["type"] == HIT_CENTRUM else m.id)
        if var:
            self.props.append([], var, comp)

    def _remove(self, bid: int):
        self.body_list = [b for b in self.body_list if b.id != bid]

    # -- Integrate / DecisionMaking ---------------------------------------------------------
    def _integrate(self, tl: TimeLine):
        st = self.sc.settings
        sx.check_type_order(self.body_list)
        system = sx.build_system(st, self.body_list, self.sc.gas)
        self.be = be = self.factory(system, st, self.dir)
        self.phases += 1
        collisions = st.collision is not None
        clock = _Clock()  # the phase-relative clock of relative_end_test
        chunked = hasattr(be, "run_until")
        try:
            be.save_phases(tl.time)
            be.save_integrals(tl.time)
            while True:
                if chunked:  # the steps without host work run on the device
                    reason = be.run_until(self, tl, clock)
                    if reason == abi.STOP_STEPS:
                        continue
                    y_start = be.step_start() if collisions and reason == abi.STOP_EVENT else None
                    events = reason == abi.STOP_EVENT
                else:
                    y_start = be.state() if collisions else None
                    tl.time, tl.h_did, tl.h_next = be.step(tl.time, tl.h_next)
                    self.steps += 1
                    tl.elapsed += tl.h_did
                    tl.last_save += tl.h_did
                    clock.all += tl.h_did
                    clock.save += tl.h_did
                    events = True
                stop = self._decision(tl, clock, y_start, events)
                if self.steps % CHECK_FOR_SMALLEST == 0:
                    be.zero_below_smallest()
                if stop:
                    break
            # UpdateBodyListAfterIntegration: the phases go back to the body list
            y = be.state()
            for k, b in enumerate(self.body_list):
                b.phase = [float(v) for v in y[6 * k:6 * k + 6]]
            be.save_phases(tl.time)
            be.save_integrals(tl.time)
        finally:
            self.rejected += getattr(be, "rejected", 0)
            be.close()
            self.be = None

    def _decision(self, tl: TimeLine, clock: "_Clock", y_start, events: bool) -> bool:
        """Simulator::DecisionMaking (Simulator.cpp:181-250) after the step's
        times are added: CheckEvent, the end test, the clamps and the record."""
        be = self.be
        if events:
            self._check_event(tl.time, y_start)
        now = clock.all if self.relative_end_test else tl.time  # 1000 YearToDay millenium + time
        since = clock.save if self.relative_end_test else tl.last_save
        if abs(now) >= abs(tl.length):
            return True
        if be.n_total() <= 1:
            self._log("The total number of bodies reduced to 1!")
            return True
        if abs(now + tl.h_next) > abs(tl.length):
            tl.h_next = tl.length - now
        if abs(since) >= abs(tl.output):
            be.save_phases(tl.time)
            be.save_integrals(tl.time)
            tl.last_save = clock.save = since = 0.0
            if self.relative_end_test:
                tl.save += tl.output
        if abs(since + tl.h_next) > abs(tl.output):
            tl.h_next = tl.output - since
        return False

    # -- Simulator::Run ------------------------------------------------------------------------
    def _synchronization(self, main: TimeLine):
        """Simulator::Synchronization (Simulator.cpp:322-390)."""
        st, sc = self.sc.settings, self.sc
        sync = dataclasses.replace(main)
        times = sx.sync_start_times(st, sc.groups, sc.time0)
        inserted = set()
        for k, t in enumerate(times):
            for g in sc.groups:
                if g.start_time == t and id(g) not in inserted:
                    self._insert(g, sync.time)
                    inserted.add(id(g))
                    self._log(f"The bodygroup ({g.description}) with epoch: {g.epoch} was included")
            if k + 1 >= len(times):
                break
            sync.length = times[k + 1] - sync.time
            sync.output = main.output if sync.forward() else -main.output
            if sync.length != 0.0 and len(self.body_list) > 1:
                sx.check_type_order(self.body_list)
                sync.h_did = 0.0
                sync.h_next = sx.first_step(self.body_list, sync.length, 50.0)
                self._integrate(sync)
        main.time = sync.time
        main.save = sync.time

    def _pre_integration(self, main: TimeLine):
        """Simulator::PreIntegration (Simulator.cpp:392-421).  The reference
        takes the shortest period of an empty body list when nothing was
        synchronised; here the list is populated first."""
        st = self.sc.settings
        pre = dataclasses.replace(main)
        pre.length = st.start - pre.time
        pre.output = main.output if pre.forward() else -main.output
        pre.h_did = 0.0
        if not self.body_list:
            self._populate(pre.time)
        sx.check_type_order(self.body_list)
        pre.h_next = sx.first_step(self.body_list, pre.length, 50.0)
        self._integrate(pre)

    def _main_integration(self, main: TimeLine):
        """Simulator::MainIntegration (Simulator.cpp:423-447)."""
        if not self.body_list:
            self._populate(main.time)
        sx.check_type_order(self.body_list)
        main.h_did = 0.0
        main.h_next = sx.first_step(self.body_list, main.length, 50000.0)
        self._integrate(main)

    def run(self) -> dict:
        st, sc = self.sc.settings, self.sc
        t_wall = _time.time()
        main = TimeLine(time=sc.time0, length=st.length, output=st.output, save=sc.time0)
        if sc.n_distinct_start_times > 1:
            self._log("The synchronization phase of the simulation begins")
            self._synchronization(main)
        if st.start_defined:
            self._log("The pre-integration phase of the simulation begins")
            self._pre_integration(main)
        if st.length != 0.0:
            self._log("The main-integration phase of the simulation begins")
            self._main_integration(main)
        return dict(steps=self.steps, rejected=self.rejected, phases=self.phases, time=main.time,
                    affairs=self.affairs, seconds=_time.time() - t_wall)


def run_file(path: str, directory: str | None = None, device: int = 0, precision: int = abi.PRECISION_FP64) -> dict:
    """Read a scenario file and run it on the device; the output files go next
    to the scenario file (as the reference writes them) unless a directory is given."""
    from . import scenario_xml
    sc = scenario_xml.load(path)
    return Simulator(sc, directory=directory, device=device, precision=precision).run()


def main(argv=None) -> int:
    """The reference program's command line (Solaris.cpp:25-75): -i <input
    file> runs the scenario on the device and writes the output files next
    to it; -h prints the usage."""
    import sys
    args = list(sys.argv[1:] if argv is None else argv)
    usage = "Usage is -i <infile>\n"
    if not args or args[0] in ("-h", "--help"):
        sys.stdout.write("Solaris:\n" + usage)
        return 0 if args else 1
    if args[0] != "-i" or len(args) != 2:
        sys.stderr.write("Invalid argument.\n" + usage)
        return 1
    try:
        r = run_file(args[1])
    except ScenarioError as e:
        sys.stderr.write(f"{e}\n")
        return 1
    sys.stderr.write(f"{r['steps']} steps to t = {r['time']} day, {len(r['affairs'])} events, "
                     f"{r['seconds']:.2f} s\n")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

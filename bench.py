#!/usr/bin/env python
"""Headline benchmark: pair interactions per second of the force-and-integrate
path, split precision (<= 1e-12 relative acceleration error) beside plain FP64.

Workload: 1 star + 65,535 self-gravitating bodies (equal mass 1e-10 Msun,
a ~ U(0.5, 5) AU, e, i Rayleigh 0.02), seeded synthetic; one step is one
RungeKutta4 driver call = 4 force evaluations of 65,535 x 65,534 direct pairs
plus the Kepler terms, and the RK4 stage sums, all on the device.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  With N > 1 (torchrun, or started by this
script itself) the system's sinks are partitioned over the GPUs, with one
all-gather of positions per RK4 stage (strong scaling), and the ensemble's
systems are split over them.
"""
from __future__ import annotations

import argparse
import csv
import hashlib
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair interactions/s, FP64 vs split-precision at <=1e-12 rel. accel error"
UNIT = "pair interactions/s"
FLOP_PER_PAIR = 20  # conventional FP64 operation count of one pair interaction
N_BODIES = 65536
WORKLOAD = ("1 star + 65,535 self-gravitating bodies (1e-10 Msun, a~U(0.5,5) AU, e,i Rayleigh 0.02); "
            "one RK4 step = 4 force evaluations + stage sums")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_BODIES, help=argparse.SUPPRESS)
    ap.add_argument("--skip-ensemble", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--drift-steps", type=int, default=0,
                    help="instead of the benchmark line: energy drift of each form over this many RK4 steps")
    ap.add_argument("--drift-forms", default="split_ff,split,fp64",
                    help="forms for --drift-steps (comma-separated: split_ff, split, fp64)")
    return ap.parse_args()


def run_drift(args, local):
    """The 65,536-body workload integrated for --drift-steps RK4 steps in each
    form from the same initial state: the relative energy drift |E - E0| / |E0|
    (sol_integrals) every tenth of the run, the wall time, and the final state's
    maximum / RMS relative acceleration error against the FP64 form evaluated
    at that state.  One JSON line."""
    import numpy as np

    from solaris_gb300 import abi
    forms = {"split_ff": abi.PRECISION_SPLIT_FF, "split": abi.PRECISION_SPLIT, "fp64": abi.PRECISION_FP64}
    unknown = [f for f in args.drift_forms.split(",") if f not in forms]
    if unknown:
        raise SystemExit(f"bench.py: unknown --drift-forms {','.join(unknown)} (split_ff, split, fp64)")
    import torch

    from solaris_gb300 import build, engine, scenarios
    build.build()
    torch.cuda.set_device(local)
    s = scenarios.config3(n=args.n)
    n_steps = args.drift_steps
    every = max(1, n_steps // 10)
    out = {"workload": WORKLOAD, "n_bodies": s.n, "integrator": "RungeKutta4", "h": s.h0, "steps": n_steps,
           "forms": {}}
    with engine.Context(s, device=local) as ctx:
        for name in args.drift_forms.split(","):
            ctx.set_precision(forms[name])
            ctx.set_state(s.y0)
            tl = abi.SolTimeLine(0.0, s.h0, 0.0)
            e0 = ctx.integrals()[15]
            drift, done = [], 0
            t0 = time.perf_counter()
            while done < n_steps:
                k = min(every, n_steps - done)
                ctx.driver(abi.RUNGE_KUTTA4, 0, 0, k, time_line=tl)
                done += k
                drift.append(abs((ctx.integrals()[15] - e0) / e0))
            wall = time.perf_counter() - t0
            y = ctx.get_state()
            a, *_ = ctx.accel(0.0, y)
            ctx.set_precision(abi.PRECISION_FP64)
            a64, *_ = ctx.accel(0.0, y)
            A, B = a.reshape(-1, 6)[1:, 3:], a64.reshape(-1, 6)[1:, 3:]
            rel = np.linalg.norm(A - B, axis=1) / np.linalg.norm(B, axis=1)
            out["forms"][name] = {"relative_energy_drift": drift, "every": every, "wall_s": wall,
                                  "final_max_rel_accel_err": float(rel.max()),
                                  "final_rms_rel_accel_err": float(np.sqrt(np.mean(rel ** 2))),
                                  "final_state_sha": hashlib.sha256(y.tobytes()).hexdigest()[:16]}
    print(json.dumps({"drift": out}))


# ---- clocks --------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.file.read())) if len(r) >= 9]
        os.unlink(self.file.name)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        under = [v for v in sm if v > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(under) if under else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


# ---- CPU baseline ----------------------------------------------------------------
def cpu_sample(system, n_sinks: int, threads: int):
    """GravityAC of the oracle port on sinks [1, 1 + n_sinks) of the workload."""
    import oracle
    o = oracle.Oracle(system)
    t0 = time.perf_counter()
    _, pairs = o.gravity_sample(system.y0, 1, 1 + n_sinks, threads)
    dt = time.perf_counter() - t0
    return pairs / dt, pairs, dt


def run_reference(args, rank, world):
    """The reference's CPU path (the oracle port of GravityAC, all host threads)
    on the same workload and metric."""
    from solaris_gb300 import replicas, scenarios
    if rank != 0:
        replicas.finalize()
        return
    s = scenarios.config3(n=args.n)
    threads = os.cpu_count() or 1
    n_sinks = min(s.n - 1, 4096 * threads)
    for _ in range(max(args.warmup, 0)):
        cpu_sample(s, min(n_sinks, 256 * threads), threads)
    pairs_total, t_total = 0, 0.0
    for _ in range(args.steps):
        _, pairs, dt = cpu_sample(s, n_sinks, threads)
        pairs_total += pairs
        t_total += dt
    v = pairs_total / t_total
    sample = f"GravityAC on sinks [1, {1 + n_sinks}) x all sources per step, {threads} OpenMP threads"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_bodies": s.n, "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    replicas.finalize()


def profile_figures(names=("pair_kernels_65536.md", "k_pairs_ff_65536.md")):
    """`key: value` lines of the committed ncu summaries (DRAM bytes per
    launch, instructions per pair measured at the bench size); later files
    override earlier ones."""
    out = {}
    for name in names:
        p = os.path.join(ROOT, "profiles", name)
        if os.path.exists(p):
            out.update(_figures(p))
    return out


def _figures(p):
    out = {}
    for line in open(p):
        line = line.strip().lstrip("-* ")
        if ":" in line and line.split(":", 1)[0].replace("_", "").isalnum():
            k, v = line.split(":", 1)
            try:
                out[k.strip()] = float(v.strip().split()[0].replace(",", ""))
            except (ValueError, IndexError):
                pass
    return out


FF_FP32_OPS_PER_PAIR = 106.5
# The FP32 pipe completes 128 lane operations per SM cycle (4 sub-partitions x
# 32 lanes; a paired FFMA2 instruction is two).
FP32_LANES_PER_SM_CYCLE = 128.0


def fp32_peak(local, clocks):
    """FP32 lane-operation peak (per second) at the SM clock sampled during the
    timed region, and the probe's measured chains beside it."""
    import torch
    from solaris_gb300 import engine
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    probe = engine.fp32_pipe_rates(local)
    mhz = (clocks or {}).get("sm_mhz") or probe["sm_mhz"] or 2070.0
    peak = FP32_LANES_PER_SM_CYCLE * nsm * mhz * 1e6
    return peak, {"sms": nsm, "sm_mhz": mhz, "lanes_per_sm_cycle": FP32_LANES_PER_SM_CYCLE,
                  "probe_ffma_per_s": probe["ffma"], "probe_ffma2_per_s": probe["ffma2"],
                  "probe_sm_mhz": probe["sm_mhz"],
                  "probe_frac_of_peak": max(probe["ffma"], probe["ffma2"]) /
                  (FP32_LANES_PER_SM_CYCLE * nsm * (probe["sm_mhz"] or mhz) * 1e6)}


def roofline_entry(name, pps, fp64_ops, fp32_ops, peak64, info64, peak32, info32, prof, ms):
    """The dominant kernel's roofline: SPLIT_FF's pair kernel is bound by the
    FP32 pipe, the other forms by the FP64 pipe."""
    traffic = {"traffic": prof.get(f"{name}_dram_bytes_per_launch"),
               "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the pair kernel and its "
                               "k_combine at 65,536 bodies (profiles/pair_kernels_65536.md, "
                               "profiles/k_pairs_ff_65536.md; SPLIT_FF with the caches as the timed step "
                               "leaves them, --cache-control none)",
               "kernel_ms_per_launch": ms}
    if name in fp32_ops:
        return {"bound": "fp32", "kernel": "k_pairs_ff (SPLIT_FF pair kernel) + k_combine",
                "achieved": pps * fp32_ops[name] / 1e9, "peak": peak32 / 1e9, "unit": "Gop/s",
                "frac": pps * fp32_ops[name] / peak32, **traffic, "fp32_ops_per_pair": fp32_ops[name],
                "fp64_instructions_per_pair_ncu": prof.get(f"{name}_fp64_instructions_per_pair"),
                "peak_source": "FP32 pipe, 128 lane operations per SM cycle x SMs x the SM clock sampled during "
                               "the timed region (probe of FFMA / FFMA2 chains beside it)",
                "peak_detail": info32}
    return {"bound": "fp64", "kernel": f"k_pairs<{name.upper()}> (pair kernel)",
            "achieved": pps * fp64_ops[name] / 1e9, "peak": peak64 / 1e9, "unit": "Gop/s",
            "frac": pps * fp64_ops[name] / peak64, **traffic, "fp64_instructions_per_pair": fp64_ops[name],
            "peak_source": "FP64 pipe issue rate, 2 thread instructions per SM cycle (ncu peak_sustained 1/16 warp "
                           "instruction), x SMs x the SM clock sampled during the timed region",
            "peak_detail": info64}


# The FP64 pipe issues 1/16 warp instruction per SM cycle (ncu
# sm__inst_executed_pipe_fp64.avg.peak_sustained = 0.0625 on the GB300):
# 2 thread instructions per SM per cycle.
FP64_LANES_PER_SM_CYCLE = 2.0


def fp64_peak(local, clocks):
    """FP64 instruction peak (thread instructions/s) at the SM clock sampled
    during the timed region, and the probe's measured chains beside it."""
    import torch
    from solaris_gb300 import engine
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    probe = engine.fp64_pipe_rates(local)
    mhz = (clocks or {}).get("sm_mhz") or probe["sm_mhz"] or 2070.0
    peak = FP64_LANES_PER_SM_CYCLE * nsm * mhz * 1e6
    return peak, {"sms": nsm, "sm_mhz": mhz, "lanes_per_sm_cycle": FP64_LANES_PER_SM_CYCLE,
                  "probe_dfma_per_s": probe["dfma"], "probe_dadd_per_s": probe["dadd"],
                  "probe_dmul_per_s": probe["dmul"], "probe_sm_mhz": probe["sm_mhz"],
                  "probe_frac_of_peak": max(probe["dfma"], probe["dadd"], probe["dmul"]) /
                  (FP64_LANES_PER_SM_CYCLE * nsm * (probe["sm_mhz"] or mhz) * 1e6)}


def ensemble_section(local):
    """Batched-ensemble figures (4,096 systems of 1 star + 2..12 planets +
    0..512 test particles, adaptive RKF78 eps 1e-10): system-steps/s of the
    persistent ensemble kernel (SPLIT_FF and FP64, launch shape autotuned),
    of serial per-system launches of the single-system path, and of the CPU
    oracle on one core."""
    import oracle
    from solaris_gb300 import abi, engine, scenarios
    systems = scenarios.config4()
    out = {"workload": "4096 systems: 1 star + U{2..12} planets + U{0..512} test particles, RKF78 eps 1e-10",
           "unit": "system-steps/s", "bodies": int(sum(x.n for x in systems))}
    steps = 10
    for name, prec in (("split_ff", abi.PRECISION_SPLIT_FF), ("fp64", abi.PRECISION_FP64)):
        with engine.Ensemble(systems, device=local, precision=prec) as ens:
            ens.set_state([x.y0 for x in systems], [0.0] * len(systems), [x.h0 for x in systems])
            threads, per_sm, _ = ens.autotune(steps=2)
            ens.advance(2)
            t0 = time.perf_counter()
            acc, rej, _ = ens.advance(steps)
            dt = time.perf_counter() - t0
            out[name] = {"value": acc / dt, "accepted": acc, "rejected": rej, "threads_per_system": threads,
                         "systems_per_sm": per_sm}
    k, acc_tot, dt_tot = 16, 0, 0.0
    for x in systems[:k]:
        with engine.Context(x, device=local) as ctx:
            ctx.set_state(x.y0)
            ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, x.h0, 2)
            t0 = time.perf_counter()
            r = ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0.0, x.h0, steps)
            dt_tot += time.perf_counter() - t0
            acc_tot += r["stats"][0]
    out["serial_single_system"] = {"value": acc_tot / dt_tot, "sample_systems": k}
    out["speedup_vs_serial"] = out["split_ff"]["value"] / out["serial_single_system"]["value"]
    k, acc_tot, dt_tot = 8, 0, 0.0
    for x in systems[:k]:
        o = oracle.Oracle(x)
        t0 = time.perf_counter()
        r = o.driver(abi.RUNGE_KUTTA_FEHLBERG78, x.y0, 0.0, x.h0, steps)
        dt_tot += time.perf_counter() - t0
        acc_tot += r["stats"][0]
    out["cpu_port_1_core"] = {"value": acc_tot / dt_tot, "sample_systems": k, "kind": "port", "cores": 1}
    return out


def adjoint_section(local):
    """Discrete adjoint of fixed-step RKF78 on the adjoint workload at its
    full length (1 star + 8 planets + 1,024 planetesimals typed ProtoPlanet,
    h = shortest period / 500, 10^4 steps, a checkpoint every 100): forward
    and backward milliseconds per step, the backward / forward cost ratio
    (bound 4), FP64 and SPLIT_FF forces; the oracle's forward step on one core
    beside it."""
    import numpy as np

    import oracle
    from solaris_gb300 import engine, scenarios
    s = scenarios.config5()
    h, n_steps, every = s.h0 * 100, 10000, 100
    out = {"workload": "1 star + 8 planets + 1,024 ProtoPlanet planetesimals, fixed-step RKF78, "
                       "h = shortest period / 500, 10^4 steps, checkpoint every 100 steps",
           "n_bodies": s.n, "steps": n_steps, "checkpoint_every": every,
           "pairs_per_step": 11 * s.pair_count()}
    rng = np.random.default_rng(1005)
    for name, prec in (("fp64", 0), ("split_ff", 2)):
        with engine.Context(s, device=local, precision=prec) as ctx:
            ctx.adjoint_forward(s.y0, h, 20, 10)  # warm-up
            t0 = time.perf_counter()
            yf = ctx.adjoint_forward(s.y0, h, n_steps, every)
            tf = time.perf_counter() - t0
            target = yf.reshape(-1, 6)[:, :3] + 1e-6 * rng.standard_normal((s.n, 3))
            g = np.zeros_like(yf).reshape(-1, 6)
            g[:, :3] = 2.0 * (yf.reshape(-1, 6)[:, :3] - target)
            t0 = time.perf_counter()
            ctx.adjoint_backward(g.reshape(-1))
            tb = time.perf_counter() - t0
        out[name] = {"forward_s": tf, "backward_s": tb, "forward_ms_per_step": 1e3 * tf / n_steps,
                     "backward_ms_per_step": 1e3 * tb / n_steps, "backward_over_forward": tb / tf,
                     "forward_pairs_per_s": out["pairs_per_step"] * n_steps / tf}
    o = oracle.Oracle(s)
    k = 3
    t0 = time.perf_counter()
    o.rkf78_fixed(s.y0, h, k)
    out["cpu_port_1_core"] = {"forward_ms_per_step": 1e3 * (time.perf_counter() - t0) / k, "kind": "port",
                              "cores": 1, "sample": f"{k} fixed RKF78 steps of the oracle"}
    return out


def config1_full_run(local):
    """The 256-body configuration over its full 1,000 years as the scenario
    file tests/golden/scenarios/config1_1000yr.xml: the device simulator, the
    oracle-driven simulator on one host core (its output files are the
    reference program's byte for byte), and the reference program's own run
    of the file (tests/golden/scenarios/config1_1000yr/summary.json: driver
    calls and force evaluations counted around its unchanged objects, wall
    time on the x86 machine that generated it)."""
    import tempfile

    import oracle
    from solaris_gb300 import scenario_xml, simulator
    xml = os.path.join(ROOT, "tests", "golden", "scenarios", "config1_1000yr.xml")
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "scenarios", "config1_1000yr", "summary.json")))

    def run(backend=None):
        sc = scenario_xml.load(xml)
        with tempfile.TemporaryDirectory() as d:
            kw = {"backend": backend} if backend else {"device": local}
            t0 = time.perf_counter()
            r = simulator.Simulator(sc, directory=d, **kw).run()
            wall = time.perf_counter() - t0
            integ = open(os.path.join(d, "Integrals.dat"), "rb").read()
        e = _energies(integ)
        return {"wall_s": wall, "accepted": r["steps"], "rejected": r["rejected"],
                "steps_per_s": r["steps"] / wall, "events": len(r["affairs"]),
                "ejected_ids": sorted(int(a["id2"]) for a in r["affairs"]),
                "energy_rel_drift": abs((e[-1] - e[0]) / e[0])}

    gpu = run()
    cpu = run(oracle.ScenarioBackend)
    cpu.update(kind="port", cores=1, sample="the full run, oracle-driven simulator (the reference's bytes)")
    want = set(e["id2"] for e in ref["events"])
    return {"workload": "1 star + 2 giants + 253 test particles, RKF78 1e-10, 1000 yr, ejection 15 AU, "
                        "hit-centrum 1 AU (scenario file)",
            "gpu": gpu, "cpu_port_1_core": cpu,
            "reference_program": {k: ref[k] for k in ("accepted", "rejected", "evaluations", "wall_s",
                                                      "energy_rel_drift", "machine")} | {"events": len(want)},
            "ejected_in_common_with_reference": len(want & set(gpu["ejected_ids"])),
            "speedup_vs_cpu_port": cpu["wall_s"] / gpu["wall_s"]}


def _energies(integrals_bytes):
    import struct
    (ln,) = struct.unpack_from("<i", integrals_bytes, 0)
    o, out = 4 + ln, []
    while o < len(integrals_bytes):
        (ne,) = struct.unpack_from("<i", integrals_bytes, o)
        vals = struct.unpack_from(f"<{ne}d", integrals_bytes, o + 4)
        out.append(vals[16])  # time, then the 16 values; the last is the total energy
        o += 4 + 8 * ne
    return out


def small_systems_section(local):
    """The latency-bound configurations at their stated lengths: the 256-body
    configuration (1 star, 2 giants, 253 test particles; adaptive RKF78 eps
    1e-10) over its 1,000 years as a scenario run, and 8,193 bodies with a gas
    nebula (1 star, 2 giants, 8,190 planetesimals with drag; eps 1e-11) for
    10^4 accepted steps, FP64, every driver call of a sequence in one
    cooperative launch of the group driver (k_group_rkf78); the oracle on one
    core beside each."""
    import oracle
    from solaris_gb300 import abi, engine, scenarios
    out = {"config1_256_bodies_1000yr": config1_full_run(local)}
    s, k, kc = scenarios.config2(), 10000, 20
    with engine.Context(s, device=local) as ctx:
        ctx.set_tolerance(s.epsilon)
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        t0 = time.perf_counter()
        r = ctx.driver(abi.RUNGE_KUTTA_FEHLBERG78, 0, 0, k, time_line=tl)
        dt = time.perf_counter() - t0
    acc, rej, evals = r["stats"]
    o = oracle.Oracle(s)
    o.set_eval_flags(abi.EVAL_ALL)
    t0 = time.perf_counter()
    ro = o.driver(abi.RUNGE_KUTTA_FEHLBERG78, s.y0, 0.0, s.h0, kc)
    dtc = time.perf_counter() - t0
    out["config2_8193_bodies_gas_1e4_steps"] = {
        "wall_s": dt, "steps_per_s": acc / dt, "evaluations_per_s": evals / dt,
        "pair_interactions_per_s": evals * s.pair_count() / dt, "body_evaluations_per_s": evals * s.n / dt,
        "accepted": acc, "rejected": rej, "simulated_days": tl.time,
        "cpu_port_1_core": {"steps_per_s": ro["stats"][0] / dtc,
                            "pair_interactions_per_s": ro["stats"][2] * s.pair_count() / dtc,
                            "kind": "port", "cores": 1, "sample": f"the first {kc} driver calls"}}
    return out


# FP64 pipe slots per state element of one RKF78 attempt's elementwise kernels:
# stage r is a0 f0 + ... (2 K_r - 1) then y0 + h acc (2): sum over the 12
# stages of 2 K_r + 1 = 122; the final sum 13, the error estimate 3 adds, 2
# multiplications and a division by 840 (~5 slots) = 10, |e / yscale| a
# division (~5) and the comparison (1) -- 151 in all.
STAGE_FP64_SLOTS = 151


def stage_sums_section(local, hbm_peak_gbs, fp64_peak_ops):
    """Elementwise kernels of an RKF78 attempt (12 stage sums, final sum with
    error estimate and scaled norm), event-timed, at the bench's 65,536 bodies
    (vectors L2-resident) and at 1,048,576 bodies (vectors far larger than
    L2): algorithmic bytes 8 * 6N * 93 per attempt against the HBM copy peak,
    and FP64 pipe slots 151 * 6N against the FP64 peak.  With ~0.2 FP64
    operations per byte against the GB300's 0.075 (505 G FP64 instructions/s
    over 6.7 TB/s), the FP64 pipe is the bound."""
    from solaris_gb300 import engine, scenarios
    out = {"bound": "fp64", "bytes_per_attempt": "8 * 6N * 93", "fp64_slots_per_element": STAGE_FP64_SLOTS,
           "hbm_peak_gbs": hbm_peak_gbs, "fp64_peak_gops": fp64_peak_ops / 1e9}
    for n in (65536, 1048576):
        s = scenarios.config3(n=n)
        with engine.Context(s, device=local) as ctx:
            ctx.set_state(s.y0)
            ms = ctx.bench_stages(20)
        gbs = 8 * 6 * n * 93 / (ms * 1e-3) / 1e9
        gops = STAGE_FP64_SLOTS * 6 * n / (ms * 1e-3) / 1e9
        out[f"n_{n}"] = {"ms_per_attempt": ms, "achieved_gbs": gbs,
                         "frac_of_hbm_peak": gbs / hbm_peak_gbs if hbm_peak_gbs else None,
                         "achieved_fp64_gops": gops, "frac_of_fp64_peak": gops * 1e9 / fp64_peak_ops}
    return out


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "MEASURED_PEAKS.json"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def relaunch_under_torchrun(args):
    """`bench.py --gpus N` (N > 1) started as a plain process: run it again
    as N ranks of torch.distributed.run on this node."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__), *sys.argv[1:]]
    os.execv(sys.executable, cmd)


def run_sharded(args, rank, world, local):
    """N > 1 GPUs: the one 65,536-body system with its sinks partitioned over
    the ranks (solaris_gb300.sharded: per RK4 stage an all-gather of the
    blocks' positions, each rank's pair kernels over its own sinks); total
    work fixed, so the scaling is strong.  The ensemble's 4,096 systems are
    split over the ranks (no exchange).  value = the system's pair
    interactions per step / the slowest rank's time."""
    import numpy as np
    import torch

    from solaris_gb300 import abi, build, engine, replicas, scenarios, sharded
    build.build()
    torch.cuda.set_device(local)
    s = scenarios.config3(n=args.n)
    pairs_step = 4 * s.pair_count()
    sh = sharded.ShardedRK4(s, device=local, precision=abi.PRECISION_SPLIT_FF)
    stream = sh.be.stream
    l2_flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    sh.set_state(s.y0)
    t = sh.step(0.0, s.h0, args.warmup)
    sampler = ClockSampler(local)
    replicas.barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = engine.kernel_launches()
    ms = 0.0
    for _ in range(args.steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t = sh.step(t, s.h0, 1)
        ev1.record(stream)
        ev1.synchronize()
        ms += ev0.elapsed_time(ev1)
    launches = engine.kernel_launches() - launches0
    torch.cuda.synchronize()
    replicas.barrier()
    clocks = sampler.stop()
    ms_step = replicas.max_over_ranks(ms / args.steps)
    # end to end: the full state from pinned host memory in and back out every step
    y_host = torch.empty(6 * s.n, dtype=torch.float64, pin_memory=True).numpy()
    y_host[:] = sh.get_state()
    ke = max(2, args.steps // 3)
    replicas.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        sh.set_state(y_host)
        t = sh.step(t, s.h0, 1)
        y_host[:] = sh.get_state()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)
    lo, hi = replicas.shard(4096, rank, world)
    systems = scenarios.config4()[lo:hi]
    with engine.Ensemble(systems, device=local, precision=abi.PRECISION_SPLIT_FF) as ens:
        ens.set_state([x.y0 for x in systems], [0.0] * len(systems), [x.h0 for x in systems])
        ens.autotune(steps=2)
        ens.advance(2)
        replicas.barrier()
        t0 = time.perf_counter()
        acc, _, _ = ens.advance(10)
        dt = replicas.max_over_ranks(time.perf_counter() - t0)
    ens_rate = replicas.sum_over_ranks(acc) / dt
    sh.close()
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": pairs_step / (ms_step * 1e-3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64+f32 (split)", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_bodies": s.n, "pairs_per_eval": s.pair_count(), "evals_per_step": 4,
                       "integrator": "RungeKutta4", "precision": "split_ff",
                       "l2": "flushed between timed steps (256 MiB write, outside the events)",
                       "parallelism": f"sinks partitioned over {world} GPUs, positions all-gathered per stage"},
            "e2e": {"value": pairs_step * ke / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * 6 * s.n,
                    "d2h_bytes_per_step": 8 * 6 * s.n, "steps": ke,
                    "api": "solaris_gb300.sharded.ShardedRK4 (host state in and out every step)"},
            "gpu_launches": launches, "clocks": clocks,
            "ensemble": {"value": ens_rate, "unit": "system-steps/s", "systems": 4096,
                         "parallelism": f"systems split over {world} GPUs"}}))
    replicas.finalize()


def main():
    args = parse()
    from solaris_gb300 import replicas
    world_env = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch_under_torchrun(args)
    if world_env > 1 and world_env != args.gpus:
        raise SystemExit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world_env}")
    rank, world, local = replicas.init()
    if args.drift_steps > 0:
        return run_drift(args, local)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        return run_sharded(args, rank, world, local)

    import numpy as np
    import torch

    from solaris_gb300 import abi, build, engine, scenarios
    build.build()
    torch.cuda.set_device(local)
    s = scenarios.config3(n=args.n)
    pairs_eval = s.pair_count()
    pairs_step = 4 * pairs_eval
    ctx = engine.Context(s, device=local, precision=abi.PRECISION_SPLIT)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    l2_flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > 129 MB L2

    def run_steps(precision, k, w, sampler=None):
        ctx.set_precision(precision)
        ctx.set_state(s.y0)
        tl = abi.SolTimeLine(0.0, s.h0, 0.0)
        for _ in range(w):
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
        e_before = ctx.integrals()[15]
        replicas.barrier()
        torch.cuda.synchronize()
        if sampler:
            sampler.start()
        launches0 = engine.kernel_launches()
        ms = 0.0
        t0 = time.perf_counter()
        for _ in range(k):
            l2_flush.zero_()
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            ctx.driver(abi.RUNGE_KUTTA4, 0, 0, 1, time_line=tl)
            ev1.record(stream)
            ev1.synchronize()
            ms += ev0.elapsed_time(ev1)
        wall = time.perf_counter() - t0
        launches = engine.kernel_launches() - launches0
        torch.cuda.synchronize()
        replicas.barrier()
        clocks = sampler.stop() if sampler else None
        e_after = ctx.integrals()[15]
        ms_max = replicas.max_over_ranks(ms)
        return dict(ms_per_step=ms_max / k, wall=wall, launches=launches, clocks=clocks, k=k,
                    energy_drift=abs((e_after - e_before) / e_before), y=ctx.get_state())

    sampler = ClockSampler(local)
    # headline form first (clocks sampled during its timed region), the others beside it
    ff = run_steps(abi.PRECISION_SPLIT_FF, args.steps, args.warmup, sampler)
    k_other = max(2, args.steps // 3)
    split = run_steps(abi.PRECISION_SPLIT, k_other, 1)
    fp64 = run_steps(abi.PRECISION_FP64, k_other, 1)

    # accuracy of both split forms against the FP64 reference form on the final state
    ctx.set_precision(abi.PRECISION_FP64)
    a64, *_ = ctx.accel(0.0, ff["y"])
    acc = {}
    for name, p in (("split_ff", abi.PRECISION_SPLIT_FF), ("split", abi.PRECISION_SPLIT)):
        ctx.set_precision(p)
        asp, *_ = ctx.accel(0.0, ff["y"])
        A, B = asp.reshape(-1, 6)[1:, 3:], a64.reshape(-1, 6)[1:, 3:]
        rel = np.linalg.norm(A - B, axis=1) / np.linalg.norm(B, axis=1)
        acc[name] = (float(rel.max()), float(np.sqrt(np.mean(rel ** 2))))
    ff_ok = acc["split_ff"][0] <= 1e-12
    head, head_name, head_prec = (ff, "split_ff", abi.PRECISION_SPLIT_FF) if ff_ok else \
        (split, "split", abi.PRECISION_SPLIT)

    # dominant kernel: the pair kernel alone, per launch, CUDA events on its stream
    ctx.set_state(s.y0)
    ms_launch = {name: ctx.bench_force(p, reps) for name, p, reps in
                 (("split_ff", abi.PRECISION_SPLIT_FF, 5), ("split", abi.PRECISION_SPLIT, 2),
                  ("fp64", abi.PRECISION_FP64, 2))}
    peak_ops, peak_info = fp64_peak(local, ff["clocks"])  # FP64 thread instructions per second
    peak32, peak32_info = fp32_peak(local, ff["clocks"])  # FP32 lane operations per second
    # FP64 instructions per pair of each form's arithmetic: SPLIT_FF none (its
    # pair runs on the FP32 pipe); SPLIT 12 (displacement 3, r^2 3, the Newton
    # residual 1, G m y^3 and its correction 2, the accumulation 3; the seed's
    # square and cube and the correction's t come from the integer pipe); the
    # reference form 14 in the pair (correctly rounded sqrt and reciprocal by
    # one FMA remainder each, the six term multiplies on the integer pipe) plus
    # the 3 in-order additions
    fp64_ops = {"split_ff": 0, "split": 12, "fp64": 17}
    # SPLIT_FF's pair (k_pairs_ff) runs on the FP32 pipe: FP32 lane operations
    # per pair of its float-float arithmetic (sol_pair.cuh): the displacement
    # from the grid triples 21, r^2 23, G m r^-3 22, the accumulation 40.5
    # (12 per component and step, a 3-operation renormalisation every second)
    fp32_ops = {"split_ff": FF_FP32_OPS_PER_PAIR}
    prof = profile_figures()

    # end to end through the C-ABI: pinned host state in, host state out, every step
    y_host = torch.empty(6 * s.n, dtype=torch.float64, pin_memory=True).numpy()
    y_host[:] = s.y0
    ctx.set_precision(head_prec)
    lib = ctx.lib
    tl = abi.SolTimeLine(0.0, s.h0, 0.0)
    st = abi.SolStepStats()
    import ctypes as C
    ke = max(2, args.steps // 3)
    lib.sol_driver_host(ctx.h, abi.RUNGE_KUTTA4, abi.f64p(y_host), C.byref(tl), 1, C.byref(st))  # warm
    replicas.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        abi.check(lib, lib.sol_driver_host(ctx.h, abi.RUNGE_KUTTA4, abi.f64p(y_host), C.byref(tl), 1, C.byref(st)))
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0)

    n_ranks = world
    rate = lambda r: n_ranks * pairs_step / (r["ms_per_step"] * 1e-3)
    value = rate(head)
    e2e_value = n_ranks * pairs_step * ke / e2e_s
    forms = {}
    for name, r in (("split_ff", ff), ("split", split), ("fp64", fp64)):
        pps = pairs_eval / (ms_launch[name] * 1e-3)
        forms[name] = {"value": rate(r), "unit": UNIT, "ms_per_step": r["ms_per_step"],
                       "kernel_ms_per_launch": ms_launch[name],
                       "fp64_instructions_per_pair": fp64_ops[name],
                       "fp64_instructions_per_pair_ncu": prof.get(f"{name}_fp64_instructions_per_pair"),
                       "fp64_pipe_frac": pps * fp64_ops[name] / peak_ops,
                       "fp32_ops_per_pair": fp32_ops.get(name),
                       "fp32_pipe_frac": pps * fp32_ops[name] / peak32 if name in fp32_ops else None,
                       "conventional_tflops": pps * FLOP_PER_PAIR / 1e12,
                       # the conventional count against the FP64 peak means something only for the
                       # forms whose pair runs on the FP64 pipe; SPLIT_FF's runs on the FP32 pipe
                       "conventional_frac_of_fp64_peak": (pps * FLOP_PER_PAIR / (2.0 * peak_ops)
                                                          if fp64_ops[name] else None),
                       "energy_drift": r["energy_drift"], "steps": r.get("k")}
        if name in acc:
            forms[name]["max_rel_accel_err"], forms[name]["rms_rel_accel_err"] = acc[name]
    pps_head = pairs_eval / (ms_launch[head_name] * 1e-3)
    ensemble = ensemble_section(local) if not args.skip_ensemble else None
    hbm_peak, hbm_src = measured_hbm_peak()
    extra = {}
    if not args.skip_ensemble:
        extra["adjoint"] = adjoint_section(local)
        extra["small_systems"] = small_systems_section(local)
        extra["stage_sums"] = dict(stage_sums_section(local, hbm_peak, peak_ops), hbm_peak_source=hbm_src)
    cpu = None
    if rank == 0:
        n_sinks = 12288
        v, pairs, dt = cpu_sample(s, n_sinks, 1)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"oracle GravityAC, sinks [1, {1 + n_sinks}) x {s.n - 1} sources ({pairs:.3e} pairs, "
                         f"{dt:.1f} s), 1 thread"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32 (split)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_bodies": s.n, "pairs_per_eval": pairs_eval, "evals_per_step": 4,
                   "integrator": "RungeKutta4", "precision": head_name,
                   "l2": "flushed between timed steps (256 MiB write, outside the events)",
                   "parallelism": "single GPU"},
        "forms": forms,
        "split_speedup_vs_fp64": value / forms["fp64"]["value"],
        "accuracy": {"bound": 1e-12, "reference_form": "fp64 (bit-identical to the reference CPU build)",
                     "split_ff_max_rel_accel_err": acc["split_ff"][0], "split_max_rel_accel_err": acc["split"][0],
                     "headline_within_bound": acc[head_name][0] <= 1e-12},
        "roofline": roofline_entry(head_name, pps_head, fp64_ops, fp32_ops, peak_ops, peak_info, peak32,
                                   peak32_info, prof, ms_launch[head_name]),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * 6 * s.n, "d2h_bytes_per_step": 8 * 6 * s.n,
                "steps": ke, "api": "sol_driver_host (pinned host y0 in/out)"},
        "gpu_launches": head["launches"],
        "clocks": head["clocks"],
        "ensemble": ensemble,
        **extra,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    replicas.finalize()


if __name__ == "__main__":
    main()

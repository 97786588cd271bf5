"""bench.py's reference arm (the reference's CPU path, timed on the host
cores) keeps the benchmark line's contract: one JSON line on rank 0 with the
metric, unit and config of the GPU arm, a cpu_baseline describing the run
and an e2e entry without device copies; under torchrun the other ranks exit
0 without work."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "3"]


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(line):
    assert line["impl"] == "reference"
    assert line["unit"] == "pair interactions/s" and line["value"] > 0
    assert line["steps"] == 1 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_reference_arm_under_torchrun_two_ranks():
    pytest.importorskip("torch.distributed.run")
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29561", "bench.py", "--gpus", "2", *ARGS]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1  # rank 0 alone prints
    _check(lines[0])
    assert lines[0]["n_gpus"] == 2


def test_gpus_flag_without_torchrun_starts_the_ranks_itself():
    """`bench.py --gpus 2` as a plain process runs again as two ranks of
    torch.distributed.run (rank 0 prints the one line with n_gpus 2)."""
    pytest.importorskip("torch.distributed.run")
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--gpus", "2", *ARGS], cwd=ROOT, capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1 and lines[0]["n_gpus"] == 2
    _check(lines[0])


def test_gpus_flag_must_match_the_world_size():
    env = dict(os.environ, WORLD_SIZE="3", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--gpus", "2", *ARGS], cwd=ROOT, capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode != 0
    assert "WORLD_SIZE=3" in r.stderr


def test_drift_mode_rejects_unknown_forms_before_any_device_work():
    r = subprocess.run([sys.executable, "bench.py", "--drift-steps", "10", "--drift-forms", "split_ff,fp32"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode != 0
    assert "unknown --drift-forms fp32" in r.stderr

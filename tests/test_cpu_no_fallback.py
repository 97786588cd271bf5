"""The product has no CPU fallback: without a GPU the engine, the simulator's
device backend and the ensemble raise instead of computing elsewhere, and a
missing library raises at load.  (On a machine with a GPU the first three
are skipped.)"""
import pytest

from solaris_gb300 import abi, engine, scenarios
from solaris_gb300 import scenario_xml as sx
from solaris_gb300 import simulator as sim
from scenario_files import xml_path


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


needs_no_gpu = pytest.mark.skipif(_gpu_present(), reason="a GPU is present")


@needs_no_gpu
def test_engine_context_raises_without_gpu():
    s = scenarios.config1()
    with pytest.raises(abi.SolError, match="CUDA"):
        with engine.Context(s) as ctx:
            ctx.accel(0.0, s.y0)


@needs_no_gpu
def test_ensemble_raises_without_gpu():
    systems = scenarios.config4(n_systems=2)
    with pytest.raises(abi.SolError, match="CUDA"):
        with engine.Ensemble(systems) as ens:
            ens.advance(1)


@needs_no_gpu
def test_simulator_device_backend_raises_without_gpu(tmp_path):
    sc = sx.load(xml_path("ejection_rkf78"))
    with pytest.raises(abi.SolError, match="CUDA"):
        sim.Simulator(sc, directory=str(tmp_path)).run()
    # nothing was integrated: no phases record beyond what the failed start wrote
    phases = tmp_path / sc.settings.phases
    assert not phases.exists() or phases.stat().st_size == 0


def test_missing_library_raises(tmp_path):
    with pytest.raises(RuntimeError, match="not built"):
        abi.load_library(str(tmp_path / "libsolaris_gb300.so"))

"""bench.py's host-side pieces that need no GPU.

- The clock record of the timed region: median SM clock, maximum clock and the throttle reasons
  seen, from nvidia-smi's CSV samples. A run that saw a thermal or hardware slowdown must say
  so in its JSON line.
- The config block of the JSON line: it names the workload and its sizes, and no model keys.
"""
import importlib.util
import os
import subprocess
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_contract", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _FinishedProcess:
    """Stands in for the nvidia-smi process once its samples are written."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _summary(tmp_path, lines):
    b = _bench()
    sampler = b.ClockSampler(0)
    path = tmp_path / "clocks.csv"
    path.write_text("".join(line + "\n" for line in lines))
    sampler.proc = _FinishedProcess()
    sampler.path = str(path)
    out = sampler.stop()
    assert not path.exists()  # the sample file is removed
    return out


IDLE = "0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"


def test_clock_summary_median_max_and_power_cap(tmp_path):
    capped = "0, 1950, 2070, 1395.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    out = _summary(tmp_path, [IDLE, capped, IDLE, "not a sample line"])
    assert out == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_summary_reports_thermal_and_hardware_slowdowns(tmp_path):
    hot = "0, 1600, 2070, 1400.0, 0x0000000000000048, Active, Not Active, Active, Not Active"
    hw_thermal = "0, 1500, 2070, 1400.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    out = _summary(tmp_path, [IDLE, hot, hw_thermal])
    assert out["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert out["sm_mhz"] == 1600.0 and out["samples"] == 3


def test_clock_summary_without_samples(tmp_path):
    assert _summary(tmp_path, []) is None


def test_clock_sampler_without_nvidia_smi(monkeypatch):
    b = _bench()

    def missing(*args, **kwargs):
        raise FileNotFoundError("nvidia-smi")

    monkeypatch.setattr(subprocess, "Popen", missing)
    sampler = b.ClockSampler(0)
    sampler.start()
    assert sampler.path is None  # the sample file is not left behind
    assert sampler.stop() is None


def test_config_block_names_the_workload():
    b = _bench()
    one = b.config_json(types.SimpleNamespace(precision="f64", mode="fast", gpus=1), 4096000)
    assert one["workload"] == "sph_lattice_3d" and one["particles"] == 4096000
    assert one["precision"] == "f64" and one["arith"] == "fast" and one["parallelism"] == "single GPU"
    assert not {"model", "global_batch", "seq_len"} & set(one)
    two = b.config_json(types.SimpleNamespace(precision="f64", mode="fast", gpus=2), 4096000)
    assert two["parallelism"] == "replicas"

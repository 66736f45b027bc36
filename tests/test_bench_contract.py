"""bench.py's reference arm (the CPU restatement on the host cores) prints one JSON line with the keys
the benchmark contract names."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(600)
def test_reference_arm_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--n", "128"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["warmup"] >= 3 and d["steps"] == 1
    assert d["value"] > 0 and d["unit"] == "GFLOP/s" and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert "workload" in d["config"] and d["config"]["workload"].startswith("128^3")


@pytest.mark.timeout(120)
def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun with N > 1, ranks other than 0 leave the reference arm at once with status 0 and
    print nothing; rank 0 alone runs and prints the line."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, cwd=ROOT, env=env,
                       timeout=120)
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_clock_sampler_parses_reasons_and_median():
    """The clock record of the timed region: median SM clock under load, the maximum, and every throttle reason
    seen active (nvidia-smi csv, noheader, nounits)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_clocks", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class _Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s = bench.ClockSampler("0")
    s.proc = _Done()
    s.lines = [
        "0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1100.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2010, 2070, 1200.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    r = s.stop()
    assert r["sm_mhz"] == 1980 and r["sm_max_mhz"] == 2070 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    s.lines.append("0, 1500, 2070, 1300.0, 0x8, Active, Not Active, Active, Not Active")
    r = s.stop()
    assert r["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]

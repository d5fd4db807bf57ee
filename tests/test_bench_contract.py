"""The reference arm of bench.py (the CPU implementation of the path, timed
on the host cores) prints one JSON line with the keys of the bench contract;
no GPU needed. The GPU arm's line is checked where it runs."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--workload", "plain2d"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "frames/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] >= 3 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and "32 elements" in d["config"]["workload"]
    assert "p50" in d["latency_ms"] and "p99" in d["latency_ms"]


def _fake_smi(tmp_path, line, delay_s, period_s=0.05):
    """A stand-in nvidia-smi on PATH: after `delay_s` it prints `line` every
    `period_s`, as the real tool does under -lms."""
    d = tmp_path / f"bin{period_s}"
    d.mkdir()
    f = d / "nvidia-smi"
    f.write_text(f"#!/bin/bash\nsleep {delay_s}\nwhile true; do echo '{line}'; sleep {period_s}; done\n")
    f.chmod(0o755)
    return str(d)


def test_clock_sampler_waits_for_its_first_sample(tmp_path, monkeypatch):
    """The sampler starts before the timed region and waits for the tool's
    first sample, so that a region of a few hundred ms holds several samples;
    a region shorter than the interval takes the first sample after it
    (in_region 0). Throttle reasons reported Active are listed."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, "1900, 2070, 600.0, Not Active, Not Active, Not Active, Active", 0.3)
                       + os.pathsep + os.environ["PATH"])
    c = bench.ClockSampler(0)
    t0 = time.time()
    c.start()
    assert time.time() - t0 >= 0.25          # waited for the first sample
    time.sleep(0.4)
    r = c.stop()
    assert r["in_region"] >= 3 and r["samples"] == r["in_region"]
    assert r["sm_mhz"] == 1900 and r["sm_max_mhz"] == 2070 and r["reasons"] == ["sw_power_cap"]
    # A region far shorter than the tool's period: the next sample, flagged.
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, "2070, 2070, 600.0, Not Active, Not Active, Not Active, Not Active",
                                         0.1, period_s=0.6) + os.pathsep + os.environ["PATH"])
    c = bench.ClockSampler(0)
    c.start()
    r = c.stop()
    assert r["in_region"] == 0 and r["samples"] == 1 and r["reasons"] == []

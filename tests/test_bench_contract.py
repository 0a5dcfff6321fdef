"""bench.py's output contract on the CPU: the reference arm prints one JSON
line with the keys of the default line, the GPU arm fails loudly without a
GPU (no CPU fallback), and the clock samples taken during the timed region
are summarised as the clocks key."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config")


def _bench(*args, timeout=300):
    return subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_line():
    p = _bench("--impl", "reference", "--steps", "1", "--warmup", "0")
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["metric"] == "frags/s" and line["unit"] == "frags/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["config"]["workload"] == "fill_stress_1080p_100k_gouraud"
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_gpu_arm_fails_loudly_without_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    p = _bench("--steps", "1", "--warmup", "1")
    assert p.returncode != 0
    assert not [l for l in p.stdout.splitlines() if l.startswith("{")]


def test_clock_samples_parsed():
    """The clocks key: median SM clock, the maximum, and the throttle reasons
    seen active, from nvidia-smi's CSV samples (here a stand-in process)."""
    sys.path.insert(0, ROOT)
    import bench
    csv = "\n".join([
        "0, 2070, 2070, 812.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1398.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2055, 2070, 1200.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, [N/A], 2070, 0.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ])

    class Proc:
        def terminate(self):
            pass

        def communicate(self, timeout=None):
            return csv, None

    c = bench.Clocks(0)
    c.p = Proc()
    r = c.stop()
    assert r == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert bench.Clocks(0).stop() is None  # never started

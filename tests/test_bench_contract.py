"""The benchmark's reference arm on the CPU: one JSON line with the contract's
keys, the workload of the GPU arm (at a small scale here), and its own
cpu_baseline / e2e records; and the clock summary parser."""

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--scale", "0.005",
                          "--steps", "3", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["unit"] == "px/s"
    assert d["steps"] == 3 and d["warmup"] == 1 and d["value"] > 0
    assert d["config"]["workload"].startswith("large_fill") and d["config"]["scale"] == 0.005
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 2
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "px/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_clock_summary_flags_throttle_reasons(tmp_path):
    sys.path.insert(0, str(ROOT))
    import bench

    c = bench.Clocks(0)
    c.path = tmp_path / "clocks.csv"
    c.path.write_text("2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                      "1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n"
                      "2070, 2070, 1200.5, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                      "garbage line\n")
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


@pytest.mark.parametrize("n", [0])
def test_empty_clock_file(tmp_path, n):
    sys.path.insert(0, str(ROOT))
    import bench

    c = bench.Clocks(0)
    c.path = tmp_path / "none.csv"
    s = c.summary()
    assert s["samples"] == n and s["sm_mhz"] is None

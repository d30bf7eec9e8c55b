"""bench.py's clock sampler on CPU, against a fake nvidia-smi on PATH: only the
samples of the timed region (plus the one after it) are summarised, throttle
reasons are parsed, and a refused short period falls back to 200 ms."""
import os
import sys
import time
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

# Prints one CSV line per period. The first line (before the timed region
# starts) reports a low idle clock, the later ones the loaded clock with
# sw_power_cap active. With REFUSE_SHORT set it exits 1 for periods below 100 ms.
FAKE = r"""#!/bin/bash
p=200
args=("$@")
for ((i=0;i<${#args[@]};i++)); do
  if [ "${args[$i]}" = "-lms" ]; then p=${args[$((i+1))]}; fi
done
if [ -n "$REFUSE_SHORT" ] && [ "$p" -lt 100 ]; then echo "bad period" >&2; exit 1; fi
s=$(printf '0.%03d' "$p")
echo "345, 2070, 150.0, 0x0, Not Active, Not Active, Not Active, Not Active"
while true; do
  sleep "$s"
  echo "2070, 2070, 900.0, 0x4, Not Active, Not Active, Not Active, Active"
done
"""


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    f = tmp_path / "nvidia-smi"
    f.write_text(FAKE)
    f.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    sys.path.insert(0, str(ROOT))
    import bench
    return bench


def test_region_samples_only(fake_smi):
    with fake_smi.ClockSampler(0) as clk:
        time.sleep(0.3)
    s = clk.summary()
    assert s["period_ms"] == 50
    assert s["samples"] >= 3
    assert s["sm_mhz"] == 2070.0  # the idle line printed before the region is left out
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_refused_period_falls_back(fake_smi, monkeypatch):
    monkeypatch.setenv("REFUSE_SHORT", "1")
    with fake_smi.ClockSampler(0) as clk:
        time.sleep(0.5)
    s = clk.summary()
    assert s["period_ms"] == 200
    assert s["samples"] >= 2
    assert s["sm_mhz"] == 2070.0


def test_missing_tool(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    sys.path.insert(0, str(ROOT))
    import bench
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary()["samples"] == 0

"""Both arms of bench.py time the same window of the same run.

`--impl reference` computes the state at the first step of the other arm's
timed window with the engine (untimed set-up), then times copies of the CPU
restatement over the following steps; the engine arm times the same steps.
Config 0's deck keeps this to seconds.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _line(args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_times_the_engine_arms_window():
    common = ["--workload", "c0", "--spinup", "60", "--warmup", "3", "--steps", "4"]
    ref = _line(["--impl", "reference", "--ref-copies", "2"] + common)
    ours = _line(common + ["--no-e2e", "--cpu-seconds", "2"])
    assert ref["impl"] == "reference"
    assert ref["config"]["window_start_step"] == ours["config"]["window_start_step"] == 63
    assert ref["steps"] == ours["steps"] == 4
    assert "the other arm's timed window" in ref["config"]["window"]
    assert ref["cpu_baseline"]["cores"] == 2 and ref["value"] > 0
    assert ref["metric"] == ours["metric"] and ref["unit"] == ours["unit"]

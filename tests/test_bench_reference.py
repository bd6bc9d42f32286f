"""bench.py's reference arm on the CPU: the JSON line the driver reads.

`--impl reference` times the CPU restatement of the reference (the oracle,
single thread) on the workload's deck; its line carries the common keys plus
`impl`, a `cpu_baseline` describing the run (copies of the single-thread
run, one per host core) and an `e2e` object with no transfers. Config 0's
small deck keeps the run to a few seconds.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c0",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "voxel-updates/s" and d["unit"] == "voxel-updates/s"
    assert d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 5
    assert d["config"]["workload"] == "c0"
    cb = d["cpu_baseline"]
    # one single-thread copy per host core (within the memory cap); the value
    # is their summed throughput
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert "copies" in cb["sample"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_ensemble_json_line():
    """Config 3's reference arm: copies of the CPU restatement on the first
    realisations, runs/s from their completed fractions."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c3",
                        "--ref-seconds", "2", "--realisations", "4", "--ref-copies", "2"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "runs/s" and d["unit"] == "runs/s"
    assert d["value"] > 0 and d["steps"] > 0
    assert d["cpu_baseline"]["cores"] == 2 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]


def test_track_steps_formula():
    """One-layer single tracks run Nsd - 1 loop iterations (Nsd laser points,
    Grid.C:83); realisation 1 of config 3 ran 672 on the GPU."""
    import tempfile

    sys.path.insert(0, ROOT)
    import bench
    from amcafe_gb300.ensemble import make_decks

    with tempfile.TemporaryDirectory() as d:
        decks = make_decks(d, n=1, sides=(96, 192), host_seed=bench.ENSEMBLE_HOST_SEED)
        assert bench._track_steps(decks[0]) == 672

"""GPU against the oracle at config-1 size (512x256x128 voxels, 16.8 M cells).

The oracle cannot run config 1 from the start in test time, so the GPU state at
a step (fields, grain table, laser and layer counters, genlayer engine state)
is handed to the oracle, both advance the same number of steps, and the
results must agree: integer fields bit-exact, floats within 1e-12 relative.
Windows: in the first track (step 300), around the run's first capture event
with a negative time (steps 341-344: the event at step 343 shrinks the front's
extents and clamps 11 of them at zero, VoxelsCA.C:511-516, which the keyed
event loop handles by forcing exact evaluations) and at the benchmark's window
(step 2000, four tracks into the first layers).
"""
import os

import numpy as np
import pytest

import cafe_oracle as orc
from _compare import compare_states

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
C1 = os.path.join(ROOT, "amcafe_gb300", "decks", "c1.in")
WINDOW = 6


def _compare_window(sim, where, n=WINDOW):
    info = sim.info()
    st = sim.state()
    cth = sim.ctheta()
    neg0 = sim.stats()["negative_dt"]
    ost, _, ostats = orc.run_window(C1, info, st, cth, n, libm=orc.LIBM_CR)
    for _ in range(n):
        sim.step()
    got = sim.state()
    compare_states(got, ost, where=where)
    assert ostats["steps"] == n, ostats
    assert sim.info()["nGrain"] == ostats["nGrain"], where
    assert sim.stats()["negative_dt"] - neg0 == ostats["negative_dt"], where
    return ostats


def test_config1_windows_match_oracle():
    from amcafe_gb300 import Simulation

    sim = Simulation(C1, device=0)
    sim.InitializeVoxels()
    sim.begin()
    sim.run(300)
    _compare_window(sim, "config 1, steps 300-%d" % (300 + WINDOW))
    sim.run(341 - 300 - WINDOW)
    ostats = _compare_window(sim, "config 1, steps 341-344", n=3)
    assert ostats["negative_dt"] >= 1 and ostats["clamped"] >= 1, ostats
    sim.run(2000 - 344)
    _compare_window(sim, "config 1, steps 2000-%d" % (2000 + WINDOW))
    stats = sim.stats()
    assert stats["exact_scan_steps"] == 0
    assert stats["events"] > 0 and stats["nucleations"] > 0, stats
    sim.close()


def test_config1_window_across_the_first_layer_change(tmp_path):
    """The oracle and the GPU both step through config 1's first layer change
    (UpdateLaser wraps to the next layer, CleanLayer renumbers the grains,
    AddLayer1 draws the new layer's Voronoi sites and orientations from
    genlayer, main1.C:75-88) from the same state a few steps before it. The
    step of the change is found by running in chunks from checkpoints."""
    from amcafe_gb300 import Simulation

    chunk = 1000
    # the checkpoint (0.7 GB) in memory where the machine offers it
    ckdir = "/dev/shm" if os.path.isdir("/dev/shm") and os.access("/dev/shm", os.W_OK) else str(tmp_path)
    ck = os.path.join(ckdir, "cafe_c1_window_%d.ckpt" % os.getpid())
    sim = Simulation(C1, device=0)
    sim.InitializeVoxels()
    sim.begin()
    layer0 = sim.info()["indlayer"]
    start = 0
    while True:
        sim.checkpoint(ck)
        sim.run(chunk)
        if sim.info()["indlayer"] != layer0:
            break
        start += chunk
        assert start < 40000, "no layer change in config 1's first 40,000 steps"
    # back to the chunk's start, find the step that changes the layer
    sim.restore(ck)
    k = start
    while sim.info()["indlayer"] == layer0:
        sim.step()
        k += 1
    # and back again, to four steps before it
    sim.restore(ck)
    if k - 4 > start:
        sim.run(k - 4 - start)
    assert sim.info()["indlayer"] == layer0
    ng0 = sim.info()["nGrain"]
    _compare_window(sim, "config 1, steps %d-%d (layer change at step %d)" % (k - 3, k + 4, k), n=8)
    info = sim.info()
    assert info["indlayer"] == layer0 + 1
    assert info["nGrain"] != ng0
    sim.close()
    os.unlink(ck)

"""The launch paths of a step give identical results: the step's CUDA graph
(cafe_sim_run and cafe_sim_step) and the ungraphed launches (phase timing on),
on a deck with rotated layers, new layers and output points every 7 steps."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def _deck(tmp_path, outint):
    src = open(os.path.join(DECKS, "layers_rot.in")).read()
    txt = "\n".join(l for l in src.splitlines() if not l.lower().startswith("outint")) + "\noutint %d\n" % outint
    p = tmp_path / ("layers_rot_out%d.in" % outint)
    p.write_text(txt)
    return str(p)


def _final(sim):
    st = sim.state()
    st["build"] = sim.build()
    st["ctheta"] = sim.ctheta()
    i = sim.info()
    st["scalars"] = np.array([i["nGrain"], i["tInd"], i["isp"], i["indlayer"], i["steps"], i["tf_tInd"]])
    return st


@pytest.mark.parametrize("outint", [7, 1000000])
def test_graphed_and_ungraphed_steps_agree(tmp_path, outint):
    from amcafe_gb300 import Simulation

    deck = _deck(tmp_path, outint)
    res = {}
    for mode in ("run", "step", "timed"):
        with Simulation(deck) as sim:
            sim.InitializeVoxels()
            sim.begin()
            if mode == "run":
                sim.run()
            else:
                if mode == "timed":
                    sim.set_timing(True)
                while not sim.step():
                    pass
                sim.CleanLayer()
            res[mode] = _final(sim)
    for mode in ("step", "timed"):
        for k, v in res["run"].items():
            assert np.array_equal(np.asarray(v), np.asarray(res[mode][k]), equal_nan=True), "%s: %s" % (mode, k)


@pytest.mark.parametrize("deck,steps", [("layers_rot.in", 0), ("odd_dims.in", 0)])
def test_fill_helper_block_changes_nothing(deck, steps):
    """The event loop with its new-row fills handed to a second block and
    with one block doing everything (the default) end in identical states."""
    from amcafe_gb300 import Simulation

    out = []
    for helper in (1, 0):
        with Simulation(os.path.join(DECKS, deck), event_fill_helper=helper) as sim:
            sim.InitializeVoxels()
            sim.begin()
            sim.run(steps)
            st = sim.state()
            st["ctheta"] = sim.ctheta()
            st["events"] = sim.stats()["events"]
            out.append(st)
    for k in out[0]:
        a, b = np.asarray(out[0][k]), np.asarray(out[1][k])
        assert np.array_equal(a, b) or (a.dtype.kind == "f" and np.array_equal(np.isnan(a), np.isnan(b)) and
                                         np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])), k

"""Checkpoint and restore (cafe_sim_checkpoint / cafe_sim_restore): a run
resumed from a checkpoint in a fresh handle reaches bit-identical results to
the uninterrupted run; bad files are refused without breaking the handle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def _final(sim):
    st = sim.state()
    st["build"] = sim.build()
    st["ctheta"] = sim.ctheta()
    i = sim.info()
    st["scalars"] = np.array([i["nGrain"], i["tInd"], i["isp"], i["indlayer"], i["steps"], i["done"],
                              i["genlayer_state"], i["inewlayerflg"], i["inewscanflg"], i["ilaserLoc"]])
    st["time"] = np.array([i["time"], i["gth"]])
    return st


@pytest.mark.parametrize("deck,k", [("layers_rot.in", 37), ("layers_rot.in", 90), ("track_nuc.in", 5)])
def test_resume_matches_uninterrupted_run(tmp_path, deck, k):
    from amcafe_gb300 import Simulation

    path = os.path.join(DECKS, deck)
    ck = str(tmp_path / "run.ckpt")
    with Simulation(path) as a:
        a.InitializeVoxels()
        a.begin()
        a.run(k)
        a.checkpoint(ck)
        a.run()
        want = _final(a)
    with Simulation(path) as b:
        b.restore(ck)
        b.run()
        got = _final(b)
    for key in want:
        assert np.array_equal(got[key], want[key], equal_nan=True), key


def test_restore_refuses_bad_files(tmp_path):
    from amcafe_gb300 import Simulation
    from amcafe_gb300._native import CafeError

    ck = str(tmp_path / "a.ckpt")
    with Simulation(os.path.join(DECKS, "track_nuc.in")) as a:
        a.InitializeVoxels()
        a.begin()
        a.run(3)
        a.checkpoint(ck)
    data = open(ck, "rb").read()
    trunc = tmp_path / "t.ckpt"
    trunc.write_bytes(data[: len(data) // 2])
    junk = tmp_path / "j.ckpt"
    junk.write_bytes(b"not a checkpoint" * 10)
    with Simulation(os.path.join(DECKS, "layers_rot.in")) as other:  # another grid
        with pytest.raises(CafeError):
            other.restore(ck)
    with Simulation(os.path.join(DECKS, "track_nuc.in")) as b:
        for bad in (str(trunc), str(junk)):
            with pytest.raises(CafeError):
                b.restore(bad)
        with pytest.raises(CafeError):
            b.step()  # unusable after a failed restore
        b.restore(ck)
        assert b.info()["steps"] == 3
        b.run()

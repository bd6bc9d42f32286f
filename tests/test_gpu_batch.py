"""Batched ensemble (cafe_batch_*): realisations stepped concurrently on one
GPU, by batched launches (one launch per step kernel for all realisations,
autotuned launch shapes) or by host round-robin, give bit-identical results
to their plain runs, and one of them matches the CPU oracle."""
import os

import numpy as np
import pytest

import cafe_oracle as orc

pytestmark = pytest.mark.gpu


def _final(sim):
    st = sim.state()
    st["ctheta"] = sim.ctheta()
    info = sim.info()
    st["nGrain"] = info["nGrain"]
    st["tInd"] = info["tInd"]
    st["steps"] = info["steps"]
    return st


@pytest.mark.parametrize("threads,helper", [(0, 0), (3, 0), (0, 1)])
def test_batch_matches_plain_runs(tmp_path, threads, helper):
    """Uneven realisations (sides 24-40 voxels, their own speeds and seeds)
    end in bit-identical states to their plain runs; with batched launches
    the autotuner tried its candidates during the run and reported them."""
    from amcafe_gb300 import Batch, Simulation
    from amcafe_gb300.ensemble import make_decks

    decks = make_decks(str(tmp_path), n=6, sides=(24, 40), host_seed=5)
    plain = []
    for d in decks:
        with Simulation(d) as sim:
            sim.InitializeVoxels()
            sim.begin()
            sim.run()
            plain.append(_final(sim))
    with Batch(decks, threads=threads, event_fill_helper=helper) as b:
        total = b.run()
        assert total > 0
        for i, want in enumerate(plain):
            assert b.finished(i)
            got = _final(b.sims[i])
            for k in want:
                assert np.array_equal(np.asarray(got[k]), np.asarray(want[k])), "realisation %d: %s" % (i, k)
        rep = b.report()
        if threads == 0:
            # every realisation takes the batched path, so a batch step steps all
            # that are still looping
            assert rep["batch_steps"] == max(p["steps"] for p in plain)
            assert rep["launches"] == 22 * rep["batch_steps"]
            tun = rep["tuning"]
            assert len(tun["candidates"]) == 6 and all(c["ms_per_batch_step"] > 0 for c in tun["candidates"])
            best = min(tun["candidates"], key=lambda c: c["ms_per_batch_step"])
            assert tun["chosen"]["grid_share_sms"] == best["grid_share_sms"]
            assert tun["event_loop_blocks"] == (2 if helper else 1)
        else:
            assert rep["launches"] == 0 and rep["tuning"] is None


def test_batch_steps_a_per_cell_field_on_the_plain_path(tmp_path):
    """A realisation under the Rosenthal field cannot take the batched graph;
    it steps on its own path within the batch and still ends as its plain run."""
    from amcafe_gb300 import Batch, Simulation
    from amcafe_gb300.ensemble import make_decks

    decks = make_decks(str(tmp_path), n=2, sides=(24, 32), host_seed=7)
    ros = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks", "track_ros.in")
    decks = decks + [ros]
    plain = []
    for d in decks:
        with Simulation(d) as sim:
            sim.InitializeVoxels()
            sim.begin()
            sim.run()
            plain.append(_final(sim))
    with Batch(decks) as b:
        b.run()
        for i, want in enumerate(plain):
            got = _final(b.sims[i])
            for k in want:
                assert np.array_equal(np.asarray(got[k]), np.asarray(want[k])), "realisation %d: %s" % (i, k)


def test_batch_realisation_matches_oracle(tmp_path):
    from amcafe_gb300 import Batch
    from amcafe_gb300.ensemble import make_decks

    decks = make_decks(str(tmp_path), n=3, sides=(24, 32), host_seed=11)
    dump = str(tmp_path / "o.bin")
    orc.run(decks[2], dump, libm=orc.LIBM_CR, dump_stride=0)
    last = orc.read_dump(dump)[-1]
    with Batch(decks) as b:
        b.run()
        got = _final(b.sims[2])
    assert got["nGrain"] == last["nGrain"]
    for k in ("gID", "vState", "buildj"):
        assert np.array_equal(got[k], last[k]), k
    assert np.allclose(got["extents"], last["extents"], rtol=1e-12, atol=0, equal_nan=True)

"""Batched ensemble (cafe_batch_*): realisations stepped concurrently on one
GPU give bit-identical results to their plain runs, and one of them matches
the CPU oracle."""
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
    return st


def test_batch_matches_plain_runs(tmp_path):
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
    with Batch(decks, threads=3) as b:
        total = b.run()
        assert total > 0
        for i, want in enumerate(plain):
            assert b.finished(i)
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

"""Host transfers through the C ABI: cafe_sim_download_state / upload_state.

The device keeps vState and BuildjID as bytes and centres as three arrays;
the ABI's host layout is int32 and interleaved x,y,z, converted on the device
in chunks. A round trip must be the identity, and values outside their range
must be rejected (CAFE_E_ARG) without leaving a half-replaced state usable.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def _advanced(deck, nsteps):
    from amcafe_gb300 import Simulation

    sim = Simulation(os.path.join(DECKS, deck), device=0)
    sim.InitializeVoxels()
    sim.begin()
    for _ in range(nsteps):
        sim.step()
    return sim


def test_upload_download_round_trip():
    from amcafe_gb300 import Simulation

    src = _advanced("track_nuc.in", 12)
    st = src.state()
    cth = src.ctheta()
    src.close()
    dst = Simulation(os.path.join(DECKS, "track_nuc.in"), device=0)
    dst.upload_state(st["gID"], st["vState"], st["extents"], st["centroid"], cth)
    back = dst.state()
    for k in ("gID", "vState", "extents", "centroid"):
        assert np.array_equal(back[k], st[k]), k
    assert np.array_equal(dst.ctheta(), cth)
    assert dst.info()["nGrain"] == len(cth) // 4
    dst.close()


def test_upload_rejects_out_of_range_values():
    from amcafe_gb300 import Simulation
    from amcafe_gb300._native import CafeError

    src = _advanced("track_r0.in", 3)
    st = src.state()
    cth = src.ctheta()
    src.close()
    sim = Simulation(os.path.join(DECKS, "track_r0.in"), device=0)
    bad = st["vState"].copy()
    bad[len(bad) // 2] = 7
    with pytest.raises(CafeError, match="vState"):
        sim.upload_state(st["gID"], bad, st["extents"], st["centroid"], cth)
    gbad = st["gID"].copy()
    gbad[0] = len(cth) // 4 + 5
    with pytest.raises(CafeError, match="gID"):
        sim.upload_state(gbad, st["vState"], st["extents"], st["centroid"], cth)
    # the rejected upload left the handle unusable until a valid one
    with pytest.raises(CafeError):
        sim.step()
    sim.upload_state(st["gID"], st["vState"], st["extents"], st["centroid"], cth)
    assert np.array_equal(sim.state()["gID"], st["gID"])
    sim.close()

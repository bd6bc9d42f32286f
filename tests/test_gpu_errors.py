"""Capacity limits and bad calls are reported as errors (never a fault): a
run whose active list outgrows the capacity it was created with stops with
CAFE_E_CAPACITY; calls out of order are refused."""
import os

import pytest

pytestmark = pytest.mark.gpu
DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def test_active_capacity_overflow_is_reported():
    from amcafe_gb300 import Simulation
    from amcafe_gb300._native import CafeError

    with Simulation(os.path.join(DECKS, "track_nuc.in"), active_capacity=64) as sim:
        sim.InitializeVoxels()
        sim.begin()
        with pytest.raises(CafeError, match="capacity"):
            sim.run()


def test_calls_out_of_order_are_refused():
    from amcafe_gb300 import Simulation
    from amcafe_gb300._native import CafeError

    with Simulation(os.path.join(DECKS, "track_nuc.in")) as sim:
        with pytest.raises(CafeError):
            sim.step()  # before InitializeVoxels/begin
        with pytest.raises(CafeError):
            sim.UpdateVoxels()  # before a temperature
        sim.InitializeVoxels()
        with pytest.raises(CafeError):
            sim.InitializeVoxels()  # twice
        sim.begin()
        assert not sim.step()

"""GB300 engine for AMCAFE's per-time-step cellular-automaton path.

`Simulation` holds one realisation (Grid, TempField, BasePlate and VoxelsCA of
AMCAFE's src/src-mpi) on one GPU; its methods are the reference's time-loop
calls (main1.C:60-96). The voxel work runs in libcafe_gpu.so (CUDA, sm_103a).
"""
from .cafe import Batch, Simulation, run_deck  # noqa: F401

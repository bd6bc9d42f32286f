"""The allocation-free CleanLayer entry point against the handle-based one.

cafe_clean_layer_noalloc() exists for callers that cannot go back to the CUDA
allocator during a run (their device memory comes from their own pool, or they
cannot afford the device-wide synchronisation of cudaFree). It must give the
same grain renumbering and orientation table as cafe_sim_clean_layer(). Two
calls are made in a row on different states, so the second also shows that the
shared scratch left by the first call does not leak into its result. Device
buffers here are torch tensors owned by the test (the caller's memory).
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
DECKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "decks")


def _state_before_clean(deck, nsteps):
    from amcafe_gb300 import Simulation

    sim = Simulation(os.path.join(DECKS, deck), device=0)
    sim.InitializeVoxels()
    sim.begin()
    for _ in range(nsteps):
        sim.step()
    st = sim.state()
    cth = sim.ctheta()
    return sim, st["gID"].copy(), cth.copy(), len(cth) // 4


def _clean_noalloc(gid_host, cth_host, ngrain):
    import torch

    from amcafe_gb300._native import check, load

    lib = load()
    gid = torch.from_numpy(gid_host.copy()).cuda()
    cth = torch.from_numpy(cth_host.copy()).cuda()
    out = ctypes.c_int(-1)
    torch.cuda.synchronize()
    check(lib.cafe_clean_layer_noalloc(ctypes.c_void_p(gid.data_ptr()), gid.numel(),
                                       ctypes.c_void_p(cth.data_ptr()), ngrain, ctypes.byref(out), None))
    return gid.cpu().numpy(), cth.cpu().numpy()[: 4 * out.value], out.value


def test_noalloc_clean_layer_matches_handle_entry():
    for deck, nsteps in (("layers_rot.in", 40), ("track_nuc.in", 6)):
        sim, gid, cth, ngrain = _state_before_clean(deck, nsteps)
        got_gid, got_cth, got_n = _clean_noalloc(gid, cth, ngrain)
        sim.CleanLayer()
        want_gid = sim.state()["gID"]
        want_cth = sim.ctheta()
        sim.close()
        assert got_n == len(want_cth) // 4, deck
        assert np.array_equal(got_gid, want_gid), deck
        assert np.array_equal(got_cth, want_cth), deck
        assert got_n < ngrain or np.array_equal(got_gid, gid), deck


def test_noalloc_rejects_oversized_grain_table():
    import torch

    from amcafe_gb300._native import load

    lib = load()
    gid = torch.zeros(8, dtype=torch.int32, device="cuda")
    cth = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = ctypes.c_int(-1)
    rc = lib.cafe_clean_layer_noalloc(ctypes.c_void_p(gid.data_ptr()), 8, ctypes.c_void_p(cth.data_ptr()),
                                      (1 << 18) + 1, ctypes.byref(out), None)
    assert rc == 3  # CAFE_E_CAPACITY
    assert b"CAFE_NOALLOC_MAX_GRAINS" in lib.cafe_last_error()


def test_noalloc_rejects_grain_ids_outside_the_table():
    """A grain ID above ngrain or below zero would index outside the caller's
    grain table; the call must refuse it and change neither array."""
    import torch

    from amcafe_gb300._native import load

    lib = load()
    ngrain = 3
    gid_host = np.array([1, 2, 0, ngrain + 1, 3, -1, 2, 1], dtype=np.int32)
    cth_host = np.arange(4 * ngrain, dtype=np.float64) + 0.5
    gid = torch.from_numpy(gid_host.copy()).cuda()
    cth = torch.from_numpy(cth_host.copy()).cuda()
    out = ctypes.c_int(-1)
    torch.cuda.synchronize()
    rc = lib.cafe_clean_layer_noalloc(ctypes.c_void_p(gid.data_ptr()), gid.numel(), ctypes.c_void_p(cth.data_ptr()),
                                      ngrain, ctypes.byref(out), None)
    assert rc == 1  # CAFE_E_ARG
    assert b"outside 0..ngrain" in lib.cafe_last_error()
    assert out.value == -1
    assert np.array_equal(gid.cpu().numpy(), gid_host)
    assert np.array_equal(cth.cpu().numpy(), cth_host)
    # a valid call right after it still gives the handle-free renumbering
    gid_ok = torch.from_numpy(np.array([0, 3, 3, 1, 0, 1], dtype=np.int32)).cuda()
    check = lib.cafe_clean_layer_noalloc(ctypes.c_void_p(gid_ok.data_ptr()), gid_ok.numel(),
                                         ctypes.c_void_p(cth.data_ptr()), ngrain, ctypes.byref(out), None)
    assert check == 0 and out.value == 2
    assert np.array_equal(gid_ok.cpu().numpy(), np.array([0, 2, 2, 1, 0, 1], dtype=np.int32))
    assert np.array_equal(cth.cpu().numpy()[:8], np.concatenate([cth_host[0:4], cth_host[8:12]]))

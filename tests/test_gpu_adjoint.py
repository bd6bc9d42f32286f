"""Adjoint extension: the hand-written CUDA values and vector-Jacobian products
(csrc/cafe_adjoint.cu) against the FP64 numpy restatement (oracle/adjoint_ref.py)
and central finite differences (h = 1e-6 relative), the adjoint's temperature
against the field the CA stepped under (deck keyword rosenthal), the segment
replay from checkpoints against one logged run, and a calibration that
recovers hidden parameters from the outputs of a CA run at those parameters."""
import os

import numpy as np
import pytest

import adjoint_ref as ref

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECK = os.path.join(ROOT, "amcafe_gb300", "decks", "c4.in")
THETA = np.array([200.0, 0.35, 1.0, 1e-5, 2.0])
# the Rosenthal pool's tail cools below the liquidus (and captures begin)
# about 300 steps into config 4's track; the adjoint window starts after
SPINUP = 400


@pytest.fixture(scope="module")
def run():
    from amcafe_gb300.adjoint import GrowthRun

    r = GrowthRun(DECK, nsteps=96, segment=32, theta=THETA, spinup=SPINUP)
    yield r
    r.close()


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def _fd(f, theta, k, h=1e-6):
    tp, tm = theta.copy(), theta.copy()
    tp[k] *= 1 + h
    tm[k] *= 1 - h
    return (f(tp) - f(tm)) / (2 * h * theta[k])


def test_pool_matches_reference_and_fd(run):
    cot = np.array([0.7, -1.3, 2.1])
    out, g = run.pool(THETA, cot)
    rout, rg = ref.pool(run.setup_dict(), THETA, cot)
    assert _rel(out, rout) < 1e-10
    assert _rel(g[:3], rg[:3]) < 1e-8 and np.all(g[3:] == 0)
    for k in range(3):
        fd = _fd(lambda th: float(cot @ run.pool(th)[0]), THETA, k)
        assert abs(g[k] - fd) <= 1e-6 * abs(fd), (k, g[k], fd)


def test_growth_matches_reference_and_fd(run):
    cells, steps, tau = run.log()
    # negative-time events shrink extents: some growth times are negative
    assert len(cells) > 500 and np.all(np.isfinite(tau)) and np.any(tau > 0)
    G, g = run.growth(THETA, cot=1.0)
    rG, rg = ref.growth(run.setup_dict(), THETA, cells, steps, tau, cot=1.0)
    assert _rel(G, rG) < 1e-10
    assert _rel(g, rg) < 1e-8
    for k in range(5):
        fd = _fd(lambda th: run.growth(th)[0], THETA, k)
        assert abs(g[k] - fd) <= 1e-6 * abs(fd), (k, g[k], fd)


def test_replayed_segments_equal_one_logged_run(run):
    """The checkpointed replay reproduces the log of an uninterrupted run."""
    import torch
    from amcafe_gb300 import Simulation

    cells, steps, tau = run.log()
    sim = Simulation(run.deck)
    sim.InitializeVoxels()
    sim.begin()
    sim.run(run.spinup)
    cap = 1 << 22
    c = torch.empty(cap, dtype=torch.int32, device="cuda")
    s = torch.empty(cap, dtype=torch.int32, device="cuda")
    t = torch.empty(cap, dtype=torch.float64, device="cuda")
    sim._lib.cafe_sim_set_growth_log(sim._h, c.data_ptr(), s.data_ptr(), t.data_ptr(), cap)
    for _ in range(run.nsteps):
        sim.step()
    import ctypes

    n = ctypes.c_longlong(0)
    assert sim._lib.cafe_sim_growth_log_count(sim._h, ctypes.byref(n)) == 0
    n = n.value
    assert np.array_equal(c[:n].cpu().numpy(), cells)
    assert np.array_equal(s[:n].cpu().numpy(), steps)
    assert np.array_equal(t[:n].cpu().numpy(), tau)
    sim.close()


def test_adjoint_temperature_is_the_cas_field(run):
    """The temperature the adjoint differentiates is the one the CA stepped
    under: at the last step, for every cell below the source plane, the FP64
    restatement of the adjoint's field equals the engine's TempCurr to 1e-12
    relative (the same formula, evaluated in another operation order)."""
    run.log()  # replays every segment: the replaying handle ends at the last step
    T_ca = run._sim.temperature()
    su = run.setup_dict()
    nx, ny, nz, dx = su["nx"], su["ny"], su["nz"], su["dx"]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x, y, z = (i.ravel() + .5) * dx, (j.ravel() + .5) * dx, (k.ravel() + .5) * dx
    below = z <= su["z_src"]
    T_adj, _ = ref.temperature(su, run.theta, x[below], y[below], z[below], su["step_final"] * su["dt"])
    assert _rel(T_adj, T_ca[below]) < 1e-12
    assert np.all(T_ca[~below] == su["T0"])
    assert np.sum(T_ca >= su["Tl"]) > 1000  # a melt pool of some thousand cells


def test_objective_gradient(run):
    import torch

    from amcafe_gb300.adjoint import Objective

    th = torch.tensor(THETA, dtype=torch.float64, requires_grad=True)
    out = Objective.apply(th, run)
    w = torch.tensor([1.0, 2.0, 3.0, 1e3], dtype=torch.float64)
    (out * w).sum().backward()
    for k in range(5):
        fd = _fd(lambda x: float((Objective.apply(torch.tensor(x), run) * w).sum()), THETA, k)
        assert abs(float(th.grad[k]) - fd) <= 1e-6 * abs(fd), k


def test_calibration_recovers_parameters_from_a_ca_run():
    """The target is the output of a CA run at the hidden parameters (its own
    temperature field's pool and its own summed growth); starting away from
    them, the calibration fits P and a with that run's event set frozen and
    recovers them."""
    from amcafe_gb300.adjoint import ca_target, calibrate

    hidden = np.array([180.0, 0.4, 1.0, 1.2e-5, 2.0])
    target, run = ca_target(DECK, 96, hidden, spinup=SPINUP)
    try:
        assert run.stats["events"] > 1000
        got, hist = calibrate(run, target, [220.0, 0.4, 1.0, 0.9e-5, 2.0], free=(0, 3))
    finally:
        run.close()
    assert abs(got[0] - 180.0) < 1e-4 * 180.0, (got, hist[-3:])
    assert abs(got[3] - 1.2e-5) < 1e-4 * 1.2e-5, (got, hist[-3:])

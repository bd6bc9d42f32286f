"""The FP64 numpy restatement of the adjoint extension (oracle/adjoint_ref.py):
its hand-written gradients against central finite differences, on CPU."""
import numpy as np

import adjoint_ref as ref

SETUP = dict(k=20.0, alpha=5e-6, T0=300.0, Tl=1609.0, tau_T=10.0, x_start=20e-6, y_src=40e-6, z_src=50e-6,
             dt=6.25e-7, dx=2.5e-6, nx=64, ny=32, nz=24, step_final=60)
THETA = np.array([200.0, 0.35, 1.0, 1e-5, 2.0])


def _fd(f, k, h=1e-6):
    tp, tm = THETA.copy(), THETA.copy()
    tp[k] *= 1 + h
    tm[k] *= 1 - h
    return (f(tp) - f(tm)) / (2 * h * THETA[k])


def test_pool_gradient_matches_finite_differences():
    cot = np.array([0.7, -1.3, 2.1])
    _, g = ref.pool(SETUP, THETA, cot)
    for k in range(3):
        fd = _fd(lambda th: float(cot @ ref.pool(SETUP, th)[0]), k)
        assert abs(g[k] - fd) <= 1e-6 * abs(fd), (k, g[k], fd)


def test_growth_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n = 5000
    cells = rng.integers(0, SETUP["nx"] * SETUP["ny"] * 18, n)
    steps = rng.integers(0, 80, n)
    tau = rng.uniform(0, 1e-7, n)
    _, g = ref.growth(SETUP, THETA, cells, steps, tau, cot=1.0)
    for k in range(5):
        fd = _fd(lambda th: ref.growth(SETUP, th, cells, steps, tau)[0], k)
        assert abs(g[k] - fd) <= 1e-6 * abs(fd), (k, g[k], fd)

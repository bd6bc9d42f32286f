"""FP64 CPU reference of the adjoint extension (test infrastructure only).

Restates in numpy the melt-pool moments and the summed growth that
amcafe_gb300/csrc/cafe_adjoint.cu evaluates (Rosenthal point source with R
clamped below at half a voxel, as the CA's field under the deck keyword
"rosenthal", soft
melt indicator, growth a (T_liq - T)^n tau over a growth log) together with
their gradients with respect to theta = (P, eta, v, a, n), written out by hand
from the formulas; tests compare the GPU kernels with it and with central
finite differences.
"""
import numpy as np


def temperature(setup, theta, x, y, z, t):
    P, eta, v = theta[0], theta[1], theta[2]
    xi = x - (setup["x_start"] + v * t)
    dy, dz = y - setup["y_src"], z - setup["z_src"]
    R = np.sqrt(xi * xi + dy * dy + dz * dz)
    clamped = R < 0.5 * setup["dx"]  # the forward field clamps R at half a voxel
    R = np.where(clamped, 0.5 * setup["dx"], R)
    q = eta * P / (2 * np.pi * setup["k"])
    U = q / R * np.exp(-v * (R + xi) / (2 * setup["alpha"]))
    dv = np.where(clamped, -(R + xi) / (2 * setup["alpha"]) + v * t / (2 * setup["alpha"]),
                  -(R + xi) / (2 * setup["alpha"]) + v * t * (1 + xi / R) / (2 * setup["alpha"]) + xi * t / (R * R))
    dT = np.stack([U / P, U / eta, U * dv])
    return setup["T0"] + U, dT


def _cells(setup):
    nx, ny, nz, dx = setup["nx"], setup["ny"], setup["nz"], setup["dx"]
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x, y, z = (i.ravel() + .5) * dx, (j.ravel() + .5) * dx, (k.ravel() + .5) * dx
    keep = z <= setup["z_src"]
    return x[keep], y[keep], z[keep]


def pool(setup, theta, cot=None):
    x, y, z = _cells(setup)
    T, dT = temperature(setup, theta, x, y, z, setup["step_final"] * setup["dt"])
    m = 1.0 / (1.0 + np.exp(-(T - setup["Tl"]) / setup["tau_T"]))
    d = setup["z_src"] - z
    f = np.stack([np.ones_like(x), x, x * x, y, y * y, d * d])
    S = f @ m
    S0, mx, my = S[0], S[1] / S[0], S[3] / S[0]
    vx, vy, ed = S[2] / S0 - mx * mx, S[4] / S0 - my * my, S[5] / S0
    out = np.array([np.sqrt(12 * vx), np.sqrt(12 * vy), np.sqrt(3 * ed)])
    if cot is None:
        return out, None
    # d out / d S by the chain rule, then d S / d theta = f . dm/dtheta
    gvx, gvy, ged = cot[0] * 6 / out[0], cot[1] * 6 / out[1], cot[2] * 1.5 / out[2]
    w = np.zeros(6)
    w[1], w[2] = gvx * (-2 * mx / S0), gvx / S0
    w[3], w[4] = gvy * (-2 * my / S0), gvy / S0
    w[5] = ged / S0
    w[0] = (gvx * (-S[2] / S0 ** 2 + 2 * mx * S[1] / S0 ** 2) + gvy * (-S[4] / S0 ** 2 + 2 * my * S[3] / S0 ** 2)
            + ged * (-S[5] / S0 ** 2))
    dm = m * (1 - m) / setup["tau_T"] * (w @ f)
    g = np.zeros(5)
    g[:3] = dT @ dm
    return out, g


def growth(setup, theta, cells, steps, tau, cot=None):
    a, n = theta[3], theta[4]
    nx, nxy, dx = setup["nx"], setup["nx"] * setup["ny"], setup["dx"]
    c = np.asarray(cells, np.int64)
    k, r = c // nxy, c % nxy
    j, i = r // nx, r % nx
    T, dT = temperature(setup, theta, (i + .5) * dx, (j + .5) * dx, (k + .5) * dx, np.asarray(steps) * setup["dt"])
    D = setup["Tl"] - T
    ta0 = np.asarray(tau)
    ok = (ta0 != 0) & np.isfinite(ta0) & (D > 0)
    D, ta, dT = D[ok], np.asarray(tau)[ok], dT[:, ok]
    pw = D ** n
    G = np.sum(a * pw * ta)
    if cot is None:
        return G, None
    dgdT = -a * n * D ** (n - 1) * ta
    g = np.zeros(5)
    g[:3] = cot * (dT @ dgdT)
    g[3] = cot * np.sum(pw * ta)
    g[4] = cot * np.sum(a * pw * ta * np.log(D))
    return G, g

"""Decks of a batched ensemble: many independent single-track realisations.

Each realisation is config 0's single track on one layer, with its own box
(sides drawn from U(lo, hi) voxels at dx = 2.5 um), laser speed v ~ U(0.5,
1.5) m/s, power P ~ U(150, 300) W, the realisation seed k (extension keyword
"seed"), the analytic pool sized to the Rosenthal isotherm at (P, v)
(rosenthal.pool) and the time step 0.25 dx / max(v, growth speed at the
solidus). The draws come from numpy's default_rng(host_seed), so a host seed
names the ensemble. A nucleation mean undercooling ~ U(5, 9) K is drawn and
recorded in each deck's comment; it has no effect (the reference's bulk
nucleation has no undercooling distribution).
"""
import os

import numpy as np

from .rosenthal import pool

DX = 2.5e-6
AVEL, NVEL, T_LIQ, T_SOL = 1e-5, 2.0, 1609.0, 1531.5


def deck_text(k, side, v, P, nuc_mean, dx=DX):
    sx, sy, sz = (int(a) for a in side)
    front, rear, width, depth = pool(P, v)
    dt = 0.25 * dx / max(v, AVEL * (T_LIQ - T_SOL) ** NVEL)
    lines = [
        "# ensemble realisation %d: %dx%dx%d voxels at %.3g um, v = %.6g m/s, P = %.6g W" % (k, sx, sy, sz, dx * 1e6, v, P),
        "# Rosenthal pool (eta 0.35, k 20 W/mK, alpha 5e-6 m^2/s): front, rear, half width, depth",
        "# nucleation mean undercooling %.6g K (recorded, not used)" % nuc_mean,
        "dx %r" % dx,
        "nX %d %d %d" % (sx, sy, sz),
        "bmV %r" % v,
        "bmP %r" % P,
        "bmDelT %r" % dt,
        "r 2e-4",
        "lT %r" % ((sz - 4) * dx),
        "bpH 10e-6",
        "tL %r" % T_LIQ,
        "tS %r" % T_SOL,
        "meltparam %r %r %r %r" % (front, rear, width, depth),
        "bhatch 1e-3",
        "mu 1.25e-4",
        "lrate 1.25e-4",
        "patternID 1",
        "outint 1000000",
        "offset 0.0 0.0 0.0",
        "gridsize %r 0" % (sx * dx),
        "gridtheta 0.0",
        "dendritegrowth2 %r %r" % (AVEL, NVEL),
        "seed %d" % k,
    ]
    return "\n".join(lines) + "\n"


def make_decks(out_dir, n=64, sides=(96, 192), host_seed=20240603):
    """Writes n decks ens_<k>.in (k = 1..n) into out_dir; returns their paths."""
    rng = np.random.default_rng(host_seed)
    os.makedirs(out_dir, exist_ok=True)
    paths = []
    for k in range(1, n + 1):
        side = rng.integers(sides[0], sides[1] + 1, 3)
        v = float(rng.uniform(0.5, 1.5))
        P = float(rng.uniform(150.0, 300.0))
        nuc = float(rng.uniform(5.0, 9.0))
        path = os.path.join(out_dir, "ens_%d.in" % k)
        with open(path, "w") as f:
            f.write(deck_text(k, side, v, P, nuc))
        paths.append(path)
    return paths

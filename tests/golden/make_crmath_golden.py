"""Correctly rounded reference values for cafe_crmath.h (tests/golden/crmath.npz).

Arguments cover the ranges the CA evaluates: atan2 of non-negative pairs and of
all sign combinations, sin/cos on [-2pi, 2pi] plus multiples of pi/2 and their
neighbours, acos on [-1, 1], x^e for e = 2..14 on [0, 1.4]. Values are
computed with mpmath at 300 bits and rounded to nearest. Needs mpmath (ships
with sympy); run from the repository root.
"""
import os

import mpmath
import numpy as np

mpmath.mp.prec = 300
HERE = os.path.dirname(os.path.abspath(__file__))


def rn(v):
    return mpmath.libmp.to_float(mpmath.mpf(v)._mpf_, rnd="n")


def main():
    rng = np.random.default_rng(20240611)
    n = 4000
    M = mpmath.mpf
    cases = {}
    y = rng.random(n) * 1e-5
    x = rng.random(n) * 1e-5
    sy = np.where(rng.random(n) < 0.3, -1.0, 1.0)
    sx = np.where(rng.random(n) < 0.3, -1.0, 1.0)
    y = y * sy
    x = x * sx
    x[:20] = 0.0
    y[20:40] = 0.0
    cases["atan2"] = (y, x, np.array([rn(mpmath.atan2(M(a), M(b))) for a, b in zip(y, x)]))
    t = rng.uniform(-2 * np.pi, 2 * np.pi, n)
    t[:40] = np.array([k * (np.pi / 2) for k in range(-4, 5)] * 5)[:40]
    t[40:80] = np.nextafter(t[:40], np.inf)
    cases["cos"] = (t, np.zeros(n), np.array([rn(mpmath.cos(M(a))) for a in t]))
    cases["sin"] = (t, np.zeros(n), np.array([rn(mpmath.sin(M(a))) for a in t]))
    u = rng.uniform(-1, 1, n)
    u[:4] = [-1.0, 1.0, 0.0, -0.0]
    u[4:10] = [np.nextafter(1.0, 0), np.nextafter(-1.0, 0), 1e-300, -1e-300, 0.5, -0.5]
    cases["acos"] = (u, np.zeros(n), np.array([rn(mpmath.acos(M(a))) for a in u]))
    r = rng.uniform(0, 1.4, n)
    e = rng.integers(1, 8, n) * 2.0
    cases["pow_int"] = (r, e, np.array([rn(M(a) ** int(b)) for a, b in zip(r, e)]))
    out = {}
    for k, (a, b, v) in cases.items():
        out[k + "_x"] = a
        out[k + "_y"] = b
        out[k + "_v"] = v
    np.savez_compressed(os.path.join(HERE, "crmath.npz"), **out)


if __name__ == "__main__":
    main()

"""Correctly rounded reference values for cafe_crmath.h (tests/golden/crmath.npz).

Arguments cover the ranges the CA evaluates: atan2 of non-negative pairs and of
all sign combinations, sin/cos on [-2pi, 2pi] plus multiples of pi/2 and their
neighbours, acos on [-1, 1], x^e for e = 2..14 on [0, 1.4], exp over its whole range and
x^(-1/2) over the double range. Values are
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


def rn_sub(v):
    """Round to nearest double, rounding once on the subnormal grid below 2^-1022."""
    v = mpmath.mpf(v)
    if v != 0 and abs(v) < mpmath.mpf(2) ** -1022:
        n = int(mpmath.nint(v * mpmath.mpf(2) ** 1074))
        return float(np.ldexp(float(n), -1074))
    return rn(v)


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
    # exp over its whole range: dense near 0, the subnormal band, near overflow
    xe = np.concatenate([rng.uniform(-750, 710, n), rng.uniform(-1, 1, n), rng.uniform(-745.2, -700, n // 2),
                         rng.uniform(700, 709.8, n // 4), -rng.uniform(0, 80, n),
                         [0.0, -0.0, 1e-300, -1e-300, 709.782712893384, -745.1332191019411, -745.1332191019412]])
    cases["exp"] = (xe, np.zeros(len(xe)), np.array([rn_sub(mpmath.exp(M(a))) for a in xe]))
    # x^(-1/2): log-uniform over the double range, the quadrature's (t - x) range, raw bit patterns
    xm = np.concatenate([10.0 ** rng.uniform(-320, 307, n), rng.uniform(1e-7, 8e-4, n),
                         (rng.integers(1, 0x7FEFFFFFFFFFFFFF, n, dtype=np.int64)).view(np.float64),
                         [1.0, 4.0, 0.25, 2.0, 5e-324, 1.7976931348623157e308]])
    cases["pow_mhalf"] = (xm, np.zeros(len(xm)), np.array([rn_sub(M(a) ** M(-0.5)) for a in xm]))
    out = {}
    for k, (a, b, v) in cases.items():
        out[k + "_x"] = a
        out[k + "_y"] = b
        out[k + "_v"] = v
    np.savez_compressed(os.path.join(HERE, "crmath.npz"), **out)


if __name__ == "__main__":
    main()

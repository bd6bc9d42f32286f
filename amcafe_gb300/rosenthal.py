"""Melt-pool size of the Rosenthal moving point source, for sizing decks.

The reference's analytic temperature (TempField::AnalyticTempCurr,
TempField.C:139-217) is a double ellipsoid given by `meltparam` (front
length, rear length, half width, depth). Decks for a given laser power P,
absorptivity eta, speed v and material (k, alpha, T_liq, T0) take those four
numbers from the liquidus isotherm of the Rosenthal solution for a point source
moving over a half space,

    T - T0 = eta P / (2 pi k R) exp(-v (R + xi) / (2 alpha)),   R = |(xi, y, z)|,

with xi the coordinate along the travel direction measured from the source:
front length = the root of T = T_liq ahead of the source on the axis, rear
length = eta P / (2 pi k (T_liq - T0)) (the exponent vanishes behind it), and
half width = depth = the largest radius of the isotherm over xi.
"""
import math


def _bisect(f, a, b, it=200):
    fa = f(a)
    for _ in range(it):
        m = 0.5 * (a + b)
        fm = f(m)
        if (fm > 0) == (fa > 0):
            a, fa = m, fm
        else:
            b = m
    return 0.5 * (a + b)


def pool(P, v, eta=0.35, k=20.0, alpha=5e-6, T_liq=1609.0, T0=300.0):
    """(front, rear, half_width, depth) in metres of the liquidus isotherm."""
    q = eta * P / (2 * math.pi * k)
    dT = T_liq - T0
    rear = q / dT

    def excess_axis(xi):  # ahead of the source, R = xi
        return q / xi * math.exp(-v * xi / alpha) - dT

    front = _bisect(excess_axis, 1e-12, rear)

    def radius(xi):  # largest r with T(xi, r) >= T_liq, 0 if none
        def excess(r):
            R = math.hypot(xi, r)
            return q / R * math.exp(-v * (R + xi) / (2 * alpha)) - dT

        if excess(0.0 if xi != 0 else 1e-15) <= 0:
            return 0.0
        return _bisect(excess, 1e-15 if xi == 0 else 0.0, rear)

    # golden-section search for the widest section, xi in (-rear, front)
    a, b = -rear, front
    g = (math.sqrt(5) - 1) / 2
    c, d = b - g * (b - a), a + g * (b - a)
    rc, rd = radius(c), radius(d)
    for _ in range(200):
        if rc > rd:
            b, d, rd = d, c, rc
            c = b - g * (b - a)
            rc = radius(c)
        else:
            a, c, rc = c, d, rd
            d = a + g * (b - a)
            rd = radius(d)
    width = max(rc, rd)
    return front, rear, width, width

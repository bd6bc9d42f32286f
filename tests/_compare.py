"""Field-by-field comparison of CA states (test helper)."""
import numpy as np

INT_FIELDS = ("gID", "vState", "buildj")
FLOAT_FIELDS = ("extents", "centroid", "temp")


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if same.all():
        return 0.0
    d = np.abs(a - b)[~same] / np.maximum(np.abs(b)[~same], 1e-300)
    return float(np.nanmax(d)) if np.isfinite(d).any() else float("inf")


def compare_states(got, ref, rtol=1e-12, where=""):
    """got/ref: dicts with gID, vState, extents, centroid (+ optional temp,
    buildj). Integer fields must match exactly; floats within rtol (relative).
    Returns the largest relative float difference."""
    worst = 0.0
    for k in INT_FIELDS:
        if k in got and k in ref:
            a, b = np.asarray(got[k]), np.asarray(ref[k])
            if not np.array_equal(a, b):
                idx = np.nonzero(a != b)[0]
                raise AssertionError("%s: %s differs at %d cells (first %s: %s vs %s)" % (
                    where, k, len(idx), idx[:5], a[idx[:5]], b[idx[:5]]))
    for k in FLOAT_FIELDS:
        if k in got and k in ref:
            r = max_rel(got[k], ref[k])
            if not r <= rtol:
                raise AssertionError("%s: %s relative difference %g > %g" % (where, k, r, rtol))
            worst = max(worst, r)
    return worst

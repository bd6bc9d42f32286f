"""The C ABI library loads and exports every function include/cafe_gpu.h
declares (no GPU calls)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_symbols_exported():
    from amcafe_gb300 import _native
    from amcafe_gb300 import build as b

    if not os.path.exists(_native.LIB_PATH):
        b.build_engine()
    lib = _native.load()
    text = open(os.path.join(ROOT, "include", "cafe_gpu.h")).read()
    names = set(re.findall(r"\b(cafe_[a-z_]+)\s*\(", text))
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), "missing export %s" % n
    assert names == set(_native.EXPORTS), "binding and header disagree: %s" % (names ^ set(_native.EXPORTS))


def test_error_reporting_without_gpu():
    import ctypes

    from amcafe_gb300 import _native

    lib = _native.load()
    h = ctypes.c_void_p()
    rc = lib.cafe_sim_create(b"/nonexistent/deck.in", None, ctypes.byref(h))
    assert rc == 5  # CAFE_E_IO
    assert b"cannot open deck" in lib.cafe_last_error()


def test_rosenthal_pool_sizes_the_config_decks():
    """The Rosenthal sizer reproduces the meltparam of the config 0 and 2 decks."""
    from amcafe_gb300.rosenthal import pool

    for P, v, want in ((200.0, 1.0, (16.31e-6, 425.5e-6, 55.11e-6)), (200.0, 0.8, (19.32e-6, 425.5e-6, 61.39e-6))):
        f, r, w, d = pool(P, v)
        assert abs(f - want[0]) < 0.01e-6 and abs(r - want[1]) < 0.1e-6 and abs(w - want[2]) < 0.01e-6 and w == d


def test_ensemble_decks_are_deterministic(tmp_path):
    from amcafe_gb300.ensemble import make_decks

    a = make_decks(str(tmp_path / "a"), n=4)
    b = make_decks(str(tmp_path / "b"), n=4)
    for x, y in zip(a, b):
        assert open(x).read() == open(y).read()
    txt = open(a[2]).read()
    assert "seed 3" in txt and "nX " in txt

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

"""Host builds of the device headers against their references (CPU only).

* cafe_rng.h must reproduce libstdc++'s std::default_random_engine +
  std::uniform_real_distribution<double>(0,1) stream exactly, both sequentially
  and by jump-ahead (the device draws ruq offsets by jump-ahead);
* cafe_crmath.h must return the correctly rounded value on the committed
  mpmath cases (tests/golden/crmath.npz).
The wrapper tests/native/hdr_check.cpp is compiled here with FP contraction
off, as the library is.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cafe_oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def hc(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hc") / "hc.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    os.path.join(HERE, "native", "hdr_check.cpp"), "-o", so], check=True)
    lib = ctypes.CDLL(so)
    f64p = ctypes.POINTER(ctypes.c_double)
    lib.hc_uniforms_at.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_long, f64p]
    lib.hc_uniforms_stream.argtypes = [ctypes.c_uint32, ctypes.c_long, f64p]
    lib.hc_eval.argtypes = [ctypes.c_int, ctypes.c_long, f64p, f64p, f64p]
    return lib


def _std_uniforms(seed, skip, n):
    out = np.empty(n)
    orc.load().cafe_oracle_std_uniforms(seed, skip, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


@pytest.mark.parametrize("seed", [1, 2912351, 2912351 + 30 * 7, 531231, 2132512 + 32 * 5 + 64 * 99, 0,
                                  2147483647, 4294967295])
def test_uniform_stream_matches_libstdcxx(hc, seed):
    n = 5000
    want = _std_uniforms(seed, 0, n)
    got = np.empty(n)
    hc.hc_uniforms_stream(seed, n, got.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert np.array_equal(got, want)
    got2 = np.empty(n)
    hc.hc_uniforms_at(seed, 0, n, got2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert np.array_equal(got2, want)


def test_uniform_jump_ahead(hc):
    for seed, skip in ((2912351, 123456), (77, 1), (2912351 + 30 * 1000, 2000000)):
        want = _std_uniforms(seed, skip, 100)
        got = np.empty(100)
        hc.hc_uniforms_at(seed, skip, 100, got.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert np.array_equal(got, want)


@pytest.mark.parametrize("fn,name", [(0, "atan2"), (1, "cos"), (2, "sin"), (3, "acos"), (5, "pow_int"), (6, "exp"),
                                     (7, "pow_mhalf")])
def test_crmath_correctly_rounded(hc, fn, name):
    g = np.load(os.path.join(HERE, "golden", "crmath.npz"))
    x = np.ascontiguousarray(g[name + "_x"])
    y = np.ascontiguousarray(g[name + "_y"])
    want = g[name + "_v"]
    got = np.empty_like(x)
    p = ctypes.POINTER(ctypes.c_double)
    hc.hc_eval(fn, len(x), x.ctypes.data_as(p), y.ctypes.data_as(p), got.ctypes.data_as(p))
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, "%s: %d of %d not correctly rounded, e.g. x=%r y=%r got %r want %r" % (
        name, len(bad), len(x), x[bad[0]], y[bad[0]], got[bad[0]], want[bad[0]])


def test_pow_half_is_pow_semantics(hc):
    x = np.array([0.0, -0.0, 4.0, 2.0, np.inf, -np.inf, -1.0])
    got = np.empty_like(x)
    p = ctypes.POINTER(ctypes.c_double)
    hc.hc_eval(4, len(x), x.ctypes.data_as(p), x.ctypes.data_as(p), got.ctypes.data_as(p))
    want = np.array([np.sqrt(v) if v >= 0 else np.nan for v in x])
    want[5] = np.inf  # pow(-inf, 0.5) = +inf
    assert np.array_equal(got[:6], want[:6]) and np.isnan(got[6])
    assert not np.signbit(got[1])

"""Python access to the CPU oracle (oracle/cafe_oracle.cpp). Test
infrastructure: imported only by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py.
"""
import ctypes
import os

from cafe_dump import read_dump  # noqa: F401  (re-exported for tests)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libcafe_oracle.so")
REF_DUMP = os.path.join(HERE, "_ref", "cafe_ref_dump")

LIBM_GLIBC, LIBM_CR, LIBM_PERTURB = 0, 1, 2
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError("oracle library not built: make -C oracle oracle")
        lib = ctypes.CDLL(LIB)
        lib.cafe_oracle_run.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_long, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_ulonglong,
                                        ctypes.POINTER(ctypes.c_longlong)]
        lib.cafe_oracle_run.restype = ctypes.c_int
        lib.cafe_oracle_std_uniforms.argtypes = [ctypes.c_uint, ctypes.c_long, ctypes.c_long,
                                                 ctypes.POINTER(ctypes.c_double)]
        lib.cafe_oracle_orientations.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_double)]
        lib.cafe_oracle_rotmat.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double)]
        _lib = lib
    return _lib


def run(deck, dump_path="", max_steps=-1, dump_stride=1, libm=LIBM_GLIBC, perturb_p=0.0, perturb_seed=0):
    """Runs the main1.C loop on `deck`; returns a stats dict."""
    st = (ctypes.c_longlong * 8)()
    rc = load().cafe_oracle_run(str(deck).encode(), str(dump_path).encode(), max_steps, dump_stride, libm,
                                perturb_p, perturb_seed, st)
    if rc != 0:
        raise RuntimeError("oracle run failed on %s" % deck)
    keys = ("steps", "events", "nucleations", "max_active", "max_front", "nGrain", "ncell")
    return dict(zip(keys, list(st)[:7]))

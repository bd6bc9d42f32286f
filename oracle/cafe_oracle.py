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


class Window(ctypes.Structure):
    _fields_ = [("isp", ctypes.c_int), ("inewscanflg", ctypes.c_int), ("inewlayerflg", ctypes.c_int),
                ("indlayer", ctypes.c_int), ("ilaserLoc", ctypes.c_int), ("tInd", ctypes.c_int),
                ("time", ctypes.c_double), ("gth", ctypes.c_double), ("genlayer_state", ctypes.c_uint),
                ("ngrain", ctypes.c_int)]


def run_window(deck, info, state, ctheta, nsteps, libm=LIBM_CR, copy=True):
    """Resumes the loop from a GPU state (info from Simulation.info(), state
    from Simulation.state()); returns (new_state, seconds, stats). The arrays
    in `state` are copied, not modified. With copy=False the arrays are passed
    as they are (they may be read-only memory maps) and new_state is None: the
    run is only timed and counted."""
    import numpy as np

    lib = load()
    lib.cafe_oracle_set_window_writeback.argtypes = [ctypes.c_int]
    lib.cafe_oracle_set_window_writeback(1 if copy else 0)
    f = lib.cafe_oracle_run_window
    i32p, f64p = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.c_char_p, ctypes.POINTER(Window), i32p, i32p, f64p, f64p, i32p, f64p, ctypes.c_long,
                  ctypes.c_int, f64p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int)]
    w = Window(info["isp"], info["inewscanflg"], info["inewlayerflg"], info["indlayer"], info["ilaserLoc"],
               info["tInd"], info["time"], info["gth"], info["genlayer_state"], info["nGrain"])
    if copy:
        st = {k: np.array(v, copy=True) for k, v in state.items()}
    else:
        st = {k: np.ascontiguousarray(v) for k, v in state.items()}
    cth = np.ascontiguousarray(ctheta, np.float64)
    sec = ctypes.c_double(0)
    stats = (ctypes.c_longlong * 10)()
    ng = ctypes.c_int(0)
    rc = f(str(deck).encode(), ctypes.byref(w), st["gID"].ctypes.data_as(i32p), st["vState"].ctypes.data_as(i32p),
           st["extents"].ctypes.data_as(f64p), st["centroid"].ctypes.data_as(f64p), st["buildj"].ctypes.data_as(i32p),
           cth.ctypes.data_as(f64p), int(nsteps), libm, ctypes.byref(sec), stats, ctypes.byref(ng))
    lib.cafe_oracle_set_window_writeback(1)
    if rc != 0:
        raise RuntimeError("oracle window run failed")
    keys = ("steps", "events", "nucleations", "max_active", "max_front", "nGrain", "ncell")
    out = dict(zip(keys, list(stats)[:7]))
    out["negative_dt"], out["clamped"] = stats[8], stats[9]
    return (st if copy else None), sec.value, out


def run(deck, dump_path="", max_steps=-1, dump_stride=1, libm=LIBM_GLIBC, perturb_p=0.0, perturb_seed=0):
    """Runs the main1.C loop on `deck`; returns a stats dict."""
    st = (ctypes.c_longlong * 10)()
    rc = load().cafe_oracle_run(str(deck).encode(), str(dump_path).encode(), max_steps, dump_stride, libm,
                                perturb_p, perturb_seed, st)
    if rc != 0:
        raise RuntimeError("oracle run failed on %s" % deck)
    keys = ("steps", "events", "nucleations", "max_active", "max_front", "nGrain", "ncell", "loop_ns",
            "negative_dt", "clamped")
    return dict(zip(keys, list(st)[:10]))


def set_output(out_dir, every=1):
    """Makes the following run() calls write the datasets of
    VoxelsCA::WriteToHDF1 as raw files <out_dir>/out<tInd>.h5.<name>.bin at
    every `every`-th output point and final.h5.<name>.bin after the closing
    CleanLayer; out_dir None turns output off."""
    lib = load()
    lib.cafe_oracle_set_output.argtypes = [ctypes.c_char_p, ctypes.c_long]
    lib.cafe_oracle_set_output(str(out_dir).encode() if out_dir else None, int(every))


def set_budget(seconds):
    """Wall-clock limit (s) for the oracle's loops; 0 = none."""
    lib = load()
    lib.cafe_oracle_set_budget.argtypes = [ctypes.c_double]
    lib.cafe_oracle_set_budget(float(seconds))

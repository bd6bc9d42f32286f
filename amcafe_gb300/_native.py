"""ctypes binding of libcafe_gpu.so (the C ABI declared in include/cafe_gpu.h).

The library is built in-tree by amcafe_gb300.build (nvcc, sm_103a). Loading
fails with an ImportError when it has not been built: there is no fallback
implementation of the GPU path.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcafe_gpu.so")

# Every symbol declared in include/cafe_gpu.h.
EXPORTS = (
    "cafe_sim_create", "cafe_sim_destroy", "cafe_sim_initialize_voxels", "cafe_sim_add_layer",
    "cafe_sim_update_laser", "cafe_sim_temperature", "cafe_sim_update_voxels",
    "cafe_sim_clean_layer", "cafe_sim_update_time", "cafe_sim_begin", "cafe_sim_step",
    "cafe_sim_run", "cafe_sim_synchronize", "cafe_sim_info", "cafe_sim_stats",
    "cafe_sim_download_state", "cafe_sim_download_temperature", "cafe_sim_download_ctheta",
    "cafe_sim_upload_state", "cafe_last_error", "cafe_sim_set_timing", "cafe_sim_phase_times",
    "cafe_sim_stream", "cafe_sim_mark", "cafe_sim_elapsed", "cafe_clean_layer_noalloc",
    "cafe_sim_set_build", "cafe_sim_download_build", "cafe_sim_download_output", "cafe_sim_write_output",
    "cafe_batch_create", "cafe_batch_run", "cafe_batch_size", "cafe_batch_sim", "cafe_batch_finished",
    "cafe_batch_destroy", "cafe_sim_checkpoint", "cafe_sim_restore", "cafe_sim_set_growth_log",
    "cafe_sim_growth_log_count", "cafe_adjoint_pool", "cafe_adjoint_growth", "cafe_sim_grid",
    "cafe_generate_samples", "cafe_batch_report", "cafe_sim_set_output",
)
PHASES = ("melt", "classify", "gather", "events", "writeback", "layer")
NPHASE = 8


class CafeOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("active_capacity", ctypes.c_longlong),
                ("grain_capacity", ctypes.c_longlong), ("event_scan", ctypes.c_int),
                ("event_fill_helper", ctypes.c_int)]


class CafeGrid(ctypes.Structure):
    _fields_ = [("nX", ctypes.c_int * 3), ("dX", ctypes.c_double * 3), ("LX", ctypes.c_double * 3),
                ("offset", ctypes.c_double * 3), ("meltparam", ctypes.c_double * 4), ("gbox", ctypes.c_double * 4),
                ("gsize", ctypes.c_double * 2)] + [
        (n, ctypes.c_double) for n in ("bmV", "bmP", "bmDelT", "bhatch", "tL", "tS", "T0", "layerT", "bpH", "mu",
                                       "lrate", "rNmax", "Avel", "nvel", "gth0", "gth", "time", "DelT")] + [
        (n, ctypes.c_int) for n in ("outint", "patternID", "outNL", "EASM_Flag", "nZlayer", "Nzhg", "Nsd", "Ntd",
                                    "NpT", "isp", "inewscanflg", "inewlayerflg", "indlayer", "ilaserLoc", "tInd",
                                    "tf_tInd", "Nzh", "nlayerTot", "seed", "tmodel")] + [
        ("ros_eta", ctypes.c_double), ("ros_k", ctypes.c_double), ("ros_alpha", ctypes.c_double),
        ("laser", ctypes.c_double * 3), ("dirp", ctypes.c_double)]


class CafeInfo(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("tInd", ctypes.c_int), ("time", ctypes.c_double),
                ("isp", ctypes.c_int), ("indlayer", ctypes.c_int), ("inewlayerflg", ctypes.c_int),
                ("inewscanflg", ctypes.c_int), ("ilaserLoc", ctypes.c_int), ("nGrain", ctypes.c_int),
                ("nlayerTot", ctypes.c_int), ("Nzh", ctypes.c_int), ("done", ctypes.c_int),
                ("steps", ctypes.c_longlong), ("gth", ctypes.c_double), ("genlayer_state", ctypes.c_uint),
                ("tf_tInd", ctypes.c_int), ("output_due", ctypes.c_int)]


class CafeAdjointSetup(ctypes.Structure):
    _fields_ = [("k", ctypes.c_double), ("alpha", ctypes.c_double), ("T0", ctypes.c_double), ("Tl", ctypes.c_double),
                ("tau_T", ctypes.c_double), ("x_start", ctypes.c_double), ("y_src", ctypes.c_double),
                ("z_src", ctypes.c_double), ("dt", ctypes.c_double), ("dx", ctypes.c_double),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("step_final", ctypes.c_int)]


class CafeStats(ctypes.Structure):
    _fields_ = [("events", ctypes.c_ulonglong), ("nucleations", ctypes.c_ulonglong),
                ("max_active", ctypes.c_ulonglong), ("max_rows", ctypes.c_ulonglong),
                ("steps", ctypes.c_ulonglong), ("negative_dt", ctypes.c_ulonglong),
                ("sum_active", ctypes.c_ulonglong), ("sum_rows", ctypes.c_ulonglong),
                ("launches", ctypes.c_ulonglong), ("exact_scan_steps", ctypes.c_ulonglong),
                ("row_evaluations", ctypes.c_ulonglong), ("cycles_select", ctypes.c_ulonglong),
                ("cycles_apply", ctypes.c_ulonglong), ("cycles_fill", ctypes.c_ulonglong),
                ("graph_captures", ctypes.c_ulonglong), ("easm_integrals", ctypes.c_ulonglong),
                ("cycles_merge", ctypes.c_ulonglong)]


_lib = None


def load():
    """Returns the loaded library; raises ImportError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libcafe_gpu.so is not built (%s); run amcafe_gb300.build.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, I, LL, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    i32p = ctypes.POINTER(ctypes.c_int32)
    f64p = ctypes.POINTER(ctypes.c_double)
    f32p = ctypes.POINTER(ctypes.c_float)
    sig = {
        "cafe_sim_create": (I, [ctypes.c_char_p, ctypes.POINTER(CafeOptions), ctypes.POINTER(P)]),
        "cafe_sim_destroy": (None, [P]),
        "cafe_sim_initialize_voxels": (I, [P]),
        "cafe_sim_add_layer": (I, [P]),
        "cafe_sim_update_laser": (I, [P]),
        "cafe_sim_temperature": (I, [P]),
        "cafe_sim_update_voxels": (I, [P]),
        "cafe_sim_clean_layer": (I, [P]),
        "cafe_sim_update_time": (I, [P]),
        "cafe_sim_begin": (I, [P]),
        "cafe_sim_step": (I, [P, ctypes.POINTER(I)]),
        "cafe_sim_run": (I, [P, LL, ctypes.POINTER(LL)]),
        "cafe_sim_synchronize": (I, [P]),
        "cafe_sim_info": (I, [P, ctypes.POINTER(CafeInfo)]),
        "cafe_sim_grid": (I, [P, ctypes.POINTER(CafeGrid)]),
        "cafe_generate_samples": (I, [I, ctypes.c_uint, P]),
        "cafe_batch_report": (I, [P, ctypes.POINTER(LL), ctypes.POINTER(LL), ctypes.c_char_p, I]),
        "cafe_sim_set_output": (I, [P, ctypes.c_char_p]),
        "cafe_sim_stats": (I, [P, ctypes.POINTER(CafeStats)]),
        "cafe_sim_download_state": (I, [P, i32p, i32p, f64p, f64p, i32p]),
        "cafe_sim_download_temperature": (I, [P, f64p]),
        "cafe_sim_download_ctheta": (I, [P, f64p, LL, ctypes.POINTER(I)]),
        "cafe_sim_upload_state": (I, [P, i32p, i32p, f64p, f64p, f64p, I]),
        "cafe_last_error": (ctypes.c_char_p, []),
        "cafe_sim_set_timing": (I, [P, I]),
        "cafe_sim_phase_times": (I, [P, f64p, ctypes.POINTER(LL), I, I]),
        "cafe_sim_stream": (I, [P, ctypes.POINTER(P)]),
        "cafe_sim_mark": (I, [P, I]),
        "cafe_sim_elapsed": (I, [P, I, I, ctypes.POINTER(D)]),
        "cafe_clean_layer_noalloc": (I, [P, LL, P, I, ctypes.POINTER(I), P]),
        "cafe_sim_set_build": (I, [P]),
        "cafe_sim_download_build": (I, [P, i32p]),
        "cafe_sim_download_output": (I, [P, f32p, f32p, f32p, f32p]),
        "cafe_sim_write_output": (I, [P, ctypes.c_char_p]),
        "cafe_batch_create": (I, [ctypes.POINTER(ctypes.c_char_p), I, ctypes.POINTER(CafeOptions), I,
                                  ctypes.POINTER(P)]),
        "cafe_batch_run": (I, [P, LL, ctypes.POINTER(LL)]),
        "cafe_batch_size": (I, [P]),
        "cafe_batch_sim": (P, [P, I]),
        "cafe_batch_finished": (I, [P, I]),
        "cafe_batch_destroy": (None, [P]),
        "cafe_sim_checkpoint": (I, [P, ctypes.c_char_p]),
        "cafe_sim_restore": (I, [P, ctypes.c_char_p]),
        "cafe_sim_set_growth_log": (I, [P, P, P, P, LL]),
        "cafe_sim_growth_log_count": (I, [P, ctypes.POINTER(LL)]),
        "cafe_adjoint_pool": (I, [ctypes.POINTER(CafeAdjointSetup), f64p, f64p, f64p, f64p, P]),
        "cafe_adjoint_growth": (I, [ctypes.POINTER(CafeAdjointSetup), f64p, P, P, P, LL, D, f64p, f64p, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class CafeError(RuntimeError):
    pass


def check(rc):
    if rc != 0:
        msg = load().cafe_last_error()
        raise CafeError("cafe error %d: %s" % (rc, msg.decode() if msg else ""))

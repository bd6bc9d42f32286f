"""Python face of libcafe_gpu.so, mirroring AMCAFE's class interface.

The reference's time loop (main1.C:18-101) reads

    Grid g(file); Partition part(g); part.PartitionGraph2(); BasePlate bp(g, part);
    TempField TempF(g, part, bp, ut); TempF.InitializeAnalytic();
    VoxelsCA vox(g, TempF, part); vox.InitializeVoxels(bp);
    vox.AddLayer1(); g.UpdateLaser();
    while (!bcheck) { TempF.AnalyticTempCurr(...); vox.UpdateVoxels(); g.UpdateLaser();
                      bcheck = g.indlayer > nlayerTot; if (g.inewlayerflg) vox.CleanLayer();
                      g.UpdateTime2(TempF.DelT); if (g.inewlayerflg) vox.AddLayer1(); }
    vox.CleanLayer();

`Simulation(deck)` performs the constructors; the same calls exist as methods
with the reference's names (InitializeVoxels, AddLayer1, UpdateLaser,
AnalyticTempCurr, UpdateVoxels, CleanLayer, UpdateTime2) and as `step()` /
`run()` for the loop body and the whole loop. The public fields (gID, vState,
extents, centroidOct, TempCurr, BuildjID, cTheta, nGrain) are read with
`state()`, `temperature()` and `ctheta()`. At the output points of the loop
(`info()["output_due"]`) `step()` has called SetBuild; `build()`, `output()`
and `WriteToHDF1(prefix)` give Build and the datasets the reference writes.
"""
import ctypes
import os

import numpy as np

from ._native import NPHASE, PHASES, CafeGrid, CafeInfo, CafeOptions, CafeStats, check, load


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None else None


class Simulation:
    def __init__(self, deck, device=0, active_capacity=0, grain_capacity=0, event_scan=0, _handle=None,
                 event_fill_helper=0):
        self._lib = load()
        self._owned = _handle is None
        if _handle is not None:  # a realisation owned by a Batch
            self._h = ctypes.c_void_p(_handle)
        else:
            self._h = ctypes.c_void_p()
            opt = CafeOptions(device, active_capacity, grain_capacity, event_scan, event_fill_helper)
            check(self._lib.cafe_sim_create(str(deck).encode(), ctypes.byref(opt), ctypes.byref(self._h)))
        inf = self.info()
        self.shape = (inf["nz"], inf["ny"], inf["nx"])
        self.ncell = inf["nx"] * inf["ny"] * inf["nz"]

    # -- reference calls -------------------------------------------------
    def InitializeVoxels(self):
        check(self._lib.cafe_sim_initialize_voxels(self._h))

    def AddLayer1(self):
        check(self._lib.cafe_sim_add_layer(self._h))

    def UpdateLaser(self):
        check(self._lib.cafe_sim_update_laser(self._h))

    def AnalyticTempCurr(self):
        check(self._lib.cafe_sim_temperature(self._h))

    def UpdateVoxels(self):
        check(self._lib.cafe_sim_update_voxels(self._h))

    def CleanLayer(self):
        check(self._lib.cafe_sim_clean_layer(self._h))

    def UpdateTime2(self):
        check(self._lib.cafe_sim_update_time(self._h))

    # -- loop helpers ----------------------------------------------------
    def begin(self):
        """InitializeVoxels() was called; AddLayer1() + first UpdateLaser() (main1.C:60-61)."""
        check(self._lib.cafe_sim_begin(self._h))

    def step(self):
        done = ctypes.c_int(0)
        check(self._lib.cafe_sim_step(self._h, ctypes.byref(done)))
        return bool(done.value)

    def run(self, max_steps=0):
        n = ctypes.c_longlong(0)
        check(self._lib.cafe_sim_run(self._h, int(max_steps), ctypes.byref(n)))
        return n.value

    def synchronize(self):
        check(self._lib.cafe_sim_synchronize(self._h))

    # -- state -------------------------------------------------------------
    def info(self):
        i = CafeInfo()
        check(self._lib.cafe_sim_info(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in CafeInfo._fields_}

    def grid(self):
        """Grid's public scalars (cafe_sim_grid): deck values, derived laser
        grid, clock and laser state, the temperature model, and the source
        position and scan direction of the next temperature call."""
        g = CafeGrid()
        check(self._lib.cafe_sim_grid(self._h, ctypes.byref(g)))
        out = {}
        for f, t in CafeGrid._fields_:
            v = getattr(g, f)
            out[f] = list(v) if hasattr(v, "__len__") else v
        return out

    def stats(self):
        s = CafeStats()
        check(self._lib.cafe_sim_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in CafeStats._fields_}

    def state(self, out=None):
        """gID, vState, extents, centroid (x,y,z interleaved) and buildj as
        numpy arrays. `out` may hold preallocated contiguous arrays under the
        same keys (for example views of pinned host memory), filled in place."""
        n = self.ncell
        shapes = dict(gID=(n, np.int32), vState=(n, np.int32), extents=(n, np.float64),
                      centroid=(3 * n, np.float64), buildj=(n, np.int32))
        arrs = {}
        for k, (m, dt) in shapes.items():
            a = None if out is None else out.get(k)
            if a is None:
                a = np.empty(m, dt)
            elif a.dtype != dt or a.size != m or not a.flags["C_CONTIGUOUS"]:
                raise ValueError("out[%r] must be a contiguous %s array of %d elements" % (k, np.dtype(dt), m))
            arrs[k] = a
        gid, vs, ext, cen, bj = (arrs[k] for k in ("gID", "vState", "extents", "centroid", "buildj"))
        check(self._lib.cafe_sim_download_state(self._h, _ptr(gid, ctypes.c_int32), _ptr(vs, ctypes.c_int32),
                                                _ptr(ext, ctypes.c_double), _ptr(cen, ctypes.c_double),
                                                _ptr(bj, ctypes.c_int32)))
        return dict(gID=gid, vState=vs, extents=ext, centroid=cen, buildj=bj)

    def temperature(self):
        t = np.empty(self.ncell, np.float64)
        check(self._lib.cafe_sim_download_temperature(self._h, _ptr(t, ctypes.c_double)))
        return t

    def ctheta(self):
        ng = ctypes.c_int(0)
        check(self._lib.cafe_sim_download_ctheta(self._h, None, 0, ctypes.byref(ng)))
        out = np.empty(4 * max(ng.value, 1), np.float64)
        check(self._lib.cafe_sim_download_ctheta(self._h, _ptr(out, ctypes.c_double), out.size, ctypes.byref(ng)))
        return out[:4 * ng.value]

    # -- output (VoxelsCA::SetBuild / WriteToHDF1) ---------------------------
    def SetBuild(self):
        check(self._lib.cafe_sim_set_build(self._h))

    def build(self):
        """VoxelsCA::Build as an int32 array."""
        b = np.empty(self.ncell, np.int32)
        check(self._lib.cafe_sim_download_build(self._h, _ptr(b, ctypes.c_int32)))
        return b

    def output(self):
        """The derived datasets of WriteToHDF1: Temperature (float32, one per
        cell) and IPFz, IPFx, IPFy (float32 RGB, 3 per cell)."""
        n = self.ncell
        t = np.empty(n, np.float32)
        z, x, y = (np.empty(3 * n, np.float32) for _ in range(3))
        f = ctypes.c_float
        check(self._lib.cafe_sim_download_output(self._h, _ptr(t, f), _ptr(z, f), _ptr(x, f), _ptr(y, f)))
        return dict(Temperature=t, IPFz=z, IPFx=x, IPFy=y)

    def set_output(self, base):
        """The loop writes the WriteToHDF1 datasets itself at its output
        points as "<base><tInd>.h5.*" (before that step's AddLayer1, as
        main1.C does), and after the closing CleanLayer of run(); None turns
        it off (cafe_sim_set_output)."""
        check(self._lib.cafe_sim_set_output(self._h, str(base).encode() if base else None))

    def WriteToHDF1(self, prefix):
        """Writes the datasets of VoxelsCA::WriteToHDF1 as raw files
        <prefix>.<dataset>.bin (prefix such as "out/run120.h5")."""
        check(self._lib.cafe_sim_write_output(self._h, os.fsencode(prefix)))

    # -- checkpoint / restore --------------------------------------------------
    def checkpoint(self, path):
        """Writes the whole loop state to `path` (cafe_sim_checkpoint)."""
        check(self._lib.cafe_sim_checkpoint(self._h, os.fsencode(path)))

    def restore(self, path):
        """Loads a checkpoint written from the same deck, in place of
        InitializeVoxels + begin (cafe_sim_restore)."""
        check(self._lib.cafe_sim_restore(self._h, os.fsencode(path)))

    def upload_state(self, gID, vState, extents, centroid, ctheta):
        gID = np.ascontiguousarray(gID, np.int32)
        vState = np.ascontiguousarray(vState, np.int32)
        extents = np.ascontiguousarray(extents, np.float64)
        centroid = np.ascontiguousarray(centroid, np.float64)
        ctheta = np.ascontiguousarray(ctheta, np.float64)
        check(self._lib.cafe_sim_upload_state(self._h, _ptr(gID, ctypes.c_int32), _ptr(vState, ctypes.c_int32),
                                              _ptr(extents, ctypes.c_double), _ptr(centroid, ctypes.c_double),
                                              _ptr(ctheta, ctypes.c_double), len(ctheta) // 4))

    # -- profiling ---------------------------------------------------------
    def set_timing(self, on=True):
        check(self._lib.cafe_sim_set_timing(self._h, 1 if on else 0))

    def phase_times(self, reset=False):
        """{phase: (milliseconds, kernel launches)} accumulated while timing was on."""
        ms = (ctypes.c_double * NPHASE)()
        nl = (ctypes.c_longlong * NPHASE)()
        check(self._lib.cafe_sim_phase_times(self._h, ms, nl, NPHASE, 1 if reset else 0))
        return {name: (ms[i], nl[i]) for i, name in enumerate(PHASES)}

    def mark(self, slot):
        check(self._lib.cafe_sim_mark(self._h, slot))

    def elapsed_ms(self, a, b):
        ms = ctypes.c_double(0)
        check(self._lib.cafe_sim_elapsed(self._h, a, b, ctypes.byref(ms)))
        return ms.value

    def stream(self):
        """The cudaStream_t (as an int) that this simulation's work runs on."""
        p = ctypes.c_void_p()
        check(self._lib.cafe_sim_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    def close(self):
        if self._h and self._owned:
            self._lib.cafe_sim_destroy(self._h)
        self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_deck(deck, max_steps=0, device=0, **kw):
    """The whole main1.C time loop on one deck; returns the Simulation."""
    sim = Simulation(deck, device=device, **kw)
    sim.InitializeVoxels()
    sim.begin()
    sim.run(max_steps)
    return sim


class Batch:
    """Independent realisations (one deck each) stepped concurrently on one GPU
    (cafe_batch_*): threads=0 launches every step kernel once for all of them
    (autotuned launch shapes), threads>=1 steps them round-robin from that many
    host threads. `sims[i]` reads realisation i like a Simulation."""

    def __init__(self, decks, device=0, threads=0, active_capacity=0, grain_capacity=0, event_scan=0,
                 event_fill_helper=0):
        self._lib = load()
        self._h = ctypes.c_void_p()
        arr = (ctypes.c_char_p * len(decks))(*[str(d).encode() for d in decks])
        opt = CafeOptions(device, active_capacity, grain_capacity, event_scan, event_fill_helper)
        check(self._lib.cafe_batch_create(arr, len(decks), ctypes.byref(opt), int(threads), ctypes.byref(self._h)))
        self.sims = [Simulation(None, _handle=self._lib.cafe_batch_sim(self._h, i)) for i in range(len(decks))]

    def run(self, max_steps=0):
        """Runs every realisation's loop to its end (or max_steps iterations
        each); returns the loop iterations of all realisations."""
        n = ctypes.c_longlong(0)
        check(self._lib.cafe_batch_run(self._h, int(max_steps), ctypes.byref(n)))
        return n.value

    def finished(self, i):
        return self._lib.cafe_batch_finished(self._h, i) == 1

    def report(self):
        """Batched launches: kernel launches and batch steps so far, and the
        autotuner's candidates and choice (cafe_batch_report)."""
        import json

        la, st = ctypes.c_longlong(0), ctypes.c_longlong(0)
        buf = ctypes.create_string_buffer(4096)
        check(self._lib.cafe_batch_report(self._h, ctypes.byref(la), ctypes.byref(st), buf, len(buf)))
        txt = buf.value.decode()
        return {"launches": la.value, "batch_steps": st.value, "tuning": json.loads(txt) if txt else None}

    def close(self):
        if self._h:
            for s in self.sims:
                s._h = ctypes.c_void_p()
            self._lib.cafe_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

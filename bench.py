#!/usr/bin/env python3
"""Throughput of AMCAFE's CA time step on GB300: voxel-updates per second.

One step is one iteration of the reference's time loop (main1.C:62-93:
AnalyticTempCurr + UpdateVoxels + UpdateLaser + layer bookkeeping) over the
whole voxel box; one voxel-update is one box voxel advanced one step, so
value = N_voxels * steps / time. The default workload is config 1
(512x256x128 voxels at 2.5 um, four layers, bidirectional hatching;
amcafe_gb300/decks/c1.in). Before timing, the run is advanced by --spinup
steps (part of setup, untimed) so that the melt pool, its liquid trail and the
solidification front are developed; then --warmup untimed steps; then --steps
timed steps. The voxel state (about 700 MB for config 1) is larger than L2.

Printed keys beyond the common contract:
  e2e        the same metric through the C ABI with host buffers: the state is
             uploaded from pinned host memory before the steps and downloaded
             after, and every step reads its summary (nGrain, flags) back to the
             host; it runs the timed window's steps first, then the engine
             is restored from a checkpoint taken one step before the window
             (in a temporary directory or /dev/shm, wherever it fits) and
             steps once, untimed, to the window's start for the device-timed
             steps; `wall` splits its time into upload, steps and download;
  roofline   for the phase with the largest device time in the timed region,
             its algorithmic bytes per launch over its mean launch time
             (CUDA events on the engine's stream), against the measured HBM
             copy bandwidth;
  event_cycles  SM cycles per capture/nucleation event of the timed steps,
             by section of the event loop (its own clock64 counters);
  cpu_baseline  the CPU oracle (a single-threaded restatement of the
             reference) resumed from the GPU state at the start of the timed
             window, for a bounded wall-clock sample.
`--impl reference` times the CPU restatement of the reference from the deck's
initial state (the reference's own CPU code path; no GPU work).
"""
import argparse
import json
import shutil
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (deck, default spin-up steps, description)
    "c1": ("amcafe_gb300/decks/c1.in", 2000, "config 1: 512x256x128 voxels @2.5um, 4 layers, hatching 100um"),
    "c2": ("amcafe_gb300/decks/c2.in", 1200, "config 2: 1024x1024x256 voxels @2.5um, 10 layers, 67 deg rotation"),
    "c0": ("amcafe_gb300/decks/c0.in", 300, "config 0: 128x64x32 voxels @2.5um, single track"),
    "c0e": ("amcafe_gb300/decks/c0_easm.in", 100, "config 0 geometry with the EASM temperature: 128x64x32 "
                                                   "voxels @2.5um, single track, 200 W"),
    "c3": (None, 0, "config 3: ensemble of single-track realisations, sides U(96,192) voxels @2.5um, "
                    "v U(0.5,1.5) m/s, P U(150,300) W, seeds 1..n, run batched on one GPU"),
}
ENSEMBLE_HOST_SEED = 20240603
ENSEMBLE_ACTIVE_CAPACITY = 1 << 18  # active cells per step of one realisation
FALLBACK_HBM_GBS = 6800.0
# EASM field: FP64 operations per quadrature node of Utilities::Integral as the
# kernel evaluates them with per-integral invariants hoisted (6 multiplies,
# 5 adds or subtracts, 3 divisions, the weighted accumulation's multiply and
# add, the final product, and exp counted as one), against the nominal FP64
# rate of GB300 in instructions (1.25 TFLOP/s counts an FMA as two flops;
# these operations are single instructions)
# the end-to-end run repeats the timed window from a checkpoint up to this
# many cells (config 1: 16.8 M, a 0.7 GB checkpoint); larger boxes time the
# steps that follow the timed window instead
E2E_REWIND_MAX = 1 << 31  # cells (the engine's limit)
# checkpoint file size per cell (gID 4, state 1, extent and centre 32, build
# flags 2, rounded up)
CKPT_BYTES_PER_CELL = 40
# host memory of one copy of the CPU restatement per cell (about 58 B measured
# on config 1)
REF_BYTES_PER_CELL = 64
# private memory of one copy resumed from shared read-only state files: the
# restatement's own fields (gID, vState, BuildjID 4 B each, extents 8,
# centroid 24, temperature 8) and per-step work arrays
REF_WINDOW_BYTES_PER_CELL = 60
EASM_OPS_PER_NODE = 18
EASM_NODES = 25
FP64_NOMINAL_GOPS = 625.0
BYTES_DENSE_PER_VOXEL = 2   # read + write of the uint8 cell state per voxel-update
BYTES_PER_FRONT_CELL = 74   # gID 4, extents 8, centroid 24, state 1; read and written


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist

    dist.init_process_group("gloo")
    return dist


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clock/throttle samples every 100 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                return float(v["value"] if isinstance(v, dict) else v), "measured"
    except Exception:
        pass
    return FALLBACK_HBM_GBS, "fallback"


def committed_traffic(workload, phase):
    """A figure from the committed ncu summaries (profiles/traffic.json), or
    None: under a phase's name its DRAM bytes per launch, under
    "<phase>_fp64_issue_frac" its FP64 issue rate on the SM it runs on."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(path))
        return d.get(workload, {}).get(phase)
    except Exception:
        return None


def committed_traffic_source(workload):
    """Where the committed figures of `workload` come from: the capture's
    command, the commit it measured and its date (profiles/traffic.json)."""
    src = committed_traffic(workload, "_source")
    if src is None:
        return None
    return dict(src, note="from a committed ncu capture, not measured in this run")


def cpu_baseline(deck, info, state, ctheta, nvox, seconds):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cafe_oracle as orc

    orc.set_budget(seconds)
    _, sec, st = orc.run_window(deck, info, state, ctheta, 1 << 30, libm=orc.LIBM_GLIBC)
    orc.set_budget(0)
    steps = st["steps"]
    return {"value": nvox * steps / sec if sec > 0 else None, "unit": "voxel-updates/s", "cores": 1,
            "kind": "port",
            "sample": "%d steps from step %d of the same run (GPU state handed over), one thread, "
                      "glibc libm, %.1f s" % (steps, info["steps"], sec)}


def _ref_sample(a):
    """One single-thread run of the CPU restatement from the deck's start, for
    at most `budget` seconds of loop time (a spawned worker of run_reference)."""
    deck, nsteps, budget = a
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cafe_oracle as orc

    orc.set_budget(budget)
    st = orc.run(deck, "", max_steps=nsteps, dump_stride=0, libm=orc.LIBM_GLIBC)
    orc.set_budget(0)
    return st["steps"], st["loop_ns"] * 1e-9, st["ncell"]


STATE_FIELDS = ("gID", "vState", "extents", "centroid", "buildj")


def _spinup_state(a):
    """Untimed set-up of the reference arm (a spawned child, so that no CUDA
    context outlives it): the engine runs the deck to the first step of the
    timed window and writes the state there as .npy files plus info.json."""
    deck, nsteps, device, outdir = a
    sys.path.insert(0, ROOT)
    import numpy as np

    from amcafe_gb300 import Simulation

    with Simulation(deck, device=device) as sim:
        sim.InitializeVoxels()
        sim.begin()
        if nsteps > 0:
            sim.run(nsteps)
        sim.synchronize()
        info = sim.info()
        st = sim.state()
        for k in STATE_FIELDS:
            np.save(os.path.join(outdir, k + ".npy"), st[k])
        np.save(os.path.join(outdir, "ctheta.npy"), sim.ctheta())
    with open(os.path.join(outdir, "info.json"), "w") as fh:
        json.dump({k: (v if not hasattr(v, "item") else v.item()) for k, v in info.items()}, fh)
    return info["steps"]


def _ref_window_sample(a):
    """One single-thread copy of the CPU restatement resumed from the state
    files of _spinup_state (read-only maps shared by all copies): up to
    `nsteps` steps within `budget` seconds of loop time."""
    deck, statedir, nsteps, budget = a
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np

    import cafe_oracle as orc

    info = json.load(open(os.path.join(statedir, "info.json")))
    state = {k: np.load(os.path.join(statedir, k + ".npy"), mmap_mode="r") for k in STATE_FIELDS}
    cth = np.load(os.path.join(statedir, "ctheta.npy"))
    orc.set_budget(budget)
    _, sec, stats = orc.run_window(deck, info, state, cth, nsteps, libm=orc.LIBM_GLIBC, copy=False)
    orc.set_budget(0)
    return stats["steps"], sec, stats["ncell"], stats["events"]


def _deck_cells(deck):
    for line in open(deck):
        f = line.split("#")[0].split()
        if len(f) >= 4 and f[0].lower() == "nx":
            return int(f[1]) * int(f[2]) * int(f[3])
    return None


def _mem_available():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except Exception:
        pass
    return None


def _host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _ref_copies(ncell, requested, bytes_per_cell=None, shared_bytes=0):
    """How many copies of the CPU run to start: one per host core (or the
    requested number), within 85 % of the available memory (less
    `shared_bytes` of shared state files) at `bytes_per_cell` each (half of it
    at REF_BYTES_PER_CELL when not given)."""
    cores = _host_cores()
    n = cores if not requested or requested <= 0 else min(requested, cores)
    avail = _mem_available()
    if avail is None or not ncell:
        return 1
    if bytes_per_cell is None:
        return max(1, min(n, int(0.5 * avail // (REF_BYTES_PER_CELL * ncell))))
    return max(1, min(n, int(0.85 * (avail - shared_bytes) // (bytes_per_cell * ncell))))


def _state_dir(nbytes):
    """A scratch directory with room for `nbytes` of state files."""
    for base in (None, "/dev/shm"):
        try:
            d = tempfile.mkdtemp(prefix="cafe_refstate_", dir=base)
        except Exception:
            continue
        if shutil.disk_usage(d).free > 1.1 * nbytes:
            return d
        shutil.rmtree(d, ignore_errors=True)
    return None


def _gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    import multiprocessing as mp

    deck_rel, spin_default, desc = WORKLOADS[args.workload]
    deck = os.path.join(ROOT, deck_rel)
    spinup = spin_default if args.spinup is None else args.spinup
    start = spinup + args.warmup  # first step of the other arm's timed window
    budget = args.ref_seconds
    ncell = _deck_cells(deck)
    t_wall0 = time.time()
    ctx = mp.get_context("spawn")
    statedir = None
    if start > 0 and _gpu_available():
        statedir = _state_dir(48 * ncell)
    if statedir is not None:
        # the same window as the other arm: the state at its first step is
        # computed by the engine (untimed set-up, in a child process that
        # exits before the CPU copies start), then every host core runs a
        # single-thread copy of the CPU restatement of the reference over the
        # same steps from that state
        with ctx.Pool(1) as pool:
            reached = pool.apply(_spinup_state, ((deck, start, 0, statedir),))
        shared = sum(os.path.getsize(os.path.join(statedir, f)) for f in os.listdir(statedir))
        ncopy = _ref_copies(ncell, getattr(args, "ref_copies", 0), bytes_per_cell=REF_WINDOW_BYTES_PER_CELL,
                            shared_bytes=shared)
        job = (deck, statedir, args.steps, budget)
        with ctx.Pool(ncopy) as pool:
            res = pool.map(_ref_window_sample, [job] * ncopy)
        shutil.rmtree(statedir, ignore_errors=True)
        window = "steps %d..%d, the other arm's timed window" % (reached + 1, reached + min(r[0] for r in res))
        sample = ("%d single-thread copies at once (one per host core within 85%% of the free memory), each "
                  "resumed from the state at step %d (computed by the engine as untimed set-up) for up to %d steps "
                  "or %.0f s of loop time, glibc libm; value = the copies' summed throughput (what as many "
                  "MPI ranks would reach at perfect scaling)" % (ncopy, reached, args.steps, budget))
    else:
        # no GPU for the set-up: the loop from the deck's initial state
        ncopy = _ref_copies(ncell, getattr(args, "ref_copies", 0))
        job = (deck, max(1, args.warmup + args.steps), budget)
        if ncopy == 1:
            res = [_ref_sample(job)]
        else:
            with ctx.Pool(ncopy) as pool:
                res = pool.map(_ref_sample, [job] * ncopy)
        reached = 0
        window = "first %d steps from the deck's initial state" % min(r[0] for r in res)
        sample = ("steps 1..%d of %s from its initial state, %d single-thread copies at once (one per host core "
                  "within half the free memory), glibc libm, up to %.1f s loop time each (init excluded); value = "
                  "the copies' summed throughput" % (min(r[0] for r in res), args.workload, ncopy,
                                                      max(r[1] for r in res)))
    steps_total = min(r[0] for r in res)
    nvox = res[0][2]
    rates = [nvox * r[0] / r[1] for r in res if r[1] > 0]
    value = sum(rates) if rates else None
    out = {
        "impl": "reference",
        "metric": "voxel-updates/s",
        "value": value,
        "unit": "voxel-updates/s",
        "n_gpus": ws,
        "steps": steps_total,
        "warmup": 0,
        "ms_per_step": 1e3 * sum(r[1] / max(1, r[0]) for r in res) / len(res),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded Voronoi microstructure and laser path from the deck)",
        "config": {"workload": args.workload, "deck": deck_rel, "description": desc, "voxels": nvox,
                   "window_start_step": reached, "window": window},
        "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": ncopy, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.time() - t_wall0,
    }
    print(json.dumps(out))
    return 0


def _final_digest(sim):
    import hashlib

    st = sim.state()
    h = hashlib.sha256()
    for k in ("gID", "vState", "extents", "centroid", "buildj"):
        h.update(st[k].tobytes())
    h.update(sim.ctheta().tobytes())
    return h.hexdigest()


def _track_steps(deck):
    """Loop iterations of a one-layer single-track deck: its Nsd laser points
    (Grid.C:83) less the one the first UpdateLaser takes before the time loop
    (main1.C:61); on the 64 decks of config 3 their sum equals the engine's
    38,643 iterations."""
    import math

    g = {}
    for line in open(deck):
        f = line.split("#")[0].split()
        if f:
            g[f[0].lower()] = f[1:]
    gs, v, dt = float(g["gridsize"][0]), float(g["bmv"][0]), float(g["bmdelt"][0])
    return int(math.ceil(gs / (v * dt)))


def run_reference_ensemble(args, ws, rank):
    """Config 3 on the CPU restatement: one copy per host core (within the
    memory cap), copy i running realisation i+1 from its deck for a bounded
    sample; runs/s is the sum over copies of completed fraction / loop time."""
    if rank != 0:
        return 0
    from amcafe_gb300.ensemble import make_decks

    t_wall0 = time.time()
    work = tempfile.mkdtemp(prefix="cafe_ens_ref_")
    n = args.realisations
    decks = make_decks(work, n=n, sides=(96, 192), host_seed=ENSEMBLE_HOST_SEED)
    ncopy = _ref_copies(max(_deck_cells(d) for d in decks), getattr(args, "ref_copies", 0))
    jobs = [(decks[i % n], -1, args.ref_seconds) for i in range(ncopy)]
    if ncopy == 1:
        res = [_ref_sample(jobs[0])]
    else:
        import multiprocessing as mp

        with mp.get_context("spawn").Pool(ncopy) as pool:
            res = pool.map(_ref_sample, jobs)
    rates = [(r[0] / _track_steps(j[0])) / r[1] for r, j in zip(res, jobs) if r[1] > 0]
    value = sum(rates) if rates else None
    steps_done = sum(r[0] for r in res)
    out = {
        "impl": "reference",
        "metric": "runs/s",
        "value": value,
        "unit": "runs/s",
        "n_gpus": ws,
        "steps": steps_done,
        "warmup": 0,
        "ms_per_step": 1e3 * sum(r[1] / max(1, r[0]) for r in res) / len(res),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded decks from amcafe_gb300.ensemble, host seed %d)" % ENSEMBLE_HOST_SEED,
        "config": {"workload": "c3", "description": WORKLOADS["c3"][2], "realisations": n},
        "cpu_baseline": {"value": value, "unit": "runs/s", "cores": ncopy, "kind": "port",
                         "sample": "realisations 1..%d, one single-thread copy each at once (one per host core "
                                   "within half the free memory), glibc libm, up to %.1f s loop time each "
                                   "(initialisation excluded); runs/s = the copies' summed completed fraction / "
                                   "time" % (ncopy, max(r[1] for r in res))},
        "e2e": {"value": value, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": time.time() - t_wall0,
    }
    print(json.dumps(out))
    shutil.rmtree(work, ignore_errors=True)
    return 0


def run_ensemble(args, ws, rank, local):
    """Config 3: runs/s of whole realisations (initialisation, the full loop
    and the closing CleanLayer), batched (cafe_batch_*) against the same
    realisations run one after another through the plain API. Each rank runs
    its own ensemble (replicas); rank 0 prints."""
    import torch

    from amcafe_gb300 import Batch, Simulation
    from amcafe_gb300.ensemble import make_decks

    dist = init_dist(ws)
    n = args.realisations
    work = tempfile.mkdtemp(prefix="cafe_ens_")
    decks = make_decks(work, n=n, sides=(96, 192), host_seed=ENSEMBLE_HOST_SEED)
    cap = ENSEMBLE_ACTIVE_CAPACITY
    # warm-up: context, allocator and code paths on three small realisations
    wdecks = make_decks(os.path.join(work, "warm"), n=3, sides=(24, 32), host_seed=1)
    for _ in range(args.warmup):
        with Batch(wdecks, device=local, active_capacity=cap) as wb:
            wb.run()
    torch.cuda.synchronize(local)
    # ---- batched (timed): all realisations in one batch
    clocks = ClockSampler(local)
    barrier(dist)
    clocks.start()
    t0 = time.time()
    b = Batch(decks, device=local, threads=args.threads, active_capacity=cap)
    iters = b.run()
    torch.cuda.synchronize(local)
    batch_s = time.time() - t0
    clk = clocks.stop()
    batch_s = reduce_max(dist, batch_s)
    digests_b = [_final_digest(s) for s in b.sims]
    nvox = [s.ncell for s in b.sims]
    steps_each = [s.info()["steps"] for s in b.sims]
    report = b.report()
    # the realisations' own launches (initialisation, layer work, plain steps)
    # and the batched launches (one per step kernel for all realisations)
    launches = sum(s.stats()["launches"] for s in b.sims) + report["launches"]
    threads = min(args.threads, n) if args.threads > 0 else 0  # 0: batched launches
    b.close()
    # ---- sequential plain runs of the same realisations (bounded by --seq-seconds)
    seq_s, seq_done, same = 0.0, 0, True
    for i, d in enumerate(decks):
        if seq_s > args.seq_seconds:
            break
        t1 = time.time()
        with Simulation(d, device=local, active_capacity=cap) as sim:
            sim.InitializeVoxels()
            sim.begin()
            sim.run()
            sim.synchronize()
            seq_s += time.time() - t1
            same = same and _final_digest(sim) == digests_b[i]
        seq_done += 1
    seq_rate = seq_done / seq_s if seq_s > 0 else None
    # ---- CPU baseline: the oracle on realisation 1 for a bounded sample
    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import cafe_oracle as orc

        orc.set_budget(args.cpu_seconds)
        st = orc.run(decks[0], "", max_steps=-1, dump_stride=0, libm=orc.LIBM_GLIBC)
        orc.set_budget(0)
        sec = st["loop_ns"] * 1e-9
        frac = st["steps"] / max(1, steps_each[0])
        cpu = {"value": frac / sec if sec > 0 else None, "unit": "runs/s", "cores": 1, "kind": "port",
               "sample": "realisation 1 (%d voxels): %d of its %d steps in %.1f s, one thread, glibc libm; "
                         "runs/s = completed fraction / time (initialisation excluded)"
                         % (nvox[0], st["steps"], steps_each[0], sec)}
    if rank == 0:
        value = ws * n / batch_s
        out = {
            "metric": "runs/s",
            "value": value,
            "unit": "runs/s",
            "n_gpus": ws,
            "steps": int(iters),
            "warmup": args.warmup,
            "ms_per_step": 1e3 * batch_s / max(1, max(steps_each)),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded decks from amcafe_gb300.ensemble, host seed %d)" % ENSEMBLE_HOST_SEED,
            "config": {"workload": "c3", "description": WORKLOADS["c3"][2], "realisations": n,
                       "voxels_total": int(sum(nvox)), "voxels_min": int(min(nvox)), "voxels_max": int(max(nvox)),
                       "host_threads": int(threads), "active_capacity": cap,
                       "l2": "each realisation's state larger than L2 or not: timing is whole runs",
                       "parallelism": "batch%d" % n},
            "sequential": {"value": seq_rate, "unit": "runs/s", "runs": seq_done, "seconds": seq_s},
            "speedup_vs_sequential": (value / ws) / seq_rate if seq_rate else None,
            "bitexact_vs_sequential": same,
            "voxel_updates_per_s": ws * sum(v * k for v, k in zip(nvox, steps_each)) / batch_s,
            "e2e": {"value": value, "unit": "runs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "whole runs from the decks: wall time of the batch including initialisation"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
            "batched": {"batch_steps": report["batch_steps"], "launches": report["launches"],
                        "autotuner": report["tuning"]},
            "wall_s_timed": batch_s,
        }
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--spinup", type=int, default=None)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-seconds", type=float, default=300.0)
    ap.add_argument("--ref-copies", type=int, default=0, help="copies of the reference arm's CPU run (0: one per core)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--realisations", type=int, default=64)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--seq-seconds", type=float, default=150.0)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist_env()
    if args.workload == "c3":
        if args.impl == "reference":
            return run_reference_ensemble(args, ws, rank)
        return run_ensemble(args, ws, rank, local)
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    dist = init_dist(ws)
    from amcafe_gb300 import Simulation

    deck_rel, spin_default, desc = WORKLOADS[args.workload]
    deck = os.path.join(ROOT, deck_rel)
    spinup = spin_default if args.spinup is None else args.spinup
    t_setup = time.time()
    sim = Simulation(deck, device=local)
    sim.InitializeVoxels()
    sim.begin()
    if spinup > 0:
        sim.run(spinup)
    nvox = sim.ncell
    # a checkpoint one step before the timed window (before the last warm-up
    # step), in a temporary directory or /dev/shm, wherever it fits: the
    # end-to-end leg runs the window first, then the engine is rewound there
    # and that one step, whose full passes a restore entails, stays untimed
    ckpt = None
    ckpt_dir = _state_dir(CKPT_BYTES_PER_CELL * nvox) if not args.no_e2e and nvox <= E2E_REWIND_MAX else None
    for i in range(args.warmup):
        if i == args.warmup - 1 and ckpt_dir is not None:
            sim.synchronize()
            ckpt = os.path.join(ckpt_dir, "window.ckpt")
            try:
                sim.checkpoint(ckpt)
            except Exception as exc:  # e.g. no room for the file: time the following steps instead
                print("bench: no checkpoint for the end-to-end run (%s)" % exc, file=sys.stderr)
                shutil.rmtree(ckpt_dir, ignore_errors=True)
                ckpt = ckpt_dir = None
        sim.step()
    sim.synchronize()
    setup_s = time.time() - t_setup
    info0 = sim.info()
    # the state at the start of the timed window, in pinned host memory (the
    # end-to-end run uploads it)
    st_host = cth_host = None
    if not args.no_e2e or (rank == 0 and not args.no_cpu):
        import torch

        def pinned(n, dt):
            return torch.empty(n, dtype=dt, pin_memory=True).numpy()

        ncell = sim.ncell
        st_host = sim.state(out=dict(gID=pinned(ncell, torch.int32), vState=pinned(ncell, torch.int32),
                                     extents=pinned(ncell, torch.float64),
                                     centroid=pinned(3 * ncell, torch.float64),
                                     buildj=pinned(ncell, torch.int32)))
        # the grain table too, in pinned memory (a pageable host buffer makes
        # the driver stage the copy and block)
        cth = sim.ctheta()
        cth_host = pinned(len(cth), torch.float64)
        cth_host[:] = cth

    def run_e2e(window):
        """The end-to-end leg through the C ABI with host buffers: upload of
        st_host, args.steps steps with each step's summary read back, download
        into st_host; wall clock."""
        h2d = sum(a.nbytes for a in (st_host["gID"], st_host["vState"], st_host["extents"], st_host["centroid"])) \
            + cth_host.nbytes
        d2h = h2d - cth_host.nbytes + st_host["buildj"].nbytes
        ke = args.steps
        sim.synchronize()
        e2e_start = sim.info()["steps"]
        ev_e0 = sim.stats()["events"]
        barrier(dist)
        te0 = time.time()
        sim.upload_state(st_host["gID"], st_host["vState"], st_host["extents"], st_host["centroid"], cth_host)
        te1 = time.time()  # (the upload returns after its copies completed)
        n_e, done_e = 0, False
        per_step_d2h = 0
        while n_e < ke and not done_e:
            done_e = sim.step()
            sim.info()  # per-step result read back to the host
            per_step_d2h += 8
            n_e += 1
        sim.synchronize()
        te2 = time.time()
        sim.state(out=st_host)
        te = time.time() - te0
        te_parts = {"upload_s": round(te1 - te0, 4), "steps_s": round(te2 - te1, 4),
                    "download_s": round(te0 + te - te2, 4)}
        te = reduce_max(dist, te)
        return {"value": ws * nvox * n_e / te, "unit": "voxel-updates/s",
                "h2d_bytes_per_step": int(h2d / max(1, n_e)),
                "d2h_bytes_per_step": int(d2h / max(1, n_e) + per_step_d2h / max(1, n_e)),
                "steps": n_e, "window_start_step": e2e_start, "window": window,
                "events_per_step": (sim.stats()["events"] - ev_e0) / max(1, n_e), "wall": te_parts}

    # ---- end to end first, from the window's start (host-to-device copies on
    # the box run slowly for a while after a restore or a large host copy),
    # then back to the step before the window (restore) and one untimed step
    # to the window's start for the device-timed steps
    e2e = None
    if ckpt is not None:
        e2e = run_e2e("the timed window, run before it (then rewound from a checkpoint)")
        sim.restore(ckpt)
        os.unlink(ckpt)
        ckpt = None
        sim.step()  # to the window's start again, untimed
        sim.synchronize()
        if sim.info()["steps"] != info0["steps"]:
            raise RuntimeError("bench: the rewind did not reach the window's start")
        st_host = sim.state(out=st_host)  # the window's start (the CPU baseline's input)
        sim.synchronize()
    snapshot = None
    if rank == 0 and not args.no_cpu:
        snapshot = (info0, st_host, cth_host)

    # ---- timed region: device time between two events on the engine's stream
    # (the product path: each step is the step's CUDA graph)
    stats0 = sim.stats()
    sim.phase_times(reset=True)
    clocks = ClockSampler(local)
    barrier(dist)
    sim.synchronize()
    clocks.start()
    import torch

    torch.cuda.profiler.start()  # the timed steps are the range a profiler captures (no-op otherwise)
    sim.mark(0)
    t0 = time.time()
    done = False
    k = 0
    while k < args.steps and not done:
        done = sim.step()
        k += 1
    sim.mark(1)
    torch.cuda.profiler.stop()
    ms = sim.elapsed_ms(0, 1)
    sim.synchronize()
    wall = time.time() - t0
    clk = clocks.stop()
    stats1 = sim.stats()
    launches = int(stats1["launches"])  # counted since the reset before the timed steps
    ms = reduce_max(dist, ms)
    barrier(dist)
    value = ws * nvox * k / (ms * 1e-3)

    # ---- phase breakdown: the next steps again with CUDA events around each
    # phase (ungraphed launches), for the roofline of the dominant phase
    kp = 0
    if not done:
        sim.set_timing(True)
        sim.phase_times(reset=True)
        statsp0 = sim.stats()
        while kp < min(args.steps, 20) and not done:
            done = sim.step()
            kp += 1
        phases = sim.phase_times()
        statsp1 = sim.stats()
        sim.set_timing(False)
    if kp == 0:
        phases, statsp0, statsp1 = {"events": (ms, k)}, stats0, stats1

    # ---- roofline of the dominant phase
    peak, peak_src = hbm_peak()
    dom = max(phases, key=lambda p: phases[p][0])
    dom_ms, dom_launches = phases[dom]
    steps_done = max(1, statsp1["steps"] - statsp0["steps"])
    avg_na = (statsp1["sum_active"] - statsp0["sum_active"]) / steps_done
    if dom in ("events", "writeback", "gather"):
        bytes_per_launch = BYTES_PER_FRONT_CELL * avg_na
    else:
        bytes_per_launch = BYTES_DENSE_PER_VOXEL * nvox
    launches_dom = max(1, dom_launches)
    per_launch_ms = dom_ms / launches_dom if dom != "events" else dom_ms / steps_done
    achieved = bytes_per_launch / (per_launch_ms * 1e-3) / 1e9
    avg_na_timed = (stats1["sum_active"] - stats0["sum_active"]) / max(1, stats1["steps"] - stats0["steps"])
    step_bytes = BYTES_DENSE_PER_VOXEL * nvox + BYTES_PER_FRONT_CELL * avg_na_timed
    easm = "easm" in open(deck).read().lower()
    if easm and dom == "melt":
        # the EASM field (k_easm) is FP64-bound: operations per step over its time
        integrals = (statsp1["easm_integrals"] - statsp0["easm_integrals"]) / steps_done
        ops = integrals * EASM_NODES * EASM_OPS_PER_NODE
        achieved = ops / (dom_ms / steps_done * 1e-3) / 1e9
        roofline = {"bound": "fp64", "achieved": achieved, "peak": FP64_NOMINAL_GOPS, "unit": "GOP/s",
                    "frac": achieved / FP64_NOMINAL_GOPS, "traffic": committed_traffic(args.workload, dom),
                    "kernel": "k_easm", "phase": dom, "phase_steps": kp,
                    "peak_source": "nominal FP64 rate in instructions (1.25 TFLOP/s with an FMA as two flops)",
                    "integrals_per_step": integrals, "ops_per_node": EASM_OPS_PER_NODE}
    else:
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": committed_traffic(args.workload, dom),
                    "traffic_source": committed_traffic_source(args.workload),
                    "kernel": {"events": "k_event_loop", "classify": "k_active_count/k_active_scatter",
                               "gather": "k_gather", "melt": "k_melt", "writeback": "k_writeback"}.get(dom, dom),
                    "phase": dom, "peak_source": peak_src,
                    "phase_steps": kp,
                    "step_achieved_GBs": step_bytes * k / (ms * 1e-3) / 1e9}
        fp64 = committed_traffic(args.workload, dom + "_fp64_issue_frac")
        if fp64 is not None:
            # the serial loop runs on one SM: its FP64 issue rate there against
            # that SM's peak (ncu, sm__inst_executed_pipe_fp64, profiles/)
            roofline["sm_fp64_issue_frac_ncu"] = fp64

    cpu = None
    if snapshot is not None:
        cpu = cpu_baseline(deck, snapshot[0], snapshot[1], snapshot[2], nvox, args.cpu_seconds)

    # ---- end to end without a checkpoint: the steps after the timed ones,
    # from the state reached there
    if e2e is None and not args.no_e2e and not done:
        st_host = sim.state(out=st_host)
        cth = sim.ctheta()
        cth_host = pinned(len(cth), torch.float64)
        cth_host[:] = cth
        e2e = run_e2e("the steps after the timed and phase-timing steps")
    if ckpt_dir is not None:
        shutil.rmtree(ckpt_dir, ignore_errors=True)
    if rank == 0:
        ev = stats1["events"] - stats0["events"]
        out = {
            "metric": "voxel-updates/s",
            "value": value,
            "unit": "voxel-updates/s",
            "n_gpus": ws,
            "steps": k,
            "warmup": args.warmup,
            "ms_per_step": ms / k,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded Voronoi microstructure and laser path from the deck)",
            "config": {"workload": args.workload, "deck": deck_rel, "description": desc,
                       "voxels": nvox, "spinup_steps": spinup, "window_start_step": info0["steps"],
                       "l2": "state larger than L2 (inputs > 129 MB)",
                       "parallelism": "replicas%d" % ws},
            "e2e": e2e,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
            "events_per_step": ev / max(1, k),
            # the event loop's own clock (thread 0 of its block), SM cycles per
            # capture/nucleation event in the timed steps, by section
            "event_cycles": {sec: round((stats1["cycles_" + key] - stats0["cycles_" + key]) / max(1, ev))
                             for sec, key in (("winner", "select"), ("capture", "apply"),
                                              ("fill_and_next_selection", "fill"), ("merge", "merge"))},
            "phase_ms": {p: round(v[0], 3) for p, v in phases.items()},
            "wall_s_timed": wall,
            "setup_s": setup_s,
        }
        print(json.dumps(out))
    sim.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

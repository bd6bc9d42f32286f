"""Gradients of the smooth part of the CA step (no counterpart in the reference).

With the capture and nucleation events held fixed, the CA's growth is the
time integral of the octahedron growth v = a dT^n of each frontier cell over
the event times it grew through (VoxelsCA.C:405, 511-516). The CA itself runs
under the Rosenthal moving point source (deck keyword "rosenthal"), so the
temperature field the adjoint differentiates is the one that decided the
events. `GrowthRun` runs the CA once at given parameters theta = (P, eta, v,
a, n) (written into the deck: bmP, the rosenthal absorptivity, bmV,
dendritegrowth2), keeping a checkpoint (cafe_sim_checkpoint) every `segment`
steps; evaluating the summed growth or its gradient replays one segment at a
time from its checkpoint with the growth log on (cafe_sim_set_growth_log), so
only one segment's log is held at a time. The melt-pool length, width and
depth come from the moments of the soft melt indicator of the same field
(cafe_adjoint_pool). Values and vector-Jacobian products are hand-written CUDA
kernels (csrc/cafe_adjoint.cu); `Objective` exposes them to torch.autograd.

`ca_target` runs the CA at hidden parameters and gives its outputs (its own
field's pool, its own summed growth) together with the run, whose event set
`calibrate` then holds fixed while it fits the parameters. The frozen event
set is what makes the growth-law coefficient identifiable: re-running the CA
at each estimate moves the capture times with the growth speed (a faster
growth reaches each capture sooner), so the summed growth of a fresh run
hardly changes with a. Only eta P enters the temperature, so P and eta are not
separately identifiable from these outputs either; P (eta fixed) and a are
fitted.
"""
import ctypes
import os
import re
import shutil
import tempfile

import numpy as np
import torch

from ._native import CafeAdjointSetup, check, load
from .cafe import Simulation


def _f64p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def deck_with_theta(deck, theta, path):
    """Writes `deck` with theta = (P, eta, v, a, n) as bmP, the absorptivity
    of the rosenthal keyword, bmV and dendritegrowth2 into `path`."""
    P, eta, v, a, n = (float(x) for x in theta)
    src = open(deck).read()
    if not re.search(r"(?mi)^\s*rosenthal\s", src):
        raise ValueError("%s: the adjoint needs the Rosenthal temperature (deck keyword rosenthal)" % deck)

    def sub(key, repl, text):
        out, k = re.subn(r"(?mi)^(\s*%s)\s+[^\n#]*" % key, lambda m: m.group(1) + " " + repl, text)
        if k != 1:
            raise ValueError("%s: keyword %s must appear once" % (deck, key))
        return out

    src = sub("bmP", repr(P), src)
    src = sub("bmV", repr(v), src)
    src = sub("dendritegrowth2", "%r %r" % (a, n), src)
    m = re.search(r"(?mi)^\s*rosenthal\s+(\S+)\s+(\S+)\s+(\S+)", src)
    src = sub("rosenthal", "%r %s %s" % (eta, m.group(2), m.group(3)), src)
    with open(path, "w") as f:
        f.write(src if src.endswith("\n") else src + "\n")
    return path


class GrowthRun:
    """The CA run of `deck` at theta (default: the deck's own parameters): after
    `spinup` steps (run, not logged), a window of `nsteps` steps with
    checkpoints every `segment`, whose event set the adjoint holds fixed."""

    def __init__(self, deck, nsteps, segment=32, device=0, tau_T=10.0, log_capacity=1 << 22, workdir=None,
                 theta=None, spinup=0):
        self.segment, self.device = int(segment), device
        self._lib = load()
        self._dir = tempfile.mkdtemp(prefix="cafe_adj_", dir=workdir)
        self.deck = str(deck)
        if theta is not None:
            self.deck = deck_with_theta(deck, theta, os.path.join(self._dir, "theta.in"))
        self.checkpoints = []  # (path, steps in the segment)
        sim = Simulation(self.deck, device=device)
        sim.InitializeVoxels()
        sim.begin()
        g0 = sim.grid()
        if spinup > 0:
            sim.run(int(spinup))
        self.spinup = sim.info()["steps"]
        done, k = sim.info()["done"] != 0, 0
        while k < nsteps and not done:
            path = os.path.join(self._dir, "seg%05d.ckpt" % len(self.checkpoints))
            sim.checkpoint(path)
            m = 0
            while m < self.segment and k < nsteps and not done:
                done = sim.step()
                m += 1
                k += 1
            self.checkpoints.append((path, m))
        self.nsteps = k
        self.step_final = sim.info()["tInd"] - 1
        self.stats = sim.stats()
        sim.close()
        self.theta = np.array([g0["bmP"], g0["ros_eta"], g0["bmV"], g0["Avel"], g0["nvel"]])
        self._sim = Simulation(self.deck, device=device)  # replays segments
        dev = torch.device("cuda", device)
        self._cells = torch.empty(log_capacity, dtype=torch.int32, device=dev)
        self._steps = torch.empty(log_capacity, dtype=torch.int32, device=dev)
        self._tau = torch.empty(log_capacity, dtype=torch.float64, device=dev)
        self._cap = log_capacity
        self.setup = self._make_setup(g0, tau_T)

    def _make_setup(self, g, tau_T):
        """The adjoint's source path from the engine's own laser state at the
        first step: a track along +x of an unrotated laser frame, source at
        laser + (v t, 0, 0) at t = tInd dt."""
        if g["tmodel"] != 2:
            raise ValueError("the adjoint needs the Rosenthal temperature (deck keyword rosenthal)")
        if g["gth"] != 0.0 or not g["dirp"] > 0:
            raise ValueError("the adjoint's source path is a track along +x of an unrotated laser frame")
        s = CafeAdjointSetup()
        s.k, s.alpha, s.T0 = g["ros_k"], g["ros_alpha"], g["T0"]
        s.Tl = g["tL"]
        s.tau_T = tau_T
        s.dt = g["DelT"]
        s.x_start = g["laser"][0] - g["bmV"] * (g["tInd"] * s.dt)
        s.y_src = g["laser"][1]
        s.z_src = g["laser"][2]
        s.dx = g["dX"][0]
        s.nx, s.ny, s.nz = g["nX"]
        s.step_final = self.step_final
        return s

    def _replay(self, i):
        """Recomputes segment i with the growth log on; returns its entry count."""
        path, m = self.checkpoints[i]
        sim = self._sim
        # (the same arrays every time: the step graph captured with them stays valid)
        check(self._lib.cafe_sim_set_growth_log(sim._h, self._cells.data_ptr(), self._steps.data_ptr(),
                                                self._tau.data_ptr(), self._cap))
        sim.restore(path)
        for _ in range(m):
            if sim.step():
                break
        n = ctypes.c_longlong(0)
        check(self._lib.cafe_sim_growth_log_count(sim._h, ctypes.byref(n)))
        return n.value

    def growth(self, theta, cot=None):
        """(G, cot * dG/dtheta or None), replaying the segments."""
        th = np.ascontiguousarray(theta, np.float64)
        G, grad = 0.0, np.zeros(5)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        for i in range(len(self.checkpoints)):
            n = self._replay(i)
            out = ctypes.c_double(0)
            g = np.zeros(5)
            check(self._lib.cafe_adjoint_growth(ctypes.byref(self.setup), _f64p(th), self._cells.data_ptr(),
                                                self._steps.data_ptr(), self._tau.data_ptr(), n,
                                                float(cot) if cot is not None else 0.0, ctypes.byref(out),
                                                _f64p(g) if cot is not None else None, stream))
            G += out.value
            grad += g
        return G, (grad if cot is not None else None)

    def log(self):
        """The whole growth log (cells, steps, tau) as numpy arrays, segment by segment."""
        parts = []
        for i in range(len(self.checkpoints)):
            n = self._replay(i)
            parts.append((self._cells[:n].cpu().numpy(), self._steps[:n].cpu().numpy(), self._tau[:n].cpu().numpy()))
        return tuple(np.concatenate([p[q] for p in parts]) for q in range(3))

    def pool(self, theta, cot=None):
        th = np.ascontiguousarray(theta, np.float64)
        out, g = np.zeros(3), np.zeros(5)
        c = np.ascontiguousarray(cot, np.float64) if cot is not None else None
        stream = torch.cuda.current_stream(self.device).cuda_stream
        check(self._lib.cafe_adjoint_pool(ctypes.byref(self.setup), _f64p(th), _f64p(c) if c is not None else None,
                                          _f64p(out), _f64p(g) if c is not None else None, stream))
        return out, (g if c is not None else None)

    def setup_dict(self):
        return {f: getattr(self.setup, f) for f, _ in CafeAdjointSetup._fields_}

    def close(self):
        if self._sim is not None:
            self._sim.close()
            self._sim = None
        shutil.rmtree(self._dir, ignore_errors=True)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Objective(torch.autograd.Function):
    """theta (5 doubles: P, eta, v, a, n) -> (length, width, depth, G)."""

    @staticmethod
    def forward(ctx, theta, run):
        th = theta.detach().cpu().numpy()
        pool, _ = run.pool(th)
        G, _ = run.growth(th)
        ctx.run = run
        ctx.save_for_backward(theta)
        return torch.tensor([pool[0], pool[1], pool[2], G], dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (theta,) = ctx.saved_tensors
        th = theta.detach().cpu().numpy()
        go = gout.detach().cpu().numpy()
        _, gp = ctx.run.pool(th, cot=go[:3])
        _, gg = ctx.run.growth(th, cot=go[3])
        return torch.tensor(gp + gg, dtype=theta.dtype), None


def calibrate(run, target, theta0, free=(0, 3), iters=30):
    """Recovers the parameters listed in `free` (indices into theta) from target
    outputs (length, width, depth, G) by L-BFGS on their logarithms, minimising
    the summed squared relative errors; returns (theta, loss history)."""
    theta0 = torch.tensor(theta0, dtype=torch.float64)
    logp = torch.log(theta0[list(free)]).clone().requires_grad_(True)
    tgt = torch.tensor(target, dtype=torch.float64)
    opt = torch.optim.LBFGS([logp], lr=1.0, max_iter=iters, tolerance_grad=1e-14, tolerance_change=1e-16,
                            line_search_fn="strong_wolfe")
    hist = []

    def closure():
        opt.zero_grad()
        th = theta0.clone()
        th[list(free)] = torch.exp(logp)
        out = Objective.apply(th, run)
        loss = torch.sum(((out - tgt) / tgt) ** 2)
        loss.backward()
        hist.append(float(loss.detach()))
        return loss

    opt.step(closure)
    th = theta0.clone()
    th[list(free)] = torch.exp(logp.detach())
    return th.numpy(), hist


def ca_target(deck, nsteps, theta, segment=32, device=0, spinup=0):
    """A CA run at theta and its outputs (length, width, depth, G): the pool of
    its own temperature field at the last step and the summed growth over its
    own event set in the window after `spinup` steps. Returns (outputs, run);
    the caller closes the run."""
    run = GrowthRun(deck, nsteps, segment=segment, device=device, theta=theta, spinup=spinup)
    pool, _ = run.pool(run.theta)
    G, _ = run.growth(run.theta)
    return np.array([pool[0], pool[1], pool[2], G]), run

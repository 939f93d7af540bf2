"""Continuous-batching serving loop for lattice solves.

Requests (a boundary composition, an initial state and a step budget) arrive
over time.  At every tick the engine admits waiting requests while their
device state fits the HBM budget and a slot is free, advances every live
request together by ``tick_steps`` steps in batched launches (one launch per
step covering all of them; a request whose budget ends inside the tick stops
at its last step), and retires the requests whose budget is spent: their
final moments are read back and their memory is freed.
Requests that arrive while others are on the GPU join at the next tick, so
their work overlaps on the device.  A request's result does not depend on
what it shared the GPU with: every lattice is updated by the same kernel and
arithmetic whatever else is in the batch.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import boundary_utils as BU
from . import scenarios as S
from .batch import Batch, Member
from .lattice import REF_SHIFTED


@dataclass
class Request:
    rid: int
    kind: str
    nx: int
    ny: int
    omega: float
    steps: int
    boundary: object
    f0: np.ndarray
    rho0: np.ndarray
    u0: np.ndarray
    arrival: float = 0.0          # seconds after the stream starts
    params: dict = field(default_factory=dict)
    init: object = None           # () -> (f0, rho0, u0): the initial state built on demand
    dev_ref: tuple = None         # reference velocity for the "f16r" / "bf16r" storages (default (0, 0))
    # filled in by the engine
    prepared: tuple = None        # the initial state on the device, built while the GPU runs a tick
    admitted: float = None
    finished: float = None
    rho: torch.Tensor = None
    u: torch.Tensor = None

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    @property
    def nodes(self):
        return self.nx * self.ny

    def initial_state(self):
        """(f0, rho0, u0): the given arrays, else built by ``init``."""
        if self.f0 is not None:
            return self.f0, self.rho0, self.u0
        return self.init()


def _rest_state(nx, ny, device="cuda"):
    """rho = 1, u = 0 and its equilibrium (the weights) on the device."""
    w = torch.tensor([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=torch.float64, device=device)
    return (w.expand(nx, ny, 9).contiguous(), torch.ones((nx, ny), dtype=torch.float64, device=device),
            torch.zeros((nx, ny, 2), dtype=torch.float64, device=device))


def request_stream(n, rate=50.0, seed=7, step_range=(1000, 50000), kinds=("couette", "poiseuille", "von_karman")):
    """The seeded draws behind ``request_mix``, host only: per request (rid,
    arrival, kind, steps, nx, ny, params).  The arrival gaps are rate-scaled
    draws of one seeded stream, so the same seed gives the same requests
    (kinds, sizes, budgets) at every rate."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        kind = kinds[int(rng.integers(0, len(kinds)))]
        steps = int(rng.integers(step_range[0], step_range[1] + 1))
        if kind == "couette":
            ny = int(rng.integers(32, 513))
            out.append((rid, t, kind, steps, ny, ny, {"u_w": float(rng.uniform(0.01, 0.1))}))
        elif kind == "poiseuille":
            nx = int(rng.integers(64, 2049))
            ny = int(rng.integers(16, 513))
            drho = float(math.exp(rng.uniform(math.log(1e-4), math.log(1e-2))))
            out.append((rid, t, kind, steps, nx, ny, {"drho": drho}))
        else:
            out.append((rid, t, kind, steps, 420, 180, {"re": 100}))
    return out


def request_mix(n, rate=50.0, seed=7, step_range=(1000, 50000), kinds=("couette", "poiseuille", "von_karman"),
                lazy=False):
    """Seeded Poisson arrivals (mean ``rate`` per second) of mixed requests:
    Couette (moving top wall u_w in [0.01, 0.1], ny in [32, 512], nx = ny),
    pressure-driven Poiseuille (delta rho log-uniform in [1e-4, 1e-2], nx x ny
    up to 2048 x 512) and the von Karman channel (420 x 180, Re 100); the same
    requests at every rate (``request_stream``).  With ``lazy`` the initial
    states are built on the device at admission (long streams would not fit
    the host memory up front).  The channel requests carry their inlet velocity
    as the reference of the reference-shifted storages."""
    out = []
    for rid, t, kind, steps, nx, ny, params in request_stream(n, rate, seed, step_range, kinds):
        if kind == "couette":
            bnd = BU.Boundary([BU.rigid_wall(_row(nx, ny, 0)),
                               BU.moving_wall(_row(nx, ny, -1), np.array([params["u_w"], 0.0]), 1.0)])
            req = Request(rid, kind, nx, ny, 1.0, steps, bnd, None, None, None, t, params,
                          init=lambda nx=nx, ny=ny: _rest_state(nx, ny))
        elif kind == "poiseuille":
            d = params["drho"]
            bnd = BU.poiseuille_flow_boundary_conditions(nx, ny, (1 + d / 2) / 3, (1 - d / 2) / 3)
            req = Request(rid, kind, nx, ny, 1.5, steps, bnd, None, None, None, t, params,
                          init=lambda nx=nx, ny=ny: _rest_state(nx, ny))
        else:
            om = 1.0 / (3.0 * (0.1 * 40 / 100.0) + 0.5)
            bnd = BU.von_karman_boundary_conditions(420, 180, 1.0, 0.1, 40, walls=True, plate_offset=1)
            req = Request(rid, kind, 420, 180, om, steps, bnd, None, None, None, t, params,
                          init=lambda rid=rid: S.von_karman_start(420, 180, 0.1, 1e-3, seed=rid),
                          dev_ref=(0.1, 0.0))
        if not lazy:
            req.f0, req.rho0, req.u0 = req.init()
        out.append(req)
    return out


def _row(nx, ny, y):
    m = np.zeros((nx, ny), dtype=bool)
    m[:, y] = True
    return m


class ServingEngine:
    """Admits, batches and retires lattice solves on one GPU."""

    def __init__(self, storage="f16", hbm_budget=64 << 30, max_slots=128, tick_steps=500, npt=0, threads=0,
                 blocks=None, device="cuda"):
        self.storage = storage
        self.hbm_budget = int(hbm_budget)
        self.max_slots = max_slots
        self.tick_steps = tick_steps
        # a plain grid of one tile per block by default (blocks None); runs per
        # tile chosen by the batch size each time the table is rebuilt (one run
        # per tile for the small batches of the tail, whose few lattices need
        # every tile they can get)
        self.batch = Batch([], storage=storage, npt=npt, threads=threads, blocks=blocks, device=device)
        self.live = []          # (Request, Member)
        self.used = 0
        self.stats = {"ticks": 0, "max_live": 0, "steps": 0}
        # host work for the next requests (boundary compile, initial state) runs
        # while the GPU runs a tick; its copies and kernels go on this stream
        self.side = torch.cuda.Stream(device=self.batch.device)

    def _next_admissions(self, waiting, extra=2):
        """The head of the queue that the next admissions can take (free slots,
        room in the HBM budget), plus ``extra`` more: the requests worth
        preparing now, with their initial states held beyond the budget for a
        few requests at most."""
        out, used, slots = [], self.used, self.max_slots - len(self.live)
        for r in waiting:
            if slots <= 0 or used + self.state_bytes(r) > self.hbm_budget:
                break
            out.append(r)
            used += self.state_bytes(r)
            slots -= 1
        return waiting[:len(out) + extra]

    def _prepare(self, reqs):
        """Compile the boundary descriptor and build the initial state on the
        device for requests about to be admitted, on the side stream."""
        for r in reqs:
            if r.prepared is not None:
                continue
            with torch.cuda.stream(self.side):
                r.boundary.geometry(r.nx, r.ny)
                state = r.initial_state()
                r.prepared = tuple(None if t is None else
                                   (t if isinstance(t, torch.Tensor) else torch.from_numpy(np.asarray(t))).to(
                                       self.batch.device, non_blocking=False)
                                   for t in state)

    def state_bytes(self, req):
        per = {"fx64": 8, "f64": 8, "f32": 4, "f16": 2, "bf16": 2, "f16r": 2, "bf16r": 2}[self.storage]
        pitch = (req.nx + 31) // 32 * 32
        return 2 * 9 * req.ny * pitch * per + 2 * 3 * req.ny * 8

    def serve(self, requests, realtime=True):
        """Run an arrival stream to completion.  With ``realtime`` the arrival
        times are wall-clock offsets from the start; otherwise every request is
        waiting from the start (a closed loop).  Returns the finished requests
        with timings and results (rho, u on the device) filled in."""
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting, done = [], []
        b = self.batch
        t0 = time.perf_counter()
        i = 0
        while i < len(pending) or waiting or self.live:
            now = time.perf_counter() - t0
            if not waiting and not self.live and i < len(pending) and realtime and pending[i].arrival > now:
                time.sleep(pending[i].arrival - now)
                now = time.perf_counter() - t0
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                waiting.append(pending[i])
                i += 1
            main = torch.cuda.current_stream(b.device)
            while waiting and len(self.live) < self.max_slots and \
                    self.used + self.state_bytes(waiting[0]) <= self.hbm_budget:
                r = waiting.pop(0)
                r.admitted = now
                self._prepare([r])
                main.wait_stream(self.side)
                f0, rho0, u0 = r.prepared
                m = b.add(Member(r.nx, r.ny, r.omega, r.boundary, steps=r.steps, f0=f0, rho0=rho0, u0=u0,
                                 dev_ref=r.dev_ref if self.storage in REF_SHIFTED else None))
                # the first step has consumed the initial state (its memory, from
                # the side stream's pool, is not reused before that step has run)
                for t in r.prepared:
                    if t is not None:
                        t.record_stream(main)
                m.f0 = m.rho0 = m.u0 = None
                r.prepared = None
                del f0, rho0, u0
                self.live.append((r, m))
                self.used += self.state_bytes(r)
            if not self.live:
                if waiting:
                    raise RuntimeError("request %d does not fit the HBM budget" % waiting[0].rid)
                continue
            # full ticks: a request whose budget ends inside the tick stops there
            # by itself (the batched step skips a lattice outside its window) and
            # retires at the tick's end, so one short request does not cut every
            # tick short
            left = max(m.s0 + m.steps - 1 - b.g for _, m in self.live)
            n = max(0, min(self.tick_steps, left))
            b.run(n)
            self.stats["ticks"] += 1
            self.stats["steps"] += n
            self.stats["max_live"] = max(self.stats["max_live"], len(self.live))
            # while the tick runs: take in the arrivals and prepare the requests
            # that the next admissions will take
            now = time.perf_counter() - t0
            while i < len(pending) and (pending[i].arrival <= now or not realtime):
                waiting.append(pending[i])
                i += 1
            self._prepare(self._next_admissions(waiting))
            finished = [(r, m) for r, m in self.live if b.done(m)]
            if finished:
                for r, m in finished:
                    _, r.rho, r.u = b.read(m, want_f=False)
                torch.cuda.synchronize()
                now = time.perf_counter() - t0
                for r, m in finished:
                    r.finished = now
                    self.used -= self.state_bytes(r)
                    b.remove(m)
                    done.append(r)
                ids = {id(m) for _, m in finished}
                self.live = [(r, m) for r, m in self.live if id(m) not in ids]
        return done


def summarize(done):
    lat = np.array([r.latency for r in done])
    span = max(r.finished for r in done) - min(r.arrival for r in done)
    nodes_steps = sum(r.nodes * r.steps for r in done)
    return {"requests": len(done), "solves_per_s": len(done) / span, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()), "span_s": span,
            "mlups": nodes_steps / span / 1e6}

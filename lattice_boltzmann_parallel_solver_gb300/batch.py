"""Many lattices of different sizes advanced together: one boundary-free
launch per time step covers every live lattice (a flat list of tiles of
consecutive node chunks walked by a grid), a second one the boundary nodes,
optionally replayed from a captured CUDA graph.

This runs what the reference does one driver loop at a time - for example
the Reynolds / blockage / width sweeps of ``x_strouhal``
(src/experiments.py:650-720, src/main.py:150-207) - as one device job.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import torch

from . import _arrays as A
from . import _lib
from .geometry import empty_geometry
from .lattice import REF_SHIFTED, SIXTEEN_BIT, STORAGES, with_dev_ref


BatchLatticeC = _lib.BatchLattice


@dataclass
class Member:
    """One lattice of a batch: its geometry, state buffers and step window."""
    nx: int
    ny: int
    omega: float
    boundary: object = None
    steps: int = 1
    probe: tuple = None          # (x, y) node whose velocity is recorded every step
    f0: object = None            # reference-layout initial populations
    rho0: object = None
    u0: object = None
    seed: int = 0                # random bits of the stochastic rounding (16-bit storages)
    dev_ref: tuple = None        # reference velocity of the "f16r" / "bf16r" storages (default (0, 0))
    # filled in by the batch
    geo: object = None
    pitch: int = 0
    pop: list = field(default_factory=list)
    aux: list = field(default_factory=list)
    probe_buf: torch.Tensor = None
    probe_count: torch.Tensor = None
    s0: int = 0

    @property
    def nodes(self) -> int:
        return self.nx * self.ny


class Batch:
    """A set of lattices sharing one storage type, advanced in lock step.
    Members can join (``add``) and leave (``remove``) between runs."""

    def __init__(self, members=(), storage: str = "f16", npt: int = 0, threads: int = 0, blocks: int = None,
                 device: str = "cuda", stochastic: bool = None, rows: int = 0, inline_bc: bool | None = None):
        """Batches of at least 2^20 nodes take each step as a boundary-free
        launch over every node followed by a pass over the boundary nodes,
        smaller ones as one launch with the boundary sources inside (same
        results); ``inline_bc`` True / False forces the one or the other.
        ``npt``, ``threads`` and ``rows`` (nodes per thread, threads per tile,
        runs of ``threads`` chunks per tile) default to what ``autotune`` picks
        for such batches (``_default_shape``; for large mixed von Karman
        batches 1 x 64 for fx64 with 4 runs, 4 x 128 for the 16-bit storages
        with 8 runs; several runs only when the batch has enough of them to
        keep every SM busy, 1 otherwise).  ``blocks``: the default (None) is a
        plain grid of one tile per block, 0 persistent blocks filling the GPU
        that walk contiguous spans of tiles, any other number that many
        persistent blocks.  The reference-shifted storages ("f16r", "bf16r",
        each member's ``dev_ref``) run at 128 threads and 2 or 4 nodes per thread."""
        A.require_cuda()
        self.stochastic = storage in SIXTEEN_BIT if stochastic is None else bool(stochastic)
        self.storage = storage
        self.store_id, self.pop_dtype, self.aux_dtype = STORAGES[storage]
        self.device = torch.device(device)
        # nodes per thread and threads per tile: the given ones, else chosen by
        # the batch size each time the work table is built
        self.inline_bc = inline_bc      # None: chosen by the batch size
        self._auto_shape = (not npt, not threads)
        self.npt, self.threads = int(npt), int(threads)
        self._default_shape(0)
        self.blocks = ONE_TILE_PER_BLOCK if blocks is None else blocks
        self.rows = int(rows)           # runs per tile (0: chosen from the batch size)
        self.bc_chunks = -1             # boundary-node plan of the work table (-1: sources in the step)
        self.gbase = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.g = 0                    # host mirror of the global step
        self.members = []
        for m in members:
            self._alloc(m)
            self.members.append(m)
        self.table = None
        self.tiles = 0
        self._dirty = True
        self._graphs = {}

    def _alloc(self, m: Member):
        m.geo = m.boundary.geometry(m.nx, m.ny) if m.boundary is not None else empty_geometry(m.nx, m.ny)
        m.geo = with_dev_ref(m.geo, self.storage, m.dev_ref)
        if not m.geo.fusable:
            raise NotImplementedError("the outlet must sit on column nx-1")
        m.pitch = (m.nx + 31) // 32 * 32
        n = 9 * m.ny * m.pitch
        m.pop = [torch.empty(n, dtype=self.pop_dtype, device=self.device) for _ in range(2)]
        m.aux = [torch.zeros(3 * m.ny, dtype=self.aux_dtype, device=self.device) for _ in range(2)]
        if m.probe is not None:
            m.probe_buf = torch.zeros(2 * max(m.steps, 1), dtype=torch.float64, device=self.device)
            m.probe_count = torch.zeros(1, dtype=torch.int32, device=self.device)

    def _init_member(self, m: Member):
        """The member's first step (collision of its initial state); its remaining
        steps are global steps [g, g + steps - 1)."""
        f = A.to_device(m.f0)
        rho = A.to_device(m.rho0) if m.rho0 is not None else None
        u = A.to_device(m.u0) if m.u0 is not None else None
        _lib.call("lbm_lattice_init", m.geo.ref, self.store_id, f.data_ptr(), A.ptr(rho), A.ptr(u), m.omega,
                  m.pop[0].data_ptr(), m.pitch, m.aux[0].data_ptr(), 0, A.stream())
        m.s0 = self.g
        if m.probe_count is not None:
            m.probe_count.zero_()

    def add(self, m: Member):
        """Admit a lattice now: allocate, take its first step, join the next launch."""
        self._alloc(m)
        self._init_member(m)
        self.members.append(m)
        self._dirty = True
        return m

    def remove(self, m: Member):
        """Drop a lattice and release its device memory."""
        self.members = [x for x in self.members if x is not m]
        m.pop, m.aux = [], []
        self._dirty = True

    def done(self, m: Member) -> bool:
        return self.g >= m.s0 + m.steps - 1

    @property
    def nodes(self) -> int:
        return sum(m.nodes for m in self.members)

    @property
    def state_bytes(self) -> int:
        return sum(t.numel() * t.element_size() for m in self.members for t in m.pop + m.aux)

    # -- work table ----------------------------------------------------------------
    def _default_shape(self, nodes: int):
        """Default nodes per thread / threads per tile: below 2^20 nodes (one
        launch per step, boundary sources inside, row-segment tiles) 2 x 128
        for the 16-bit storages and 1 x 128 for fx64; above (boundary-free step
        over runs across row ends, then the boundary-node pass) 4 x 128 and
        1 x 64 (the reference-shifted 16-bit storages as the others)."""
        split = self.inline_bc is False or (self.inline_bc is None and nodes >= (1 << 20))
        if self._auto_shape[0]:
            self.npt = {"fx64": 1, "f64": 2}.get(self.storage, 4 if split or self.storage == "f32" else 2)
        if self._auto_shape[1]:
            self.threads = {"fx64": 64 if split else 128}.get(self.storage, 128)

    def _rows(self) -> int:
        """Runs per tile (a run: ``threads`` consecutive chunks of ``npt``
        nodes, row by row): the given number, else (when the batch has at
        least 64 runs per SM) 8 for the 16-bit storages and 4 for the others,
        else 1."""
        if self.rows > 0:
            return self.rows
        runs = sum(-(-(-(-m.nx // self.npt) * m.ny) // self.threads) for m in self.members)
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        if runs < 64 * sms:
            return 1
        return 8 if self.storage in SIXTEEN_BIT else 4

    def _build(self, with_probes=True):
        n = len(self.members)
        self._default_shape(self.nodes)
        rows = self._rows()
        arr = (BatchLatticeC * n)()
        self._keep = []
        for j, m in enumerate(self.members):
            c = arr[j]
            c.g = ctypes.addressof(m.geo.struct)
            c.pop_a, c.pop_b = m.pop[0].data_ptr(), m.pop[1].data_ptr()
            c.aux_a, c.aux_b = m.aux[0].data_ptr(), m.aux[1].data_ptr()
            c.pitch, c.omega = m.pitch, m.omega
            c.s0, c.s_end = m.s0, m.s0 + max(m.steps - 1, 0)
            if with_probes and m.probe is not None:
                c.probe_x, c.probe_y = int(m.probe[0]), int(m.probe[1])
                c.probe_cap = m.probe_buf.numel() // 2
                c.probe_buf, c.probe_count = m.probe_buf.data_ptr(), m.probe_count.data_ptr()
            else:
                c.probe_x = c.probe_y = -1
            c.seed = int(m.seed) & 0xFFFFFFFF
            c.flags = (_lib.FLAG_STOCHASTIC if self.stochastic else 0) | \
                {True: _lib.FLAG_BC_INLINE, False: _lib.FLAG_BC_SPLIT}.get(self.inline_bc, 0)
            c.rows = rows
        size = int(_lib.load().lbm_batch_table_bytes(n))
        self.table = torch.empty(size, dtype=torch.uint8, device=self.device)
        tiles, chunks = ctypes.c_int32(0), ctypes.c_int32(0)
        _lib.call("lbm_batch_build", arr, n, self.npt, self.threads, self.table.data_ptr(), size,
                  ctypes.byref(tiles), ctypes.byref(chunks), A.stream())
        self.tiles, self.bc_chunks = tiles.value, chunks.value
        self._graphs.clear()
        self._dirty = False

    # -- state ---------------------------------------------------------------------
    def start(self):
        """Take every member's first step and arm the batch at the current global step."""
        for m in self.members:
            self._init_member(m)
        self._build()
        return self

    @property
    def remaining(self) -> int:
        return max((m.s0 + m.steps - 1 for m in self.members), default=self.g) - self.g

    def run(self, nsteps: int = None):
        """Advance nsteps global steps (default: until every member is done)."""
        n = self.remaining if nsteps is None else int(nsteps)
        if self._dirty and self.members:
            self._build()
        if n > 0 and self.members:
            _lib.call("lbm_batch_run", self.table.data_ptr(), len(self.members), self.tiles, self.bc_chunks,
                      self.store_id, self.npt, self.threads, self.gbase.data_ptr(), n, self.blocks, A.stream())
            self.g += n
        return self

    def run_graph(self, nsteps: int = None, chunk: int = 100):
        """Like run(), replaying a captured graph of ``chunk`` steps."""
        n = self.remaining if nsteps is None else int(nsteps)
        if self._dirty and self.members:
            self._build()
        full, rest = divmod(max(n, 0), chunk)
        if full:
            g = self._graphs.get(chunk)
            if g is None:
                # a zero-step call outside capture settles the default grid size
                _lib.call("lbm_batch_run", self.table.data_ptr(), len(self.members), self.tiles, self.bc_chunks,
                          self.store_id, self.npt, self.threads, self.gbase.data_ptr(), 0, self.blocks, A.stream())
                g = torch.cuda.CUDAGraph()
                side = torch.cuda.Stream()
                side.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(side):
                    with torch.cuda.graph(g, stream=side):
                        _lib.call("lbm_batch_run", self.table.data_ptr(), len(self.members), self.tiles,
                                  self.bc_chunks, self.store_id, self.npt, self.threads, self.gbase.data_ptr(),
                                  chunk, self.blocks, side.cuda_stream)
                torch.cuda.current_stream().wait_stream(side)
                self._graphs[chunk] = g
            for _ in range(full):
                g.replay()
            self.g += full * chunk
        if rest:
            self.run(rest)
        return self

    def current(self, m: Member) -> int:
        """Index of the buffer holding member m's state at the current global step."""
        done = min(max(self.g - m.s0, 0), max(m.steps - 1, 0))
        return done % 2

    def read(self, j, want_f: bool = True):
        """(f, rho, u) of member j (an index or the Member) in the reference layout (float64, device)."""
        m = self.members[j] if isinstance(j, int) else j
        k = self.current(m)
        f = torch.empty((m.nx, m.ny, 9), dtype=torch.float64, device=self.device) if want_f else None
        rho = torch.empty((m.nx, m.ny), dtype=torch.float64, device=self.device)
        u = torch.empty((m.nx, m.ny, 2), dtype=torch.float64, device=self.device)
        _lib.call("lbm_lattice_read", m.geo.ref, self.store_id, m.pop[k].data_ptr(), m.pitch, m.aux[k].data_ptr(),
                  A.ptr(f), rho.data_ptr(), u.data_ptr(), A.stream())
        return f, rho, u

    def probe_trace(self, j: int) -> torch.Tensor:
        """Velocity (ux, uy) recorded at member j's probe, one row per batched step."""
        m = self.members[j]
        n = min(int(m.probe_count.item()), m.probe_buf.numel() // 2)
        return m.probe_buf[: 2 * n].view(n, 2)


# a grid size above half the tile count gives one tile per block: a plain
# (non-persistent) grid walked by the hardware block scheduler
ONE_TILE_PER_BLOCK = 1 << 24


def autotune(batch: Batch, candidates=None, steps: int = 6, warmup: int = 2):
    """Pick nodes per thread, threads per block, grid size (0: one persistent
    block per resident slot; ONE_TILE_PER_BLOCK) and runs per tile for a
    batch by timing each candidate on the batch itself.  Call it before
    ``start()``: the timed steps run on the members' uninitialised buffers
    (probes off) and the global step counter is reset afterwards."""
    sms = torch.cuda.get_device_properties(batch.device).multi_processor_count
    if candidates is None:
        npts = {"fx64": (1, 2), "f16": (2, 4, 8), "bf16": (2, 4, 8)}.get(batch.storage, (2, 4))
        threads = (128,) if batch.storage in REF_SHIFTED else (64, 128, 256)
        candidates = [(p, t, b, r) for p in npts for t in threads for b in (0, 8 * sms, ONE_TILE_PER_BLOCK)
                      for r in (1, 2, 4, 8, 16)]
    best, results = None, []
    for cand in candidates:
        npt, threads, blocks = cand[:3]
        rows = cand[3] if len(cand) > 3 else 1
        batch.npt, batch.threads, batch.blocks, batch.rows = npt, threads, blocks, rows
        batch._auto_shape = (False, False)
        try:
            batch._build(with_probes=False)
        except (AssertionError, NotImplementedError):
            continue
        batch.run(warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        batch.run(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        results.append({"npt": npt, "threads": threads, "blocks": blocks, "rows": rows, "ms_per_step": ms,
                        "glups": batch.nodes / (ms * 1e-3) / 1e9})
        if best is None or ms < best[0]:
            best = (ms, npt, threads, blocks, rows)
        del t0
    batch.g = 0
    batch.gbase.zero_()
    _, batch.npt, batch.threads, batch.blocks, batch.rows = best
    batch.tuning = results
    return results

"""Device-resident lattice: the hot loop of the reference's drivers
(for example experiments.py:83-84, 324-325, 766-767) without host round trips.

The populations live on the device as structure-of-arrays planes
pop[9][ny][pitch] (x contiguous, pitch a multiple of 32 elements) in one of
seven storage forms:

  "fx64"  round((f_i - w_i) 2^56) in int64, exact integer moments and
          linear relaxation, float-float quadratic term: float64 accuracy
          without float64 instructions (72 B per node; the default)
  "f64"   float64 storage and arithmetic, the drop-in's form (72 B)
  "f32"   float32 storage and arithmetic (36 B)
  "f16"   float32 arithmetic, f_i - w_i stored in binary16 (18 B)
  "bf16"  float32 arithmetic, f_i - w_i stored in bfloat16 (18 B)
  "f16r", "bf16r"  as "f16" / "bf16" with w_i replaced by c_i, the
          equilibrium at rho = 1 and a reference velocity (``dev_ref``): a
          flow near a uniform velocity (a channel at its inlet velocity) keeps
          smaller stored deviations and smaller rounding errors

One fused kernel per step reads the previous post-collision populations
once, streams them by pulling, applies the boundary descriptor, forms the
moments, collides and writes the new post-collision populations once.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _arrays as A
from . import _lib
from .geometry import empty_geometry

STORAGES = {
    "fx64": (_lib.STORE_FX64, torch.int64, torch.int64),
    "f64": (_lib.STORE_F64, torch.float64, torch.float64),
    "f32": (_lib.STORE_F32, torch.float32, torch.float32),
    "f16": (_lib.STORE_F16S, torch.float16, torch.float32),
    "bf16": (_lib.STORE_BF16S, torch.bfloat16, torch.float32),
    "f16r": (_lib.STORE_F16R, torch.float16, torch.float32),
    "bf16r": (_lib.STORE_BF16R, torch.bfloat16, torch.float32),
}
BYTES_PER_NODE = {"fx64": 144, "f64": 144, "f32": 72, "f16": 36, "bf16": 36, "f16r": 36, "bf16r": 36}
# the storages that keep 16-bit deviations (stochastic rounding on by default)
SIXTEEN_BIT = ("f16", "bf16", "f16r", "bf16r")
# the reference-shifted ones
REF_SHIFTED = ("f16r", "bf16r")


def with_dev_ref(geo, storage: str, dev_ref):
    """The geometry to pass with ``storage``: for the reference-shifted
    storages a copy carrying the reference velocity ``dev_ref`` (default
    (0, 0)); the geometry itself otherwise, where ``dev_ref`` must be None."""
    if storage in REF_SHIFTED:
        ux, uy = dev_ref if dev_ref is not None else (0.0, 0.0)
        return geo.with_dev_ref(ux, uy)
    if dev_ref is not None:
        raise ValueError("dev_ref applies to the reference-shifted storages %s only" % (REF_SHIFTED,))
    return geo


class Lattice:
    """An nx x ny D2Q9 lattice with a fused boundary composition, resident on the device."""

    def __init__(self, nx: int, ny: int, omega: float, boundary=None, storage: str = None,
                 exact: bool = False, device: str = "cuda", generic: bool = False, npt: int = 0,
                 stochastic: bool = None, seed: int = 0, bc_inline: bool | None = None,
                 probe: tuple = None, probe_cap: int = 0, dev_ref: tuple = None):
        """``generic`` forces the one-node-per-thread kernel; ``npt`` sets the
        nodes per thread of the vectorised kernel (0 = the default for the storage).
        ``stochastic`` (default: on for the 16-bit storages) rounds the stored
        deviations stochastically, which keeps increments smaller than half a
        16-bit step from being lost; ``seed`` seeds its random bits.
        Large lattices (from 2^22 nodes in the 16-bit storages, 2^25 in the
        others) run the vectorised step without boundary work and then a pass
        over the boundary nodes; smaller ones apply the boundary sources inside
        the step (same results).  ``bc_inline`` True / False forces the one or
        the other.  The
        default storage is "fx64", or "f64" with ``exact`` (the reference's
        float64 operation order, bit for bit).  ``probe`` = (x, y) records the
        velocity of that node at every fused step, up to ``probe_cap`` steps
        (``probe_trace``): the per-step probe of the reference's drivers
        (src/experiments.py:690,703-704) kept on the device.  ``dev_ref`` =
        (ux, uy): the reference velocity of the "f16r" / "bf16r" storages
        (default (0, 0)); they run at 4 nodes per thread (``npt`` ignored)."""
        A.require_cuda()
        assert 0 < omega < 2
        if storage is None:
            storage = "f64" if exact else "fx64"
        assert storage in STORAGES, "storage must be one of %s" % sorted(STORAGES)
        assert not (exact and storage != "f64"), "exact arithmetic needs float64 storage"
        self.nx, self.ny, self.omega = int(nx), int(ny), float(omega)
        self.storage = storage
        self.store_id, self.pop_dtype, self.aux_dtype = STORAGES[storage]
        if stochastic is None:
            stochastic = storage in SIXTEEN_BIT
        self.flags = (_lib.FLAG_EXACT if exact else 0) | (_lib.FLAG_GENERIC if generic else 0) | \
            ((int(npt) & 15) << _lib.FLAG_NPT_SHIFT) | (_lib.FLAG_STOCHASTIC if stochastic else 0) | \
            {True: _lib.FLAG_BC_INLINE, False: _lib.FLAG_BC_SPLIT}.get(bc_inline, 0)
        self.seed = int(seed) & 0xFFFFFFFF
        self.pitch = (self.nx + 31) // 32 * 32
        self.device = torch.device(device)
        self.boundary = boundary
        self.geo = boundary.geometry(self.nx, self.ny) if boundary is not None else empty_geometry(self.nx, self.ny)
        self.geo = with_dev_ref(self.geo, storage, dev_ref)
        self.dev_ref = None if storage not in REF_SHIFTED else (self.geo.struct.dev_ref_ux, self.geo.struct.dev_ref_uy)
        if not self.geo.fusable:
            raise NotImplementedError("the outlet must sit on column nx-1 for the resident lattice")
        n = 9 * self.ny * self.pitch
        self.pop = [torch.empty(n, dtype=self.pop_dtype, device=self.device) for _ in range(2)]
        self.aux = [torch.zeros(3 * self.ny, dtype=self.aux_dtype, device=self.device) for _ in range(2)]
        self.cur = 0
        self.t = 0
        self._init = None
        self._graphs = {}
        self._stepdev = None
        self.probe = None if probe is None else (int(probe[0]), int(probe[1]))
        if self.probe is not None:
            assert 0 <= self.probe[0] < self.nx and 0 <= self.probe[1] < self.ny, "probe outside the lattice"
            self.probe_buf = torch.zeros(2 * max(int(probe_cap), 1), dtype=torch.float64, device=self.device)
            self.probe_count = torch.zeros(1, dtype=torch.int32, device=self.device)

    # -- state ------------------------------------------------------------------
    def set_state(self, f, density=None, velocity=None):
        """Start from a reference-layout state f[nx, ny, 9]; the first step's
        collision uses ``density``/``velocity`` when given (as the reference's
        step does), else their moments."""
        f = A.to_device(f)
        assert tuple(f.shape) == (self.nx, self.ny, 9)
        rho = A.to_device(density) if density is not None else None
        u = A.to_device(velocity) if velocity is not None else None
        if rho is not None:
            assert tuple(rho.shape) == (self.nx, self.ny) and tuple(u.shape) == (self.nx, self.ny, 2)
        self._init = (f.clone(), None if rho is None else rho.clone(), None if u is None else u.clone())
        self.t = 0
        self.cur = 0
        self._graphs.clear()
        if self.probe is not None:
            self.probe_count.zero_()
        return self

    @property
    def state_bytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in self.pop + self.aux)

    # -- stepping ---------------------------------------------------------------
    def _first(self):
        f, rho, u = self._init
        _lib.call("lbm_lattice_init", self.geo.ref, self.store_id, f.data_ptr(), A.ptr(rho), A.ptr(u),
                  self.omega, self.pop[self.cur].data_ptr(), self.pitch, self.aux[self.cur].data_ptr(),
                  self.flags, A.stream())
        self._init = None
        self.t += 1

    def _options(self, counter=None):
        """lbm_run_options for the probe and/or a device step counter (None: neither)."""
        if self.probe is None and counter is None:
            return None
        o = _lib.RunOptions()
        o.step_counter = None if counter is None else counter.data_ptr()
        o.probe_x, o.probe_y = self.probe if self.probe is not None else (-1, -1)
        if self.probe is not None:
            o.probe_cap = self.probe_buf.numel() // 2
            o.probe_buf, o.probe_count = self.probe_buf.data_ptr(), self.probe_count.data_ptr()
        return o

    def _run(self, n: int, rho_out=None, u_out=None):
        a, b = self.cur, 1 - self.cur
        opts = self._options()
        _lib.call("lbm_lattice_run_opts", self.geo.ref, self.store_id, self.pop[a].data_ptr(),
                  self.pop[b].data_ptr(), self.pitch, self.aux[a].data_ptr(), self.aux[b].data_ptr(), self.omega,
                  int(n), A.ptr(rho_out), A.ptr(u_out), self.flags, (self.seed + self.t - 1) & 0xFFFFFFFF,
                  None if opts is None else ctypes.byref(opts), A.stream())
        if n % 2:
            self.cur = b
        self.t += n

    def step(self, n: int = 1):
        """Advance n time steps (asynchronous on the current stream)."""
        if n <= 0:
            return self
        if self._init is not None:
            self._first()
            n -= 1
        if n > 0:
            self._run(n)
        return self

    def step_graph(self, n: int, chunk: int = 64):
        """Advance n steps replaying a captured CUDA graph of ``chunk`` fused
        steps (chunk even, so the buffers return to their places); for small
        lattices where launch latency would dominate.  Results equal step(n)
        bit for bit: with stochastic rounding the captured steps read the step
        index from a device counter, so every replay draws the random bits that
        step() would."""
        assert chunk % 2 == 0 and chunk > 0
        if self._init is not None:
            self._first()
            n -= 1
        full, rest = divmod(max(n, 0), chunk)
        if full:
            counted = bool(self.flags & _lib.FLAG_STOCHASTIC)
            if counted:
                if self._stepdev is None:
                    self._stepdev = torch.zeros(1, dtype=torch.int32, device=self.device)
                # the step index the captured launches add to the seed (ordered before the replays)
                self._stepdev.fill_(self.t - 1)
            key = (chunk, self.cur)
            g = self._graphs.get(key)
            if g is None:
                g = torch.cuda.CUDAGraph()
                side = torch.cuda.Stream()
                side.wait_stream(torch.cuda.current_stream())
                opts = self._options(self._stepdev if counted else None)
                seed = self.seed if counted else (self.seed + self.t - 1) & 0xFFFFFFFF
                with torch.cuda.stream(side):
                    with torch.cuda.graph(g, stream=side):
                        _lib.call("lbm_lattice_run_opts", self.geo.ref, self.store_id,
                                  self.pop[self.cur].data_ptr(), self.pop[1 - self.cur].data_ptr(), self.pitch,
                                  self.aux[self.cur].data_ptr(), self.aux[1 - self.cur].data_ptr(), self.omega,
                                  chunk, 0, 0, self.flags, seed, None if opts is None else ctypes.byref(opts),
                                  side.cuda_stream)
                torch.cuda.current_stream().wait_stream(side)
                self._graphs[key] = g
            for _ in range(full):
                g.replay()
            self.t += full * chunk
        if rest:
            self._run(rest)
        return self

    def probe_trace(self) -> torch.Tensor:
        """(ux, uy) recorded at the probe node, one row per fused step: row k is the
        velocity of the state after k + 1 steps (the first step only collides
        the initial state; the velocity after the last step is read())."""
        assert self.probe is not None, "the lattice has no probe"
        n = min(int(self.probe_count.item()), self.probe_buf.numel() // 2)
        return self.probe_buf[: 2 * n].view(n, 2)

    # -- read-out ---------------------------------------------------------------
    def read(self, want_f: bool = True):
        """(f[nx, ny, 9], rho[nx, ny], u[nx, ny, 2]) of the current state, float64,
        reference layout, on the device."""
        if self._init is not None:
            f, rho, u = self._init
            from .lattice_boltzmann_method import compute_density, compute_velocity_field
            r = compute_density(f)
            return (f.clone() if want_f else None), r, compute_velocity_field(r, f)
        f = torch.empty((self.nx, self.ny, 9), dtype=torch.float64, device=self.device) if want_f else None
        rho = torch.empty((self.nx, self.ny), dtype=torch.float64, device=self.device)
        u = torch.empty((self.nx, self.ny, 2), dtype=torch.float64, device=self.device)
        _lib.call("lbm_lattice_read", self.geo.ref, self.store_id, self.pop[self.cur].data_ptr(), self.pitch,
                  self.aux[self.cur].data_ptr(), A.ptr(f), rho.data_ptr(), u.data_ptr(), A.stream())
        return f, rho, u

    def moments(self):
        _, rho, u = self.read(want_f=False)
        return rho, u

    # -- checkpoint / resume -----------------------------------------------------
    def checkpoint(self) -> dict:
        """The resident state (populations, outlet memory, step count) as host
        arrays; ``restore`` continues bit for bit from it."""
        if self._init is not None:
            f, rho, u = self._init
            return {"pending": np.asarray(1), "f": f.cpu().numpy(),
                    "rho": None if rho is None else rho.cpu().numpy(),
                    "u": None if u is None else u.cpu().numpy(), "t": np.asarray(self.t)}
        pop = self.pop[self.cur]
        pop = pop.view(torch.int16).cpu().numpy().view(np.uint16) if self.pop_dtype == torch.bfloat16 \
            else pop.cpu().numpy()
        return {"pending": np.asarray(0), "pop": pop,
                "aux": self.aux[self.cur].cpu().numpy(), "t": np.asarray(self.t),
                "storage": np.asarray(self.storage), "nx": np.asarray(self.nx), "ny": np.asarray(self.ny),
                "dev_ref": None if self.dev_ref is None else np.asarray(self.dev_ref, dtype=np.float64)}

    def restore(self, ck: dict):
        if int(ck["pending"]):
            self.set_state(ck["f"], ck.get("rho"), ck.get("u"))
            self.t = int(ck["t"])
            return self
        assert str(ck["storage"]) == self.storage and int(ck["nx"]) == self.nx and int(ck["ny"]) == self.ny
        if self.dev_ref is not None:
            # the stored numbers are deviations from the equilibrium at this reference velocity
            saved = ck.get("dev_ref")
            assert saved is not None and tuple(float(v) for v in np.asarray(saved)) == tuple(self.dev_ref), \
                "the checkpoint was written with another reference velocity"
        self._init = None
        self.cur = 0
        pop = np.asarray(ck["pop"])
        src = torch.from_numpy(pop.view(np.int16)).view(torch.bfloat16) if pop.dtype == np.uint16 \
            else torch.from_numpy(pop)
        self.pop[0].copy_(src)
        self.aux[0].copy_(torch.from_numpy(np.asarray(ck["aux"])))
        self.t = int(ck["t"])
        self._graphs.clear()
        return self

    def save(self, path: str):
        """Write a checkpoint file (.npz)."""
        ck = self.checkpoint()
        np.savez(path, **{k: v for k, v in ck.items() if v is not None})

    def load(self, path: str):
        with np.load(path, allow_pickle=False) as z:
            ck = {k: z[k] for k in z.files}
        ck.setdefault("rho", None)
        ck.setdefault("u", None)
        ck.setdefault("dev_ref", None)
        if "pop" in ck and self.pop_dtype == torch.bfloat16:
            ck["pop"] = ck["pop"].view(np.uint16)
        return self.restore(ck)

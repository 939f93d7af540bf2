"""Drop-in for the reference's ``src/boundary_utils.py`` (scenario boundary
compositions) plus the restated scenarios the reference has no composition
for (sliding-lid cavity, von Karman channel with walls).

A composition is a ``Boundary``: an ordered list of boundary closures
(later ones win where they write the same population, as in the
reference), optionally preceded by the pre-streaming pressure rewrite.
Called with the reference hook signature
``boundary(f_pre, f_post, density, velocity, f_prev)`` it behaves like the
reference closure; passed to ``lattice_boltzmann_step`` or to a
``Lattice`` it is compiled into the per-node descriptor of the fused kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _arrays as A
from . import _lib
from .boundary_conditions import (_Closure, _PressurePeriodic, inlet, moving_wall, outlet,
                                  periodic_with_pressure_variations, rigid_wall)
from .geometry import BOUNCE, CONST, OUTLET, CompiledGeometry


class Boundary:
    """Ordered boundary composition, fusable into the step kernels."""

    _lbm_gb300_hook = True

    def __init__(self, closures=(), pressure: _PressurePeriodic = None, padded: bool = False):
        self.closures = list(closures)
        self.pressure = pressure
        self.padded = padded
        self._geo = {}

    def sources(self, nx, ny):
        out = []
        for c in self.closures:
            out += c.sources(nx, ny)
        return out

    def geometry(self, nx: int, ny: int) -> CompiledGeometry:
        key = (int(nx), int(ny))
        if key not in self._geo:
            spec = self.pressure.spec if self.pressure is not None else None
            self._geo[key] = CompiledGeometry(nx, ny, self.sources(nx, ny), pressure=spec)
        return self._geo[key]

    def __call__(self, f_pre_streaming, f_post_streaming, density=None, velocity=None, f_prev=None):
        kind = A.kind_of(f_post_streaming)
        pre = A.to_device(f_pre_streaming)
        post = A.to_device(f_post_streaming)
        nx, ny = int(post.shape[0]), int(post.shape[1])
        g = self.geometry(nx, ny)
        s = A.stream()
        if self.pressure is not None:
            # the rewrite acts on f_pre in place, then the composition streams again
            # (boundary_utils.py:103-104)
            rho, u = A.to_device(density), A.to_device(velocity)
            _lib.call("lbm_pressure_prestream_f64", g.ref, pre.data_ptr(), rho.data_ptr(), u.data_ptr(), s)
            A.write_back(f_pre_streaming, pre)
            post = torch.empty_like(pre)
            _lib.call("lbm_streaming_f64", pre.data_ptr(), post.data_ptr(), nx, ny, s)
        prev = A.to_device(f_prev) if f_prev is not None else None
        _lib.call("lbm_apply_boundary_f64", g.ref, pre.data_ptr(), A.ptr(prev), post.data_ptr(), s)
        if self.pressure is None:
            return A.write_back(f_post_streaming, post)
        return A.to_kind(post, kind)


def _row(lx, ly, y):
    m = np.zeros((lx, ly), dtype=bool)
    m[:, y] = True
    return m


def couette_flow_boundary_conditions(lx, ly, U, avg_density):
    """Rigid top wall, then moving bottom wall u_w = (U, 0) (boundary_utils.py:9-55)."""
    return Boundary([rigid_wall(_row(lx, ly, -1)), moving_wall(_row(lx, ly, 0), np.array([U, 0]), avg_density)])


def poiseuille_flow_boundary_conditions(lx, ly, p_in, p_out):
    """Pressure-periodic in x, re-stream, rigid bottom then top wall (boundary_utils.py:58-110)."""
    m = np.zeros((lx, ly), dtype=bool)
    m[0, :] = True
    m[-1, :] = True
    return Boundary([rigid_wall(_row(lx, ly, 0)), rigid_wall(_row(lx, ly, -1))],
                    pressure=periodic_with_pressure_variations(m, p_in, p_out))


class _Sources(_Closure):
    """A closure given directly as descriptor sources."""

    def __init__(self, fn):
        self.fn = fn

    def sources(self, nx, ny):
        return self.fn(nx, ny)


def plate_rows(ly, plate_size):
    """Plate face rows [y_min, y_max) and corner rows (upper, lower) (boundary_utils.py:145, 184-201)."""
    return (ly // 2 - plate_size // 2 + 1, ly // 2 + plate_size // 2 - 1,
            ly // 2 + plate_size // 2 - 1, ly // 2 - plate_size // 2)


def _vk_closures(lx, ly, density_in, velocity_in, plate_size, off=0, plate_x=None, walls=False, feq_in=None,
                 plate_offset=0):
    """Inlet, outlet, plate left face + corners, plate right face + corners, on
    a domain whose interior starts at index ``off`` (1 for ghost-padded arrays).
    ``feq_in`` (the 9 inlet populations) is computed on the device when not given;
    ``plate_offset`` shifts the plate rows."""
    px = (lx // 4 if plate_x is None else plate_x) + off
    y_min, y_max, y_up, y_lo = (r + plate_offset for r in plate_rows(ly, plate_size))
    if feq_in is None:
        feq_in = inlet((1, ly), density_in, velocity_in).values

    def srcs(nx, ny):
        out = []
        m = np.zeros((nx, ny), dtype=bool)
        m[off, off:off + ly] = True
        out += [(m, i, CONST, float(feq_in[i])) for i in range(9)]
        m = np.zeros((nx, ny), dtype=bool)
        m[off + lx - 1, off:off + ly] = True
        out += [(m, i, OUTLET, 0.0) for i in (3, 6, 7)]
        for x, face, up, lo in ((px, ((3, 1), (7, 5), (6, 8)), ((3, 1), (6, 8)), ((3, 1), (7, 5))),
                                (px + 1, ((1, 3), (5, 7), (8, 6)), ((1, 3), (5, 7)), ((1, 3), (8, 6)))):
            m = np.zeros((nx, ny), dtype=bool)
            m[x, off + y_min:off + y_max] = True
            out += [(m, a, BOUNCE, 0.0) for a, _ in face]
            m = np.zeros((nx, ny), dtype=bool)
            m[x, off + y_up] = True
            out += [(m, a, BOUNCE, 0.0) for a, _ in up]
            m = np.zeros((nx, ny), dtype=bool)
            m[x, off + y_lo] = True
            out += [(m, a, BOUNCE, 0.0) for a, _ in lo]
        if walls:
            # rigid bottom and top rows with the reference rigid_wall mapping
            for y, dirs in ((off, (4, 7, 8)), (off + ly - 1, (2, 5, 6))):
                m = np.zeros((nx, ny), dtype=bool)
                m[off:off + lx, y] = True
                out += [(m, int(_lib_opp(i)), BOUNCE, 0.0) for i in dirs]
        return out
    return [_Sources(srcs)]


def _lib_opp(i):
    return (0, 3, 4, 1, 2, 7, 8, 5, 6)[i]


def parallel_von_karman_boundary_conditions(coord2d, n_local_x, n_local_y, lx, ly, x_size, y_size,
                                            density_in, velocity_in, plate_size):
    """The von Karman composition on ghost-padded (n_local_x+2, n_local_y+2, 9)
    arrays (boundary_utils.py:113-205).  One GPU holds the whole domain, so
    only the single-rank decomposition (x_size = y_size = 1) exists here."""
    if x_size != 1 or y_size != 1 or n_local_x != lx or n_local_y != ly:
        raise NotImplementedError("one device holds the whole lattice: use x_size = y_size = 1")
    return Boundary(_vk_closures(lx, ly, density_in, velocity_in, plate_size, off=1), padded=True)


def von_karman_boundary_conditions(lx, ly, density_in, velocity_in, plate_size, plate_x=None, walls=False,
                                   plate_offset=0):
    """The same composition on an unpadded periodic lx x ly lattice (fusable).
    ``walls=True`` adds rigid bottom/top rows after the plate; ``plate_offset``
    moves the plate by that many rows."""
    return Boundary(_vk_closures(lx, ly, density_in, velocity_in, plate_size, off=0, plate_x=plate_x,
                                 walls=walls, plate_offset=plate_offset))


def cavity_boundary_conditions(nx, ny, u_lid=0.1, avg_density=1.0):
    """Sliding-lid cavity (no reference composition exists): lateral walls
    bounce their incoming links (x=0: 1,5,8 from 3,7,6; x=-1: 3,7,6 from
    1,5,8), then the reference rigid bottom wall, then the reference moving
    lid u_w = (u_lid, 0); later walls win at the corners."""
    def lateral(nxx, nyy):
        out = []
        m = np.zeros((nxx, nyy), dtype=bool)
        m[0, :] = True
        out += [(m, a, BOUNCE, 0.0) for a in (1, 5, 8)]
        m = np.zeros((nxx, nyy), dtype=bool)
        m[-1, :] = True
        out += [(m, a, BOUNCE, 0.0) for a in (3, 7, 6)]
        return out
    return Boundary([_Sources(lateral), rigid_wall(_row(nx, ny, 0)),
                     moving_wall(_row(nx, ny, -1), np.array([u_lid, 0.0]), avg_density)])


class _HaloExchange:
    """Single-rank periodic ghost exchange on a padded array, in place
    (parallelization_utils.py:23-50 with this rank as every neighbour)."""

    _lbm_gb300_hook = True

    def __call__(self, f):
        dev = A.to_device(f)
        _lib.call("lbm_halo_fill_f64", dev.data_ptr(), int(dev.shape[0]), int(dev.shape[1]), A.stream())
        return A.write_back(f, dev)


def communication(comm=None):
    """The halo hook of the reference's decomposition (parallelization_utils.py:6-52)
    for the one-device domain."""
    return _HaloExchange()

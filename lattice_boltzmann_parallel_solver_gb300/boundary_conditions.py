"""Drop-in for the reference's ``src/boundary_conditions.py``.

Each factory keeps the reference's name, arguments and closure signature
and returns a callable object.  Called on its own it applies the condition
with a CUDA kernel and, like the reference closure, updates and returns its
argument.  Composed (``boundary_utils.Boundary``) it contributes its
per-node sources to the descriptor the fused step kernels read.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _arrays as A
from . import _lib
from .geometry import BOUNCE, CONST, OUTLET, CompiledGeometry
from .lattice_boltzmann_method import get_velocity_sets, get_w_i, vel_to_opp_vel_mapping

_OPP = vel_to_opp_vel_mapping()
_CS = 1 / np.sqrt(3)


def get_wall_indices(boundary) -> np.ndarray:
    """Directions bounced at a wall; one wall per mask, first match wins, with
    the reference's mapping of the x-walls (boundary_conditions.py:8-28)."""
    b = np.asarray(boundary)
    index_list = []
    if np.all(b[0, :]):
        index_list += [1, 5, 8]
    elif np.all(b[-1, :]):
        index_list += [3, 6, 7]
    elif np.all(b[:, 0]):
        index_list += [4, 7, 8]
    elif np.all(b[:, -1]):
        index_list += [2, 5, 6]
    return np.array(index_list)


def get_corner_indices(boundary) -> list:
    """Corner nodes of a one-column object with the two directions each bounces (:31-56)."""
    b = np.asarray(boundary)
    assert b.ndim == 2
    idx = np.argwhere(b)
    x0, x1 = int(idx[:, 0].min()), int(idx[:, 0].max()) + 1
    y0, y1 = int(idx[:, 1].min()), int(idx[:, 1].max())
    return [((x0, y1), (1, 8)), ((x0, y0), (1, 5)), ((x1, y1), (3, 7)), ((x1, y0), (3, 6))]


def remove_corner_indices_from_boundary(boundary, corner_indices):
    """Clears the corner nodes in place and returns the mask (:59-75)."""
    assert len(boundary.shape) == 2
    for (cx, cy), _ in corner_indices:
        boundary[cx, cy] = False
    return boundary


def _host_mask(boundary) -> np.ndarray:
    if isinstance(boundary, torch.Tensor):
        return boundary.detach().cpu().numpy()
    return np.asarray(boundary)


class _Closure:
    """Base of the boundary objects: descriptor sources plus standalone application."""

    _lbm_gb300_hook = True
    shape = None

    def sources(self, nx: int, ny: int):
        raise NotImplementedError

    def _geometry(self, nx, ny):
        cache = self.__dict__.setdefault("_geo", {})
        if (nx, ny) not in cache:
            cache[(nx, ny)] = CompiledGeometry(nx, ny, self.sources(nx, ny))
        return cache[(nx, ny)]

    def _apply(self, f_pre, f_prev, f_post):
        dev = A.to_device(f_post)
        pre = A.to_device(f_pre) if f_pre is not None else dev
        prev = A.to_device(f_prev) if f_prev is not None else None
        assert pre.shape == dev.shape
        nx, ny = int(dev.shape[0]), int(dev.shape[1])
        g = self._geometry(nx, ny)
        _lib.call("lbm_apply_boundary_f64", g.ref, pre.data_ptr(), A.ptr(prev), dev.data_ptr(), A.stream())
        return A.write_back(f_post, dev)


def _bounce_sources(mask, dirs, k=None):
    """f_post[mask, opp(i)] = f_pre[mask, i] - k_i for each i in dirs."""
    out = []
    for i in dirs:
        out.append((mask, int(_OPP[i]), BOUNCE, 0.0 if k is None else float(k[i])))
    return out


class _RigidWall(_Closure):
    def __init__(self, boundary):
        self.mask = _host_mask(boundary)
        assert self.mask.dtype == bool
        self.dirs = get_wall_indices(self.mask)

    def sources(self, nx, ny):
        return _bounce_sources(self.mask, self.dirs)

    def __call__(self, f_pre_streaming, f_post_streaming):
        assert self.mask.shape == tuple(f_pre_streaming.shape[0:2])
        assert self.mask.shape == tuple(f_post_streaming.shape[0:2])
        return self._apply(f_pre_streaming, None, f_post_streaming)


def rigid_wall(boundary):
    """Half-way bounce-back f_post[b, opp(i)] = f_pre[b, i] (:78-113)."""
    return _RigidWall(boundary)


class _RigidObject(_Closure):
    def __init__(self, boundary):
        assert boundary.dtype == bool
        corners = get_corner_indices(boundary)
        b = remove_corner_indices_from_boundary(boundary, corners)
        self.left = _host_mask(b).copy()
        self.right = np.roll(self.left, 1, axis=0)
        self.corners = corners

    def sources(self, nx, ny):
        src = _bounce_sources(self.left, (1, 5, 8)) + _bounce_sources(self.right, (3, 6, 7))
        for (cx, cy), dirs in self.corners:
            m = np.zeros((nx, ny), dtype=bool)
            m[cx, cy] = True
            src += _bounce_sources(m, dirs)
        return src

    def __call__(self, f_pre_streaming, f_post_streaming):
        assert self.left.shape == tuple(f_pre_streaming.shape[0:2])
        assert self.left.shape == tuple(f_post_streaming.shape[0:2])
        return self._apply(f_pre_streaming, None, f_post_streaming)


def rigid_object(boundary):
    """Bounce-back around a one-column object away from the walls; like the
    reference, the corner nodes are removed from ``boundary`` in place (:116-167)."""
    return _RigidObject(boundary)


def moving_wall_terms(boundary, u_w, avg_density) -> dict:
    """Per bounced direction i the term 2 w_i rho_avg (c_i.u_w)/c_s^2, evaluated
    with the reference's float64 expression (:186-210)."""
    c_i, w_i = get_velocity_sets(), get_w_i()
    u_w = np.asarray(u_w)
    return {int(i): 2 * w_i[i] * avg_density * np.divide(c_i[i] @ u_w, _CS ** 2)
            for i in get_wall_indices(boundary)}


class _MovingWall(_Closure):
    def __init__(self, boundary, u_w, avg_density):
        self.mask = _host_mask(boundary)
        assert self.mask.dtype == bool
        self.k = moving_wall_terms(self.mask, u_w, avg_density)

    def sources(self, nx, ny):
        return _bounce_sources(self.mask, list(self.k.keys()), self.k)

    def __call__(self, f_pre_streaming, f_post_streaming):
        assert self.mask.shape == tuple(f_pre_streaming.shape[0:2])
        assert self.mask.shape == tuple(f_post_streaming.shape[0:2])
        return self._apply(f_pre_streaming, None, f_post_streaming)


def moving_wall(boundary, u_w, avg_density):
    """f_post[b, opp(i)] = f_pre[b, i] - 2 w_i rho_avg c_i.u_w / c_s^2 (:170-214)."""
    return _MovingWall(boundary, u_w, avg_density)


def inlet_populations(density_in, velocity_in) -> np.ndarray:
    """The 9 equilibrium populations at (density_in, (velocity_in, 0)), from the
    same kernel as equilibrium_distr_func (:231-237)."""
    from .lattice_boltzmann_method import equilibrium_distr_func
    u = torch.zeros((1, 1, 2), dtype=torch.float64, device="cuda")
    u[..., 0] = velocity_in
    rho = torch.ones((1, 1), dtype=torch.float64, device="cuda") * density_in
    return equilibrium_distr_func(rho, u).reshape(9).cpu().numpy()


class _Inlet(_Closure):
    def __init__(self, lattice_grid_shape, density_in, velocity_in):
        self.shape = tuple(int(s) for s in lattice_grid_shape)
        self.values = inlet_populations(density_in, velocity_in)

    def sources(self, nx, ny):
        m = np.zeros((nx, ny), dtype=bool)
        m[0, :] = True
        return [(m, i, CONST, float(self.values[i])) for i in range(9)]

    def __call__(self, f_post_streaming):
        return self._apply(None, None, f_post_streaming)


def inlet(lattice_grid_shape, density_in, velocity_in):
    """All 9 populations of column x=0 set to the inlet equilibrium (:217-254)."""
    return _Inlet(lattice_grid_shape, density_in, velocity_in)


class _Outlet(_Closure):
    dirs = (3, 6, 7)

    def sources(self, nx, ny):
        m = np.zeros((nx, ny), dtype=bool)
        m[-1, :] = True
        return [(m, i, OUTLET, 0.0) for i in self.dirs]

    def __call__(self, f_previous, f_post_streaming):
        return self._apply(f_post_streaming, f_previous, f_post_streaming)


def outlet():
    """Column x=-1 takes directions 3, 6, 7 from column x=-2 of the previous state (:257-283)."""
    return _Outlet()


class _PressurePeriodic:
    """Pre-streaming rewrite of columns 0 and -1 (:286-348)."""

    _lbm_gb300_hook = True

    def __init__(self, boundary, p_in, p_out):
        b = _host_mask(boundary)
        assert b.dtype == bool
        assert np.all(b[0, :] == b[-1, :]) or np.all(b[:, 0] == b[:, -1])
        self.shape = b.shape
        self.rho_in = np.divide(p_in, _CS ** 2)
        self.rho_out = np.divide(p_out, _CS ** 2)
        if np.all(b[0, :] == b[-1, :]):
            self.n_rows = b.shape[1]
            self.dirs_in, self.dirs_out = [1, 5, 8], [3, 6, 7]
        else:
            # the reference still rewrites columns 0 and -1 here, with density
            # arrays sized by nx: it only runs when nx == ny
            self.n_rows = b.shape[0]
            self.dirs_in, self.dirs_out = [2, 5, 6], [4, 7, 8]

    @property
    def spec(self):
        return (self.dirs_in, self.dirs_out, self.rho_in, self.rho_out)

    def __call__(self, f_pre_streaming, density, velocity):
        assert self.shape == tuple(f_pre_streaming.shape[0:2])
        dev = A.to_device(f_pre_streaming)
        rho, u = A.to_device(density), A.to_device(velocity)
        nx, ny = int(dev.shape[0]), int(dev.shape[1])
        assert self.n_rows == ny, "density_in has %d entries for %d rows" % (self.n_rows, ny)
        g = CompiledGeometry(nx, ny, (), pressure=self.spec)
        _lib.call("lbm_pressure_prestream_f64", g.ref, dev.data_ptr(), rho.data_ptr(), u.data_ptr(), A.stream())
        return A.write_back(f_pre_streaming, dev)


def periodic_with_pressure_variations(boundary, p_in, p_out):
    """Periodic boundary with an inlet/outlet density difference (:286-348)."""
    return _PressurePeriodic(boundary, p_in, p_out)

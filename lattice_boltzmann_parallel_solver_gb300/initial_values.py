"""Drop-in for the reference's ``src/initial_values.py``: initial density and
velocity fields (host arrays, float64, reference layout)."""
from __future__ import annotations

import numpy as np


def sinusoidal_density_x(lattice_grid_shape, initial_p0, epsilon, check: bool = True):
    """rho = p0 + eps sin(2 pi x / lx), u = 0 (:38-64).  ``check`` keeps the
    reference's range asserts (p0 + eps < 1, p0 - eps > 0)."""
    if check:
        assert initial_p0 + epsilon < 1, "rho can potentially be >= 1"
        assert initial_p0 - epsilon > 0, "rho can potentially be <= 0"
    x = np.arange(0, lattice_grid_shape[0])
    rho_x = initial_p0 + epsilon * np.sin(np.divide(2 * np.pi * x, lattice_grid_shape[0]))
    rho = np.tile(rho_x, (lattice_grid_shape[1], 1)).T
    return rho, np.zeros(tuple(lattice_grid_shape) + (2,))


def sinusoidal_velocity_x(lattice_grid_shape, epsilon):
    """rho = 1, u_x = eps sin(2 pi y / ly) (:67-93)."""
    assert np.abs(epsilon) < 0.1, "|u| can potentially be >= 0.1"
    y = np.arange(0, lattice_grid_shape[1])
    ux = np.tile(epsilon * np.sin(np.divide(2 * np.pi * y, lattice_grid_shape[1])), (lattice_grid_shape[0], 1))
    return np.ones(lattice_grid_shape), np.dstack([ux, np.zeros(lattice_grid_shape)])


def density_1_velocity_0_initial(lattice_grid_shape):
    """rho = 1, u = 0 (:96-106)."""
    return np.ones(lattice_grid_shape), np.zeros(tuple(lattice_grid_shape) + (2,))


def density_1_velocity_x_u0_velocity_y_0_initial(lattice_grid_shape, u0):
    """rho = 1, u = (u0, 0) (:109-123)."""
    u = np.empty(tuple(lattice_grid_shape) + (2,))
    u[..., 0] = u0
    u[..., 1] = 0
    return np.ones(lattice_grid_shape), u

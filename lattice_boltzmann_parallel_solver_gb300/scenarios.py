"""Builders for the benchmark scenarios: initial fields (float64, reference
layout) and boundary compositions.  Seeded inputs stand in for datasets,
none exists for this path."""
from __future__ import annotations

import math

import numpy as np

from . import boundary_utils as BU


def equilibrium_np(rho, u):
    """Reference equilibrium on the host, for building initial states
    (src/lattice_boltzmann_method.py:162-188)."""
    c = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])
    w = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36])
    cu = u @ c.T
    usq = np.power(np.linalg.norm(u, axis=-1), 2)
    return w[None, None, :] * rho[..., None] * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * usq[..., None])


def shear_wave(n=64, eps=0.01):
    """rho = 1 + eps sin(2 pi x / n), u = 0, f = feq (64x64, omega 1.0 in the config)."""
    x = np.arange(n)
    rho = np.tile(1.0 + eps * np.sin(np.divide(2 * np.pi * x, n)), (n, 1)).T
    u = np.zeros((n, n, 2))
    return equilibrium_np(rho, u), rho, u


def cavity(n, u_lid=0.1):
    """Sliding-lid cavity: rho = 1, u = 0 start, three walls and a moving lid."""
    rho, u = np.ones((n, n)), np.zeros((n, n, 2))
    return equilibrium_np(rho, u), rho, u, BU.cavity_boundary_conditions(n, n, u_lid, 1.0)


def von_karman_start(lx, ly, u_in=0.1, noise=1e-3, seed=0):
    """Start of the channel study: rho = 1, u = (u_in, U(-noise, noise)) with u_y
    drawn by numpy.random.default_rng(seed), f = f_eq(rho, u)."""
    rng = np.random.default_rng(seed)
    rho = np.ones((lx, ly))
    u = np.zeros((lx, ly, 2))
    u[..., 0] = u_in
    u[..., 1] = rng.uniform(-noise, noise, (lx, ly))
    return equilibrium_np(rho, u), rho, u


def von_karman(lx=420, ly=180, plate=40, re=100.0, u_in=0.1, noise=1e-3, seed=0, plate_offset=1,
               walls=True, plate_x=None):
    """Channel with a flat plate (the precision study's form): inlet (u_in, 0), the
    reference's outlet, top/bottom bounce-back, plate of ``plate`` rows at x = lx//4
    shifted by ``plate_offset`` rows, nu = u_in * plate / re, seeded U(-noise, noise)
    on u_y."""
    nu = u_in * plate / re
    omega = 1.0 / (3.0 * nu + 0.5)
    f, rho, u = von_karman_start(lx, ly, u_in, noise, seed)
    bnd = BU.von_karman_boundary_conditions(lx, ly, 1.0, u_in, plate, plate_x=plate_x, walls=walls,
                                            plate_offset=plate_offset)
    return f, rho, u, omega, bnd


def batch_sweep_params(n=256, seed=2024):
    """The batched sweep: nx ~ U{200..1200}, ny = nx U(0.3, 0.5) rounded to even,
    plate = ny U(0.1, 0.3), Re log-uniform in [40, 250], inlet 0.1."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.integers(200, 1201))
        ny = int(round(nx * rng.uniform(0.3, 0.5) / 2) * 2)
        plate = max(2, int(round(ny * rng.uniform(0.1, 0.3))))
        re = float(math.exp(rng.uniform(math.log(40), math.log(250))))
        nu = 0.1 * plate / re
        omega = 1.0 / (3 * nu + 0.5)
        out.append({"nx": nx, "ny": ny, "plate": plate, "re": re, "omega": omega, "risky": omega > 1.95})
    return out


def von_karman_device(lx, ly, plate, re, u_in=0.1, noise=1e-3, seed=0, plate_offset=1, walls=True,
                      device="cuda"):
    """von_karman() built on the device (torch generator for the u_y noise, the
    package's equilibrium kernel), for many or large lattices."""
    import torch
    from .lattice_boltzmann_method import equilibrium_distr_func
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    nu = u_in * plate / re
    omega = 1.0 / (3.0 * nu + 0.5)
    rho = torch.ones((lx, ly), dtype=torch.float64, device=device)
    u = torch.zeros((lx, ly, 2), dtype=torch.float64, device=device)
    u[..., 0] = u_in
    u[..., 1] = (torch.rand((lx, ly), generator=gen, dtype=torch.float64, device=device) * 2 - 1) * noise
    bnd = BU.von_karman_boundary_conditions(lx, ly, 1.0, u_in, plate, walls=walls, plate_offset=plate_offset)
    return equilibrium_distr_func(rho, u), rho, u, omega, bnd

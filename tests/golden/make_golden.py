"""Generate the golden fixtures in this folder by running the REFERENCE solver.

Run from the repository root in a container where the reference checkout is
available (it is read, never modified):

    python tests/golden/make_golden.py <path of the reference checkout>

The reference is pure Python/NumPy.  Its ``boundary_utils`` and
``parallelization_utils`` modules import ``mpi4py``; a single-rank stand-in
(every neighbour is the rank itself, Sendrecv copies the send buffer into the
receive buffer) is placed on ``sys.path`` so that the reference's own
von Karman composition and halo exchange run unchanged on one process.

Every fixture holds the reference's outputs for seeded inputs; the oracle is
pinned to them in ``tests/test_oracle_golden.py``.  The missing upstream
fixtures ``tests/von_karman_vortex_shedding/f_0..f_10.npy`` are regenerated
here (as checksums and a reduced-size full field) with the reference's
single-rank path, and the regenerated probe trace is checked against the
upstream ``vel_at_p.npy`` before it is written.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_mpi_stub():
    mpi = types.ModuleType("mpi4py.MPI")

    class _Cart:
        def Get_coords(self, rank):
            return [0, 0]

        def Shift(self, direction, disp):
            return 0, 0

        def Sendrecv(self, sendbuf, dest, recvbuf=None, source=None):
            recvbuf[...] = sendbuf

    class _World(_Cart):
        def Get_size(self):
            return 1

        def Get_rank(self):
            return 0

        def Create_cart(self, dims, periods, reorder=False):
            return _Cart()

    mpi.COMM_WORLD = _World()
    mpi.Intracomm = _Cart
    pkg = types.ModuleType("mpi4py")
    pkg.MPI = mpi
    sys.modules["mpi4py"] = pkg
    sys.modules["mpi4py.MPI"] = mpi


def main(ref_root):
    _install_mpi_stub()
    sys.path.insert(0, os.path.join(ref_root, "src"))
    if not hasattr(np, "bool"):
        np.bool = bool
    import lattice_boltzmann_method as L
    import boundary_conditions as B
    import boundary_utils as U
    import parallelization_utils as P

    rng = np.random.default_rng(20261203)
    out = {}

    # ---- component functions on seeded random inputs --------------------
    nx, ny = 7, 5
    f = rng.uniform(0.01, 0.3, (nx, ny, 9))
    rho = rng.uniform(0.8, 1.2, (nx, ny))
    u = rng.normal(0.0, 0.05, (nx, ny, 2))
    f_zero_rho = f.copy()
    f_zero_rho[2, 3, :] = 0.0
    rho0 = L.compute_density(f_zero_rho)
    out.update(fn_f=f, fn_rho=rho, fn_u=u,
               fn_density=L.compute_density(f),
               fn_velocity=L.compute_velocity_field(L.compute_density(f), f),
               fn_f_zero_rho=f_zero_rho,
               fn_velocity_zero_rho=L.compute_velocity_field(rho0, f_zero_rho),
               fn_streaming=L.streaming(f),
               fn_feq=L.equilibrium_distr_func(rho, u),
               fn_feq_1d=L.equilibrium_distr_func(rho[3], u[3]),
               fn_step_f=L.lattice_boltzmann_step(f, rho, u, 1.3)[0],
               fn_step_rho=L.lattice_boltzmann_step(f, rho, u, 1.3)[1],
               fn_step_u=L.lattice_boltzmann_step(f, rho, u, 1.3)[2])

    # ---- boundary primitives -------------------------------------------------
    nx, ny = 9, 6
    f_pre = rng.uniform(0.01, 0.3, (nx, ny, 9))
    f_post = rng.uniform(0.01, 0.3, (nx, ny, 9))
    f_prev = rng.uniform(0.01, 0.3, (nx, ny, 9))
    rho = rng.uniform(0.9, 1.1, (nx, ny))
    u = rng.normal(0.0, 0.04, (nx, ny, 2))
    out.update(bc_f_pre=f_pre, bc_f_post=f_post, bc_f_prev=f_prev, bc_rho=rho, bc_u=u)
    edges = {"x0": (0, None), "x1": (-1, None), "y0": (None, 0), "y1": (None, -1)}
    for name, (ex, ey) in edges.items():
        m = np.zeros((nx, ny), dtype=bool)
        if ex is not None:
            m[ex, :] = True
        else:
            m[:, ey] = True
        out["bc_rigid_" + name] = B.rigid_wall(m)(f_pre, f_post.copy())
        out["bc_moving_" + name] = B.moving_wall(m, np.array([0.07, -0.03]), 1.1)(f_pre, f_post.copy())
    plate = np.zeros((nx, ny), dtype=bool)
    plate[3, 1:5] = True
    out["bc_object_mask"] = plate.copy()
    out["bc_object"] = B.rigid_object(plate.copy())(f_pre, f_post.copy())
    out["bc_inlet"] = B.inlet((nx, ny), 1.05, 0.08)(f_post.copy())
    out["bc_outlet"] = B.outlet()(f_prev, f_post.copy())
    pm = np.zeros((nx, ny), dtype=bool)
    pm[0, :] = True
    pm[-1, :] = True
    out["bc_pressure"] = B.periodic_with_pressure_variations(pm, 0.34, 0.33)(f_pre.copy(), rho, u)

    # ---- scenarios ------------------------------------------------------------
    # shear wave (64x64, omega 1, rho = 1 + 0.01 sin(2 pi x/64), u = 0, f = feq)
    n = 64
    x = np.arange(n)
    rho = np.tile(1.0 + 0.01 * np.sin(np.divide(2 * np.pi * x, n)), (n, 1)).T
    u = np.zeros((n, n, 2))
    f = L.equilibrium_distr_func(rho, u)
    amp = [np.abs(rho - 1.0).max()]
    for k in range(2000):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, 1.0)
        amp.append(np.abs(rho - 1.0).max())
        if k + 1 == 100:
            out["shear_f100"] = f.copy()
    out["shear_amp"] = np.array(amp)

    # Couette 20x30, U = 0.05, omega 1 (experiments.py:304-325)
    lx, ly = 20, 30
    rho, u = np.ones((lx, ly)), np.zeros((lx, ly, 2))
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.couette_flow_boundary_conditions(lx, ly, 0.05, np.mean(rho))
    for k in range(200):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, 1.0, bnd)
        if k + 1 in (1, 200):
            out["couette_f%d" % (k + 1)] = f.copy()

    # Poiseuille 40x20, omega 1.5, delta_p 1e-3 (experiments.py:377-406)
    lx, ly = 40, 20
    p_in, p_out = (1 + 1.5e-3) / 3, (1 - 1.5e-3) / 3
    rho, u = np.ones((lx, ly)), np.zeros((lx, ly, 2))
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.poiseuille_flow_boundary_conditions(lx, ly, p_in, p_out)
    for k in range(200):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, 1.5, bnd)
        if k + 1 in (1, 200):
            out["poiseuille_f%d" % (k + 1)] = f.copy()

    # Von Karman, reference single-rank parallel path on ghost-padded arrays
    def vk_parallel(lx, ly, d, steps):
        u0, kin = 0.1, 0.04
        omega = np.reciprocal(3 * kin + 0.5)
        comm = sys.modules["mpi4py"].MPI.COMM_WORLD
        cart = comm.Create_cart(dims=[1, 1], periods=[True, True], reorder=False)
        c2 = cart.Get_coords(0)
        nlx, nly = P.get_local_coords(c2, lx, ly, 1, 1)
        rho = np.ones((nlx + 2, nly + 2))
        u = np.zeros((nlx + 2, nly + 2, 2))
        u[..., 0] = u0
        f = L.equilibrium_distr_func(rho, u)
        _, px, py = P.global_coord_to_local_coord(c2, 3 * lx // 4, ly // 2, lx, ly, 1, 1)
        probe = [np.linalg.norm(u[px, py, ...])]
        bnd = U.parallel_von_karman_boundary_conditions(c2, nlx, nly, lx, ly, 1, 1, 1.0, u0, d)
        com = P.communication(cart)
        for _ in range(steps):
            f, rho, u = L.lattice_boltzmann_step(f, rho, u, omega, bnd, com)
            probe.append(np.linalg.norm(u[px, py, ...]))
        return f, rho, u, np.array(probe)

    f, rho, u, probe = vk_parallel(420, 180, 40, 11)
    upstream = np.load(os.path.join(ref_root, "tests", "von_karman_vortex_shedding", "vel_at_p.npy"))
    assert np.array_equal(probe, upstream), "regenerated probe trace differs from upstream"
    core = f[1:-1, 1:-1, :]
    out["vk420_probe"] = probe
    out["vk420_f11_sum"] = np.array([core.sum(), (core * core).sum(), core.max(), core.min()])
    out["vk420_f11_sample"] = core[::7, ::5, :].copy()
    f, rho, u, probe = vk_parallel(84, 36, 8, 30)
    out["vk84_f30_padded"] = f.copy()
    out["vk84_rho30_padded"] = rho.copy()
    out["vk84_u30_padded"] = u.copy()

    # serial von Karman with rigid_object (milestoneQuickFunctionCalls.py:293-326), 84x36, d=8
    lx, ly, d, u0 = 84, 36, 8, 0.1
    omega = np.reciprocal(3 * 0.04 + 0.5)

    def bnd_serial(f_pre, f_post, density=None, velocity=None, f_previous=None):
        f_post = B.inlet((lx, ly), 1.0, u0)(f_post)
        f_post = B.outlet()(f_previous, f_post)
        pl = np.zeros((lx, ly))
        pl[lx // 4, ly // 2 - d // 2:ly // 2 + d // 2] = 1
        return B.rigid_object(pl.astype(bool))(f_pre, f_post)

    rho = np.ones((lx, ly))
    u = np.zeros((lx, ly, 2))
    u[..., 0] = u0
    f = L.equilibrium_distr_func(rho, u)
    for _ in range(30):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, omega, bnd_serial)
    out["vk84_serial_f30"] = f.copy()

    # sliding-lid cavity 32x32, omega 1.7, lid 0.1: reference streaming/collision,
    # reference rigid_wall (bottom) and moving_wall (lid), restated lateral walls
    n = 32
    rho, u = np.ones((n, n)), np.zeros((n, n, 2))
    f = L.equilibrium_distr_func(rho, u)
    mb = np.zeros((n, n), dtype=bool)
    mb[:, 0] = True
    mt = np.zeros((n, n), dtype=bool)
    mt[:, -1] = True
    bottom = B.rigid_wall(mb)
    lid = B.moving_wall(mt, np.array([0.1, 0.0]), 1.0)
    opp = L.vel_to_opp_vel_mapping()

    def bnd_cavity(f_pre, f_post, density=None, velocity=None, f_previous=None):
        for a in (1, 5, 8):
            f_post[0, :, a] = f_pre[0, :, opp[a]]
        for a in (3, 7, 6):
            f_post[-1, :, a] = f_pre[-1, :, opp[a]]
        f_post = bottom(f_pre, f_post)
        return lid(f_pre, f_post)

    for k in range(100):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, 1.7, bnd_cavity)
    out["cavity_f100"] = f.copy()

    # mass preservation (tests/test_mass_preservation.py:22-34): 50x50, omega 0.5
    rho = np.ones((50, 50)) * 0.5
    rho[24, 24] = 0.6
    u = np.zeros((50, 50, 2))
    f = L.equilibrium_distr_func(rho, u)
    mass = [rho.sum()]
    for k in range(10000):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, 0.5)
        if (k + 1) % 100 == 0:
            mass.append(rho.sum())
    out["mass_trace"] = np.array(mass)
    out["mass_rho10000"] = rho.copy()

    path = os.path.join(HERE, "reference_fixtures.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])

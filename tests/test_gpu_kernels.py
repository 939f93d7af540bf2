"""The vectorised fused kernel (several nodes per thread, warp-shuffled x
shifts) against the one-node-per-thread kernel, for every storage and
nodes-per-thread choice, on geometries with walls, inlet/outlet, plate and
the pressure rewrite, and on widths that leave partial warps and rows that
are only two chunks wide."""
import numpy as np
import pytest
import torch

from oracle import lbm_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    import lattice_boltzmann_parallel_solver_gb300 as P
    P._lib.load()
    return P


def geometries(pkg, nx, ny):
    U = pkg.boundary_utils
    yield "periodic", None
    yield "cavity", U.cavity_boundary_conditions(nx, ny, 0.1, 1.0)
    yield "poiseuille", U.poiseuille_flow_boundary_conditions(nx, ny, (1 + 3e-3) / 3, (1 - 3e-3) / 3)
    yield "vk", U.von_karman_boundary_conditions(nx, ny, 1.0, 0.1, max(2, ny // 5), walls=True)


def start(nx, ny, seed):
    rng = np.random.default_rng(seed)
    rho = 1 + rng.normal(0, 0.01, (nx, ny))
    u = rng.normal(0, 0.03, (nx, ny, 2))
    return O.equilibrium(rho, u), rho, u


TOL = {"fx64": 1e-13, "f64": 1e-13, "f32": 1e-6, "f16": 1e-3, "bf16": 1e-2}


@pytest.mark.parametrize("storage,npt", [("fx64", 1), ("fx64", 2), ("fx64", 4), ("f64", 2), ("f64", 4), ("f32", 2), ("f32", 4), ("f16", 4),
                                         ("f16", 8), ("bf16", 4), ("bf16", 8)])
@pytest.mark.parametrize("nx,ny", [(16, 9), (48, 20), (520, 12), (1040, 7)])
def test_vectorised_matches_generic(pkg, storage, npt, nx, ny):
    if nx < 2 * npt or nx % npt:
        pytest.skip("width not supported by this chunk size")
    f, rho, u = start(nx, ny, nx * 7 + ny)
    for name, bnd in geometries(pkg, nx, ny):
        a = pkg.Lattice(nx, ny, 1.3, bnd, storage=storage, generic=True, stochastic=False).set_state(f, rho, u).step(25)
        b = pkg.Lattice(nx, ny, 1.3, bnd, storage=storage, npt=npt, stochastic=False).set_state(f, rho, u).step(25)
        fa, ra, ua = a.read()
        fb, rb, ub = b.read()
        err = float((fa - fb).abs().max() / fa.abs().max())
        assert err <= TOL[storage], "%s %s: %.3e" % (name, storage, err)


@pytest.mark.parametrize("storage", ["fx64", "f64"])
def test_vectorised_f64_against_oracle_with_pressure_and_outlet(pkg, storage):
    nx, ny = 64, 18
    U = pkg.boundary_utils
    f, rho, u = start(nx, ny, 3)
    for obnd, bnd in ((O.poiseuille_boundary(nx, ny, 0.34, 0.33), U.poiseuille_flow_boundary_conditions(nx, ny, 0.34, 0.33)),
                      (O.von_karman_boundary(nx, ny, 1.0, 0.1, 6), U.von_karman_boundary_conditions(nx, ny, 1.0, 0.1, 6))):
        ref = O.run(f, rho, u, 1.4, 40, obnd)
        lat = pkg.Lattice(nx, ny, 1.4, bnd, storage=storage, npt=2).set_state(f, rho, u).step(40)
        got = lat.read()[0].cpu().numpy()
        assert np.abs(got - ref[0]).max() / np.abs(ref[0]).max() <= 1e-12


def test_stochastic_rounding_keeps_slow_flows_accurate(pkg):
    """Couette flow from rest (64x64, moving wall 0.05, 3000 steps): binary16
    storage with stochastic rounding stays within 1e-3 relative velocity L2 of
    float64; round-to-nearest loses the small increments near the diffusion front."""
    n, uw = 64, 0.05
    m0 = np.zeros((n, n), bool)
    m0[:, 0] = True
    m1 = np.zeros((n, n), bool)
    m1[:, -1] = True
    B = pkg.boundary_conditions
    bnd = pkg.boundary_utils.Boundary([B.rigid_wall(m0), B.moving_wall(m1, np.array([uw, 0.0]), 1.0)])
    rho, u = np.ones((n, n)), np.zeros((n, n, 2))
    f = O.equilibrium(rho, u)
    ref = pkg.Lattice(n, n, 1.0, bnd, storage="f64").set_state(f, rho, u).step(3000).moments()[1]
    errs = {}
    for st in ("f16", "bf16"):
        for sr in (True, False):
            got = pkg.Lattice(n, n, 1.0, bnd, storage=st, stochastic=sr).set_state(f, rho, u).step(3000).moments()[1]
            errs[(st, sr)] = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
    assert errs[("f16", True)] <= 1e-3, errs
    assert errs[("f16", True)] < errs[("f16", False)], errs
    assert errs[("bf16", True)] < errs[("bf16", False)], errs


@pytest.mark.parametrize("name", ["cavity", "poiseuille", "vk"])
def test_fixed_point_matches_native_and_oracle(pkg, name):
    """The fixed-point storage and the float64 storage (FMA collision) both
    stay within 1e-12 of the oracle over 500 steps."""
    nx, ny = 72, 40
    geo = dict(geometries(pkg, nx, ny))
    obnd = {"cavity": O.cavity_boundary(nx, ny, 0.1, 1.0),
            "poiseuille": O.poiseuille_boundary(nx, ny, (1 + 3e-3) / 3, (1 - 3e-3) / 3),
            "vk": None}[name]
    if name == "vk":
        bnd = pkg.boundary_utils.von_karman_boundary_conditions(nx, ny, 1.0, 0.1, 8)
        obnd = O.von_karman_boundary(nx, ny, 1.0, 0.1, 8)
    else:
        bnd = geo[name]
    f, rho, u = start(nx, ny, 11)
    ref = O.run(f, rho, u, 1.6, 500, obnd)[0]
    for storage in ("fx64", "f64"):
        got = pkg.Lattice(nx, ny, 1.6, bnd, storage=storage).set_state(f, rho, u).step(500)
        err = float(np.abs(got.read()[0].cpu().numpy() - ref).max() / np.abs(ref).max())
        assert err <= 1e-12, (storage, err)


def test_fixed_point_falls_back_outside_its_range(pkg):
    """Populations scaled by 10 (rho >= 8) take the float64 collision; BGK is
    homogeneous in f, so the result is 10 times the unscaled one."""
    nx, ny = 40, 24
    f, rho, u = start(nx, ny, 5)
    ref = O.run(10 * f, 10 * rho, u, 1.3, 50)[0]
    got = pkg.Lattice(nx, ny, 1.3, storage="fx64").set_state(10 * f, 10 * rho, u).step(50).read()[0].cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12


def test_fixed_point_fast_nodes_and_nan(pkg):
    """Nodes with |ux| + |uy| > 0.49 take the float64 collision and stay within
    1e-12 of the oracle; a NaN population stays NaN (and spreads) instead of
    turning into a number."""
    nx, ny = 40, 24
    rng = np.random.default_rng(9)
    rho = 1 + rng.normal(0, 0.01, (nx, ny))
    u = rng.normal(0, 0.03, (nx, ny, 2))
    u[5:9, 3:7] = (0.3, -0.28)
    f = O.equilibrium(rho, u)
    ref = O.run(f, rho, u, 1.1, 20)[0]
    got = pkg.Lattice(nx, ny, 1.1, storage="fx64").set_state(f, rho, u).step(20).read()[0].cpu().numpy()
    assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12
    g = f.copy()
    g[10, 10, 0] = np.nan
    out = pkg.Lattice(nx, ny, 1.1, storage="fx64").set_state(g).step(3).read()[0].cpu().numpy()
    assert np.isnan(out[10, 10]).any() and np.isnan(out).sum() > 9 and np.isfinite(out[30, 5]).all()


@pytest.mark.parametrize("storage", ["fx64", "f64", "f32", "f16", "bf16"])
@pytest.mark.parametrize("name", ["cavity", "poiseuille", "vk"])
def test_boundary_node_pass_equals_inline_sources(pkg, storage, name):
    """The step as a boundary-free pass over every node plus a pass over the
    listed boundary nodes gives the same bits as the boundary sources applied
    inside the step (moments of the last step included)."""
    nx, ny = 1024, 1024  # below the default size of the pass: forced
    bnd = dict(geometries(pkg, nx, ny))[name]
    geo = bnd.geometry(nx, ny)
    assert 0 < geo.struct.n_bcnodes * 8 <= nx * ny
    f, rho, u = start(nx, ny, 21)
    a = pkg.Lattice(nx, ny, 1.3, bnd, storage=storage, bc_inline=False).set_state(f, rho, u).step(30)
    b = pkg.Lattice(nx, ny, 1.3, bnd, storage=storage, bc_inline=True).set_state(f, rho, u).step(30)
    for x, y in zip(a.read(), b.read()):
        assert torch.equal(x, y)
    assert torch.equal(a.pop[a.cur], b.pop[b.cur])

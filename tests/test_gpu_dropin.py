"""GPU parity of the drop-in modules against the reference's own outputs
(tests/golden fixtures made by running the reference) and its unit-test
known answers.  Component functions and the exact-arithmetic step must be
bit-identical to NumPy; the FMA form of the step must stay within 1e-12
relative max error."""
import numpy as np
import pytest
import torch

from oracle import lbm_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12  # max|f_gpu - f_ref| / max|f_ref|


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def pkg():
    import lattice_boltzmann_parallel_solver_gb300 as P
    P._lib.load()
    return P


def test_component_functions_bit_exact(pkg, golden):
    L = pkg.lattice_boltzmann_method
    g = golden
    assert np.array_equal(L.compute_density(g["fn_f"]), g["fn_density"])
    assert np.array_equal(L.compute_velocity_field(L.compute_density(g["fn_f"]), g["fn_f"]), g["fn_velocity"])
    rz = L.compute_density(g["fn_f_zero_rho"])
    assert np.array_equal(L.compute_velocity_field(rz, g["fn_f_zero_rho"]), g["fn_velocity_zero_rho"])
    assert np.array_equal(L.streaming(g["fn_f"]), g["fn_streaming"])
    assert np.array_equal(L.equilibrium_distr_func(g["fn_rho"], g["fn_u"]), g["fn_feq"])
    feq1 = L.equilibrium_distr_func(g["fn_rho"][3], g["fn_u"][3])
    assert feq1.shape == g["fn_feq_1d"].shape and np.array_equal(feq1, g["fn_feq_1d"])
    f, r, u = L.lattice_boltzmann_step(g["fn_f"], g["fn_rho"], g["fn_u"], 1.3)
    assert np.array_equal(f, g["fn_step_f"]) and np.array_equal(r, g["fn_step_rho"])
    assert np.array_equal(u, g["fn_step_u"])
    f, r, u = L.lattice_boltzmann_step(g["fn_f"], g["fn_rho"], g["fn_u"], 1.3, exact=False)
    assert rel(f, g["fn_step_f"]) <= TOL


def test_torch_inputs_return_torch(pkg, golden):
    L = pkg.lattice_boltzmann_method
    f = torch.from_numpy(golden["fn_f"]).cuda()
    rho = L.compute_density(f)
    assert isinstance(rho, torch.Tensor) and rho.is_cuda
    assert np.array_equal(rho.cpu().numpy(), golden["fn_density"])


def test_boundary_closures_bit_exact(pkg, golden):
    B = pkg.boundary_conditions
    g = golden
    nx, ny = g["bc_f_pre"].shape[:2]
    for name, (ex, ey) in {"x0": (0, None), "x1": (-1, None), "y0": (None, 0), "y1": (None, -1)}.items():
        m = np.zeros((nx, ny), dtype=bool)
        if ex is not None:
            m[ex, :] = True
        else:
            m[:, ey] = True
        post = g["bc_f_post"].copy()
        out = B.rigid_wall(m)(g["bc_f_pre"], post)
        assert out is post and np.array_equal(post, g["bc_rigid_" + name])
        post = g["bc_f_post"].copy()
        B.moving_wall(m, np.array([0.07, -0.03]), 1.1)(g["bc_f_pre"], post)
        assert np.array_equal(post, g["bc_moving_" + name])
    post = g["bc_f_post"].copy()
    B.rigid_object(g["bc_object_mask"].copy())(g["bc_f_pre"], post)
    assert np.array_equal(post, g["bc_object"])
    post = g["bc_f_post"].copy()
    B.inlet((nx, ny), 1.05, 0.08)(post)
    assert np.array_equal(post, g["bc_inlet"])
    post = g["bc_f_post"].copy()
    B.outlet()(g["bc_f_prev"], post)
    assert np.array_equal(post, g["bc_outlet"])
    pm = np.zeros((nx, ny), dtype=bool)
    pm[0, :] = True
    pm[-1, :] = True
    pre = g["bc_f_pre"].copy()
    B.periodic_with_pressure_variations(pm, 0.34, 0.33)(pre, g["bc_rho"], g["bc_u"])
    assert np.array_equal(pre, g["bc_pressure"])


def test_known_answers(pkg):
    """tests/test_boundary_conditions.py:12-121 of the reference."""
    B, L = pkg.boundary_conditions, pkg.lattice_boltzmann_method
    shape = (10, 10)
    u = np.zeros(shape + (2,))
    u[..., 0] = 0.1
    feq = L.equilibrium_distr_func(np.ones(shape), u)
    f = B.inlet(shape, 1, 0.1)(np.zeros(shape + (9,)))
    assert np.allclose(f[0], feq[0]) and np.allclose(f[1:], 0)
    f = B.outlet()(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    for i in range(9):
        assert np.allclose(f[-1, :, i], 1.0 if i in (3, 6, 7) else 0.0)
    m = np.zeros(shape, dtype=bool)
    m[:, -1] = True
    f = B.rigid_wall(m)(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    for i in range(9):
        assert np.allclose(f[m, i], 1.0 if i in (4, 7, 8) else 0.0)
    f = B.moving_wall(m, np.array([2, 0]), 1)(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    assert np.allclose(f[m, 4], 1) and np.allclose(f[m, 7], 1 - 1 / 3) and np.allclose(f[m, 8], 1 + 1 / 3)
    pm = np.zeros(shape, dtype=bool)
    pm[0, :] = True
    pm[-1, :] = True
    f = B.periodic_with_pressure_variations(pm, 1, 0.1)(np.ones(shape + (9,)), np.ones(shape), u)
    assert np.allclose(f[0, :, 1], 1.29555)
    assert np.allclose(f[0, :, 5], 1.073888) and np.allclose(f[0, :, 8], 1.073888)
    assert np.allclose(f[-1, :, 3], 0.943222)
    assert np.allclose(f[-1, :, 6], 0.9858) and np.allclose(f[-1, :, 7], 0.9858)


def _drive(L, f, rho, u, omega, steps, bnd=None, comm=None, exact=True):
    for _ in range(steps):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, omega, bnd, comm, exact=exact)
    return f, rho, u


@pytest.mark.parametrize("exact", [True, False])
def test_step_scenarios_against_reference_outputs(pkg, golden, exact):
    L, U = pkg.lattice_boltzmann_method, pkg.boundary_utils
    check = (lambda a, b: np.array_equal(a, b)) if exact else (lambda a, b: rel(a, b) <= TOL)
    # shear wave 64x64, 100 steps
    x = np.arange(64)
    rho = np.tile(1.0 + 0.01 * np.sin(np.divide(2 * np.pi * x, 64)), (64, 1)).T
    u = np.zeros((64, 64, 2))
    f = L.equilibrium_distr_func(rho, u)
    assert check(_drive(L, f, rho, u, 1.0, 100, exact=exact)[0], golden["shear_f100"])
    # Couette 20x30 (boundary_utils.py:9-55)
    rho, u = np.ones((20, 30)), np.zeros((20, 30, 2))
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.couette_flow_boundary_conditions(20, 30, 0.05, 1.0)
    out = _drive(L, f, rho, u, 1.0, 1, bnd, exact=exact)
    assert check(out[0], golden["couette_f1"])
    assert check(_drive(L, *out, 1.0, 199, bnd, exact=exact)[0], golden["couette_f200"])
    # Poiseuille 40x20 (boundary_utils.py:58-110)
    rho, u = np.ones((40, 20)), np.zeros((40, 20, 2))
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.poiseuille_flow_boundary_conditions(40, 20, (1 + 1.5e-3) / 3, (1 - 1.5e-3) / 3)
    out = _drive(L, f, rho, u, 1.5, 1, bnd, exact=exact)
    assert check(out[0], golden["poiseuille_f1"])
    assert check(_drive(L, *out, 1.5, 199, bnd, exact=exact)[0], golden["poiseuille_f200"])
    # cavity 32x32
    rho, u = np.ones((32, 32)), np.zeros((32, 32, 2))
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.cavity_boundary_conditions(32, 32, 0.1, 1.0)
    assert check(_drive(L, f, rho, u, 1.7, 100, bnd, exact=exact)[0], golden["cavity_f100"])


def test_von_karman_padded_with_halo_hook(pkg, golden):
    """The reference's parallel VK path on one rank: padded arrays, halo hook, unfused."""
    L, U = pkg.lattice_boltzmann_method, pkg.boundary_utils
    lx, ly, d = 84, 36, 8
    rho, u = pkg.initial_values.density_1_velocity_x_u0_velocity_y_0_initial((lx + 2, ly + 2), 0.1)
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.parallel_von_karman_boundary_conditions([0, 0], lx, ly, lx, ly, 1, 1, 1.0, 0.1, d)
    comm = U.communication(None)
    omega = np.reciprocal(3 * 0.04 + 0.5)
    f, rho, u = _drive(L, f, rho, u, omega, 30, bnd, comm)
    assert np.array_equal(f, golden["vk84_f30_padded"])
    assert np.array_equal(rho, golden["vk84_rho30_padded"])
    assert np.array_equal(u, golden["vk84_u30_padded"])


def test_von_karman_fused_unpadded(pkg, golden):
    L, U = pkg.lattice_boltzmann_method, pkg.boundary_utils
    lx, ly, d = 84, 36, 8
    rho, u = pkg.initial_values.density_1_velocity_x_u0_velocity_y_0_initial((lx, ly), 0.1)
    f = L.equilibrium_distr_func(rho, u)
    bnd = U.von_karman_boundary_conditions(lx, ly, 1.0, 0.1, d)
    omega = np.reciprocal(3 * 0.04 + 0.5)
    f, _, _ = _drive(L, f, rho, u, omega, 30, bnd)
    assert np.array_equal(f, golden["vk84_serial_f30"])


def test_reference_vk_integration_420x180(pkg, golden):
    """tests/test_parallelization_von_karman.py:18-66: 11 steps, probe trace and populations."""
    L, U = pkg.lattice_boltzmann_method, pkg.boundary_utils
    lx, ly = 420, 180
    rho, u = pkg.initial_values.density_1_velocity_x_u0_velocity_y_0_initial((lx + 2, ly + 2), 0.1)
    f = torch.from_numpy(L.equilibrium_distr_func(rho, u)).cuda()
    rho, u = torch.from_numpy(rho).cuda(), torch.from_numpy(u).cuda()
    bnd = U.parallel_von_karman_boundary_conditions([0, 0], lx, ly, lx, ly, 1, 1, 1.0, 0.1, 40)
    comm = U.communication(None)
    omega = np.reciprocal(3 * 0.04 + 0.5)
    px, py = 3 * lx // 4 + 1, ly // 2 + 1
    probe = [float(np.linalg.norm(u[px, py].cpu().numpy()))]
    for _ in range(11):
        f, rho, u = L.lattice_boltzmann_step(f, rho, u, omega, bnd, comm)
        probe.append(float(np.linalg.norm(u[px, py].cpu().numpy())))
    assert np.array_equal(np.array(probe), golden["vk420_probe"])
    core = f[1:-1, 1:-1].cpu().numpy()
    assert np.array_equal(core[::7, ::5], golden["vk420_f11_sample"])


def test_argument_errors(pkg):
    L = pkg.lattice_boltzmann_method
    f = np.ones((4, 5, 9)) / 9
    rho, u = np.ones((4, 5)), np.zeros((4, 5, 2))
    with pytest.raises(AssertionError):
        L.lattice_boltzmann_step(f, rho, u, 2.0)
    with pytest.raises(AssertionError):
        L.lattice_boltzmann_step(f, np.ones((4, 4)), u, 1.0)
    with pytest.raises(AssertionError):
        L.compute_density(np.ones((4, 5, 8)))
    with pytest.raises(AssertionError):
        pkg.boundary_conditions.rigid_wall(np.zeros((4, 5)))


@pytest.mark.parametrize("name", ["none", "cavity", "poiseuille", "vk"])
@pytest.mark.parametrize("slabs", [1, 3, 8])
def test_host_buffer_step_matches_device_step(name, slabs):
    """The slab-pipelined step on host buffers gives the device step's result
    bit for bit (exact and FMA forms), whatever the slab count."""
    import lattice_boltzmann_parallel_solver_gb300.boundary_utils as U
    from lattice_boltzmann_parallel_solver_gb300 import lattice_boltzmann_method as M
    nx, ny = 67, 40
    bnd = {"none": None, "cavity": U.cavity_boundary_conditions(nx, ny, 0.1, 1.0),
           "poiseuille": U.poiseuille_flow_boundary_conditions(nx, ny, 0.34, 0.33),
           "vk": U.von_karman_boundary_conditions(nx, ny, 1.0, 0.1, 8)}[name]
    rng = np.random.default_rng(slabs)
    rho = 1 + rng.normal(0, 0.01, (nx, ny))
    u = rng.normal(0, 0.03, (nx, ny, 2))
    f = O.equilibrium(rho, u)
    for exact in (True, False):
        dev = M.lattice_boltzmann_step(torch.from_numpy(f).cuda(), torch.from_numpy(rho).cuda(),
                                       torch.from_numpy(u).cuda(), 1.3, bnd, exact=exact)
        geo = bnd.geometry(nx, ny) if bnd is not None else M.empty_geometry(nx, ny)
        flags = M._lib.FLAG_EXACT if exact else 0
        host = M._step_host(geo, f, rho, u, 1.3, flags, M.A.NUMPY, slabs=slabs)
        for a, b in zip(host, dev):
            assert np.array_equal(a, b.cpu().numpy())
    if slabs == 8:
        # the public call on NumPy arrays takes this path and matches the oracle bit for bit
        got = M.lattice_boltzmann_step(f, rho, u, 1.3, bnd)
        assert isinstance(got[0], np.ndarray)
        if name in ("none", "cavity"):
            ref = O.run(f, rho, u, 1.3, 1, None if name == "none" else O.cavity_boundary(nx, ny, 0.1, 1.0))
            for a, b in zip(got, ref):
                assert np.array_equal(a, b)


@pytest.mark.parametrize("shape", [(1, 1), (2, 3), (5, 130), (33, 7), (130, 5)])
@pytest.mark.parametrize("slabs", [0, 4, 64])
def test_host_buffer_step_edge_sizes(shape, slabs):
    """Tiny and ragged lattices, and more slabs than columns: the host-buffer
    step still equals the device step bit for bit, and the oracle in exact mode."""
    from lattice_boltzmann_parallel_solver_gb300 import lattice_boltzmann_method as M
    nx, ny = shape
    rng = np.random.default_rng(nx * 100 + ny)
    rho = rng.uniform(0.9, 1.1, shape)
    u = rng.normal(0, 0.03, shape + (2,))
    f = O.equilibrium(rho, u) + rng.normal(0, 1e-3, shape + (9,))
    geo = M.empty_geometry(nx, ny)
    host = M._step_host(geo, f, rho, u, 1.2, M._lib.FLAG_EXACT, M.A.NUMPY, slabs=slabs)
    ref = O.run(f, rho, u, 1.2, 1)
    for a, b in zip(host, ref):
        assert np.array_equal(a, b)


def test_host_buffer_step_rejects_bad_shapes():
    from lattice_boltzmann_parallel_solver_gb300 import lattice_boltzmann_method as M
    f = np.ones((4, 5, 8))
    with pytest.raises(AssertionError):
        M.lattice_boltzmann_step(f, np.ones((4, 5)), np.zeros((4, 5, 2)), 1.0)
    f = np.ones((4, 5, 9))
    with pytest.raises(AssertionError):
        M.lattice_boltzmann_step(f, np.ones((4, 6)), np.zeros((4, 5, 2)), 1.0)
    with pytest.raises(AssertionError):
        M.lattice_boltzmann_step(f, np.ones((4, 5)), np.zeros((4, 5, 2)), 2.5)

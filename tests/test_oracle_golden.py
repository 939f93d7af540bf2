"""Pins the CPU oracle to the reference: fixtures produced by running the
reference (tests/golden/make_golden.py) and the known answers of the
reference's own unit tests (tests/test_*.py in the reference checkout)."""
import numpy as np
import pytest

from oracle import lbm_oracle as O


def test_functions_bit_exact(golden):
    g = golden
    assert np.array_equal(O.density(g["fn_f"]), g["fn_density"])
    assert np.array_equal(O.velocity(O.density(g["fn_f"]), g["fn_f"]), g["fn_velocity"])
    rz = O.density(g["fn_f_zero_rho"])
    assert np.array_equal(O.velocity(rz, g["fn_f_zero_rho"]), g["fn_velocity_zero_rho"])
    assert np.array_equal(O.streaming(g["fn_f"]), g["fn_streaming"])
    assert np.array_equal(O.equilibrium(g["fn_rho"], g["fn_u"]), g["fn_feq"])
    assert np.array_equal(O.equilibrium(g["fn_rho"][3], g["fn_u"][3]), g["fn_feq_1d"])
    f, r, u = O.step(g["fn_f"], g["fn_rho"], g["fn_u"], 1.3)
    assert np.array_equal(f, g["fn_step_f"])
    assert np.array_equal(r, g["fn_step_rho"])
    assert np.array_equal(u, g["fn_step_u"])


def test_boundary_primitives_bit_exact(golden):
    g = golden
    nx, ny = g["bc_f_pre"].shape[:2]
    for name, (ex, ey) in {"x0": (0, None), "x1": (-1, None), "y0": (None, 0), "y1": (None, -1)}.items():
        m = np.zeros((nx, ny), dtype=bool)
        if ex is not None:
            m[ex, :] = True
        else:
            m[:, ey] = True
        assert np.array_equal(O.rigid_wall(m)(g["bc_f_pre"], g["bc_f_post"].copy()), g["bc_rigid_" + name])
        got = O.moving_wall(m, np.array([0.07, -0.03]), 1.1)(g["bc_f_pre"], g["bc_f_post"].copy())
        assert np.array_equal(got, g["bc_moving_" + name])
    got = O.rigid_object(g["bc_object_mask"].copy())(g["bc_f_pre"], g["bc_f_post"].copy())
    assert np.array_equal(got, g["bc_object"])
    assert np.array_equal(O.inlet((nx, ny), 1.05, 0.08)(g["bc_f_post"].copy()), g["bc_inlet"])
    assert np.array_equal(O.outlet()(g["bc_f_prev"], g["bc_f_post"].copy()), g["bc_outlet"])
    pm = np.zeros((nx, ny), dtype=bool)
    pm[0, :] = True
    pm[-1, :] = True
    got = O.periodic_with_pressure_variations(pm, 0.34, 0.33)(g["bc_f_pre"].copy(), g["bc_rho"], g["bc_u"])
    assert np.array_equal(got, g["bc_pressure"])


def test_shear_wave_trace(golden):
    n = 64
    rho, u = O.sinusoidal_density_x((n, n), 1.0, 0.01, check=False)
    f = O.equilibrium(rho, u)
    amp = [np.abs(rho - 1).max()]
    for k in range(300):
        f, rho, u = O.step(f, rho, u, 1.0)
        amp.append(np.abs(rho - 1).max())
        if k + 1 == 100:
            assert np.array_equal(f, golden["shear_f100"])
    assert np.array_equal(np.array(amp), golden["shear_amp"][:301])


@pytest.mark.parametrize("steps", [1, 200])
def test_couette(golden, steps):
    lx, ly = 20, 30
    rho, u = O.density_1_velocity_0((lx, ly))
    f = O.equilibrium(rho, u)
    f, _, _ = O.run(f, rho, u, 1.0, steps, O.couette_boundary(lx, ly, 0.05, 1.0))
    assert np.array_equal(f, golden["couette_f%d" % steps])


@pytest.mark.parametrize("steps", [1, 200])
def test_poiseuille(golden, steps):
    lx, ly = 40, 20
    rho, u = O.density_1_velocity_0((lx, ly))
    f = O.equilibrium(rho, u)
    bnd = O.poiseuille_boundary(lx, ly, (1 + 1.5e-3) / 3, (1 - 1.5e-3) / 3)
    f, _, _ = O.run(f, rho, u, 1.5, steps, bnd)
    assert np.array_equal(f, golden["poiseuille_f%d" % steps])


def _vk_padded(lx, ly, d, steps):
    omega = np.reciprocal(3 * 0.04 + 0.5)
    rho, u = O.density_1_velocity_u0((lx + 2, ly + 2), 0.1)
    f = O.equilibrium(rho, u)
    px, py = 3 * lx // 4 + 1, ly // 2 + 1
    probe = [np.linalg.norm(u[px, py])]
    bnd = O.von_karman_boundary_padded(lx, ly, 1.0, 0.1, d)
    for _ in range(steps):
        f, rho, u = O.step(f, rho, u, omega, bnd, O.halo_fill)
        probe.append(np.linalg.norm(u[px, py]))
    return f, rho, u, np.array(probe)


def test_von_karman_padded_small(golden):
    f, rho, u, _ = _vk_padded(84, 36, 8, 30)
    assert np.array_equal(f, golden["vk84_f30_padded"])
    assert np.array_equal(rho, golden["vk84_rho30_padded"])
    assert np.array_equal(u, golden["vk84_u30_padded"])


def test_von_karman_unpadded_equals_padded_interior(golden):
    lx, ly, d = 84, 36, 8
    omega = np.reciprocal(3 * 0.04 + 0.5)
    rho, u = O.density_1_velocity_u0((lx, ly), 0.1)
    f = O.equilibrium(rho, u)
    f, _, _ = O.run(f, rho, u, omega, 30, O.von_karman_boundary(lx, ly, 1.0, 0.1, d))
    assert np.array_equal(f, golden["vk84_f30_padded"][1:-1, 1:-1])
    # the serial rigid_object form of the same scenario is identical too
    assert np.array_equal(f, golden["vk84_serial_f30"])


def test_von_karman_420x180_reference_test(golden):
    """The reference's integration test (tests/test_parallelization_von_karman.py:18-66):
    420x180, d=40, 11 steps; probe trace and a checksum of the final populations."""
    f, _, _, probe = _vk_padded(420, 180, 40, 11)
    assert np.array_equal(probe, golden["vk420_probe"])
    core = f[1:-1, 1:-1]
    assert np.array_equal(core[::7, ::5], golden["vk420_f11_sample"])
    s = golden["vk420_f11_sum"]
    assert core.sum() == s[0] and (core * core).sum() == s[1]


def test_cavity(golden):
    n = 32
    rho, u = O.density_1_velocity_0((n, n))
    f = O.equilibrium(rho, u)
    f, _, _ = O.run(f, rho, u, 1.7, 100, O.cavity_boundary(n, n, 0.1, 1.0))
    assert np.array_equal(f, golden["cavity_f100"])


def test_mass_preservation_reference_trace(golden):
    rho = np.ones((50, 50)) * 0.5
    rho[24, 24] = 0.6
    u = np.zeros((50, 50, 2))
    f = O.equilibrium(rho, u)
    mass = [rho.sum()]
    for k in range(1000):
        f, rho, u = O.step(f, rho, u, 0.5)
        if (k + 1) % 100 == 0:
            mass.append(rho.sum())
    assert np.array_equal(np.array(mass), golden["mass_trace"][:11])


# ---- known answers from the reference's unit tests --------------------------
def test_known_answer_boundaries():
    # tests/test_boundary_conditions.py:12-28 (inlet)
    shape = (10, 10)
    u = np.zeros(shape + (2,))
    u[..., 0] = 0.1
    feq = O.equilibrium(np.ones(shape), u)
    f = O.inlet(shape, 1, 0.1)(np.zeros(shape + (9,)))
    assert np.allclose(f[0], feq[0]) and np.allclose(f[1:], 0)
    # :30-42 (outlet)
    f = O.outlet()(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    for i in range(9):
        assert np.allclose(f[-1, :, i], 1.0 if i in (3, 6, 7) else 0.0)
    # :44-59 (rigid top wall)
    m = np.zeros(shape, dtype=bool)
    m[:, -1] = True
    f = O.rigid_wall(m)(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    for i in range(9):
        assert np.allclose(f[m, i], 1.0 if i in (4, 7, 8) else 0.0)
    # :62-85 (moving top wall u_w = (2, 0)); direction 7 -> 1 - 1/3, 8 -> 1 + 1/3
    f = O.moving_wall(m, np.array([2, 0]), 1)(np.ones(shape + (9,)), np.zeros(shape + (9,)))
    assert np.allclose(f[m, 4], 1) and np.allclose(f[m, 7], 1 - 1 / 3) and np.allclose(f[m, 8], 1 + 1 / 3)
    # :87-121 (pressure-periodic p_in = 1, p_out = 0.1, u = (0.1, 0))
    pm = np.zeros(shape, dtype=bool)
    pm[0, :] = True
    pm[-1, :] = True
    f = O.periodic_with_pressure_variations(pm, 1, 0.1)(np.ones(shape + (9,)), np.ones(shape), u)
    assert np.allclose(f[0, :, 1], 1.29555)
    assert np.allclose(f[0, :, 5], 1.073888) and np.allclose(f[0, :, 8], 1.073888)
    assert np.allclose(f[-1, :, 3], 0.943222)
    assert np.allclose(f[-1, :, 6], 0.9858) and np.allclose(f[-1, :, 7], 0.9858)


def test_known_answer_initial_values():
    # tests/test_initial_values.py:12-63
    rho, u = O.sinusoidal_density_x((10, 10), 0.5, 0.3)
    ref = [0.5, 0.676, 0.785, 0.785, 0.676, 0.5, 0.324, 0.215, 0.215, 0.324]
    assert np.allclose(rho[:, 0], ref, atol=5e-4) and np.all(u == 0)
    rho, u = O.sinusoidal_velocity_x((10, 10), 0.05)
    ref = [0.0, 0.029, 0.048, 0.048, 0.029, 0.0, -0.029, -0.048, -0.048, -0.029]
    assert np.allclose(u[0, :, 0], ref, atol=5e-4) and np.all(rho == 1)
    with pytest.raises(AssertionError):
        O.sinusoidal_density_x((10, 10), 1.0, 0.01)


def test_known_answer_conservation():
    # tests/test_navier_stokes_eq.py, tests/test_streaming_func.py
    f = np.random.default_rng(1).random((10, 10, 9)) / 9
    rho = O.density(f)
    u = O.velocity(rho, f)
    feq = O.equilibrium(rho, u)
    assert np.allclose(feq.sum(-1), rho, rtol=0, atol=1e-15)
    assert np.allclose(feq @ O.C, rho[..., None] * u, rtol=0, atol=1e-15)
    assert abs(O.streaming(f).sum() - f.sum()) < 1e-12

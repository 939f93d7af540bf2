"""The package's initial-value functions (host code, no GPU) against the
known answers of the reference's tests/test_initial_values.py:12-63 and, bit
for bit, against the oracle's restatement of src/initial_values.py:38-123;
the channel-form start of the von Karman study built by the package's
scenario builder equals the oracle's."""
import numpy as np
import pytest

from lattice_boltzmann_parallel_solver_gb300 import initial_values as IV
from lattice_boltzmann_parallel_solver_gb300 import scenarios
from oracle import lbm_oracle as O


def test_sinusoidal_density_known_answer():
    # tests/test_initial_values.py:12-37: 10x10, p0 0.5, eps 0.3
    shape = (10, 10)
    rho, u = IV.sinusoidal_density_x(lattice_grid_shape=shape, initial_p0=0.5, epsilon=0.3)
    assert rho.shape == shape and u.shape == shape + (2,)
    rho_true = [0.5, 0.676, 0.785, 0.785, 0.676, 0.5, 0.324, 0.215, 0.215, 0.324]
    for i in range(shape[0]):
        for j in range(shape[1]):
            assert rho[i, j] == pytest.approx(rho[i, 0], abs=5e-4)
            assert u[i, j, 0] == pytest.approx(0, abs=5e-4) and u[i, j, 1] == pytest.approx(0, abs=5e-4)
        assert rho[i, 0] == pytest.approx(rho_true[i], abs=5e-4)


def test_sinusoidal_velocity_known_answer():
    # tests/test_initial_values.py:39-63: 10x10, eps 0.05
    shape = (10, 10)
    rho, u = IV.sinusoidal_velocity_x(lattice_grid_shape=shape, epsilon=0.05)
    assert rho.shape == shape and u.shape == shape + (2,)
    u_true = [0.0, 0.029, 0.048, 0.048, 0.029, 0.0, -0.029, -0.048, -0.048, -0.029]
    for i in range(shape[0]):
        for j in range(shape[1]):
            assert u[j, i, 0] == pytest.approx(u[0, i, 0], abs=5e-4)
            assert rho[i, j] == pytest.approx(1.0, abs=5e-4)
        assert u[0, i, 0] == pytest.approx(u_true[i], abs=5e-4)


def test_range_asserts_like_the_reference():
    # initial_values.py:55-56, 84: the reference rejects p0 + eps >= 1, p0 - eps <= 0, |eps| >= 0.1
    with pytest.raises(AssertionError):
        IV.sinusoidal_density_x((10, 10), 1.0, 0.01)
    with pytest.raises(AssertionError):
        IV.sinusoidal_density_x((10, 10), 0.2, 0.3)
    with pytest.raises(AssertionError):
        IV.sinusoidal_velocity_x((10, 10), 0.1)
    rho, _ = IV.sinusoidal_density_x((64, 64), 1.0, 0.01, check=False)  # the shear-wave config's start
    assert np.array_equal(rho, O.sinusoidal_density_x((64, 64), 1.0, 0.01, check=False)[0])


@pytest.mark.parametrize("shape", [(10, 10), (7, 13), (64, 64)])
def test_bit_identical_to_oracle(shape):
    a = IV.sinusoidal_density_x(shape, 0.5, 0.3)
    b = O.sinusoidal_density_x(shape, 0.5, 0.3)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    a = IV.sinusoidal_velocity_x(shape, 0.05)
    b = O.sinusoidal_velocity_x(shape, 0.05)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    a = IV.density_1_velocity_0_initial(shape)
    b = O.density_1_velocity_0(shape)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    a = IV.density_1_velocity_x_u0_velocity_y_0_initial(shape, 0.1)
    b = O.density_1_velocity_u0(shape, 0.1)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_channel_start_matches_oracle():
    f, rho, u = scenarios.von_karman_start(60, 30, 0.1, 1e-3, seed=3)
    fo, ro, uo = O.von_karman_channel_start(60, 30, 0.1, 1e-3, 3)
    assert np.array_equal(rho, ro) and np.array_equal(u, uo) and np.array_equal(f, fo)
    assert np.abs(u[..., 1]).max() <= 1e-3

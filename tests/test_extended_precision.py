"""The oracle (the reference's float64 NumPy algorithm) against the
extended-precision fixtures: float64 rounding alone moves the density-wave
amplitude trace by about 1e-13 over 2000 steps.  This is the scale of the
float64 gate used by the GPU tests, and the reason the fixed-point storage is
compared with the extended-precision runs at 1e-15 instead."""
import numpy as np

from oracle import lbm_oracle as O


def test_oracle_density_wave_drift_is_float64_rounding(extended):
    n = 64
    rho, u = O.sinusoidal_density_x((n, n), 1.0, 0.01, check=False)
    f = O.equilibrium(rho, u)
    rho, u = O.density(f), O.velocity(O.density(f), f)
    amp = []
    for _ in range(20):
        f, rho, u = O.run(f, rho, u, 1.0, 100)
        amp.append(np.abs(rho - 1).max())
    d = np.abs(np.array(amp) - extended["density_wave_amp"]).max()
    assert 1e-15 < d < 1e-12, d


def test_extended_fixture_shapes(extended):
    assert extended["density_wave_amp"].shape == (20,)
    assert extended["density_wave_rho_x"].shape == (64,)
    assert extended["random_f"].shape == (32, 24, 9)
    # the density wave decays monotonically between its oscillation extrema
    assert extended["density_wave_amp"][0] > extended["density_wave_amp"][-1]

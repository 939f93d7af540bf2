"""The Strouhal post-processing on the host (no GPU): the reference's argmax
estimate is quantised to one FFT bin, the sub-bin spectral peak estimate
(Hann window, zero padding, Gaussian interpolation) resolves the frequency of
a noisy two-harmonic trace to better than 1e-5 relative."""
import numpy as np
import pytest

from lattice_boltzmann_parallel_solver_gb300 import analysis


@pytest.mark.parametrize("f", [1.13e-3, 7.77e-4, 3.83e-4, 2.5e-3])
def test_subbin_estimate_resolves_the_frequency(f):
    n = 130001
    t = np.arange(n)
    rng = np.random.default_rng(int(f * 1e6))
    x = 0.1 + 0.01 * np.sin(2 * np.pi * f * t + 0.3) + 0.003 * np.sin(4 * np.pi * f * t) + \
        1e-4 * rng.normal(size=n)
    fe, b, pb = analysis.spectral_peak(x)
    assert b == 1.0 / n and pb == 1.0 / (16 * n)
    assert abs(fe - f) <= 1e-5 * f
    st = analysis.strouhal(x, 40, 0.1, method="interp")
    assert st == pytest.approx(f * 400, rel=1e-5)
    # the reference's estimate: the nearest FFT bin
    assert abs(analysis.strouhal(x, 40, 0.1) - f * 400) <= 0.5 * 400 / n + 1e-12


def test_start_offset_and_argument_checks():
    t = np.arange(50000)
    x = np.where(t < 20000, 0.0, np.sin(2 * np.pi * 2e-3 * t))
    fe, _, _ = analysis.spectral_peak(x, start=20000)
    assert abs(fe - 2e-3) <= 1e-6
    with pytest.raises(AssertionError):
        analysis.strouhal(x, 40, 0.1, method="nearest")

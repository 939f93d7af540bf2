"""Generate ``extended_precision.npz``: periodic D2Q9 BGK runs in x86 80-bit
extended precision (numpy.longdouble, 64-bit significand), the yardstick for
how close a float64-class solver stays to the exact arithmetic of the
reference's equations (src/lattice_boltzmann_method.py:93-228: moments,
equilibrium, BGK relaxation, periodic streaming).

    python tests/golden/make_extended.py

The initial states are the oracle's float64 ones, so the float64 runs start
from the same numbers.  Fixtures:
  density_wave_amp    max |rho - 1| every 100 steps, 2000 steps, of the
                      density wave rho = 1 + 0.01 sin(2 pi x / 64), u = 0,
                      64 x 64, omega 1 (20 values)
  density_wave_rho_x  rho(x, 0) after 2000 steps (64 values)
  random_f            f after 500 steps of a 32 x 24 state with
                      rho ~ U(0.95, 1.05), u ~ N(0, 0.05), omega 1.3
Running the generator on a machine whose long double is not the x86
extended format changes the last bits of the fixtures (the tests compare at
1e-15, far above either format's error).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])


def step_ld(f, omega):
    """One collide-then-stream step in long double."""
    dt = np.longdouble
    w = np.array([4, 1, 1, 1, 1, 0.25, 0.25, 0.25, 0.25], dtype=dt) / dt(9)
    rho = f.sum(-1)
    ux = (f * CX).sum(-1) / rho
    uy = (f * CY).sum(-1) / rho
    cu = ux[..., None] * CX + uy[..., None] * CY
    feq = w * rho[..., None] * (1 + 3 * cu + dt(4.5) * cu * cu - dt(1.5) * (ux * ux + uy * uy)[..., None])
    f = f + (feq - f) * dt(omega)
    for i in range(9):
        f[..., i] = np.roll(np.roll(f[..., i], CX[i], axis=0), CY[i], axis=1)
    return f


def main():
    from oracle import lbm_oracle as O
    out = {}
    n = 64
    rho, u = O.sinusoidal_density_x((n, n), 1.0, 0.01, check=False)
    f = O.equilibrium(rho, u).astype(np.longdouble)
    amp = []
    for k in range(2000):
        f = step_ld(f, 1.0)
        if (k + 1) % 100 == 0:
            amp.append(np.abs(f.sum(-1) - 1).max())
    out["density_wave_amp"] = np.array(amp, dtype=np.float64)
    out["density_wave_rho_x"] = f.sum(-1)[:, 0].astype(np.float64)

    rng = np.random.default_rng(0)
    rho = rng.uniform(0.95, 1.05, (32, 24))
    u = rng.normal(0, 0.05, (32, 24, 2))
    f = O.equilibrium(rho, u).astype(np.longdouble)
    for _ in range(500):
        f = step_ld(f, 1.3)
    out["random_f"] = f.astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "extended_precision.npz"), **out)


if __name__ == "__main__":
    main()

"""The fixed-point collision's arithmetic (lbm_fx.cuh, the code the fx64
kernels run) compiled for the host: periodic runs against the 80-bit
extended-precision fixtures (1e-15) and the NumPy oracle (the 1e-12 float64
gate), and a few identities of its integer helpers."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import lbm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def stepper(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("fx") / "fx_step")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "fx_host", "fx_step.cpp"),
                           "-o", exe])
    return exe


def run(stepper, f, omega, steps, tmp_path):
    nx, ny = f.shape[:2]
    src, dst = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    np.ascontiguousarray(f, dtype=np.float64).tofile(src)
    out = subprocess.run([stepper, str(nx), str(ny), str(steps), repr(omega), src, dst], capture_output=True,
                         text=True, check=True)
    return np.fromfile(dst).reshape(f.shape), int(out.stdout.strip())


def test_density_wave_tracks_extended_precision(stepper, extended, tmp_path):
    n = 64
    rho, u = O.sinusoidal_density_x((n, n), 1.0, 0.01, check=False)
    f = O.equilibrium(rho, u)
    got, fallback = run(stepper, f, 1.0, 2000, tmp_path)
    assert fallback == 0
    assert np.abs(got.sum(-1)[:, 0] - extended["density_wave_rho_x"]).max() <= 1e-15
    ref = O.run(f, O.density(f), O.velocity(O.density(f), f), 1.0, 2000)[0]
    assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12


def test_random_state_tracks_extended_precision(stepper, extended, tmp_path):
    rng = np.random.default_rng(0)
    rho = rng.uniform(0.95, 1.05, (32, 24))
    u = rng.normal(0, 0.05, (32, 24, 2))
    got, _ = run(stepper, O.equilibrium(rho, u), 1.3, 500, tmp_path)
    assert np.abs(got - extended["random_f"]).max() <= 1e-15


def test_fast_nodes_fall_back_and_stay_accurate(stepper, tmp_path):
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.9, 1.1, (24, 20))
    u = rng.normal(0, 0.02, (24, 20, 2))
    u[3:6, 4:8] = (0.3, 0.25)  # |ux| + |uy| > 0.35: the float64 collision
    f = O.equilibrium(rho, u)
    got, fallback = run(stepper, f, 1.2, 30, tmp_path)
    assert fallback > 0
    ref = O.run(f, O.density(f), O.velocity(O.density(f), f), 1.2, 30)[0]
    assert np.abs(got - ref).max() / np.abs(ref).max() <= 1e-12

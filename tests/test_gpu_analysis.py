"""Exact global moments, device post-processing, checkpoint/resume and frame export."""
import os

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


def test_mass_momentum_exact_and_order_free(pkg):
    an = pkg.analysis
    rng = np.random.default_rng(0)
    f = rng.uniform(0.01, 0.3, (300, 77, 9))
    m, px, py = an.mass_momentum(f)
    F = np.round(np.ldexp(f, 53)).astype(object)
    ref = [sum(F.reshape(-1, 9).sum(axis=0)[i] for i in range(9))]
    exact_m = float(sum(int(v) for v in F.reshape(-1))) / 2.0 ** 53
    assert abs(m - exact_m) <= abs(exact_m) * 2 ** -52
    perm = f.reshape(-1, 9)[rng.permutation(300 * 77)].reshape(300, 77, 9)
    assert an.mass_momentum(perm) == (m, px, py)
    jx = f[..., [1, 5, 8]].sum() - f[..., [3, 6, 7]].sum()
    assert abs(px - jx) < 1e-9 and abs(py - (f[..., [2, 5, 6]].sum() - f[..., [4, 7, 8]].sum())) < 1e-9
    del ref


def test_mass_conservation_of_the_cavity_exact(pkg):
    an, S = pkg.analysis, pkg.scenarios
    f, rho, u, bnd = S.cavity(96)
    m0 = an.mass_momentum(f)[0]
    lat = pkg.Lattice(96, 96, 1.7, bnd).set_state(f, rho, u).step(3000)
    m1 = an.mass_momentum(lat.read()[0])[0]
    assert abs(m1 - m0) / m0 <= 1e-12


def test_strouhal_and_decay_fit(pkg):
    an = pkg.analysis
    t = np.arange(20000)
    trace = 0.1 + 0.02 * np.sin(2 * np.pi * t / 250.0)
    assert abs(an.strouhal(trace, 40, 0.1) - (1 / 250.0) * 40 / 0.1) < 0.01
    k2 = (2 * np.pi / 64) ** 2
    amp = 0.01 * np.exp(-0.1666 * k2 * t[:2000])
    assert abs(an.fit_decay_viscosity(amp, t[:2000], 0.01, 64) - 0.1666) < 1e-9


@pytest.mark.parametrize("storage", ["fx64", "f64", "f16", "bf16", "f16r"])
def test_checkpoint_resume_is_bit_exact(pkg, storage, tmp_path):
    S = pkg.scenarios
    f, rho, u, om, bnd = S.von_karman(120, 50, plate=10, re=80, seed=3)
    kw = {"dev_ref": (0.1, 0.0)} if storage == "f16r" else {}
    a = pkg.Lattice(120, 50, om, bnd, storage=storage, **kw).set_state(f, rho, u).step(300)
    path = os.path.join(tmp_path, "ck.npz")
    a.step(100)
    a.save(path)
    a.step(77)
    b = pkg.Lattice(120, 50, om, bnd, storage=storage, **kw).load(path).step(77)
    assert a.t == b.t == 477
    assert torch.equal(a.read()[0], b.read()[0])
    if storage == "f16r":
        # the stored numbers only mean something with the reference they were written with
        with pytest.raises(AssertionError, match="reference velocity"):
            pkg.Lattice(120, 50, om, bnd, storage=storage, dev_ref=(0.05, 0.0)).load(path)


def test_frame_and_field_export(pkg, tmp_path):
    an = pkg.analysis
    u = torch.zeros((40, 30, 2), dtype=torch.float64, device="cuda")
    u[..., 0] = torch.linspace(0, 0.1, 40, dtype=torch.float64, device="cuda")[:, None]
    p = os.path.join(tmp_path, "f.png")
    an.save_velocity_frame(p, u)
    data = open(p, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n" and len(data) > 60
    q = os.path.join(tmp_path, "rho.npy")
    an.save_field_npy(q, torch.ones((40, 30), dtype=torch.float64, device="cuda"))
    assert np.load(q).shape == (40, 30)

"""The benchmark configurations themselves against the NumPy oracle:

* the von Karman channel of the precision study (420x180, rigid top and
  bottom rows through the reference's rigid_wall, plate 40 moved up one row,
  seeded U(-1e-3, 1e-3) u_y, Re 100): bit-identical in exact float64
  arithmetic and within 1e-12 relative max error in the FMA form and the
  fixed-point (fx64) storage after 1, 10 and 100 steps, and after 2000 steps on
  a reduced channel of the same form; a batched member of the same form
  within 1e-12 (the batch sweep and the serving loop run this composition);
* the sliding-lid cavity at 1024^2 (the smallest size of the bandwidth
  benchmark), 12 steps: bit-identical in exact arithmetic, within 1e-12 in
  fx64 and the FMA form.

Steps are run as one call (the resident lattice), so 1 + 9 + 90 steps hit the
same states as separate runs of 1, 10 and 100 steps."""
import numpy as np
import pytest

from oracle import lbm_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.fixture(scope="module")
def pkg():
    import lattice_boltzmann_parallel_solver_gb300 as P
    P._lib.load()
    return P


def channel(pkg, lx, ly, plate, seed=0):
    """(omega, f0, rho0, u0, oracle boundary, package boundary) of the channel form."""
    f, rho, u, omega, bnd = pkg.scenarios.von_karman(lx, ly, plate=plate, re=100, seed=seed)
    fo, ro, uo = O.von_karman_channel_start(lx, ly, 0.1, 1e-3, seed)
    assert np.array_equal(f, fo) and np.array_equal(u, uo)
    obnd = O.von_karman_boundary(lx, ly, 1.0, 0.1, plate, walls=True, plate_offset=1)
    return omega, f, rho, u, obnd, bnd


@pytest.fixture(scope="module")
def channel_420(pkg):
    omega, f, rho, u, obnd, bnd = channel(pkg, 420, 180, 40)
    refs, state = {}, (f, rho, u)
    done = 0
    for n in (1, 10, 100):
        state = O.run(*state, omega, n - done, obnd)
        done = n
        refs[n] = state
    return omega, f, rho, u, bnd, refs


@pytest.mark.parametrize("storage,exact", [("f64", True), ("f64", False), ("fx64", False)])
def test_channel_420x180_against_oracle(pkg, channel_420, storage, exact):
    omega, f, rho, u, bnd, refs = channel_420
    lat = pkg.Lattice(420, 180, omega, bnd, storage=storage, exact=exact).set_state(f, rho, u)
    done = 0
    for n in (1, 10, 100):
        lat.step(n - done)
        done = n
        got = [t.cpu().numpy() for t in lat.read()]
        ref = refs[n]
        if exact:
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), n
        else:
            assert rel(got[0], ref[0]) <= TOL, (storage, n, rel(got[0], ref[0]))
            assert rel(got[1], ref[1]) <= TOL, (storage, n)
            assert rel(got[2], ref[2]) <= 1e-10, (storage, n, rel(got[2], ref[2]))


@pytest.mark.parametrize("storage,exact", [("f64", True), ("f64", False), ("fx64", False)])
def test_channel_reduced_2000_steps(pkg, storage, exact):
    omega, f, rho, u, obnd, bnd = channel(pkg, 105, 46, 10, seed=4)
    ref = O.run(f, rho, u, omega, 2000, obnd)
    lat = pkg.Lattice(105, 46, omega, bnd, storage=storage, exact=exact).set_state(f, rho, u).step(2000)
    got = [t.cpu().numpy() for t in lat.read()]
    if exact:
        assert np.array_equal(got[0], ref[0])
    else:
        assert rel(got[0], ref[0]) <= TOL, rel(got[0], ref[0])


@pytest.mark.parametrize("storage", ["f64", "fx64"])
def test_channel_batch_member_against_oracle(pkg, channel_420, storage):
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    omega, f, rho, u, bnd, refs = channel_420
    small = channel(pkg, 105, 46, 10, seed=5)
    ms = [Member(420, 180, omega, bnd, steps=100, f0=f, rho0=rho, u0=u),
          Member(105, 46, small[0], small[5], steps=100, f0=small[1], rho0=small[2], u0=small[3])]
    b = Batch(ms, storage=storage).start()
    b.run()
    got = b.read(0)[0].cpu().numpy()
    assert rel(got, refs[100][0]) <= TOL
    ref = O.run(small[1], small[2], small[3], small[0], 100, small[4])
    assert rel(b.read(1)[0].cpu().numpy(), ref[0]) <= TOL


def test_cavity_1024_against_oracle(pkg):
    n, steps = 1024, 12
    rho, u = O.density_1_velocity_0((n, n))
    f = O.equilibrium(rho, u)
    ref = O.run(f, rho, u, 1.7, steps, O.cavity_boundary(n, n, 0.1, 1.0))
    bnd = pkg.boundary_utils.cavity_boundary_conditions(n, n, 0.1, 1.0)
    lat = pkg.Lattice(n, n, 1.7, bnd, storage="f64", exact=True).set_state(f, rho, u).step(steps)
    got = [t.cpu().numpy() for t in lat.read()]
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    for storage in ("fx64", "f64"):
        lat = pkg.Lattice(n, n, 1.7, bnd, storage=storage).set_state(f, rho, u).step(steps)
        got = [t.cpu().numpy() for t in lat.read()]
        assert rel(got[0], ref[0]) <= TOL, storage
        assert rel(got[1], ref[1]) <= TOL, storage


@pytest.mark.parametrize("storage,l2_2k,l2_5k,st_tol", [("f16", 1e-3, 1.5e-3, 2e-3), ("bf16", 8e-3, 2e-2, 1e-2)])
def test_channel_16bit_accuracy(pkg, storage, l2_2k, l2_5k, st_tol):
    """The 16-bit deviation storages on the channel form against fx64 (float64
    accuracy): velocity L2 before the onset of shedding (measured f16 4.8e-4 at
    2000 steps and 8.7e-4 at 5000; bf16 4.1e-3, 1.0e-2) and the Strouhal number
    of u_y at (300, 90) over 100 000 steps by the sub-bin estimate (measured f16
    0.063 %, bf16 0.43 %)."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300 import analysis
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    f, rho, u, omega, bnd = pkg.scenarios.von_karman(420, 180, plate=40, re=100, seed=0)
    res = {}
    for st in ("fx64", storage):
        m = Member(420, 180, omega, bnd, steps=100000, probe=(300, 90), f0=f, rho0=rho, u0=u)
        b = Batch([m], storage=st).start()
        us = {}
        for upto in (2000, 5000):
            b.run_graph(upto - 1 - b.g, chunk=1000)
            us[upto] = b.read(0, want_f=False)[2]
        b.run_graph(chunk=1000)
        uy = b.probe_trace(0)[:, 1]
        res[st] = (us, analysis.spectral_peak(uy, start=uy.numel() // 2)[0])
    (u64, f64_), (u16, f16_) = res["fx64"], res[storage]
    e2 = float(torch.linalg.norm(u16[2000] - u64[2000]) / torch.linalg.norm(u64[2000]))
    e5 = float(torch.linalg.norm(u16[5000] - u64[5000]) / torch.linalg.norm(u64[5000]))
    est = abs(f16_ - f64_) / f64_
    print("%s: L2 %.2e at 2000, %.2e at 5000, St %.3e" % (storage, e2, e5, est))
    assert e2 <= l2_2k and e5 <= l2_5k and est <= st_tol

"""Serving loop: a request gives the same result alone and in a mix where
others arrive before and after it and share its launches; results agree with
a standalone resident lattice; admission keeps to the HBM budget."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    import lattice_boltzmann_parallel_solver_gb300 as P
    P._lib.load()
    return P


def small_mix(pkg, n=7, seed=3):
    from lattice_boltzmann_parallel_solver_gb300.serving import request_mix
    reqs = request_mix(n, rate=1e6, seed=seed, step_range=(40, 400), kinds=("couette", "poiseuille"))
    for r in reqs:  # keep the lattices small for a quick test
        if r.nx * r.ny > 300 * 200:
            r.nx, r.ny = min(r.nx, 300), min(r.ny, 200)
            rebuilt = _rebuild(pkg, r)
            r.boundary, r.f0, r.rho0, r.u0 = rebuilt
    return reqs


def _rebuild(pkg, r):
    S, U = pkg.scenarios, pkg.boundary_utils
    rho, u = np.ones((r.nx, r.ny)), np.zeros((r.nx, r.ny, 2))
    if r.kind == "poiseuille":
        d = r.params["drho"]
        bnd = U.poiseuille_flow_boundary_conditions(r.nx, r.ny, (1 + d / 2) / 3, (1 - d / 2) / 3)
    else:
        m0 = np.zeros((r.nx, r.ny), bool)
        m0[:, 0] = True
        m1 = np.zeros((r.nx, r.ny), bool)
        m1[:, -1] = True
        bnd = U.Boundary([pkg.boundary_conditions.rigid_wall(m0),
                          pkg.boundary_conditions.moving_wall(m1, np.array([r.params["u_w"], 0.0]), 1.0)])
    return bnd, S.equilibrium_np(rho, u), rho, u


def clone(r, rid, arrival):
    from lattice_boltzmann_parallel_solver_gb300.serving import Request
    return Request(rid, r.kind, r.nx, r.ny, r.omega, r.steps, r.boundary, r.f0, r.rho0, r.u0, arrival, dict(r.params),
                   dev_ref=r.dev_ref)


@pytest.mark.parametrize("storage", ["f16", "fx64", "f16r"])
def test_same_result_alone_and_in_mix(pkg, storage):
    """(f16r: the request carries its own reference velocity, the others the default.)"""
    from lattice_boltzmann_parallel_solver_gb300.serving import ServingEngine
    reqs = small_mix(pkg)
    target = reqs[3]
    if storage == "f16r":
        target.dev_ref = (0.03, 0.0)
    alone = ServingEngine(storage=storage, tick_steps=64).serve([clone(target, 100, 0.0)], realtime=False)[0]
    mix = [clone(r, r.rid, 0.0) for r in reqs]
    eng = ServingEngine(storage=storage, tick_steps=37, max_slots=4)
    done = eng.serve(mix, realtime=False)
    assert len(done) == len(mix) and eng.stats["max_live"] > 1
    got = [r for r in done if r.rid == target.rid][0]
    assert torch.equal(got.u, alone.u) and torch.equal(got.rho, alone.rho)


def test_served_results_match_resident_lattice(pkg):
    from lattice_boltzmann_parallel_solver_gb300.serving import ServingEngine
    reqs = small_mix(pkg, n=4, seed=5)
    done = ServingEngine(storage="f32", tick_steps=50).serve([clone(r, r.rid, 0.0) for r in reqs], realtime=False)
    for r in done:
        lat = pkg.Lattice(r.nx, r.ny, r.omega, r.boundary, storage="f32", npt=4)
        rho, u = lat.set_state(r.f0, r.rho0, r.u0).step(r.steps).moments()
        assert float((u - r.u).abs().max()) <= 1e-6
        assert float((rho - r.rho).abs().max()) <= 1e-6


def test_admission_respects_budget(pkg):
    from lattice_boltzmann_parallel_solver_gb300.serving import ServingEngine
    reqs = small_mix(pkg, n=5, seed=9)
    eng = ServingEngine(storage="f16", tick_steps=100)
    eng.hbm_budget = max(eng.state_bytes(r) for r in reqs)
    done = eng.serve([clone(r, r.rid, 0.0) for r in reqs], realtime=False)
    assert len(done) == 5 and eng.stats["max_live"] == 1 and eng.used == 0


def test_realtime_stream_latency_accounting(pkg):
    from lattice_boltzmann_parallel_solver_gb300.serving import ServingEngine, summarize
    reqs = small_mix(pkg, n=6, seed=11)
    for k, r in enumerate(reqs):
        r.arrival = 0.02 * k
    done = ServingEngine(storage="f16", tick_steps=50).serve(reqs, realtime=True)
    s = summarize(done)
    assert s["requests"] == 6 and s["p99_s"] >= s["p50_s"] > 0
    assert all(r.finished >= r.admitted >= r.arrival - 1e-9 for r in done)

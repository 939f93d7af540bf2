"""The fused step without allocation (lbm_step_f64_noalloc), for callers that
cannot allocate device memory, e.g. code running where cudaMalloc is not
allowed or whose host application owns all device memory.  Called through
the C ABI, it must give exactly what the allocating entry point lbm_step_f64
gives (which the other tests pin to the reference), on two calls in a row
that share its static scratch, and must reject lattices too large for that
scratch.  This file sorts last so that a run stopping at the first failure
has run every other test before it."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _cases():
    from lattice_boltzmann_parallel_solver_gb300 import boundary_utils as U
    from lattice_boltzmann_parallel_solver_gb300 import initial_values as I
    from lattice_boltzmann_parallel_solver_gb300 import lattice_boltzmann_method as L
    out = []
    # von Karman channel (inlet, outlet, plate): the outlet column uses the scratch tail
    rho, u = I.density_1_velocity_x_u0_velocity_y_0_initial((84, 36), 0.1)
    out.append((U.von_karman_boundary_conditions(84, 36, 1.0, 0.1, 8), rho, u, 1 / (3 * 0.04 + 0.5)))
    # Poiseuille (pre-streaming pressure rewrite, walls)
    rho, u = I.density_1_velocity_0_initial((40, 20))
    out.append((U.poiseuille_flow_boundary_conditions(40, 20, (1 + 1.5e-3) / 3, (1 - 1.5e-3) / 3), rho, u, 1.5))
    # fully periodic, odd sizes, perturbed state
    rng = np.random.default_rng(7)
    rho = rng.uniform(0.9, 1.1, (33, 17))
    u = rng.normal(0, 0.03, (33, 17, 2))
    out.append((None, rho, u, 1.3))
    return [(b, L.equilibrium_distr_func(r, v), r, v, om) for b, r, v, om in out]


def test_noalloc_step_matches_allocating_step_twice():
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    from lattice_boltzmann_parallel_solver_gb300.geometry import empty_geometry
    lib = _lib.load()
    s = torch.cuda.current_stream().cuda_stream
    for bnd, f0, rho0, u0, omega in _cases():
        nx, ny = f0.shape[:2]
        geo = bnd.geometry(nx, ny) if bnd is not None else empty_geometry(nx, ny)
        for exact in (True, False):
            flags = _lib.FLAG_EXACT if exact else 0
            a = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (f0, rho0, u0)]
            b = [t.clone() for t in a]
            scratch = torch.empty(int(lib.lbm_step_scratch_bytes(nx, ny)), dtype=torch.uint8, device="cuda")
            for _ in range(2):  # two calls in a row share the static scratch
                oa = [torch.empty_like(t) for t in a]
                ob = [torch.empty_like(t) for t in b]
                _lib.check(lib.lbm_step_f64(geo.ref, *[t.data_ptr() for t in a], omega,
                                            *[t.data_ptr() for t in oa], scratch.data_ptr(), flags, s))
                _lib.check(lib.lbm_step_f64_noalloc(geo.ref, *[t.data_ptr() for t in b], omega,
                                                    *[t.data_ptr() for t in ob], flags, s))
                torch.cuda.synchronize()
                for x, y in zip(oa, ob):
                    assert torch.equal(x, y)
                a, b = oa, ob


def _step_both(lib, geo, f0, rho0, u0, omega, flags, device):
    """One call of each entry point on ``device``; the two outputs."""
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    nx, ny = f0.shape[:2]
    with torch.cuda.device(device):
        s = torch.cuda.current_stream().cuda_stream
        a = [torch.from_numpy(np.ascontiguousarray(x)).to(device) for x in (f0, rho0, u0)]
        scratch = torch.empty(int(lib.lbm_step_scratch_bytes(nx, ny)), dtype=torch.uint8, device=device)
        oa = [torch.empty_like(t) for t in a]
        ob = [torch.empty_like(t) for t in a]
        _lib.check(lib.lbm_step_f64(geo.ref, *[t.data_ptr() for t in a], omega, *[t.data_ptr() for t in oa],
                                    scratch.data_ptr(), flags, s))
        _lib.check(lib.lbm_step_f64_noalloc(geo.ref, *[t.data_ptr() for t in a], omega,
                                            *[t.data_ptr() for t in ob], flags, s))
        torch.cuda.synchronize()
    return oa, ob


def test_noalloc_at_the_exact_size_limit():
    """The largest lattice the static scratch holds, with an outlet (its column
    memory takes the scratch tail): pitch 96 (nx 65..96) and ny = 1209 need
    (9 * 96 + 3) * 1209 * 8 = 8 385 624 bytes of the 8 388 608; one row more is
    rejected."""
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    from lattice_boltzmann_parallel_solver_gb300 import boundary_utils as U
    from lattice_boltzmann_parallel_solver_gb300 import initial_values as I
    from lattice_boltzmann_parallel_solver_gb300 import lattice_boltzmann_method as L
    lib = _lib.load()
    assert (9 * 96 + 3) * 1209 * 8 <= 8 << 20 < (9 * 96 + 3) * 1210 * 8
    for nx in (96, 65):
        rho, u = I.density_1_velocity_x_u0_velocity_y_0_initial((nx, 1209), 0.1)
        f0 = L.equilibrium_distr_func(rho, u)
        bnd = U.von_karman_boundary_conditions(nx, 1209, 1.0, 0.1, 40)
        oa, ob = _step_both(lib, bnd.geometry(nx, 1209), f0, rho, u, 1.5, _lib.FLAG_EXACT, 0)
        for x, y in zip(oa, ob):
            assert torch.equal(x, y)
    geo = U.von_karman_boundary_conditions(96, 1210, 1.0, 0.1, 40).geometry(96, 1210)
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.lbm_step_f64_noalloc(geo.ref, t.data_ptr(), t.data_ptr(), t.data_ptr(), 1.0, t.data_ptr(),
                                  t.data_ptr(), t.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.LBM_ERR_ARG and b"static scratch" in lib.lbm_last_error()


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs two GPUs")
def test_noalloc_on_two_devices():
    """Each device has its own copy of the static scratch: calls on device 0, then
    device 1, then device 0 again each match the allocating step there."""
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    from lattice_boltzmann_parallel_solver_gb300.geometry import CompiledGeometry
    lib = _lib.load()
    for bnd, f0, rho0, u0, omega in _cases()[:1]:
        nx, ny = f0.shape[:2]
        for dev in (0, 1, 0):
            geo = CompiledGeometry(nx, ny, bnd.sources(nx, ny), device="cuda:%d" % dev)
            oa, ob = _step_both(lib, geo, f0, rho0, u0, omega, 0, dev)
            for x, y in zip(oa, ob):
                assert torch.equal(x, y)


def test_noalloc_rejects_lattices_beyond_the_static_scratch():
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    from lattice_boltzmann_parallel_solver_gb300.geometry import empty_geometry
    lib = _lib.load()
    nx = ny = 512  # 9 * 512 * 512 * 8 bytes > 8 MiB
    geo = empty_geometry(nx, ny)
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.lbm_step_f64_noalloc(geo.ref, t.data_ptr(), t.data_ptr(), t.data_ptr(), 1.0, t.data_ptr(),
                                  t.data_ptr(), t.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.LBM_ERR_ARG
    assert b"static scratch" in lib.lbm_last_error()

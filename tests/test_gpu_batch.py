"""Batched lattices (one launch per step over many uneven lattices): each
member's result equals the same lattice run alone, float64 members match the
oracle, per-lattice step budgets stop on time, graph replay equals plain
launches, probes record the per-step velocity, and the autotuner returns a
working configuration."""
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


def members(pkg, steps=(30, 30, 30, 30, 30)):
    S, U = pkg.scenarios, pkg.boundary_utils
    from lattice_boltzmann_parallel_solver_gb300.batch import Member
    out = []
    f, rho, u, om, bnd = S.von_karman(203, 62, plate=12, re=120, seed=1)
    out.append(Member(203, 62, om, bnd, steps=steps[0], f0=f, rho0=rho, u0=u, probe=(150, 31)))
    f, rho, u, om, bnd = S.von_karman(96, 40, plate=8, re=60, seed=2, plate_offset=0, walls=False)
    out.append(Member(96, 40, om, bnd, steps=steps[1], f0=f, rho0=rho, u0=u))
    f, rho, u, bnd = S.cavity(37)
    out.append(Member(37, 37, 1.7, bnd, steps=steps[2], f0=f, rho0=rho, u0=u))
    rho, u = np.ones((50, 18)), np.zeros((50, 18, 2))
    out.append(Member(50, 18, 1.5, U.poiseuille_flow_boundary_conditions(50, 18, (1 + 3e-3) / 3, (1 - 3e-3) / 3),
                      steps=steps[3], f0=S.equilibrium_np(rho, u), rho0=rho, u0=u))
    f, rho, u = S.shear_wave(64)
    out.append(Member(64, 64, 1.0, None, steps=steps[4], f0=f, rho0=rho, u0=u))
    return out


def alone(pkg, m, storage, npt):
    lat = pkg.Lattice(m.nx, m.ny, m.omega, m.boundary, storage=storage, npt=npt)
    return lat.set_state(m.f0, m.rho0, m.u0).step(m.steps)


@pytest.mark.parametrize("storage,npt,threads,rows", [("fx64", 1, 128, 1), ("fx64", 2, 64, 3), ("f64", 2, 128, 1),
                                                      ("f32", 4, 64, 2), ("f16", 4, 128, 1), ("f16", 8, 256, 4),
                                                      ("bf16", 2, 128, 5)])
def test_batch_members_equal_lone_runs(pkg, storage, npt, threads, rows):
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch
    ms = members(pkg, steps=(30, 17, 25, 30, 4))
    b = Batch(ms, storage=storage, npt=npt, threads=threads, rows=rows).start()
    b.run()
    for j, m in enumerate(ms):
        got = b.read(j)[0]
        ref = alone(pkg, m, storage, npt).read()[0]
        err = float((got - ref).abs().max() / ref.abs().max())
        assert err <= (1e-13 if storage in ("f64", "fx64") else 1e-6), (j, err)


@pytest.mark.parametrize("storage", ["fx64", "f64"])
def test_batch_f64_against_oracle(pkg, storage):
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch
    ms = members(pkg)
    b = Batch(ms, storage=storage).start()
    b.run()
    cav = ms[2]
    ref = O.run(cav.f0, cav.rho0, cav.u0, 1.7, cav.steps, O.cavity_boundary(37, 37, 0.1, 1.0))
    got = b.read(2)[0].cpu().numpy()
    assert np.abs(got - ref[0]).max() / np.abs(ref[0]).max() <= 1e-12
    she = ms[4]
    ref = O.run(she.f0, she.rho0, she.u0, 1.0, she.steps)
    got = b.read(4)[0].cpu().numpy()
    assert np.abs(got - ref[0]).max() / np.abs(ref[0]).max() <= 1e-12


def test_graph_replay_and_probe(pkg):
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch
    ms = members(pkg, steps=(241, 241, 241, 241, 241))
    a = Batch(ms, storage="f32").start()
    a.run()
    ms2 = members(pkg, steps=(241, 241, 241, 241, 241))
    b = Batch(ms2, storage="f32").start()
    b.run_graph(chunk=40)
    for j in range(len(ms)):
        assert torch.equal(a.read(j)[0], b.read(j)[0])
    tr = b.probe_trace(0)
    assert tr.shape == (240, 2)
    # the last recorded probe is the velocity of the last step's pre-collision state,
    # i.e. of the state one step before the final one
    m = ms2[0]
    lat = pkg.Lattice(m.nx, m.ny, m.omega, m.boundary, storage="f32").set_state(m.f0, m.rho0, m.u0).step(240)
    u = lat.moments()[1][150, 31]
    assert torch.allclose(tr[-1], u.to(tr.dtype), rtol=0, atol=1e-6)


def test_autotune_picks_a_working_config(pkg):
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, autotune
    ms = members(pkg, steps=(20, 20, 20, 20, 20))
    b = Batch(ms, storage="f16")
    res = autotune(b, steps=3, warmup=1)
    assert res and all(r["ms_per_step"] > 0 for r in res)
    b.start().run()
    for j, m in enumerate(ms):
        ref = alone(pkg, m, "f16", b.npt).read()[0]
        assert float((b.read(j)[0] - ref).abs().max()) <= 1e-6


@pytest.mark.parametrize("storage", ["fx64", "f64", "f32", "f16", "bf16", "f16r"])
def test_boundary_node_pass_equals_inline_sources(pkg, storage):
    """The default batched step (a boundary-free launch, then the pass over the
    listed boundary nodes) gives bit-identical states and probe traces to the
    step with the boundary sources inside it, for walls, the moving lid, the
    pressure rewrite, inlet/outlet and the plate; the probes sit on a lid node,
    an inlet node and a pressure-column node, which the pass records."""
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch
    npt = {"fx64": 1, "f64": 2, "f32": 2}.get(storage, 4)
    threads = 128 if storage == "f16r" else 64  # the reference-shifted storages run at 128 threads
    runs = []
    for inline in (True, False):
        ms = members(pkg, steps=(40, 33, 40, 40, 40))
        ms[1].probe = (0, 20)
        ms[2].probe = (18, 36)
        ms[3].probe = (48, 9)
        if storage == "f16r":
            ms[0].dev_ref = (0.1, 0.0)
        b = Batch(ms, storage=storage, npt=npt, threads=threads, rows=2, inline_bc=inline).start()
        assert (b.bc_chunks == -1) == inline and (inline or b.bc_chunks > 0)
        b.run()
        runs.append((b, ms))
    (a, _), (b, ms) = runs
    for j, m in enumerate(ms):
        fa, ra, ua = a.read(j)
        fb, rb, ub = b.read(j)
        assert torch.equal(fa, fb) and torch.equal(ua, ub), (storage, j)
        if m.probe is not None:
            ta, tb = a.probe_trace(j), b.probe_trace(j)
            assert ta.shape[0] == m.steps - 1 and torch.equal(ta, tb), (storage, j)


@pytest.mark.parametrize("storage", ["fx64", "f16", "f32"])
@pytest.mark.parametrize("probe", [(202, 30), (0, 0), (202, 61), (0, 17), (1, 17), (201, 30)])
def test_plain_edge_columns_equal_inline_sources(pkg, storage, probe):
    """The batched boundary-free step applies the plain inlet and outlet columns
    itself and the pass skips them: bit-identical to the sources inside the
    step, with the probe on a plain outlet node, on the corners where the walls
    override the inlet / outlet (nodes the pass recomputes), on a plain inlet
    node and next to both columns."""
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch
    npt = {"fx64": 1, "f32": 2}.get(storage, 4)
    runs = []
    for inline in (True, False):
        ms = members(pkg, steps=(60, 3, 3, 3, 3))[:1]
        ms[0].probe = probe
        b = Batch(ms, storage=storage, npt=npt, threads=64, rows=2, inline_bc=inline).start()
        if not inline:
            g = ms[0].geo.struct
            assert g.n_bcnodes_edge == 2 * (62 - 2) and g.edge_inlet_desc and g.edge_outlet_desc
        b.run()
        runs.append(b)
    a, b = runs
    assert torch.equal(a.read(0)[0], b.read(0)[0])
    ta, tb = a.probe_trace(0), b.probe_trace(0)
    assert ta.shape[0] == 59 and torch.equal(ta, tb)


@pytest.mark.parametrize("storage,inline", [("f16", False), ("fx64", False), ("f16", True)])
def test_persistent_spans_equal_plain_grid(pkg, storage, inline):
    """The persistent form (blocks walking contiguous spans of tiles, spans that
    cross lattices) gives the same bits as the plain grid of one tile per block."""
    from lattice_boltzmann_parallel_solver_gb300.batch import ONE_TILE_PER_BLOCK, Batch
    npt = 1 if storage == "fx64" else 4
    runs = []
    for blocks in (ONE_TILE_PER_BLOCK, 0, 7):
        ms = members(pkg, steps=(30, 17, 25, 30, 9))
        b = Batch(ms, storage=storage, npt=npt, threads=64, rows=2, blocks=blocks, inline_bc=inline).start()
        b.run()
        runs.append([b.read(j)[0] for j in range(len(ms))])
    for other in runs[1:]:
        for x, y in zip(runs[0], other):
            assert torch.equal(x, y)


def test_batch_plan_follows_the_size(pkg):
    """Below 2^20 nodes in total a batch keeps the boundary sources inside one
    launch per step; from 2^20 it runs the boundary-free step and the pass."""
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    S = pkg.scenarios
    f, rho, u, bnd = S.cavity(64)
    small = Batch([Member(64, 64, 1.7, bnd, steps=3, f0=f, rho0=rho, u0=u)], storage="f16").start()
    assert small.bc_chunks == -1
    big_nodes = 1056 * 1000
    rho, u = np.ones((1056, 1000)), np.zeros((1056, 1000, 2))
    bnd = pkg.boundary_utils.cavity_boundary_conditions(1056, 1000, 0.1, 1.0)
    big = Batch([Member(1056, 1000, 1.7, bnd, steps=3, f0=S.equilibrium_np(rho, u), rho0=rho, u0=u)],
                storage="fx64").start()
    assert big.nodes == big_nodes >= 1 << 20 and big.bc_chunks > 0
    big.run()
    ref = alone(pkg, big.members[0], "fx64", big.npt).read()[0]
    assert float((big.read(0)[0] - ref).abs().max() / ref.abs().max()) <= 1e-13


@pytest.mark.parametrize("nx", [4, 5])
def test_pass_pressure_columns_on_narrow_lattices(pkg, nx):
    """Under the pressure rewrite the pass recomputes columns 1 and nx-2; on
    4- and 5-column lattices (adjacent columns, one between) the split step
    still equals the step with the sources inside it."""
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    U, S = pkg.boundary_utils, pkg.scenarios
    runs = []
    for inline in (True, False):
        rho, u = np.ones((nx, 12)), np.zeros((nx, 12, 2))
        bnd = U.poiseuille_flow_boundary_conditions(nx, 12, (1 + 3e-3) / 3, (1 - 3e-3) / 3)
        m = Member(nx, 12, 1.3, bnd, steps=25, f0=S.equilibrium_np(rho, u), rho0=rho, u0=u, probe=(1, 5))
        b = Batch([m], storage="fx64", npt=1, threads=64, inline_bc=inline).start()
        b.run()
        runs.append(b)
    a, b = runs
    assert torch.equal(a.read(0)[0], b.read(0)[0])
    assert torch.equal(a.probe_trace(0), b.probe_trace(0)) and a.probe_trace(0).shape[0] == 24


def test_three_column_pressure_lattice(pkg):
    """On a 3-column lattice under the pressure rewrite column 1 feeds both
    column 0 (inlet side) and column 2 (outlet side), as in the reference: a
    resident lattice takes the one-node-per-thread kernel and matches the
    oracle, and a batch, whose vectorised bodies give a node one rewrite,
    refuses the lattice."""
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    U, S = pkg.boundary_utils, pkg.scenarios
    p_in, p_out = (1 + 3e-3) / 3, (1 - 3e-3) / 3
    rho, u = np.ones((3, 12)), np.zeros((3, 12, 2))
    f0 = S.equilibrium_np(rho, u)
    ref = O.run(f0, rho, u, 1.3, 25, O.poiseuille_boundary(3, 12, p_in, p_out))
    bnd = U.poiseuille_flow_boundary_conditions(3, 12, p_in, p_out)
    for storage in ("fx64", "f64"):
        got = pkg.Lattice(3, 12, 1.3, bnd, storage=storage).set_state(f0, rho, u).step(25).read()[0].cpu().numpy()
        assert np.abs(got - ref[0]).max() / np.abs(ref[0]).max() <= 1e-12, storage
    with pytest.raises(NotImplementedError):
        Batch([Member(3, 12, 1.3, bnd, steps=5, f0=f0, rho0=rho, u0=u)], storage="fx64", npt=1).start()

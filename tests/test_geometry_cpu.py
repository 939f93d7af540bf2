"""Host logic of the boundary compiler (no GPU): the compiled per-node
descriptor, applied by a NumPy emulation of the kernels' source semantics,
must reproduce the oracle's boundary closures on random arrays for every
composition, including precedence where closures overlap."""
import numpy as np
import pytest

from lattice_boltzmann_parallel_solver_gb300 import boundary_conditions as BC
from lattice_boltzmann_parallel_solver_gb300 import boundary_utils as BU
from lattice_boltzmann_parallel_solver_gb300.geometry import BOUNCE, CONST, OUTLET, CompiledGeometry
from oracle import lbm_oracle as O


def apply_descriptor(g: CompiledGeometry, f_pre, f_post, f_prev):
    """What apply_boundary_kernel does, in NumPy."""
    out = f_post.copy()
    if g.desc is None:
        return out
    nx, ny = g.nx, g.ny
    desc = g.desc.cpu().numpy().T
    mask = g.bcmask.cpu().numpy()
    bits = ((mask[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(ny, -1)[:, :nx].T.astype(bool)
    k = np.array(g.struct.kconst)
    c = np.array(g.struct.cconst)
    for x, y in zip(*np.nonzero(bits)):
        d = int(desc[x, y])
        ks, cs = (d >> 18) & 15, (d >> 22) & 15
        for i in range(9):
            s = (d >> (2 * i)) & 3
            if s == BOUNCE:
                out[x, y, i] = f_pre[x, y, O.OPP[i]] - k[ks, i]
            elif s == CONST:
                out[x, y, i] = c[cs, i]
            elif s == OUTLET:
                out[x, y, i] = f_prev[x - 1, y, i]
    return out


def rand3(shape, seed):
    rng = np.random.default_rng(seed)
    return [rng.uniform(0.01, 0.3, shape + (9,)) for _ in range(3)]


def compiled(boundary, nx, ny):
    return CompiledGeometry(nx, ny, boundary.sources(nx, ny), device="cpu")


def test_wall_indices_match_reference_quirk():
    for edge, dirs in (((0, None), [1, 5, 8]), ((-1, None), [3, 6, 7]), ((None, 0), [4, 7, 8]),
                       ((None, -1), [2, 5, 6])):
        m = np.zeros((6, 5), dtype=bool)
        if edge[0] is not None:
            m[edge[0], :] = True
        else:
            m[:, edge[1]] = True
        assert list(BC.get_wall_indices(m)) == dirs == O.wall_directions(m)


def test_moving_wall_terms_bit_exact():
    m = np.zeros((10, 10), dtype=bool)
    m[:, -1] = True
    for u_w, rho in ((np.array([2, 0]), 1), (np.array([0.07, -0.03]), 1.1), (np.array([0.1, 0.0]), 1.0)):
        assert BC.moving_wall_terms(m, u_w, rho) == O.moving_wall_constants(m, u_w, rho)


@pytest.mark.parametrize("edge", ["x0", "x1", "y0", "y1"])
def test_single_walls(edge):
    nx, ny = 9, 6
    m = np.zeros((nx, ny), dtype=bool)
    {"x0": lambda: m.__setitem__((0, slice(None)), True), "x1": lambda: m.__setitem__((-1, slice(None)), True),
     "y0": lambda: m.__setitem__((slice(None), 0), True), "y1": lambda: m.__setitem__((slice(None), -1), True)}[edge]()
    pre, post, prev = rand3((nx, ny), 1)
    g = CompiledGeometry(nx, ny, BC.rigid_wall(m).sources(nx, ny), device="cpu")
    assert np.array_equal(apply_descriptor(g, pre, post, prev), O.rigid_wall(m)(pre, post.copy()))
    uw = np.array([0.07, -0.03])
    g = CompiledGeometry(nx, ny, BC.moving_wall(m, uw, 1.1).sources(nx, ny), device="cpu")
    assert np.array_equal(apply_descriptor(g, pre, post, prev), O.moving_wall(m, uw, 1.1)(pre, post.copy()))


def test_rigid_object_and_outlet():
    nx, ny = 9, 6
    plate = np.zeros((nx, ny), dtype=bool)
    plate[3, 1:5] = True
    pre, post, prev = rand3((nx, ny), 2)
    g = CompiledGeometry(nx, ny, BC.rigid_object(plate.copy()).sources(nx, ny), device="cpu")
    assert np.array_equal(apply_descriptor(g, pre, post, prev), O.rigid_object(plate.copy())(pre, post.copy()))
    g = CompiledGeometry(nx, ny, BC.outlet().sources(nx, ny), device="cpu")
    assert np.array_equal(apply_descriptor(g, pre, post, prev), O.outlet()(prev, post.copy()))


def test_couette_and_poiseuille_walls():
    lx, ly = 10, 7
    pre, post, prev = rand3((lx, ly), 3)
    b = BU.couette_flow_boundary_conditions(lx, ly, 0.05, 1.0)
    got = apply_descriptor(compiled(b, lx, ly), pre, post, prev)
    assert np.array_equal(got, O.couette_boundary(lx, ly, 0.05, 1.0)(pre, post.copy()))
    # Poiseuille: after its pressure rewrite and re-stream, the two rigid walls
    b = BU.poiseuille_flow_boundary_conditions(lx, ly, 0.34, 0.33)
    want = O.rigid_wall(np.pad(np.ones((lx, 1), bool), ((0, 0), (0, ly - 1))))(pre, post.copy())
    want = O.rigid_wall(np.pad(np.ones((lx, 1), bool), ((0, 0), (ly - 1, 0))))(pre, want)
    assert np.array_equal(apply_descriptor(compiled(b, lx, ly), pre, post, prev), want)
    assert b.pressure.dirs_in == [1, 5, 8] and b.pressure.dirs_out == [3, 6, 7]


def test_cavity_precedence():
    n = 8
    pre, post, prev = rand3((n, n), 4)
    b = BU.cavity_boundary_conditions(n, n, 0.1, 1.0)
    got = apply_descriptor(compiled(b, n, n), pre, post, prev)
    assert np.array_equal(got, O.cavity_boundary(n, n, 0.1, 1.0)(pre, post.copy()))


def test_von_karman_unpadded_and_padded():
    lx, ly, d = 84, 36, 8
    feq_in = O.inlet_populations((1, 1), 1.0, 0.1)[0, 0]
    pre, post, prev = rand3((lx, ly), 5)
    b = BU.Boundary(BU._vk_closures(lx, ly, 1.0, 0.1, d, feq_in=feq_in))
    got = apply_descriptor(compiled(b, lx, ly), pre, post, prev)
    assert np.array_equal(got, O.von_karman_boundary(lx, ly, 1.0, 0.1, d)(pre, post.copy(), None, None, prev))
    pre, post, prev = rand3((lx + 2, ly + 2), 6)
    b = BU.Boundary(BU._vk_closures(lx, ly, 1.0, 0.1, d, off=1, feq_in=feq_in), padded=True)
    g = compiled(b, lx + 2, ly + 2)
    assert not g.fusable
    got = apply_descriptor(g, pre, post, prev)
    want = O.von_karman_boundary_padded(lx, ly, 1.0, 0.1, d)(pre, post.copy(), None, None, prev)
    assert np.array_equal(got, want)


def test_outlet_fusable_only_on_last_column():
    lx, ly = 6, 4
    g = CompiledGeometry(lx, ly, BC.outlet().sources(lx, ly), device="cpu")
    assert g.outlet and g.fusable
    m = np.zeros((lx, ly), dtype=bool)
    m[2, :] = True
    assert not CompiledGeometry(lx, ly, [(m, 3, OUTLET, 0.0)], device="cpu").fusable


def test_too_many_constant_sets():
    lx, ly = 40, 4
    src = []
    for x in range(20):
        m = np.zeros((lx, ly), dtype=bool)
        m[x, :] = True
        src.append((m, 2, CONST, 0.01 * x))
    with pytest.raises(NotImplementedError):
        CompiledGeometry(lx, ly, src, device="cpu")


@pytest.mark.parametrize("name", ["couette", "poiseuille", "cavity", "vk", "channel"])
def test_boundary_node_list_matches_the_mask(name):
    """The boundary-node pass recomputes exactly the listed nodes: the list
    holds the linear indices y*nx + x of the mask's set bits, the plain inlet
    and outlet nodes (n_bcnodes_edge of them) last, each part ascending, and
    covers at most an eighth of these lattices."""
    lx, ly = 70, 33
    feq_in = O.inlet_populations((1, 1), 1.0, 0.1)[0, 0]
    if name == "couette":
        b = BU.couette_flow_boundary_conditions(lx, ly, 0.05, 1.0)
    elif name == "poiseuille":
        b = BU.poiseuille_flow_boundary_conditions(lx, ly, 0.34, 0.33)
    elif name == "cavity":
        b = BU.cavity_boundary_conditions(lx, ly, 0.1, 1.0)
    elif name == "vk":
        b = BU.Boundary(BU._vk_closures(lx, ly, 1.0, 0.1, 8, feq_in=feq_in))
    else:
        b = BU.Boundary(BU._vk_closures(lx, ly, 1.0, 0.1, 8, feq_in=feq_in, walls=True, plate_offset=1))
    g = compiled(b, lx, ly)
    mask = g.bcmask.cpu().numpy()
    bits = ((mask[:, :, None] >> np.arange(32, dtype=np.uint32)) & 1).reshape(ly, -1)[:, :lx].astype(bool)
    want = np.flatnonzero(bits.reshape(-1))
    got = g.bcnodes.cpu().numpy()
    n_edge = g.struct.n_bcnodes_edge
    core, tail = got[:got.size - n_edge], got[got.size - n_edge:]
    assert got.dtype == np.int32 and np.array_equal(np.sort(got), want)
    assert np.all(np.diff(core) > 0) and np.all(np.diff(tail) > 0)
    assert g.struct.n_bcnodes == want.size and 0 < want.size * 8 <= lx * ly
    desc = g.desc.cpu().numpy().reshape(-1)
    if name in ("vk", "channel"):
        # every inlet / outlet node without other sources is a plain edge node
        edge_rows = ly if name == "vk" else ly - 2
        assert n_edge == 2 * edge_rows
        x = tail % lx
        assert set(x.tolist()) == {0, lx - 1}
        assert np.all(desc[tail[x == 0]] == g.struct.edge_inlet_desc)
        assert np.all(desc[tail[x == lx - 1]] == g.struct.edge_outlet_desc)
        assert g.struct.edge_inlet_desc & 0x3FFFF == 0x2AAAA and g.struct.edge_outlet_desc & 0x3FFFF == 0xF0C0
        # the corners (walls over inlet / outlet) stay in the pass
        assert not np.isin(tail, core).any()
    else:
        assert n_edge == 0 and g.struct.edge_inlet_desc == 0 and g.struct.edge_outlet_desc == 0


def test_edge_columns_need_a_descriptor_on_every_node():
    """An inlet on part of column 0 is no plain edge column: the kernel would
    apply it to the nodes without one."""
    lx, ly = 20, 10
    m = np.zeros((lx, ly), dtype=bool)
    m[0, 2:8] = True
    src = [(m, i, CONST, 0.1 + 0.01 * i) for i in range(9)]
    g = CompiledGeometry(lx, ly, src, device="cpu")
    assert g.struct.edge_inlet_desc == 0 and g.struct.n_bcnodes_edge == 0
    m[0, :] = True
    src = [(m, i, CONST, 0.1 + 0.01 * i) for i in range(9)]
    g = CompiledGeometry(lx, ly, src, device="cpu")
    assert g.struct.edge_inlet_desc != 0 and g.struct.n_bcnodes_edge == ly


@pytest.mark.parametrize("offset", [0, 1])
def test_von_karman_channel_form(offset):
    """The channel form (rigid bottom/top rows after the plate, plate moved by
    ``offset`` rows) compiles to the oracle's composition of the reference's
    closures, corners included."""
    lx, ly, d = 84, 36, 8
    feq_in = O.inlet_populations((1, 1), 1.0, 0.1)[0, 0]
    pre, post, prev = rand3((lx, ly), 7 + offset)
    b = BU.Boundary(BU._vk_closures(lx, ly, 1.0, 0.1, d, feq_in=feq_in, walls=True, plate_offset=offset))
    got = apply_descriptor(compiled(b, lx, ly), pre, post, prev)
    want = O.von_karman_boundary(lx, ly, 1.0, 0.1, d, walls=True, plate_offset=offset)(pre, post.copy(), None,
                                                                                         None, prev)
    assert np.array_equal(got, want)


def test_reference_velocity_copy_shares_the_descriptor():
    from lattice_boltzmann_parallel_solver_gb300.lattice import with_dev_ref
    geo = compiled(BU.couette_flow_boundary_conditions(60, 30, 0.05, 1.0), 60, 30)
    r = with_dev_ref(geo, "f16r", (0.1, -0.02))
    assert (r.struct.dev_ref_ux, r.struct.dev_ref_uy) == (0.1, -0.02)
    assert (geo.struct.dev_ref_ux, geo.struct.dev_ref_uy) == (0.0, 0.0)
    assert r.desc is geo.desc and r.struct.desc == geo.struct.desc and r.struct.n_bcnodes == geo.struct.n_bcnodes
    z = with_dev_ref(geo, "bf16r", None)
    assert (z.struct.dev_ref_ux, z.struct.dev_ref_uy) == (0.0, 0.0)
    assert with_dev_ref(geo, "f16", None) is geo
    with pytest.raises(ValueError):
        with_dev_ref(geo, "f16", (0.1, 0.0))
    with pytest.raises(AssertionError):
        with_dev_ref(geo, "f16r", (0.6, 0.0))

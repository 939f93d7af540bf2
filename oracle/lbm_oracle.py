"""CPU oracle for the D2Q9 BGK hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain NumPy/float64, the algorithm of the reference
solver's hot path so that the CUDA implementation can be checked against it.
It is imported only by ``tests/``, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``; the product package never imports it.

Parity pin: the functions below are checked bit-for-bit against fixtures that
``tests/golden/make_golden.py`` generated by running the reference itself
(``src/lattice_boltzmann_method.py``, ``src/boundary_conditions.py`` and
``src/boundary_utils.py`` with a single-rank MPI stand-in), and against the
known answers in the reference's unit tests (``tests/test_boundary_conditions.py``,
``tests/test_initial_values.py``, ``tests/test_mass_preservation.py``).

Layout everywhere is the reference's: ``f[nx, ny, 9]`` (x is axis 0, the
direction index fastest), ``rho[nx, ny]``, ``u[nx, ny, 2]``.
"""
from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------
# D2Q9 constants  (src/lattice_boltzmann_method.py:5-52)
# ---------------------------------------------------------------------------
C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1],
              [1, 1], [-1, 1], [-1, -1], [1, -1]])            # :14-26
OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])                    # :37-39
W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9,
              1 / 36, 1 / 36, 1 / 36, 1 / 36])                  # :50-52
CS = 1 / np.sqrt(3)                                            # boundary_conditions.py:186,304


def velocity_set():
    return C.copy()


def opposite():
    return OPP.copy()


def weights():
    return W.copy()


def reynolds_number(L, u, v):                                   # :55-71
    return np.divide(L * u, v)


def strouhal_number(f, L, u):                                   # :74-90
    return np.divide(f * L, u)


# ---------------------------------------------------------------------------
# Moments, equilibrium, streaming, step  (src/lattice_boltzmann_method.py)
# ---------------------------------------------------------------------------
def density(f):
    """rho = sum_i f_i over the last axis (:93-105)."""
    assert f.shape[-1] == 9
    return np.sum(f, axis=-1)


def velocity(rho, f):
    """u = (sum f c)/rho, 0 where rho == 0 (:108-137)."""
    assert f.shape[-1] == 9
    jx = np.sum(f[..., [1, 5, 8]], axis=-1) - np.sum(f[..., [3, 6, 7]], axis=-1)
    jy = np.sum(f[..., [2, 5, 6]], axis=-1) - np.sum(f[..., [4, 7, 8]], axis=-1)
    ux = np.divide(jx, rho, out=np.zeros_like(rho), where=rho != 0)
    uy = np.divide(jy, rho, out=np.zeros_like(rho), where=rho != 0)
    return np.stack((ux, uy), axis=-1)


def streaming(f):
    """Periodic shift of every population plane by its velocity (:140-159)."""
    assert f.shape[-1] == 9
    out = np.zeros_like(f)
    for i in range(9):
        out[..., i] = np.roll(f[..., i], C[i], axis=(0, 1))
    return out


def equilibrium(rho, u):
    """f_eq = w rho (1 + 3 c.u + 9/2 (c.u)^2 - 3/2 |u|^2) (:162-188).

    |u|^2 is formed as norm(u)**2 (square root, then square) exactly as the
    reference does, and c.u through a matmul with the integer velocity set.
    """
    assert rho.shape == u.shape[:-1]
    cu = u @ C.T
    usq = np.power(np.linalg.norm(u, axis=-1), 2)
    # the weights carry two leading axes, so a 1-D (n,) input yields (1, n, 9)
    return W[np.newaxis, np.newaxis, :] * np.expand_dims(rho, -1) * (
        1 + 3 * cu + (9 / 2) * np.power(cu, 2) - (3 / 2) * np.expand_dims(usq, -1))


def collide(f, rho, u, omega):
    """Post-collision populations f + (f_eq - f) omega (:213-215)."""
    feq = equilibrium(rho, u)
    return f + (feq - f) * omega


def step(f, rho, u, omega, boundary=None, communicate=None):
    """One BGK step: collide with the passed-in rho,u, optional halo hook,
    stream, boundary hook, moments (:191-228)."""
    assert f.shape[0:2] == rho.shape
    assert f.shape[0:2] == u.shape[0:2]
    assert 0 < omega < 2
    f_pre = collide(f, rho, u, omega)
    if communicate is not None:
        f_pre = communicate(f_pre)
    f_post = streaming(f_pre)
    if boundary is not None:
        f_post = boundary(f_pre, f_post, rho, u, f)
    rho_new = density(f_post)
    return f_post, rho_new, velocity(rho_new, f_post)


# ---------------------------------------------------------------------------
# Boundary-condition closures  (src/boundary_conditions.py)
# ---------------------------------------------------------------------------
def wall_directions(mask):
    """Outgoing directions bounced at a wall; one wall per mask, first match
    wins, x-walls mapped exactly as the reference maps them (:8-28)."""
    if np.all(mask[0, :]):
        return [1, 5, 8]
    if np.all(mask[-1, :]):
        return [3, 6, 7]
    if np.all(mask[:, 0]):
        return [4, 7, 8]
    if np.all(mask[:, -1]):
        return [2, 5, 6]
    return []


def rigid_wall(mask):
    """Half-way bounce-back on mask nodes: f_post[b, opp(i)] = f_pre[b, i] (:78-113)."""
    assert mask.dtype == bool
    dirs = wall_directions(mask)

    def bc(f_pre, f_post):
        assert mask.shape == f_pre.shape[0:2] == f_post.shape[0:2]
        for i in dirs:
            f_post[mask, OPP[i]] = f_pre[mask, i]
        return f_post
    return bc


def moving_wall_constants(mask, u_w, avg_density):
    """Per bounced direction i: 2 w_i rho_avg (c_i.u_w)/c_s^2 (:186-210)."""
    out = {}
    for i in wall_directions(mask):
        out[i] = 2 * W[i] * avg_density * np.divide(C[i] @ np.asarray(u_w), CS ** 2)
    return out


def moving_wall(mask, u_w, avg_density):
    """f_post[b, opp(i)] = f_pre[b, i] - 2 w_i rho_avg c_i.u_w / c_s^2 (:170-214)."""
    assert mask.dtype == bool
    k = moving_wall_constants(mask, u_w, avg_density)

    def bc(f_pre, f_post):
        assert mask.shape == f_pre.shape[0:2] == f_post.shape[0:2]
        for i, ki in k.items():
            f_post[mask, OPP[i]] = f_pre[mask, i] - ki
        return f_post
    return bc


def object_corners(mask):
    """Corner nodes of a one-column object and the two directions each bounces (:31-56)."""
    idx = np.argwhere(mask)
    x0, x1 = idx[:, 0].min(), idx[:, 0].max() + 1
    y0, y1 = idx[:, 1].min(), idx[:, 1].max()
    return [((x0, y1), (1, 8)), ((x0, y0), (1, 5)), ((x1, y1), (3, 7)), ((x1, y0), (3, 6))]


def rigid_object(mask):
    """Thin-plate bounce-back: left column bounces 1,5,8, the column to its right
    bounces 3,6,7, corners bounce two links each (:116-167).  Like the
    reference, the corner nodes are removed from ``mask`` in place."""
    assert mask.dtype == bool
    corners = object_corners(mask)
    for (cx, cy), _ in corners:
        mask[cx, cy] = False
    left = mask
    right = np.roll(mask, 1, axis=0)

    def bc(f_pre, f_post):
        for m, dirs in ((left, (1, 5, 8)), (right, (3, 6, 7))):
            for i in dirs:
                f_post[m, OPP[i]] = f_pre[m, i]
        for (cx, cy), dirs in corners:
            for i in dirs:
                f_post[cx, cy, OPP[i]] = f_pre[cx, cy, i]
        return f_post
    return bc


def inlet_populations(shape, density_in, velocity_in):
    """Equilibrium at (density_in, (velocity_in, 0)) on the whole grid (:231-237)."""
    u = np.zeros(tuple(shape) + (2,))
    u[..., 0] = velocity_in
    return equilibrium(np.ones(tuple(shape)) * density_in, u)


def inlet(shape, density_in, velocity_in):
    """All 9 populations of column x=0 set to the inlet equilibrium (:217-254)."""
    feq = inlet_populations(shape, density_in, velocity_in)

    def bc(f_post):
        for i in range(f_post.shape[-1]):
            f_post[0, ..., i] = feq[0, ..., i]
        return f_post
    return bc


def outlet():
    """Column x=-1 takes directions 3,6,7 from column x=-2 of the step's input (:257-283)."""
    def bc(f_prev, f_post):
        for i in (3, 6, 7):
            f_post[-1, :, i] = f_prev[-2, :, i]
        return f_post
    return bc


def pressure_setup(mask, p_in, p_out):
    """Orientation test, inlet/outlet densities and direction sets (:300-318)."""
    assert mask.dtype == bool
    assert np.all(mask[0, :] == mask[-1, :]) or np.all(mask[:, 0] == mask[:, -1])
    rho_in = np.divide(p_in, CS ** 2)
    rho_out = np.divide(p_out, CS ** 2)
    if np.all(mask[0, :] == mask[-1, :]):
        n = mask.shape[1]
        return np.ones(n) * rho_in, np.ones(n) * rho_out, [1, 5, 8], [3, 6, 7]
    n = mask.shape[0]
    return np.ones(n) * rho_in, np.ones(n) * rho_out, [2, 5, 6], [4, 7, 8]


def periodic_with_pressure_variations(mask, p_in, p_out):
    """Pre-stream rewrite of columns 0 and -1 from columns -2 and 1 with the
    inlet/outlet densities and the step's input rho,u (:286-348)."""
    rho_in, rho_out, d1, d2 = pressure_setup(mask, p_in, p_out)

    def bc(f_pre, rho, u):
        assert mask.shape == f_pre.shape[0:2]
        feq = equilibrium(rho, u)
        feq_in = equilibrium(rho_in, u[-2, ...]).squeeze()
        f_pre[0, ..., d1] = feq_in[..., d1].T + (f_pre[-2, ..., d1] - feq[-2, ..., d1])
        feq_out = equilibrium(rho_out, u[1, ...]).squeeze()
        f_pre[-1, ..., d2] = feq_out[..., d2].T + (f_pre[1, ..., d2] - feq[1, ..., d2])
        return f_pre
    return bc


# ---------------------------------------------------------------------------
# Scenario compositions  (src/boundary_utils.py) and restated scenarios
# ---------------------------------------------------------------------------
def _row_mask(lx, ly, y):
    m = np.zeros((lx, ly), dtype=bool)
    m[:, y] = True
    return m


def _col_mask(lx, ly, x):
    m = np.zeros((lx, ly), dtype=bool)
    m[x, :] = True
    return m


def couette_boundary(lx, ly, U, avg_density):
    """Rigid top wall, then moving bottom wall u_w=(U,0) (boundary_utils.py:9-55)."""
    top = rigid_wall(_row_mask(lx, ly, -1))
    bottom = moving_wall(_row_mask(lx, ly, 0), np.array([U, 0]), avg_density)

    def boundary(f_pre, f_post, rho=None, u=None, f_prev=None):
        f_post = top(f_pre, f_post)
        return bottom(f_pre, f_post)
    return boundary


def poiseuille_boundary(lx, ly, p_in, p_out):
    """Pressure-periodic x, re-stream, rigid bottom, rigid top (boundary_utils.py:58-110)."""
    m = np.zeros((lx, ly), dtype=bool)
    m[0, :] = True
    m[-1, :] = True
    pressure = periodic_with_pressure_variations(m, p_in, p_out)
    bottom = rigid_wall(_row_mask(lx, ly, 0))
    top = rigid_wall(_row_mask(lx, ly, -1))

    def boundary(f_pre, f_post, rho, u, f_prev=None):
        f_pre = pressure(f_pre, rho, u)
        f_post = streaming(f_pre)
        f_post = bottom(f_pre, f_post)
        return top(f_pre, f_post)
    return boundary


def plate_rows(ly, plate_size):
    """Plate face rows [y_min, y_max) and the two corner rows (boundary_utils.py:145,184-201)."""
    y_min, y_max = ly // 2 - plate_size // 2 + 1, ly // 2 + plate_size // 2 - 1
    return y_min, y_max, ly // 2 + plate_size // 2 - 1, ly // 2 - plate_size // 2


def von_karman_boundary(lx, ly, density_in, velocity_in, plate_size, plate_x=None, walls=False,
                        plate_offset=0):
    """Inlet, outlet, thin plate left/right faces and corners on an unpadded
    periodic domain; the single-rank interior of boundary_utils.py:113-205.

    The channel form of the von Karman study (no reference composition exists
    for it) adds, after the plate, a rigid bottom row and a rigid top row
    through the reference's rigid_wall closure (boundary_conditions.py:78-113;
    a y-wall mask picks directions 4,7,8 at y=0 and 2,5,6 at y=ly-1,
    :18-27), with ``walls=True``; ``plate_offset`` moves the plate's rows by that
    many nodes (rows 71..110 instead of 70..109 at ly=180 for +1)."""
    px = lx // 4 if plate_x is None else plate_x
    y_min, y_max, y_up, y_lo = (r + plate_offset for r in plate_rows(ly, plate_size))
    feq_in = inlet_populations((1, ly), density_in, velocity_in)[0]
    wall_bcs = [rigid_wall(_row_mask(lx, ly, 0)), rigid_wall(_row_mask(lx, ly, -1))] if walls else []

    def boundary(f_pre, f_post, rho=None, u=None, f_prev=None):
        f_post[0, :, :] = feq_in
        for i in (3, 6, 7):
            f_post[-1, :, i] = f_prev[-2, :, i]
        for a, b in zip([3, 7, 6], [1, 5, 8]):
            f_post[px, y_min:y_max, a] = f_pre[px, y_min:y_max, b]
        f_post[px, y_up, [3, 6]] = f_pre[px, y_up, [1, 8]]
        f_post[px, y_lo, [3, 7]] = f_pre[px, y_lo, [1, 5]]
        for a, b in zip([1, 5, 8], [3, 7, 6]):
            f_post[px + 1, y_min:y_max, a] = f_pre[px + 1, y_min:y_max, b]
        f_post[px + 1, y_up, [1, 5]] = f_pre[px + 1, y_up, [3, 7]]
        f_post[px + 1, y_lo, [1, 8]] = f_pre[px + 1, y_lo, [3, 6]]
        for wall in wall_bcs:
            f_post = wall(f_pre, f_post)
        return f_post
    return boundary


def halo_fill(f):
    """Single-rank periodic ghost exchange of a padded array
    (parallelization_utils.py:23-50 with every neighbour being the rank itself)."""
    f[-1, ...] = f[1, ...]
    f[0, ...] = f[-2, ...]
    f[:, -1, :] = f[:, 1, :]
    f[:, 0, :] = f[:, -2, :]
    return f


def von_karman_boundary_padded(lx, ly, density_in, velocity_in, plate_size):
    """The single-rank form of parallel_von_karman_boundary_conditions on a
    ghost-padded (lx+2, ly+2, 9) array (boundary_utils.py:113-205)."""
    inner = von_karman_boundary(lx, ly, density_in, velocity_in, plate_size)

    def boundary(f_pre, f_post, rho=None, u=None, f_prev=None):
        core = f_post[1:-1, 1:-1, :]
        core[...] = inner(f_pre[1:-1, 1:-1, :], core.copy(), None, None, f_prev[1:-1, 1:-1, :])
        return f_post
    return boundary


def cavity_boundary(n_x, n_y, u_lid=0.1, avg_density=1.0):
    """Sliding-lid cavity (restated; no reference composition exists): the
    lateral walls bounce the incoming links (x=0: 1,5,8 from 3,7,6; x=-1:
    3,7,6 from 1,5,8), then the reference rigid bottom wall, then the
    reference moving lid u_w=(u_lid,0); later walls win at corners."""
    bottom = rigid_wall(_row_mask(n_x, n_y, 0))
    lid = moving_wall(_row_mask(n_x, n_y, -1), np.array([u_lid, 0.0]), avg_density)

    def boundary(f_pre, f_post, rho=None, u=None, f_prev=None):
        for a in (1, 5, 8):
            f_post[0, :, a] = f_pre[0, :, OPP[a]]
        for a in (3, 7, 6):
            f_post[-1, :, a] = f_pre[-1, :, OPP[a]]
        f_post = bottom(f_pre, f_post)
        return lid(f_pre, f_post)
    return boundary


def von_karman_channel_start(lx, ly, velocity_in, noise, seed):
    """Start of the channel form: rho = 1, u = (velocity_in, U(-noise, noise)) with
    the u_y field drawn by numpy.random.default_rng(seed).uniform over (lx, ly),
    f = f_eq(rho, u) (the reference's initial value
    density_1_velocity_x_u0_velocity_y_0_initial, initial_values.py:109-123,
    with the seeded transverse perturbation that breaks the symmetry)."""
    rng = np.random.default_rng(seed)
    rho = np.ones((lx, ly))
    u = np.zeros((lx, ly, 2))
    u[..., 0] = velocity_in
    u[..., 1] = rng.uniform(-noise, noise, (lx, ly))
    return equilibrium(rho, u), rho, u


# ---------------------------------------------------------------------------
# Initial values  (src/initial_values.py)
# ---------------------------------------------------------------------------
def sinusoidal_density_x(shape, p0, eps, check=True):
    """rho = p0 + eps sin(2 pi x / lx), u = 0 (:38-64); ``check`` keeps the
    reference's range asserts (config 1 uses p0=1, which they reject)."""
    if check:
        assert p0 + eps < 1 and p0 - eps > 0
    x = np.arange(0, shape[0])
    rho = np.tile(p0 + eps * np.sin(np.divide(2 * np.pi * x, shape[0])), (shape[1], 1)).T
    return rho, np.zeros(tuple(shape) + (2,))


def sinusoidal_velocity_x(shape, eps):
    """rho = 1, u_x = eps sin(2 pi y / ly) (:67-93)."""
    assert np.abs(eps) < 0.1
    y = np.arange(0, shape[1])
    ux = np.tile(eps * np.sin(np.divide(2 * np.pi * y, shape[1])), (shape[0], 1))
    return np.ones(shape), np.dstack([ux, np.zeros(shape)])


def density_1_velocity_0(shape):                                 # :96-106
    return np.ones(shape), np.zeros(tuple(shape) + (2,))


def density_1_velocity_u0(shape, u0):                            # :109-123
    u = np.empty(tuple(shape) + (2,))
    u[..., 0] = u0
    u[..., 1] = 0
    return np.ones(shape), u


# ---------------------------------------------------------------------------
# Post-processing  (src/experiments.py, src/visualizations_utils.py)
# ---------------------------------------------------------------------------
def strouhal_from_trace(trace, L, u):
    """Dominant frequency |fftfreq[argmax |fft(trace - mean)|]| times L/u
    (visualizations_utils.py:149-167)."""
    t = np.asarray(trace, dtype=np.float64)
    yf = np.fft.fft(t - t.mean())
    freq = np.fft.fftfreq(len(t), 1)
    return strouhal_number(np.abs(freq[np.argmax(np.abs(yf))]), L, u)


def run(f, rho, u, omega, steps, boundary=None, communicate=None):
    for _ in range(steps):
        f, rho, u = step(f, rho, u, omega, boundary, communicate)
    return f, rho, u

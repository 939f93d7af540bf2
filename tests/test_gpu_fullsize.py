"""The headline workload at its full size (sliding-lid cavity 8192x8192, omega
1.7, lid u = (0.1, 0)), checked through properties that do not depend on the
size: the oracle finishes small lattices only, and the step is the same local
arithmetic at every node of any lattice.

* Mass: bounce-back walls and the moving lid (whose two slanted terms cancel)
  conserve the total mass; the fixed-point storage keeps it to 1e-14 relative
  (its moments are exact integer sums, the relaxation rounds zero-mean).
* Two independent arithmetic paths agree: the fixed-point kernel (integer and
  float-float collision) and the float64 FMA kernel stay within the float64
  gate of 1e-12 relative max error of each other after 200 steps, as each
  does against the NumPy oracle on the small cases of the other tests.
* The boundary-node pass: at this size the step is two launches; with the
  sources inside the step instead (LBM_FLAG_BC_INLINE) the state is
  bit-identical.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu

N, STEPS = 8192, 200


@pytest.fixture(scope="module")
def pkg():
    import lattice_boltzmann_parallel_solver_gb300 as P
    P._lib.load()
    return P


def _cavity(pkg, storage, **kw):
    from lattice_boltzmann_parallel_solver_gb300.boundary_utils import cavity_boundary_conditions
    bnd = cavity_boundary_conditions(N, N, 0.1, 1.0)
    w = torch.tensor([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=torch.float64, device="cuda")
    return pkg.Lattice(N, N, 1.7, bnd, storage=storage, **kw).set_state(w.expand(N, N, 9).contiguous())


def test_full_size_cavity_mass_and_two_arithmetic_paths(pkg):
    an = pkg.analysis
    fx = _cavity(pkg, "fx64").step(STEPS)
    f_fx = fx.read()[0]
    del fx
    m0 = float(N * N)  # rho = 1 everywhere at the start
    m1 = an.mass_momentum(f_fx)[0]
    assert abs(m1 - m0) / m0 <= 1e-14
    fl = _cavity(pkg, "f64").step(STEPS)
    f_fl = fl.read()[0]
    del fl
    err = float((f_fx - f_fl).abs().max() / f_fl.abs().max())
    assert err <= 1e-12, err
    # the lid has set the fluid moving
    assert float((f_fx[:, -2, 5] - f_fx[:, -2, 6]).abs().max()) > 1e-4


@pytest.mark.parametrize("storage", ["fx64", "f16"])
def test_full_size_boundary_node_pass_bit_identical(pkg, storage):
    a = _cavity(pkg, storage).step(20)
    b = _cavity(pkg, storage, bc_inline=True).step(20)
    fa, fb = a.read()[0], b.read()[0]
    assert torch.equal(fa, fb)

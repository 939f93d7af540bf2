"""Drop-in for the reference's ``src/lattice_boltzmann_method.py``.

Same names, signatures, layouts (f[nx, ny, 9], rho[nx, ny], u[nx, ny, 2],
float64) and error behaviour (AssertionError on shape or omega violations);
the arithmetic runs in the CUDA kernels of ``liblbm_gb300.so`` and follows
NumPy's float64 operation order.  Inputs may be NumPy arrays or torch tensors;
results come back in the caller's kind.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _arrays as A
from . import _lib
from .geometry import empty_geometry

# ---------------------------------------------------------------------------
# D2Q9 constants (lattice_boltzmann_method.py:5-52)
# ---------------------------------------------------------------------------
_C = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])
_OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])
_W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36])


def get_velocity_sets() -> np.ndarray:
    """D2Q9 velocity set c_i (:5-26)."""
    return _C.copy()


def vel_to_opp_vel_mapping() -> np.ndarray:
    """Index of the opposite direction (:29-39)."""
    return _OPP.copy()


def get_w_i() -> np.ndarray:
    """D2Q9 weights (:42-52)."""
    return _W.copy()


def reynolds_number(L, u, v):
    """Re = L u / nu (:55-71)."""
    return np.divide(L * u, v)


def strouhal_number(f, L, u):
    """St = f L / u (:74-90)."""
    return np.divide(f * L, u)


# ---------------------------------------------------------------------------
# component operators
# ---------------------------------------------------------------------------
def compute_density(prob_densitiy_func):
    """rho = sum_i f_i (:93-105)."""
    kind = A.kind_of(prob_densitiy_func)
    f = A.to_device(prob_densitiy_func)
    assert f.shape[-1] == 9
    rho = torch.empty(f.shape[:-1], dtype=torch.float64, device=f.device)
    _lib.call("lbm_density_f64", f.data_ptr(), rho.data_ptr(), rho.numel(), A.stream())
    return A.to_kind(rho, kind)


def compute_velocity_field(density_func, prob_density_func):
    """u = sum_i c_i f_i / rho, 0 where rho == 0 (:108-137)."""
    kind = A.kind_of(prob_density_func)
    f = A.to_device(prob_density_func)
    assert f.shape[-1] == 9
    assert f.dim() == 3, "compute_velocity_field indexes f[:, :, dirs]"
    rho = A.to_device(density_func)
    assert tuple(rho.shape) == tuple(f.shape[:-1])
    u = torch.empty(tuple(f.shape[:-1]) + (2,), dtype=torch.float64, device=f.device)
    _lib.call("lbm_velocity_f64", rho.data_ptr(), f.data_ptr(), u.data_ptr(), rho.numel(), A.stream())
    return A.to_kind(u, kind)


def streaming(prob_density_func):
    """Periodic streaming into a new array (:140-159)."""
    kind = A.kind_of(prob_density_func)
    f = A.to_device(prob_density_func)
    assert f.shape[-1] == 9
    assert f.dim() == 3, "streaming rolls axes 0 and 1 of f[nx, ny, 9]"
    out = torch.empty_like(f)
    _lib.call("lbm_streaming_f64", f.data_ptr(), out.data_ptr(), f.shape[0], f.shape[1], A.stream())
    return A.to_kind(out, kind)


def equilibrium_distr_func(density_func, velocity_field):
    """f_eq = w rho (1 + 3 c.u + 9/2 (c.u)^2 - 3/2 |u|^2) (:162-188).

    The weights broadcast as (1, 1, 9) exactly like the reference, so a 1-D
    input of n nodes yields shape (1, n, 9)."""
    kind = A.kind_of(velocity_field)
    rho = A.to_device(density_func)
    u = A.to_device(velocity_field)
    assert tuple(rho.shape) == tuple(u.shape[:-1])
    assert u.shape[-1] == 2
    out_shape = np.broadcast_shapes((1, 1, 9), tuple(rho.shape) + (1,))
    feq = torch.empty(out_shape, dtype=torch.float64, device=rho.device)
    _lib.call("lbm_equilibrium_f64", rho.data_ptr(), u.data_ptr(), feq.data_ptr(), rho.numel(), A.stream())
    return A.to_kind(feq, kind)


def collision(f, density, velocity, omega, exact=True):
    """f + (f_eq(rho, u) - f) omega, the collision line of the step (:213-215)."""
    kind = A.kind_of(f)
    ft = A.to_device(f)
    rho = A.to_device(density)
    u = A.to_device(velocity)
    out = torch.empty_like(ft)
    _lib.call("lbm_collide_f64", ft.data_ptr(), rho.data_ptr(), u.data_ptr(), float(omega), out.data_ptr(),
              rho.numel(), _lib.FLAG_EXACT if exact else 0, A.stream())
    return A.to_kind(out, kind)


# ---------------------------------------------------------------------------
# the step
# ---------------------------------------------------------------------------
_SCRATCH = {}


def _scratch(nx, ny, device, host=False):
    key = (nx, ny, str(device), host)
    t = _SCRATCH.get(key)
    if t is None:
        lib = _lib.load()
        n = int(lib.lbm_step_host_scratch_bytes(nx, ny) if host else lib.lbm_step_scratch_bytes(nx, ny))
        _SCRATCH.clear()
        t = torch.empty(n, dtype=torch.uint8, device=device)
        _SCRATCH[key] = t
    return t


def _host_f64(a) -> torch.Tensor:
    """Contiguous float64 CPU tensor viewing ``a`` where it can (NumPy arrays
    are not copied; pinned tensors stay pinned, which lets the copies overlap)."""
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64))
    return t.to(torch.float64).contiguous()


def _step_host(geo, f, rho, u, omega, flags, kind, slabs=0):
    """The fused step on host arrays: slabs of x copied in, stepped and copied
    out with the copies and kernels overlapped (lbm_step_f64_host; ``slabs`` 0
    takes its default)."""
    fh, rh, uh = _host_f64(f), _host_f64(rho), _host_f64(u)
    assert tuple(fh.shape[0:2]) == tuple(rh.shape) and tuple(fh.shape[0:2]) == tuple(uh.shape[0:2])
    assert fh.dim() == 3 and fh.shape[-1] == 9
    nx, ny = int(fh.shape[0]), int(fh.shape[1])
    outs = [torch.empty(t.shape, dtype=torch.float64, pin_memory=True) for t in (fh, rh, uh)]
    scratch = _scratch(nx, ny, torch.device("cuda"), host=True)
    _lib.call("lbm_step_f64_host", geo.ref, fh.data_ptr(), rh.data_ptr(), uh.data_ptr(), float(omega),
              outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), scratch.data_ptr(), scratch.numel(),
              flags, int(slabs), A.stream())
    torch.cuda.current_stream().synchronize()
    return tuple(o if kind == A.TORCH_CPU else o.numpy() for o in outs)


def _is_own_hook(obj) -> bool:
    return getattr(obj, "_lbm_gb300_hook", False)


def _call_foreign(hook, kind, *tensors):
    """Call a caller-supplied callable with arrays of the caller's kind."""
    if kind == A.TORCH_CUDA:
        return A.to_device(hook(*tensors))
    args = [None if t is None else A.to_kind(t, kind) for t in tensors]
    return A.to_device(hook(*args))


def lattice_boltzmann_step(f, density, velocity, omega, boundary=None, parallel_communication=None,
                           exact: bool = True):
    """One BGK step (:191-228): collide with the passed-in density and velocity,
    optional halo hook, stream, boundary hook, moments.

    ``boundary`` built by this package's factories (boundary_utils, or
    ``Boundary([...])``) and no halo hook run fused: two kernels for the whole
    step; on host arrays (NumPy, CPU tensors) the copies in and out are cut
    into slabs of x and overlapped with the kernels.  Any other callable, or a
    halo hook, runs the unfused sequence collide -> hook -> stream -> boundary
    -> moments on device arrays.
    ``exact=True`` (the default) keeps NumPy's float64 operation order, so the
    result is bit-for-bit the reference's; ``exact=False`` uses the FMA form.
    """
    kind = A.kind_of(f)
    assert 0 < omega < 2
    if kind != A.TORCH_CUDA and parallel_communication is None:
        # host arrays and a fusable boundary: the pipelined host-buffer step
        A.require_cuda()
        shp = np.shape(f)
        assert len(shp) == 3 and shp[-1] == 9
        nx, ny = int(shp[0]), int(shp[1])
        if boundary is None:
            hgeo = empty_geometry(nx, ny)
        elif _is_own_hook(boundary) and hasattr(boundary, "geometry"):
            hgeo = boundary.geometry(nx, ny)
            hgeo = hgeo if hgeo.fusable else None
        else:
            hgeo = None
        if hgeo is not None:
            return _step_host(hgeo, f, density, velocity, omega, _lib.FLAG_EXACT if exact else 0, kind)
    ft, rho, u = A.to_device(f), A.to_device(density), A.to_device(velocity)
    assert tuple(ft.shape[0:2]) == tuple(rho.shape)
    assert tuple(ft.shape[0:2]) == tuple(u.shape[0:2])
    assert 0 < omega < 2
    assert ft.dim() == 3 and ft.shape[-1] == 9
    nx, ny = int(ft.shape[0]), int(ft.shape[1])
    flags = _lib.FLAG_EXACT if exact else 0
    s = A.stream()

    geo = None
    if parallel_communication is None:
        if boundary is None:
            geo = empty_geometry(nx, ny)
        elif _is_own_hook(boundary) and hasattr(boundary, "geometry"):
            g = boundary.geometry(nx, ny)
            geo = g if g.fusable else None
    if geo is not None:
        f_out = torch.empty_like(ft)
        rho_out = torch.empty_like(rho)
        u_out = torch.empty_like(u)
        _lib.call("lbm_step_f64", geo.ref, ft.data_ptr(), rho.data_ptr(), u.data_ptr(), float(omega),
                  f_out.data_ptr(), rho_out.data_ptr(), u_out.data_ptr(), _scratch(nx, ny, ft.device).data_ptr(),
                  flags, s)
        return A.to_kind(f_out, kind), A.to_kind(rho_out, kind), A.to_kind(u_out, kind)

    # unfused sequence (same operations, one kernel each)
    f_pre = torch.empty_like(ft)
    _lib.call("lbm_collide_f64", ft.data_ptr(), rho.data_ptr(), u.data_ptr(), float(omega), f_pre.data_ptr(),
              nx * ny, flags, s)
    if parallel_communication is not None:
        if _is_own_hook(parallel_communication):
            f_pre = parallel_communication(f_pre)
        else:
            f_pre = _call_foreign(parallel_communication, kind, f_pre)
    f_post = torch.empty_like(f_pre)
    _lib.call("lbm_streaming_f64", f_pre.data_ptr(), f_post.data_ptr(), nx, ny, s)
    if boundary is not None:
        if _is_own_hook(boundary):
            f_post = boundary(f_pre, f_post, rho, u, ft)
        else:
            f_post = _call_foreign(boundary, kind, f_pre, f_post, rho, u, ft)
    rho_out = torch.empty((nx, ny), dtype=torch.float64, device=ft.device)
    u_out = torch.empty((nx, ny, 2), dtype=torch.float64, device=ft.device)
    _lib.call("lbm_density_f64", f_post.data_ptr(), rho_out.data_ptr(), nx * ny, s)
    _lib.call("lbm_velocity_f64", rho_out.data_ptr(), f_post.data_ptr(), u_out.data_ptr(), nx * ny, s)
    return A.to_kind(f_post, kind), A.to_kind(rho_out, kind), A.to_kind(u_out, kind)

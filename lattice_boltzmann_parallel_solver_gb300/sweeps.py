"""Strouhal-number sweeps of the von Karman flow as one device job.

The reference runs each point of its Reynolds-number, channel-length and
blockage sweeps as a separate MPI job of ``x_strouhal`` (src/experiments.py:650-720,
parameters from src/main.py:150-207) and post-processes the saved |u| probe
traces afterwards (src/visualizations_utils.py:135-260).  Here every point
of a sweep is a member of one ``Batch``: all lattices advance in the same
launches, the probe velocity is recorded on the device every step, and the
Strouhal number is formed from the trace by the reference's own
post-processing (argmax of the FFT magnitude after a per-point start sample)
and by the sub-bin estimate of ``analysis.spectral_peak``.
"""
from __future__ import annotations

import numpy as np
import torch

from . import analysis
from . import boundary_utils as BU
from .batch import Batch, Member
from .lattice import REF_SHIFTED

PLATE = 40          # the plate size every sweep keeps (x_strouhal's default)


def sweep_points(kind: str, values=None, lattice_grid_shape=(420, 180), inlet_velocity=0.1,
                 kinematic_viscosity=0.04):
    """The sweep's points as dicts (lx, ly, u, nu, start, label), following
    src/main.py:150-207 and the post-processing starts of
    src/visualizations_utils.py:135-260.

    kind "reynolds": Re in ``values`` (default 40, 70, 100, 140, 170, 200) on
    420 x 180; Re <= 130 keeps u = 0.1 and sets nu = 40 u / Re, larger Re keep
    nu = 0.03 and set u = Re nu / 40.  kind "nx": channel lengths (default 260
    ... 1250) at ly = 180.  kind "blockage": channel heights (default 60 ... 260)
    at lx = 420."""
    lx0, ly0 = lattice_grid_shape
    pts = []
    if kind == "reynolds":
        for re_ in (values or (40, 70, 100, 140, 170, 200)):
            if re_ > 130:
                nu, u = 0.03, re_ * 0.03 / 40
            else:
                nu, u = 40 * 0.1 / re_, inlet_velocity
            start = {40: 150000, 70: 125000}.get(int(re_), 70000)
            pts.append({"lx": lx0, "ly": ly0, "u": u, "nu": nu, "start": start, "label": re_})
    elif kind == "nx":
        for lx in (values or (260, 300, 350, 420, 500, 750, 1000, 1250)):
            start = {260: 125000, 300: 90000, 350: 90000, 700: 90000, 100: 175000}.get(int(lx), 75000)
            pts.append({"lx": int(lx), "ly": 180, "u": inlet_velocity, "nu": kinematic_viscosity, "start": start,
                        "label": lx})
    elif kind == "blockage":
        for ly in (values or (60, 100, 140, 180, 260)):
            pts.append({"lx": 420, "ly": int(ly), "u": inlet_velocity, "nu": kinematic_viscosity, "start": 90000,
                        "label": PLATE / ly})
    else:
        raise ValueError("kind is 'reynolds', 'nx' or 'blockage'")
    return pts


def _uniform_flow(lx, ly, u_in, device):
    """rho = 1, u = (u_in, 0) and its equilibrium, the reference's start
    (initial_values.py:109-123, lattice_boltzmann_method.py:162-188), on the device."""
    from .lattice_boltzmann_method import equilibrium_distr_func
    rho = torch.ones((lx, ly), dtype=torch.float64, device=device)
    u = torch.zeros((lx, ly, 2), dtype=torch.float64, device=device)
    u[..., 0] = u_in
    return equilibrium_distr_func(rho, u), rho, u


def strouhal_sweep(kind: str, values=None, steps: int = 200000, storage: str = "fx64", device: str = "cuda",
                   chunk: int = 1000):
    """Runs every point of the sweep for ``steps`` steps in one batch and returns,
    per point, its parameters, the |u| trace at (3 lx / 4, ly / 2) (the
    reference's vel_at_p: steps + 1 samples) and the Strouhal numbers
    St = f d / u with d = 40: by the reference's post-processing
    (``strouhal_argmax``) and by the sub-bin estimate (``strouhal``).  With a
    reference-shifted storage ("f16r", "bf16r") each point's reference velocity
    is its inlet velocity."""
    pts = sweep_points(kind, values)
    members = []
    for p in pts:
        lx, ly = p["lx"], p["ly"]
        omega = float(np.reciprocal(3 * p["nu"] + 0.5))           # experiments.py:671
        bnd = BU.von_karman_boundary_conditions(lx, ly, 1.0, p["u"], PLATE)
        f0, rho0, u0 = _uniform_flow(lx, ly, p["u"], device)
        members.append(Member(lx, ly, omega, bnd, steps=steps, probe=(3 * lx // 4, ly // 2), f0=f0, rho0=rho0,
                              u0=u0, dev_ref=(p["u"], 0.0) if storage in REF_SHIFTED else None))
    b = Batch(members, storage=storage, device=device).start()
    b.run_graph(chunk=chunk)
    out = []
    for j, (p, m) in enumerate(zip(pts, members)):
        uv = b.probe_trace(j)
        last = b.read(j, want_f=False)[2][m.probe[0], m.probe[1]]
        uv = torch.cat([uv, last[None, :]], 0)
        tr = torch.cat([torch.tensor([abs(p["u"])], dtype=torch.float64, device=uv.device),
                        torch.sqrt(uv[:, 0] * uv[:, 0] + uv[:, 1] * uv[:, 1])])
        r = dict(p)
        r["trace"] = tr
        if steps > p["start"] + 16:
            r["strouhal_argmax"] = analysis.strouhal(tr, PLATE, p["u"], start=p["start"])
            f, binw, pbin = analysis.spectral_peak(tr, start=p["start"])
            r["strouhal"] = f * PLATE / p["u"]
            r["strouhal_bin"] = binw * PLATE / p["u"]
        out.append(r)
    return out

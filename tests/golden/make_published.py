"""Extract the reference's PUBLISHED physics results into a small fixture.

    python tests/golden/make_published.py <path of the reference checkout>

The reference ships the outputs of its long runs under ``figures/``; this
script reads them (the checkout is never modified) and writes
``tests/golden/published_physics.npz``, which the GPU tests compare against
(the reference checkout does not exist where those tests run):

* von Karman, Re = 100 (``src/experiments.py:650-704`` x_strouhal: 420x180,
  plate 40 at x = 105, inlet (0.1, 0), nu = 0.04, 200 000 steps, |u| probed
  at (315, 90) each step; the published trace
  ``figures/von_karman_vortex_shedding/reynold_strouhal/vel_at_p_100.npy``):
  every 50th sample, the sum and the sum of squares of all 200 001 samples,
  and its Strouhal number by the reference's post-processing
  (``src/visualizations_utils.py:149-167``: argmax of the FFT magnitude after
  sample 70 000, L = 40, u = 0.1) and by the package's sub-bin estimate;
* the serial run of the same flow (``src/milestoneQuickFunctionCalls.py:294-341``,
  100 000 steps): SHA-256 of the raw float64 bytes of the published final
  ``velocity.py.npy`` [420, 180, 2] and ``density.py.npy`` [420, 180], a
  strided sample of both, and the published 100 001-sample probe trace as
  every 50th sample with its sum;
* the Reynolds sweep (``src/main.py:150-177``: Re 40, 70, 100 with u = 0.1,
  Re 140, 170, 200 with nu = 0.03 and u = Re nu / 40): each trace's Strouhal
  number by the reference's post-processing, with its per-Re start sample,
  and by the sub-bin estimate;
* Couette flow (``src/experiments.py:304-363``): slope, intercept and r of
  ``figures/couette_flow/linregress.csv``;
* Poiseuille flow (``src/experiments.py:377-492``): the inlet and middle flux
  areas and their ratio (``figures/poiseuille_flow/areas.csv``) and the
  quadratic fit (``curve_fit.csv``, printed to 9 digits there).
"""
from __future__ import annotations

import csv
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def reference_strouhal(trace, start, length, velocity):
    """visualizations_utils.py:149-167, restated."""
    v = np.array(trace[start:], dtype=np.float64)
    v -= np.mean(v)
    yf = np.fft.fft(v)
    freq = np.fft.fftfreq(len(v), 1)
    return float(np.abs(freq[np.argmax(np.abs(yf))]) * length / velocity)


def sha256_of(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def main(ref):
    from lattice_boltzmann_parallel_solver_gb300.analysis import spectral_peak

    vk = os.path.join(ref, "figures", "von_karman_vortex_shedding")
    out = {}

    trace = np.load(os.path.join(vk, "reynold_strouhal", "vel_at_p_100.npy"))
    assert trace.shape == (200001,)
    out["vk100_trace_every50"] = trace[::50].copy()
    out["vk100_trace_sum"] = np.float64(np.sum(trace))
    out["vk100_trace_sumsq"] = np.float64(np.sum(trace * trace))
    out["vk100_st_argmax"] = np.float64(reference_strouhal(trace, 70000, 40, 0.1))
    f, b, pb = spectral_peak(trace, start=70000)
    out["vk100_st_interp"] = np.float64(f * 40 / 0.1)

    vel = np.load(os.path.join(vk, "velocity.py.npy"))
    rho = np.load(os.path.join(vk, "density.py.npy"))
    ser = np.load(os.path.join(vk, "vel_at_p.py.npy"))
    assert vel.shape == (420, 180, 2) and rho.shape == (420, 180) and ser.shape == (100001,)
    out["vk_serial_velocity_sha256"] = np.array(sha256_of(vel))
    out["vk_serial_density_sha256"] = np.array(sha256_of(rho))
    out["vk_serial_velocity_every7"] = vel[::7, ::7].copy()
    out["vk_serial_density_every7"] = rho[::7, ::7].copy()
    out["vk_serial_trace_every50"] = ser[::50].copy()
    out["vk_serial_trace_sum"] = np.float64(np.sum(ser))

    res, st_ref, st_int, starts, vels = [], [], [], [], []
    for re_ in (40, 70, 100, 140, 170, 200):
        t = np.load(os.path.join(vk, "reynold_strouhal", "vel_at_p_%d.npy" % re_))
        start = {40: 150000, 70: 125000}.get(re_, 70000)
        u = re_ * 0.03 / 40 if re_ > 130 else 0.1
        res.append(re_)
        starts.append(start)
        vels.append(u)
        st_ref.append(reference_strouhal(t, start, 40, u))
        st_int.append(spectral_peak(t, start=start)[0] * 40 / u)
    out["re_sweep_re"] = np.array(res)
    out["re_sweep_start"] = np.array(starts)
    out["re_sweep_u"] = np.array(vels)
    out["re_sweep_st_argmax"] = np.array(st_ref)
    out["re_sweep_st_interp"] = np.array(st_int)

    with open(os.path.join(ref, "figures", "couette_flow", "linregress.csv")) as fh:
        row = next(csv.DictReader(fh))
    out["couette_slope"] = np.float64(row["slope"])
    out["couette_intercept"] = np.float64(row["intercept"])
    out["couette_rvalue"] = np.float64(row["rvalue"])

    with open(os.path.join(ref, "figures", "poiseuille_flow", "areas.csv")) as fh:
        row = next(csv.DictReader(fh))
    out["poiseuille_area_inlet"] = np.float64(row["inlet"])
    out["poiseuille_area_middle"] = np.float64(row["middle"])
    out["poiseuille_area_ratio"] = np.float64(row["relative_difference"])
    with open(os.path.join(ref, "figures", "poiseuille_flow", "curve_fit.csv")) as fh:
        row = next(csv.DictReader(fh))
    out["poiseuille_popt"] = np.array([float(v) for v in row["popt"].strip("[]").split()])

    path = os.path.join(HERE, "published_physics.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, "(%d bytes)" % os.path.getsize(path))
    for k in sorted(out):
        v = out[k]
        if np.ndim(v) == 0 or (np.ndim(v) == 1 and len(v) <= 6):
            print(" ", k, v)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_published.py <path of the reference checkout>")
    main(sys.argv[1])

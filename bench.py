"""Benchmark of the D2Q9 hot path on the sliding-lid cavity (8192^2, omega 1.7,
lid u = (0.1, 0), rho = 1, u = 0 at start): MLUPS of the resident fused step
at float64 accuracy (fx64 storage), its HBM roofline fraction, the reduced-precision storages, the
end-to-end drop-in call with host buffers, and the NumPy path on host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one lattice time step over the whole domain.  Under torchrun each
rank runs its own replica of the workload on its GPU (weak scaling); the
timed region is bracketed by a barrier and a device synchronize on both
sides and the slowest rank's time counts.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_NODE = {"fx64": 144, "f64": 144, "f32": 72, "f16": 36, "bf16": 36}
# arithmetic of each storage's collision
DTYPES = {"fx64": "int64+f32x2", "f64": "f64", "f32": "f32", "f16": "f32 (f16 storage)", "bf16": "f32 (bf16 storage)",
          "f16r": "f32 (f16 storage, shifted)", "bf16r": "f32 (bf16 storage, shifted)"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=8192, help="cavity side")
    p.add_argument("--storage", default="fx64", choices=sorted(BYTES_PER_NODE))
    p.add_argument("--exact", action="store_true", help="NumPy-order float64 arithmetic")
    p.add_argument("--bc", default="auto", choices=["auto", "split", "inline"],
                   help="boundary sources: a separate pass over the boundary nodes (split), inside the step "
                        "(inline), or chosen by the lattice size (auto)")
    p.add_argument("--no-extras", action="store_true", help="skip variants, e2e, CPU baseline and the other configs")
    p.add_argument("--workload", default="cavity",
                   choices=["cavity", "shear", "vk", "vk_seeds", "batch", "serve", "serve_sweep", "batch_step"],
                   help="cavity: the headline line; the others print one config's results and exit")
    p.add_argument("--configs", default="shear,vk,batch,serve", help="other configs added to the headline line")
    return p.parse_args()


# ---------------------------------------------------------------------------
# the other configurations (reported beside the headline)
# ---------------------------------------------------------------------------
def timed_ms(fn):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def bench_shear(P):
    """Shear-wave decay, fx64 storage, 64x64 periodic, omega 1.0, 2000 steps: amplitude
    decay and the fitted viscosity by the reference's method
    (experiments.py:195-210) against (1/omega - 1/2)/3; also the velocity shear wave."""
    import torch
    from scipy.optimize import curve_fit
    from scipy.signal import argrelextrema
    n, omega, steps = 64, 1.0, 2000
    f, rho, u = P.scenarios.shear_wave(n, 0.01)
    lat = P.Lattice(n, n, omega).set_state(f, rho, u)
    amp = []
    t0 = time.perf_counter()
    for _ in range(steps):
        lat.step(1)
        amp.append(lat.moments()[0] - 1.0)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    a = torch.stack(amp)
    dens = torch.where(a.amin(dim=(1, 2)).abs() > a.amax(dim=(1, 2)).abs(), a.amin(dim=(1, 2)).abs(),
                       a.amax(dim=(1, 2)).abs()).cpu().numpy()
    idx = argrelextrema(dens, np.greater)[0]
    k2 = (2 * np.pi / n) ** 2
    nu_d = float(curve_fit(lambda t, v: 0.01 * np.exp(-v * k2 * t), idx, dens[idx], p0=[0.1])[0][0])
    ux = P.initial_values.sinusoidal_velocity_x((n, n), 0.01)
    lat = P.Lattice(n, n, omega).set_state(P.scenarios.equilibrium_np(*ux), *ux)
    vel = []
    for _ in range(400):
        lat.step(5)
        vel.append(float(lat.moments()[1][..., 0].abs().max()))
    t = 5 * np.arange(1, 401)
    nu_v = float(curve_fit(lambda t, v: 0.01 * np.exp(-v * k2 * t), t, np.array(vel), p0=[0.1])[0][0])
    theory = (1 / omega - 0.5) / 3
    return {"workload": "shear wave 64x64, omega 1.0, rho = 1 + 0.01 sin(2 pi x/64), 2000 steps, fx64 storage",
            "amplitude_first_last": [float(dens[0]), float(dens[-1])], "nu_theory": theory,
            "nu_fit_density_wave_reference_method": nu_d, "nu_fit_velocity_wave": nu_v,
            "velocity_wave_rel_err": abs(nu_v - theory) / theory, "wall_s_with_per_step_readout": wall}


def strouhal(trace, L=40, u=0.1, start=None):
    """St from the FP64 FFT of a probe trace by the reference's argmax
    (visualizations_utils.py:157-160): quantised to one FFT bin."""
    t = np.asarray(trace, dtype=np.float64)
    if start is not None:
        t = t[start:]
    yf = np.fft.fft(t - t.mean())
    freq = np.fft.fftfreq(len(t), 1)
    return float(np.abs(freq[np.argmax(np.abs(yf))]) * L / u)


def strouhal_subbin(P, trace, L=40, u=0.1, start=0):
    """(St, St of one FFT bin, St of one padded bin) by the sub-bin spectral
    peak estimate (Hann window, 16x zero padding, Gaussian interpolation)."""
    f, b, pb = P.analysis.spectral_peak(trace, start=start)
    return f * L / u, b * L / u, pb * L / u


def phase_lag(ref, other, period_guess, window):
    """Lag tau (steps, |tau| <= half a period) maximising the correlation of
    other(t) with ref(t + tau) over the ``window`` samples that end half a
    period before the end of the traces (so that every shifted window of ref
    lies inside it)."""
    ref = np.asarray(ref, dtype=np.float64)
    other = np.asarray(other, dtype=np.float64)
    half = int(period_guess // 2)
    end = min(len(ref), len(other)) - half
    a = other[end - window:end] - other[end - window:end].mean()
    best, lag = -np.inf, 0
    for tau in range(-half, half + 1):
        b = ref[end - window + tau:end + tau]
        b = b - b.mean()
        # normalised: a window of larger amplitude must not win by its energy
        c = float(np.dot(a, b)) / max(float(np.linalg.norm(b)), 1e-300)
        if c > best:
            best, lag = c, tau
    return lag


def bench_vk_seeds(P, steps=100000, seeds=8):
    """Spread of the 16-bit storages' errors over stochastic-rounding seeds on
    the von Karman precision study (420x180, Re 100): ``seeds`` members with
    seeds 1000.. in one batch per storage (f16, f16r, bf16, bf16r; the shifted
    ones with the inlet velocity (0.1, 0) as the reference) against one fx64
    run: velocity L2 at 2000, 5000 and 10000 steps and the Strouhal error of
    u_y at (300, 90) over ``steps`` steps (sub-bin estimate), each as
    (mean, min, max)."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    f, rho, u, omega, bnd = P.scenarios.von_karman(420, 180, plate=40, re=100, seed=0)
    cps = (2000, 5000, 10000)

    def run(storage, n):
        ms = [Member(420, 180, omega, bnd, steps=steps, probe=(300, 90), f0=f, rho0=rho, u0=u, seed=1000 + k,
                     dev_ref=(0.1, 0.0) if storage in ("f16r", "bf16r") else None) for k in range(n)]
        b = Batch(ms, storage=storage).start()
        us = {}
        for c in cps:
            b.run_graph(c - 1 - b.g, chunk=1000)
            us[c] = [b.read(j, want_f=False)[2] for j in range(n)]
        b.run_graph(chunk=1000)
        sts = []
        for j in range(n):
            uy = b.probe_trace(j)[:, 1]
            sts.append(P.analysis.spectral_peak(uy, start=uy.numel() // 2)[0])
        return us, sts

    def spread(v):
        return [float(np.mean(v)), float(np.min(v)), float(np.max(v))]

    ref_us, ref_st = run("fx64", 1)
    out = {"seeds": seeds, "steps": steps}
    for st in ("f16", "f16r", "bf16", "bf16r"):
        us, sts = run(st, seeds)
        r = {"velocity_l2_rel_err_%d" % c: spread([float(torch.linalg.norm(x - ref_us[c][0]) /
                                                        torch.linalg.norm(ref_us[c][0])) for x in us[c]])
             for c in cps}
        r["strouhal_rel_err"] = spread([abs(x - ref_st[0]) / ref_st[0] for x in sts])
        out[st] = r
    return out


def bench_vk(P, steps=100000):
    """Von Karman precision study: 420x180, plate 40 at x=105 offset +1, inlet
    (0.1, 0) with seeded U(-1e-3, 1e-3) u_y, the reference's outlet,
    top/bottom bounce-back, Re 100; float64 storage against fx64 / float32 / f16 / bf16
    storage and the reference-shifted f16r / bf16r (reference velocity the
    inlet's (0.1, 0)): velocity L2 error at fixed steps (before and after the onset of
    shedding), the Strouhal number of u_y at (300, 90) by a sub-bin estimate
    with its resolution, and the error split into phase (the lag of the
    shedding cycle) and the rest (the L2 error against the float64 field at
    the lagged step)."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    lx, ly = 420, 180
    f, rho, u, omega, bnd = P.scenarios.von_karman(lx, ly, plate=40, re=100, seed=0)
    checkpoints = [s for s in (2000, 5000, 10000, 50000, steps) if s <= steps]
    out, ref_u, traces = {}, {}, {}

    def run(storage, upto, cps):
        m = Member(lx, ly, omega, bnd, steps=upto, probe=(300, 90), f0=f, rho0=rho, u0=u,
                   dev_ref=(0.1, 0.0) if storage in ("f16r", "bf16r") else None)
        b = Batch([m], storage=storage).start()
        us, ms_total, done = {}, 0.0, 1
        for c in cps:
            ms_total += timed_ms(lambda: b.run_graph(c - done, chunk=1000))
            done = c
            us[c] = b.read(0, want_f=False)[2]
        return b, us, ms_total

    for storage in ("f64", "fx64", "f32", "f16", "bf16", "f16r", "bf16r"):
        b, us, ms_total = run(storage, steps, checkpoints)
        uy = b.probe_trace(0)[:, 1].cpu().numpy()
        traces[storage] = uy
        st, st_bin, st_pbin = strouhal_subbin(P, uy, start=len(uy) // 2)
        res = {"mlups": lx * ly * (steps - 1) / (ms_total / 1e3) / 1e6,
               "strouhal": st, "strouhal_fft_bin": st_bin, "strouhal_padded_bin": st_pbin,
               "strouhal_argmax": strouhal(uy, start=len(uy) // 2),
               "uy_probe_rms_last_half": float(np.std(uy[len(uy) // 2:]))}
        if storage == "f64":
            ref_u = us
        else:
            res["velocity_l2_rel_err"] = {str(c): float(torch.linalg.norm(us[c] - ref_u[c]) / torch.linalg.norm(ref_u[c]))
                                          for c in checkpoints}
            res["strouhal_rel_err"] = abs(st - out["f64"]["strouhal"]) / out["f64"]["strouhal"]
            res["uy_rms_rel_err"] = abs(res["uy_probe_rms_last_half"] - out["f64"]["uy_probe_rms_last_half"]) / \
                out["f64"]["uy_probe_rms_last_half"]
            # phase: lag of this storage's shedding cycle behind float64's at the
            # last step (cross-correlation of the probe traces); the rest: the L2
            # error against the float64 field at the best-aligned step within
            # `near` steps of that lag
            period = 1.0 / max(st * 0.1 / 40, 1e-9)
            lag = phase_lag(traces["f64"], uy, period, window=min(len(uy) // 3, int(4 * period)))
            res["phase_lag_steps_probe"] = lag
            near = 25
            first = max(2, steps + lag - near)
            m = Member(lx, ly, omega, bnd, steps=steps + lag + near + 1, f0=f, rho0=rho, u0=u)
            b64 = Batch([m], storage="f64").start()
            b64.run_graph(first - 1, chunk=1000)
            best = (np.inf, 0)
            for t in range(first, steps + lag + near + 1):
                ref_l = b64.read(0, want_f=False)[2]
                e = float(torch.linalg.norm(us[steps] - ref_l) / torch.linalg.norm(ref_l))
                best = min(best, (e, t - steps))
                b64.run(1)
            del b64
            res["phase_lag_steps"] = best[1]
            res["phase_lag_periods"] = best[1] / period
            res["velocity_l2_rel_err_at_lag"] = best[0]
        out[storage] = res
        del b
    return {"workload": "von Karman 420x180 channel, Re 100, %d steps, probe u_y at (300,90); Strouhal by a "
                        "sub-bin spectral peak (Hann window, 16x zero padding, Gaussian interpolation) of the "
                        "last half of the trace" % steps, "storages": out}


def bench_batch(P, steps=20000, n=256):
    """Batched sweep: 256 von Karman lattices (nx ~ U{200..1200}, ny = nx U(0.3,0.5)
    even, plate ny U(0.1,0.3), Re log-uniform [40, 250], inlet 0.1), f16 storage,
    autotuned tiles, graph-captured; against the same lattices solved one by one
    at float64 accuracy (fx64 storage, timed on a sample, extrapolated)."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member, autotune
    params = P.scenarios.batch_sweep_params(n)
    members = []
    for j, q in enumerate(params):
        f, rho, u, om, bnd = P.scenarios.von_karman_device(q["nx"], q["ny"], q["plate"], q["re"], seed=j)
        members.append(Member(q["nx"], q["ny"], om, bnd, steps=steps, f0=f, rho0=rho, u0=u))
    b = Batch(members, storage="f16")
    tune = autotune(b, steps=4, warmup=2)
    b.start()
    ms = timed_ms(lambda: b.run_graph(chunk=200))
    nodes = sum(m.nodes for m in members)
    agg = nodes * (steps - 1) / (ms / 1e3) / 1e6
    del b
    for m in members:
        m.pop, m.aux = [], []
    torch.cuda.empty_cache()
    # the same lattices one at a time, each on its own resident lattice, on a
    # sample: plain float64 (the drop-in's storage and FMA collision) and fx64
    rng = np.random.default_rng(1)
    sample = rng.choice(n, size=12, replace=False)
    seq = {}
    for storage in ("f64", "fx64"):
        t64, nodes64 = 0.0, 0
        for j in sample:
            m = members[j]
            lat = P.Lattice(m.nx, m.ny, m.omega, m.boundary, storage=storage).set_state(m.f0, m.rho0, m.u0)
            lat.step(3)
            k = 300
            t64 += timed_ms(lambda: lat.step_graph(k, chunk=100)) / 1e3
            nodes64 += m.nodes * k
            del lat
        rate = nodes64 / t64
        seq[storage] = {"sequential_mlups": rate / 1e6, "sequential_wall_s_extrapolated": nodes * steps / rate,
                        "speedup_of_batch": nodes * steps / rate / (ms / 1e3)}
    best = min(tune, key=lambda r: r["ms_per_step"])
    return {"workload": "%d von Karman lattices, %d steps each, %.1f M nodes, f16 storage" % (n, steps, nodes / 1e6),
            "aggregate_mlups": agg, "batch_wall_s": ms / 1e3, "autotuned": best,
            "hbm_frac": agg * 1e6 * 36 / 1e9 / peaks()[0],
            "fastest_candidates": sorted(tune, key=lambda r: r["ms_per_step"])[:8],
            "candidates": len(tune), "sequential": seq,
            "omega_range": [min(q["omega"] for q in params), max(q["omega"] for q in params)],
            "stability_risk_instances": sum(q["risky"] for q in params)}


def batch_step(P, steps=8):
    """The 256-lattice batch (f16, 4 nodes per thread, 128 threads, 8 runs per
    tile, one tile per block: the autotuner's pick) set up and advanced a few
    steps without the autotuner: the case the batch kernels' ncu captures run."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300.batch import Batch, Member
    params = P.scenarios.batch_sweep_params(256)
    members = []
    for j, q in enumerate(params):
        f, rho, u, om, bnd = P.scenarios.von_karman_device(q["nx"], q["ny"], q["plate"], q["re"], seed=j)
        members.append(Member(q["nx"], q["ny"], om, bnd, steps=2 * steps, f0=f, rho0=rho, u0=u))
    from lattice_boltzmann_parallel_solver_gb300.batch import ONE_TILE_PER_BLOCK
    b = Batch(members, storage="f16", npt=4, threads=128, rows=8, blocks=ONE_TILE_PER_BLOCK).start()
    ms = timed_ms(lambda: b.run(steps))
    torch.cuda.synchronize()
    return {"workload": "256 von Karman lattices, f16, npt 4, 128 threads, 8 runs per tile, one tile per block, "
                        "%d steps (no autotuning)" % steps, "nodes": b.nodes, "ms_per_step": ms / steps}


def serve_rate(P, storage, rate, n, seed=7):
    """One run of the serving loop: the first n requests of the seeded stream
    (the same requests for every storage and rate), arriving as a Poisson stream
    of the given mean rate."""
    import torch
    from lattice_boltzmann_parallel_solver_gb300.serving import ServingEngine, request_mix, summarize
    reqs = request_mix(n, rate=rate, seed=seed, lazy=True)
    eng = ServingEngine(storage=storage, hbm_budget=64 << 30, tick_steps=500)
    done = eng.serve(reqs, realtime=True)
    s = summarize(done)
    s.update({"offered_per_s": rate, "arrival_window_s": reqs[-1].arrival, "max_live": eng.stats["max_live"]})
    # latency of the second half of the stream: past the start-up transient
    lat = sorted(r.latency for r in done if r.rid >= n // 2)
    s["p99_second_half_s"] = float(np.percentile(lat, 99))
    return s, done


def bench_serve(P, n=60, rates=None):
    """Serving: seeded Poisson arrivals of Couette / Poiseuille / von Karman
    requests with 1k-50k steps, continuous batching under an HBM budget; the
    same n requests through f16 storage, fx64 and plain float64 (f64), each at
    offered loads below its capacity (per-rate rows); error of f16 results
    against their solo fx64 solve on a sample."""
    import torch
    rates = rates or {"f16": (8.0, 16.0), "fx64": (4.0,), "f64": (1.5,)}
    out = {}
    for storage, rs in rates.items():
        rows = []
        for rate in rs:
            s, done = serve_rate(P, storage, rate, n)
            rows.append(s)
            if storage == "f16" and rate == rs[0]:
                errs, budget = {}, 0.0
                for r in sorted(done, key=lambda r: r.nodes * r.steps):
                    if budget > 20.0 or len(errs) >= 9:
                        break
                    lat = P.Lattice(r.nx, r.ny, r.omega, r.boundary, storage="fx64").set_state(*r.initial_state())
                    t = timed_ms(lambda: lat.step(r.steps)) / 1e3
                    budget += t
                    u64 = lat.moments()[1]
                    errs.setdefault(r.kind, []).append(float(torch.linalg.norm(r.u - u64) / torch.linalg.norm(u64)))
                    del lat
                out["f16_velocity_l2_rel_err_vs_solo_fx64"] = {k: max(v) for k, v in errs.items()}
            del done
            torch.cuda.empty_cache()
        out[storage] = rows
    return {"workload": "the same %d seeded requests (Couette / Poiseuille / von Karman, 1k-50k steps) at "
                        "each offered Poisson rate, HBM budget 64 GB" % n, "results": out}


def bench_serve_sweep(P, window_s=60.0, rates=None):
    """Offered load swept up to and beyond each storage's capacity, every rate
    with at least ``window_s`` seconds of arrivals (n = rate x window requests,
    a prefix of one seeded stream): solves/s, p50 and p99 latency per rate."""
    rates = rates or {"f16": (8.0, 16.0, 24.0, 32.0, 40.0), "fx64": (3.0, 6.0, 9.0, 12.0),
                      "f64": (1.0, 2.0, 3.0)}
    out = {}
    for storage, rs in rates.items():
        out[storage] = []
        for rate in rs:
            s, done = serve_rate(P, storage, rate, max(60, int(rate * window_s)))
            out[storage].append(s)
            del done
    return {"workload": "offered-load sweep, >= %.0f s of arrivals per rate" % window_s, "results": out}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_node(storage):
    """Per-node DRAM bytes of the fused kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic_per_node.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        d = json.load(fh)
    return d.get(storage)


class Clocks:
    """Samples SM clock and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.reader.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baselines (the oracle, i.e. the reference's NumPy algorithm restated)
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    n, steps, warm = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import lbm_oracle as O
    rho, u = O.density_1_velocity_0((n, n))
    f = O.equilibrium(rho, u)
    bnd = O.cavity_boundary(n, n, 0.1, 1.0)
    f, rho, u = O.run(f, rho, u, 1.7, warm, bnd)
    t0 = time.perf_counter()
    O.run(f, rho, u, 1.7, steps, bnd)
    return n * n * steps, time.perf_counter() - t0


def cpu_baseline_single(n=1024, steps=40):
    nodes, dt = _cpu_worker((n, steps, 1))
    return {"value": nodes / dt / 1e6, "unit": "MLUPS", "cores": 1, "kind": "port",
            "sample": "NumPy oracle, one process, cavity %dx%d, %d steps after 1 warm-up step" % (n, n, steps)}


def reference_arm(args):
    """The reference's NumPy algorithm on all host cores: one worker process per
    core, each stepping its own cavity sample; aggregate MLUPS."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    # per-process sample side: the smallest cavity of the bandwidth benchmark
    # (1024^2) for short runs, smaller ones so that the whole --steps run stays
    # within a few minutes
    n = 1024 if args.steps + args.warmup <= 100 else (512 if args.steps <= 600 else (256 if args.steps <= 3000 else 128))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_cpu_worker, [(64, 1, 0)] * cores)
        t0 = time.perf_counter()
        res = pool.map(_cpu_worker, [(n, args.steps, args.warmup)] * cores)
        wall = time.perf_counter() - t0
    nodes = sum(r[0] for r in res)
    # each worker's own timed span excludes its warm-up; the slowest one bounds the job
    span = max(r[1] for r in res)
    value = nodes / span / 1e6
    sample = ("NumPy oracle (the reference's algorithm), %d concurrent processes, each a %dx%d cavity, "
              "%d steps after %d warm-up steps; wall %.1f s" % (cores, n, n, args.steps, args.warmup, wall))
    line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": span / max(args.steps, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "sliding-lid cavity, omega 1.7, lid u=(0.1,0), float64 (sampled at %dx%d)" % (n, n)},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# ranks (one replica per GPU under torchrun)
# ---------------------------------------------------------------------------
def rank_barrier(world, dist, sync=None):
    """All ranks meet (when there are several), then the device drains."""
    if world > 1:
        dist.barrier()
    if sync is not None:
        sync()


def slowest_over_ranks(seconds, world, dist, device="cuda"):
    """The maximum of the ranks' timed spans: the whole job took that long."""
    if world == 1:
        return seconds
    import torch
    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mlups(world, nodes, steps, seconds):
    """Lattice updates of all ranks (each runs its own replica) per second, in millions."""
    return world * nodes * steps / seconds / 1e6


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return

    import torch
    import torch.distributed as dist

    from lattice_boltzmann_parallel_solver_gb300 import _build
    _build.build()
    import lattice_boltzmann_parallel_solver_gb300 as P
    from lattice_boltzmann_parallel_solver_gb300 import _lib
    from lattice_boltzmann_parallel_solver_gb300.boundary_utils import cavity_boundary_conditions
    from lattice_boltzmann_parallel_solver_gb300.lattice_boltzmann_method import lattice_boltzmann_step

    torch.cuda.set_device(local)
    if args.workload != "cavity":
        fn = {"shear": bench_shear, "vk": bench_vk, "vk_seeds": bench_vk_seeds, "batch": bench_batch,
              "serve": bench_serve, "serve_sweep": bench_serve_sweep, "batch_step": batch_step}[args.workload]
        print(json.dumps(fn(P)), flush=True)
        return
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        rank_barrier(world, dist, torch.cuda.synchronize)

    def slowest(seconds):
        return slowest_over_ranks(seconds, world, dist)

    n = args.n
    bnd = cavity_boundary_conditions(n, n, 0.1, 1.0)
    w = torch.tensor([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=torch.float64, device="cuda")

    bc_inline = {"auto": None, "split": False, "inline": True}[args.bc]

    def make(storage, exact=False):
        lat = P.Lattice(n, n, 1.7, bnd, storage=storage, exact=exact, bc_inline=bc_inline)
        f0 = w.expand(n, n, 9).contiguous()  # equilibrium at rho = 1, u = 0
        lat.set_state(f0)
        del f0
        return lat

    def timed(lat, steps, warm):
        lat.step(warm)
        barrier()
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        before = _lib.launches()
        e0.record(stream)
        lat.step(steps)
        e1.record(stream)
        barrier()
        launches = _lib.launches() - before
        return e0.elapsed_time(e1) / 1e3, launches

    hbm, peak_kind = peaks()
    lat = make(args.storage, args.exact)
    with Clocks(local) as clk:
        secs, launches = timed(lat, args.steps, args.warmup)
    secs = slowest(secs)
    nodes = n * n
    per_launch = secs / args.steps
    algo = BYTES_PER_NODE[args.storage] * nodes
    achieved = algo / per_launch / 1e9
    tpn = profile_traffic_per_node(args.storage)
    value = job_mlups(world, nodes, args.steps, secs)
    del lat
    torch.cuda.empty_cache()

    extras = {}
    if not args.no_extras:
        # the other storages on the same workload; each one's velocity error
        # against a float64-accurate (fx64) run of the same steps
        kv = max(50, args.steps // 2)
        ref = make("fx64").step(5 + kv)
        u_ref = ref.moments()[1]
        del ref
        torch.cuda.empty_cache()
        variants = {}
        for st in ("fx64", "f64", "f32", "f16", "bf16"):
            if st == args.storage:
                continue
            v = make(st)
            s, _ = timed(v, kv, 5)
            s = slowest(s)
            u_v = v.moments()[1]
            err = float(torch.linalg.norm(u_v - u_ref) / torch.linalg.norm(u_ref))
            variants[st] = {"mlups": world * nodes * kv / s / 1e6,
                            "hbm_frac": BYTES_PER_NODE[st] * nodes / (s / kv) / 1e9 / hbm,
                            "velocity_l2_rel_err_vs_fx64": err, "steps": 5 + kv}
            del v, u_v
            torch.cuda.empty_cache()
        del u_ref
        extras["variants"] = variants

        # the other cavity sizes of the bandwidth bench
        sizes = {}
        for m in (1024, 4096):
            if m == n:
                continue
            bm = cavity_boundary_conditions(m, m, 0.1, 1.0)
            sizes[str(m)] = {}
            for st in ("fx64", "f64", "f32"):
                k = min(args.steps, 2000)
                lat_m = P.Lattice(m, m, 1.7, bm, storage=st).set_state(w.expand(m, m, 9).contiguous())
                s_m, _ = timed(lat_m, k, 5)
                s_m = slowest(s_m)
                sizes[str(m)][st] = {"mlups": world * m * m * k / s_m / 1e6, "steps": k,
                                     "hbm_frac": BYTES_PER_NODE[st] * m * m / (s_m / k) / 1e9 / hbm}
                del lat_m
            torch.cuda.empty_cache()
        extras["cavity_sizes"] = sizes

        # end to end: the reference-facing drop-in call with pinned host buffers
        f_h = torch.empty((n, n, 9), dtype=torch.float64).pin_memory()
        f_h.copy_(w.cpu().expand(n, n, 9))
        rho_h = torch.ones((n, n), dtype=torch.float64).pin_memory()
        u_h = torch.zeros((n, n, 2), dtype=torch.float64).pin_memory()
        e2e_steps = 10
        # two untimed calls: the results of consecutive calls are both alive, so
        # the pinned host allocator caches two sets of result buffers
        state = lattice_boltzmann_step(f_h, rho_h, u_h, 1.7, bnd)
        state = lattice_boltzmann_step(*state, 1.7, bnd)
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            # inputs come from pinned host memory, results land in pinned host memory
            state = lattice_boltzmann_step(*state, 1.7, bnd)
        barrier()
        e2e_secs = slowest(time.perf_counter() - t0)
        bytes_io = (f_h.numel() + rho_h.numel() + u_h.numel()) * 8
        extras["e2e"] = {"value": world * nodes * e2e_steps / e2e_secs / 1e6, "unit": "MLUPS",
                         "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                         "path": "lattice_boltzmann_step(f, rho, u, omega, boundary) on pinned host tensors, "
                                 "exact float64, %d steps (slab-pipelined copies, lbm_step_f64_host)" % e2e_steps}
        del f_h, rho_h, u_h, state
        if rank == 0 and world == 1:
            extras["cpu_baseline"] = cpu_baseline_single()
        if rank == 0:
            configs = {}
            for name in [c for c in args.configs.split(",") if c]:
                fn = {"shear": bench_shear, "vk": bench_vk, "batch": bench_batch, "serve": bench_serve}[name]
                try:
                    configs[name] = fn(P)
                except Exception as exc:  # a side configuration must not lose the headline line
                    configs[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}
                torch.cuda.empty_cache()
            extras["configs"] = configs

    if rank != 0:
        return
    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_launch * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[args.storage], "data": "synthetic",
        "config": {"workload": "sliding-lid cavity %dx%d, omega 1.7, lid u=(0.1,0), rho=1 u=0 start, %s storage%s"
                   % (n, n, args.storage, ", exact arithmetic" if args.exact else ""),
                   "nx": n, "ny": n, "l2": "state %.1f GB, larger than L2" % (2 * BYTES_PER_NODE[args.storage] / 2 * nodes / 1e9),
                   "parallelism": "replica per GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_kind,
                     "traffic": None if tpn is None else tpn * nodes,
                     "algorithmic_bytes_per_node": BYTES_PER_NODE[args.storage]},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

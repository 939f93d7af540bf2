"""Benchmark of the D2Q9 hot path on the sliding-lid cavity (8192^2, omega 1.7,
lid u = (0.1, 0), rho = 1, u = 0 at start): MLUPS of the resident float64
fused step, its HBM roofline fraction, the reduced-precision storages, the
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

BYTES_PER_NODE = {"f64": 144, "f32": 72, "f16": 36, "bf16": 36}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=8192, help="cavity side")
    p.add_argument("--storage", default="f64", choices=sorted(BYTES_PER_NODE))
    p.add_argument("--exact", action="store_true", help="NumPy-order float64 arithmetic")
    p.add_argument("--no-extras", action="store_true", help="skip variants, e2e and CPU baseline")
    return p.parse_args()


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


def cpu_baseline_single(n=1024, steps=3):
    nodes, dt = _cpu_worker((n, steps, 1))
    return {"value": nodes / dt / 1e6, "unit": "MLUPS", "cores": 1, "kind": "port",
            "sample": "NumPy oracle, one process, cavity %dx%d, %d steps after 1 warm-up step" % (n, n, steps)}


def reference_arm(args):
    """The reference's NumPy algorithm on all host cores: one worker process per
    core, each stepping its own cavity sample; aggregate MLUPS."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    n = 512 if args.steps <= 600 else 256
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
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def slowest(seconds):
        if world == 1:
            return seconds
        t = torch.tensor([seconds], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    n = args.n
    bnd = cavity_boundary_conditions(n, n, 0.1, 1.0)
    w = torch.tensor([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4, dtype=torch.float64, device="cuda")

    def make(storage, exact=False):
        lat = P.Lattice(n, n, 1.7, bnd, storage=storage, exact=exact)
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
    value = world * nodes * args.steps / secs / 1e6
    del lat
    torch.cuda.empty_cache()

    extras = {}
    if not args.no_extras:
        # reduced-precision storages on the same workload
        variants = {}
        for st in ("f32", "f16", "bf16"):
            if st == args.storage:
                continue
            v = make(st)
            s, _ = timed(v, max(50, args.steps // 2), 5)
            s = slowest(s)
            variants[st] = {"mlups": world * nodes * max(50, args.steps // 2) / s / 1e6,
                            "hbm_frac": BYTES_PER_NODE[st] * nodes / (s / max(50, args.steps // 2)) / 1e9 / hbm}
            del v
            torch.cuda.empty_cache()
        extras["variants"] = variants

        # end to end: the reference-facing drop-in call with pinned host buffers
        f_h = torch.empty((n, n, 9), dtype=torch.float64).pin_memory()
        f_h.copy_(w.cpu().expand(n, n, 9))
        rho_h = torch.ones((n, n), dtype=torch.float64).pin_memory()
        u_h = torch.zeros((n, n, 2), dtype=torch.float64).pin_memory()
        e2e_steps = 3
        state = lattice_boltzmann_step(f_h, rho_h, u_h, 1.7, bnd)
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            state = lattice_boltzmann_step(f_h, rho_h, u_h, 1.7, bnd)
            f_h.copy_(state[0])
            rho_h.copy_(state[1])
            u_h.copy_(state[2])
        barrier()
        e2e_secs = slowest(time.perf_counter() - t0)
        bytes_io = (f_h.numel() + rho_h.numel() + u_h.numel()) * 8
        extras["e2e"] = {"value": world * nodes * e2e_steps / e2e_secs / 1e6, "unit": "MLUPS",
                         "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                         "path": "lattice_boltzmann_step(f, rho, u, omega, boundary) on pinned host tensors, "
                                 "exact float64, %d steps" % e2e_steps}
        del f_h, rho_h, u_h, state
        if rank == 0 and world == 1:
            extras["cpu_baseline"] = cpu_baseline_single()

    if rank != 0:
        return
    line = {
        "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_launch * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.storage, "data": "synthetic",
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

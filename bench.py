"""Benchmark of the DFSPH step: particle-steps/s on the 1M-particle dam break.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dam1m|dam128k|puddle]

A step is one DFSPHSolver::step of the whole scene. The workload is the dam
break at scale (80 x 160 x 80 = 1,024,000 fluid particles, r = 0.0025 m, 766,098
wall particles, dt = 2.5e-4 s) in the reference's mode: 4 fixed density
iterations (eta = 0) and no divergence iterations, synthetic seeded inputs.
One JSON line is printed by rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam1m", choices=["dam1m", "dam128k", "puddle"])
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference CUDA kernels")
    return ap.parse_args()


def make_scene(name):
    from water_simulation_gb300 import scenes

    if name == "dam1m":
        return scenes.dam_break(scale=2, reference_mode=True)
    if name == "dam128k":
        return scenes.dam_break(scale=1, reference_mode=True)
    sc = scenes.puddle()
    sc.max_density_iters, sc.max_divergence_iters, sc.eta_density, sc.eta_divergence = 4, 0, 0.0, 0.0
    return sc


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def bench_ours(args, rank, world):
    import torch

    from water_simulation_gb300 import _build, _lib
    from water_simulation_gb300.solver import solver_for

    _build.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    sc = make_scene(args.workload)
    stream = torch.cuda.current_stream()
    s = solver_for(sc, stream=stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        s.step(sc.dt)
    torch.cuda.synchronize()
    l0 = s.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler() as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (256 MB > 129 MB L2)
            ev[k][0].record(stream)
            s.step(sc.dt)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    launches = s.kernel_launches() - l0
    res = {"ms_total": ms, "ms_per_step": ms / args.steps, "wall_s": wall, "launches": launches,
           "clocks": clk.summary(), "n": sc.n, "nb": sc.nb}
    s.close()
    return sc, res


def bench_ref_cuda(sc, steps):
    from oracle import oracle as O
    from oracle import reference as R

    if not R.available():
        return None
    from water_simulation_gb300 import _lib
    from water_simulation_gb300.solver import Solver

    probe = Solver(sc.config())
    inv = probe.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    probe.close()
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    ref = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary)
    ref.step(sc.dt, 1)
    ms = ref.time_steps(sc.dt, steps)
    ref.close()
    return {"value": sc.n * steps / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms / steps,
            "steps": steps}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "CPU baseline arm not wired yet"}))
        return
    sc, res = bench_ours(args, rank, world)
    line = {
        "metric": "particle-steps/s @1M dam break",
        "value": sc.n * args.steps / (res["ms_total"] * 1e-3),
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": res["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": sc.name, "particles": sc.n, "boundary_particles": sc.nb,
                   "density_iters": sc.max_density_iters, "divergence_iters": sc.max_divergence_iters,
                   "dt": sc.dt, "l2": "flushed between timed steps (256 MB write)"},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
    }
    if not args.no_ref_cuda:
        line["ref_cuda"] = bench_ref_cuda(sc, 3 if sc.n > 500000 else 10)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()

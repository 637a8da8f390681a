"""Benchmark of the DFSPH step: particle-steps/s on the 1M-particle dam break.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload dam1m|dam128k|dam128k_div|puddle|puddle_adaptive]

A step is one DFSPHSolver::step of the whole scene. The default workload is the
dam break at scale: an 80 x 160 x 80 column (1,024,000 fluid particles,
r = 0.0025 m) against the x = 0 wall of a 1.6 x 1.0 x 0.6 m tank sampled by
766,098 wall particles, dt = 2.5e-4 s, in the reference's step: 4 fixed density
iterations (eta = 0), no divergence iterations. Inputs are seeded synthetic
(water_simulation_gb300.scenes). Rank 0 prints one JSON line.

value      device time of K steps (CUDA events on the solver's stream), inputs
           resident in HBM; L2 flushed (256 MB write) before every timed step.
e2e        the same metric through the C ABI with host buffers: every step
           uploads x, v from pinned host memory (dfsph_set_fluid), steps, and
           reads x, v back (dfsph_get_state).
drop_in    DFSPHSolver::step on a ParticleStore, i.e. dfsph_step_store on the
           caller's device AoS arrays (gather in, one step, scatter x, v and
           the density / alpha / kappa / density_adv attributes back).
roofline   the dominant kernel class, timed live with CUDA events over as
           many steps again right after the timed ones (events inside the
           timed steps would slow them); algorithmic bytes per launch from the
           per-stage byte counts (x, v, rho, alpha, kappa read/written once,
           16 B per active wall particle), against the measured HBM copy
           bandwidth.
issue_roofline  the same launches against the SMs' instruction-issue rate:
           warp instructions per launch (ncu) over the launch time.
cpu_baseline  the FP32 C++/OpenMP restatement of the reference step (oracle/)
           on all host cores, on a bounded sample of the same workload.
batched    64 independent scenes in one context (one CUDA graph of two steps)
           against 64 single-scene contexts stepped one after another.
precision  FP32 and FP32 + Kahan density sums against the FP64 build of the
           same kernels after 50 steps of the workload.
frames     sim_cli's frame loop on the puddle block: substeps chosen on the
           device inside one graph launch per frame, against the host loop.
adjoint    the differentiable drop (32,768 particles, 200 steps, checkpoint
           every 20): backward time over forward time.
dam1m_adaptive  the same dam break with the reference's default solve
           (adaptive density solve at 0.1 %, at most 100 iterations), against
           the reference's kernels over the same steps.
puddle_adaptive  the settled puddle with the reference's adaptive density
           solve (its own CPU-runnable case), against the reference's kernels
           over the same steps.
lbvh       SpatialAccel::build on the workload's fluid positions: this
           build's dfsph_lbvh_build (+ boxes) and dfsph_lbvh_refit against the
           reference's own kernels under its restated orchestration, outputs
           compared bit for bit.
ref_cuda   the reference's own CUDA kernels (compiled from its sources for
           sm_103a, oracle/_ref) under its restated host orchestration, timed on
           the same GPU in the same run.
--impl reference  the reference arm: the reference step has no CPU code, so the
           arm times the FP32 restatement (kind "port") on all host cores.
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

FALLBACK_HBM_GBS = 6800.0

# DRAM bytes (read + write) per fluid particle of one launch of each kernel
# class, from `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum` on the
# 1M dam break (one launch per kernel). The traffic of a launch on another
# workload is scaled by its particle count.
NCU_TRAFFIC_PER_PARTICLE: dict = {
    "pressure_rate": 46.0, "pressure_apply": 40.2, "density_alpha": 25.02, "forces_xsph": 38.34,
    "grid_reorder": 52.3, "grid_scatter": 17.55, "grid_count": 20.96,
}


# Warp instructions per fluid particle of one launch of each neighbour pass,
# from `ncu --metrics smsp__inst_executed.sum` on the 1M dam break (the apply
# class averages three apply passes and the fused last apply + integrator).
NCU_WARP_INST_PER_PARTICLE: dict = {
    "pressure_rate": 43.14e6 / 1024000, "pressure_apply": (3 * 35.06e6 + 39.59e6) / 4 / 1024000,
    "density_alpha": 43.63e6 / 1024000, "forces_xsph": 45.12e6 / 1024000,
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dam1m",
                    choices=["dam1m", "dam128k", "dam128k_div", "puddle", "puddle_adaptive"])
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference CUDA kernels")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched comparison")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-drop timing")
    ap.add_argument("--no-precision", action="store_true", help="skip the FP32 vs FP64 field errors")
    ap.add_argument("--no-frames", action="store_true", help="skip the device-stepped frame timing")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default 128-thread neighbour passes")
    ap.add_argument("--no-lbvh", action="store_true", help="skip the LBVH build/refit timing")
    ap.add_argument("--no-puddle", action="store_true", help="skip the adaptive-puddle leg")
    ap.add_argument("--no-dam-adaptive", action="store_true", help="skip the adaptive 1M dam-break leg")
    ap.add_argument("--no-morton", action="store_true", help="skip the Morton slot-order comparison")
    ap.add_argument("--slot-order", default="cell_key", choices=["cell_key", "morton"],
                    help="slot order of the timed context (the reference's is cell_key)")
    return ap.parse_args()


def make_scene(name, sampler=None):
    """The named workload; `sampler` samples the walls (default: the library's
    sample_aabb_boundary; the reference arm passes the oracle's, so that it
    never loads the library)."""
    from water_simulation_gb300 import scenes

    if name == "dam1m":
        return scenes.dam_break(scale=2, reference_mode=True, sampler=sampler)
    if name == "dam128k":
        return scenes.dam_break(scale=1, reference_mode=True, sampler=sampler)
    if name == "dam128k_div":  # with 2 divergence-solver iterations (the reference has none)
        return scenes.dam_break(scale=1, reference_mode=False, sampler=sampler)
    if name == "dam1m_adaptive":  # the reference's default solve: adaptive density at 0.1 %, <= 100 iterations
        sc = scenes.dam_break(scale=2, reference_mode=True, sampler=sampler)
        sc.max_density_iters, sc.eta_density = 100, 1e-3
        sc.name = "dam_break_1024000_adaptive"
        return sc
    sc = scenes.puddle(sampler=sampler)
    if name == "puddle_adaptive":  # the settled puddle as the reference runs it: adaptive density solve
        sc.max_divergence_iters, sc.eta_divergence = 0, 0.0  # (0.01 %, <= 100 iterations), no divergence solver
        sc.name = "puddle_4913_adaptive"
        return sc
    sc.max_density_iters, sc.max_divergence_iters, sc.eta_density, sc.eta_divergence = 4, 0, 0.0, 0.0
    return sc


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def issue_roofline(kclass: str, n: int, avg_ms: float, clocks: dict, sms: int) -> dict | None:
    """The roof these neighbour passes actually meet: warp instructions
    issued per launch (ncu smsp__inst_executed.sum of one launch on the 1M dam
    break, per particle, scaled by the particle count) over the launch's mean
    duration, against the SMs' issue capacity at the sampled clock (4
    schedulers per SM, one warp instruction per scheduler per cycle)."""
    per = NCU_WARP_INST_PER_PARTICLE.get(kclass)
    mhz = (clocks or {}).get("sm_mhz")
    if not per or not mhz or not avg_ms:
        return None
    inst = per * n
    achieved = inst / (avg_ms * 1e-3)
    peak = 4.0 * sms * mhz * 1e6
    return {"kernel": kclass, "warp_instructions_per_launch": inst, "achieved": achieved, "peak": peak,
            "unit": "warp instructions/s", "frac": achieved / peak, "sm_mhz": mhz, "sms": sms,
            "source": "ncu smsp__inst_executed.sum of one launch on the 1M dam break, scaled by particle count"}


def algorithmic_bytes(kclass: str, n: int, nb_active: int, cells: int) -> float | None:
    """Bytes one launch must move at minimum (x 12, v 12, rho/alpha/kappa 4 B,
    each array once; 16 B (x, m_b) per wall particle near the fluid)."""
    per = {
        "density_alpha": 20 * n + 16 * nb_active,     # x -> rho, alpha
        "pressure_rate": 40 * n + 16 * nb_active,     # x, v, rho, alpha -> kappa, rho*
        "pressure_apply": 44 * n + 16 * nb_active,    # x, v, rho, kappa -> v
        "forces_xsph": 40 * n,                        # x, v, rho -> v
        "advect": 48 * n,                             # x, v -> x, v
        "grid_count": 20 * n,                         # x -> key, rank
        "grid_scatter": 12 * n,
        "grid_reorder": 56 * n,                       # x, v, id -> sorted x, v, id
        "grid_scan": 8 * (cells + 1),                 # counts -> cell_start
    }
    return per.get(kclass)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        for line in self._proc.stdout:
            if line.strip():
                self.samples.append([x.strip() for x in line.split(",")])
            if self._stop.is_set():
                break

    def __enter__(self):
        self._proc = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)  # let the sampler start before the timed region
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        self._t.join(timeout=10)

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(s[0]) for s in self.samples) if v is not None]
        smax = [v for v in (num(s[1]) for s in self.samples if len(s) > 1) if v is not None]
        reasons = sorted({self.NAMES[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup(args):
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()




def bench_ours(args, rank, world):
    """Replicas only: every rank steps its own copy of the scene on its own GPU."""
    import torch

    from water_simulation_gb300 import _build, _lib
    from water_simulation_gb300.solver import solver_for

    _build.build()
    local = int(os.environ.get("LOCAL_RANK", rank)) if world > 1 else 0
    torch.cuda.set_device(local)
    sc = make_scene(args.workload)
    stream = torch.cuda.current_stream()
    if args.slot_order == "morton":
        from water_simulation_gb300.solver import Solver

        cfg = sc.config()
        cfg.slot_order = _lib.ORDER_MORTON
        s = Solver(cfg, device=local, stream=stream.cuda_stream)
        s.set_boundary(sc.boundary)
        s.set_fluid(sc.fluid, sc.velocity)
    else:
        s = solver_for(sc, stream=stream.cuda_stream, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # launch shapes of the neighbour passes, measured on this workload (the
    # state is restored afterwards)
    tuned = s.autotune(sc.dt, 3) if not args.no_autotune else s.block_sizes()
    # the solves of a small scene run as one cooperative launch each, which a
    # profiled pass would split: one plain step tells (the library counts them)
    c0 = s.scalar(_lib.SCALAR_COOP_SOLVES)
    s.step(sc.dt)
    coop = s.scalar(_lib.SCALAR_COOP_SOLVES) > c0
    # warm-up, with every kernel class profiled to find the dominant one
    s.profile_enable((1 << _lib.KERNEL_CLASSES) - 1)
    for _ in range(args.warmup):
        flush.zero_()
        s.step(sc.dt)
    torch.cuda.synchronize()
    share = {}
    for k in range(_lib.KERNEL_CLASSES):
        share[_lib.KERNEL_NAMES[k]] = s.profile_read(k)
    dominant = max(share, key=lambda k: share[k][0])
    dom_id = _lib.KERNEL_NAMES.index(dominant)
    # the timed steps run unprofiled: events bracketing a pass would keep it
    # from overlapping its launch with the drain of the pass before it
    # (programmatic dependent launch)
    s.profile_enable(0)
    nb_active = s.active_boundary()
    l0 = s.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (256 MB > 129 MB L2)
            ev[k][0].record(stream)
            s.step(sc.dt)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier(world)
    launches = s.kernel_launches() - l0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    # the dominant pass's launch time: the same number of steps again, live,
    # with that pass bracketed by CUDA events on the solver's stream (a
    # cooperative solve would be split into its passes by profiling: its
    # launch time comes from the profiled warm-up)
    if coop:
        dom_ms, dom_launches = share[dominant]
    else:
        # every class bracketed, so every launch runs alone (with one class
        # bracketed, the pass after it, launched with programmatic stream
        # serialization, could start beside it and slow it)
        s.profile_enable((1 << _lib.KERNEL_CLASSES) - 1)
        for _ in range(args.steps):
            flush.zero_()
            s.step(sc.dt)
        torch.cuda.synchronize()
        dom_ms, dom_launches = s.profile_read(dom_id)
        for k in range(_lib.KERNEL_CLASSES):
            if k != dom_id:
                s.profile_read(k)  # forget the other classes' records
        s.profile_enable(0)
    from water_simulation_gb300 import replicas

    ms_max, work = replicas.aggregate(ms, float(sc.n) * args.steps, world)
    res = {"ms_total": ms_max, "work": work, "wall_s": wall, "launches": launches, "clocks": clk.summary(),
           "sms": torch.cuda.get_device_properties(local).multi_processor_count,
           "dominant": dominant, "dominant_ms": dom_ms, "dominant_launches": dom_launches,
           "dominant_timed_in": "warm-up steps (passes apart)" if coop else
                                "as many steps again after the timed ones, every pass bracketed by CUDA events "
                                "(the timed steps run unprofiled)",
           "nb_active": nb_active,
           "block_sizes": {k: tuned[k] for k in ("density_alpha", "pressure_rate", "pressure_apply", "forces_xsph")},
           "warmup_raw": share,
           "warmup_share": {k: round(v[0] / max(sum(x[0] for x in share.values()), 1e-9), 4)
                            for k, v in share.items() if v[1]}}
    if not args.no_e2e:
        res["e2e"] = bench_e2e(s, sc, max(3, min(args.steps, 20)))
        res["drop_in"] = bench_drop_in(s, sc, max(3, min(args.steps, 20)), ms_max / args.steps)
    s.close()
    return sc, res


def bench_drop_in(s, sc, steps, resident_ms):
    """The reference-facing C++ path: DFSPHSolver::step on the caller's
    ParticleStore is one dfsph_step_store call on its device AoS arrays
    (gather into the sorted state, one step, scatter positions, velocities
    and the density / alpha / kappa / density_adv attributes back). Timed
    with CUDA events on the solver's stream, inputs resident in HBM."""
    import ctypes

    import torch

    dev = torch.device("cuda")
    x = torch.tensor(sc.fluid, device=dev)
    v = torch.tensor(sc.velocity, device=dev)
    attrs = [torch.empty(sc.n, dtype=torch.float32, device=dev) for _ in range(4)]
    stream = torch.cuda.current_stream()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def one():
        s._check(s._lib.dfsph_step_store(s._ctx, ptr(x), ptr(v), sc.n, ctypes.c_float(sc.dt), *map(ptr, attrs)))

    for _ in range(3):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": sc.n / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms, "steps": steps,
            "over_resident_step": ms / resident_ms,
            "path": "DFSPHSolver::step -> dfsph_step_store on device AoS arrays (ParticleStore in place)"}


def bench_e2e(s, sc, steps):
    """Host buffers in, host buffers out, every step, through the C ABI:
    dfsph_set_fluid from page-locked x and v, one dfsph_step, dfsph_get_state
    back into the same arrays (the next step's input)."""
    import torch

    from water_simulation_gb300 import _lib

    x = torch.from_numpy(sc.fluid.copy()).pin_memory()
    v = torch.from_numpy(sc.velocity.copy()).pin_memory()
    lib = s._lib
    import ctypes

    nbytes = x.numel() * 4
    # one untimed round trip
    for k in range(2):
        s._check(lib.dfsph_set_fluid(s._ctx, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(v.data_ptr()), sc.n,
                                     _lib.MEM_HOST))
        s.step(sc.dt)
        s._check(lib.dfsph_get_state(s._ctx, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                     _lib.MEM_HOST))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        s._check(lib.dfsph_set_fluid(s._ctx, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(v.data_ptr()), sc.n,
                                     _lib.MEM_HOST))
        s.step(sc.dt)
        s._check(lib.dfsph_get_state(s._ctx, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                     _lib.MEM_HOST))
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    return {"value": sc.n * steps / sec, "unit": "particle-steps/s", "h2d_bytes_per_step": 2 * nbytes,
            "d2h_bytes_per_step": 2 * nbytes, "steps": steps}


def bench_batch(steps, n_scenes=64, warmup=3):
    """64 independent falling-block scenes (2,000-60,000 particles each): one
    batched context replaying a captured CUDA graph of two steps, against 64
    single-scene contexts stepped one after another with plain launches. Also
    the batched kernels' own time per step, and the fraction of the replayed
    step that is not kernel time (launch gaps)."""
    import torch

    from water_simulation_gb300 import scenes
    from water_simulation_gb300.solver import Solver, solver_for

    scs, eps = scenes.batched_blocks(n_scenes=n_scenes)
    n_total = sum(s.n for s in scs)
    stream = torch.cuda.current_stream()
    cfg = scs[0].config(capacity=n_total)
    cfg.n_scenes = n_scenes
    cfg.use_cuda_graph = 1
    b = Solver(cfg, stream=stream.cuda_stream)
    b.set_boundary(scs[0].boundary)
    b.set_fluid_batch([s.fluid for s in scs], [s.velocity for s in scs])
    b.set_scene_viscosity(eps)
    steps = steps + (steps % 2)  # whole graph replays
    b.step(scs[0].dt, warmup + 1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = b.kernel_launches()
    e0.record(stream)
    b.step(scs[0].dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_batch = e0.elapsed_time(e1)
    launches_batch = b.kernel_launches() - l0
    # the kernels' own time per step (every launch bracketed by CUDA events,
    # which replaces the graph with plain launches): what is left of the
    # replayed step is launch gaps, the most a single persistent launch of the
    # whole step could remove
    from water_simulation_gb300 import _lib

    b.profile_enable((1 << _lib.KERNEL_CLASSES) - 1)
    b.step(scs[0].dt, steps)
    torch.cuda.synchronize()
    kernel_ms = sum(b.profile_read(k)[0] for k in range(_lib.KERNEL_CLASSES))
    b.profile_enable(0)
    b.close()
    singles = [solver_for(s, stream=stream.cuda_stream) for s in scs]
    for s in singles:
        s.step(scs[0].dt, warmup)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        for s in singles:
            s.step(scs[0].dt)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1)
    for s in singles:
        s.close()
    return {"scenes": n_scenes, "particles": n_total, "steps": steps,
            "batched_particle_steps_per_s": n_total * steps / (ms_batch * 1e-3),
            "batched_scene_steps_per_s": n_scenes * steps / (ms_batch * 1e-3),
            "sequential_particle_steps_per_s": n_total * steps / (ms_seq * 1e-3),
            "speedup_vs_sequential": ms_seq / ms_batch, "batched_launches": launches_batch,
            "batched_ms_per_step": ms_batch / steps, "sequential_ms_per_step": ms_seq / steps,
            "batched_kernel_ms_per_step": kernel_ms / steps,
            "launch_gap_fraction": max(0.0, 1.0 - kernel_ms / ms_batch)}


def _frames_run(sc, label, n_frames):
    from water_simulation_gb300.solver import Solver

    out = {"workload": label, "frames": n_frames}
    final = {}
    for name, graph in (("device", True), ("host_loop", False)):
        cfg = sc.config()
        cfg.use_cuda_graph = 1 if graph else 0
        s = Solver(cfg)
        s.set_boundary(sc.boundary)
        s.set_fluid(sc.fluid, sc.velocity)
        s.step_frames(1)  # warm-up (and graph capture)
        s.synchronize()
        t0 = time.perf_counter()
        subs = s.step_frames(n_frames)
        s.synchronize()
        t1 = time.perf_counter()
        x = s.positions()
        final[name] = (list(subs), x, s.velocities())
        out[name] = {"ms_per_frame": 1e3 * (t1 - t0) / n_frames, "substeps": int(subs.sum()),
                     "ms_per_substep": 1e3 * (t1 - t0) / max(int(subs.sum()), 1),
                     "on_device": s.frames_on_device(), "min_y_m": float(x[:, 1].min())}
        s.close()
    out["speedup"] = out["host_loop"]["ms_per_frame"] / out["device"]["ms_per_frame"]
    a, b = final["device"], final["host_loop"]
    out["same_substeps"] = a[0] == b[0]
    out["same_state"] = bool(np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]))
    return out


def bench_frames(n_frames=24):
    """sim_cli's frame loop (24 fps) on the settled-puddle scene: every
    substep size chosen on the device, one graph launch per frame, against the
    reference's host loop (max |v| read back before every substep). Wall time
    of n_frames frames from rest. Both paths take e^{-d dt} from the same
    device function, so they take the same substeps and iterations and end in
    the same state (checked: same_substeps, same_state). Two settings: the
    settled puddle with the reference's adaptive solvers (4,913 particles;
    density eta 1e-4, divergence eta 1e-3, at most 100 iterations each; both
    solves run as device-resident loops, the host loop reads the error after
    every iteration), and, with short substeps, a 16^3 block falling with
    N(0, 0.5^2) m/s velocities and fixed iterations (4 density, no divergence)
    for 6 frames."""
    from water_simulation_gb300 import scenes

    out = _frames_run(scenes.puddle(), "puddle_4913, adaptive solvers, 24 fps", n_frames)
    block = scenes.falling_block(n_side=(16, 16, 16), velocity_sigma=0.5)
    out["fixed_iterations"] = _frames_run(block, "falling block 4,096, 4 fixed density iterations, 24 fps", 6)
    return out


def bench_precision(sc, checkpoints=(50, 500)):
    """Field error of the FP32 step (plain, with Kahan density sums, and with
    Kahan density sums and compensated position updates; all with FP64
    convergence reductions) against the FP64 build of the same kernels. Every build bins and centres the stencil with the same float
    arithmetic, so from identical inputs the builds visit identical neighbour
    sets and differ by rounding only ("one_step_from_same_input"). Along one
    trajectory (the checkpoints) the positions drift apart by rounding, and a
    particle near a cell face can then see a different candidate set in the
    two builds (the stencil is truncated at one cell of length l against a
    support of 2l, so such a pair enters one sum with a jump). The FP32 and
    FP64 runs are stepped in lockstep for the first checkpoint and compare
    their candidate-set signatures after every step: "flipped" particles saw
    a different set at some step, "near_flip" ones shared a cell
    neighbourhood (27 cells) with a flipped particle at the end."""
    import time as _time

    from water_simulation_gb300 import _lib
    from water_simulation_gb300.solver import Solver, solver_for

    def snap(s):
        return {"x": s.field(_lib.FIELD_POSITION).astype(np.float64),
                "v": s.field(_lib.FIELD_VELOCITY).astype(np.float64),
                "rho": s.field(_lib.FIELD_DENSITY).astype(np.float64)}

    def errors(f, ref, mask=None):
        vs = np.linalg.norm(ref["v"], axis=1).max()
        rel = np.abs(f["rho"] - ref["rho"]) / np.abs(ref["rho"])
        out = {
            "density_max_rel": float(rel.max()),
            "density_rel_p50": float(np.percentile(rel, 50)),
            "density_rel_p99": float(np.percentile(rel, 99)),
            "density_frac_over_1e-4": float(np.mean(rel > 1e-4)),
            "density_rms_rel": float(np.sqrt(np.mean(((f["rho"] - ref["rho"]) / ref["rho"]) ** 2))),
            "position_max_abs_m": float(np.abs(f["x"] - ref["x"]).max()),
            "velocity_max_abs_rel_to_max_speed": float(np.abs(f["v"] - ref["v"]).max() / max(vs, 1e-30)),
        }
        if mask is not None:
            out["density_max_rel_without_flips"] = float(rel[~mask].max()) if (~mask).any() else 0.0
        return out, rel

    ctxs = {name: solver_for(sc, precision=prec, diagnostics=name in ("fp64", "fp32"))
            for name, prec in (("fp64", _lib.PRECISION_FP64), ("fp32", _lib.PRECISION_FP32),
                               ("fp32_kahan", _lib.PRECISION_FP32_KAHAN),
                               ("fp32_compensated", _lib.PRECISION_FP32_COMPENSATED))}
    # lockstep to the first checkpoint, candidate-set signatures compared every step
    first = checkpoints[0]
    flipped = np.zeros(sc.n, bool)
    flips_per_step = []
    t0 = _time.perf_counter()
    for _ in range(first):
        for s in ctxs.values():
            s.step(sc.dt)
        d = ctxs["fp32"].field(_lib.FIELD_NBR_SIGNATURE) != ctxs["fp64"].field(_lib.FIELD_NBR_SIGNATURE)
        flips_per_step.append(int(d.sum()))
        flipped |= d
    lockstep_s = _time.perf_counter() - t0
    # particles within one cell (27-cell neighbourhood) of a flipped particle
    s64 = ctxs["fp64"]
    dims = s64.dims
    keys = s64.field(_lib.FIELD_CELL_KEY).astype(np.int64)
    total = int(dims[0]) * int(dims[1]) * int(dims[2])
    grid = np.zeros(total + 1, bool)
    grid[keys[flipped]] = True
    g3 = grid[:total].reshape(dims)
    for ax in range(3):
        a = g3.copy()
        sl = [slice(None)] * 3
        sl[ax] = slice(1, None)
        src = [slice(None)] * 3
        src[ax] = slice(None, -1)
        a[tuple(sl)] |= g3[tuple(src)]
        a[tuple(src)] |= g3[tuple(sl)]
        g3 = a
    grid[:total] = g3.ravel()
    near = grid[keys] | flipped
    f = {name: snap(s) for name, s in ctxs.items()}
    out = {}
    for name in ("fp32", "fp32_kahan", "fp32_compensated"):
        e, rel = errors(f[name], f["fp64"], flipped)
        e["density_max_rel_away_from_flips"] = float(rel[~near].max()) if (~near).any() else 0.0
        e["over_1e-4"] = int((rel > 1e-4).sum())
        e["over_1e-4_flipped"] = int((rel[flipped] > 1e-4).sum())
        e["over_1e-4_near_flip"] = int((rel[near] > 1e-4).sum())
        out[name] = e
    out["flipped_particles"] = int(flipped.sum())
    out["near_flip_particles"] = int(near.sum())
    out["flips_per_step_max"] = int(max(flips_per_step)) if flips_per_step else 0
    out["flips_first_step"] = next((k for k, c in enumerate(flips_per_step) if c), None)
    # one step of each build from the same (FP32) state: rounding only
    x32, v32 = f["fp32"]["x"].astype(np.float32), f["fp32"]["v"].astype(np.float32)
    probe = {}
    for name, prec in (("fp64", _lib.PRECISION_FP64), ("fp32", _lib.PRECISION_FP32)):
        s = solver_for(sc, precision=prec, diagnostics=True)
        s.set_fluid(x32, v32)
        s.step(sc.dt)
        probe[name] = snap(s)
        probe[name]["sig"] = s.field(_lib.FIELD_NBR_SIGNATURE)
        s.close()
    e1, _ = errors(probe["fp32"], probe["fp64"])
    e1["candidate_sets_differ"] = int((probe["fp32"]["sig"] != probe["fp64"]["sig"]).sum())
    out[f"one_step_from_same_input_at_step_{first}"] = e1
    # the rest of the trajectory, each form's steps timed with CUDA events
    import torch

    stream = torch.cuda.current_stream()
    ms_per_step = {}
    for c in checkpoints[1:]:
        for name, s in ctxs.items():
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            s.step(sc.dt, c - first)
            e1.record(stream)
            torch.cuda.synchronize()
            ms_per_step[name] = e0.elapsed_time(e1) / (c - first)
        g = {name: snap(s) for name, s in ctxs.items()}
        for name in ("fp32", "fp32_kahan", "fp32_compensated"):
            out[f"{name}_at_{c}_steps"] = errors(g[name], g["fp64"])[0]
    for s in ctxs.values():
        s.close()
    # the flow's own sensitivity: FP32 against FP32 from positions one ulp
    # away, at the last checkpoint
    import copy

    moved = copy.copy(sc)
    moved.fluid = np.nextafter(sc.fluid, np.float32(np.inf)).astype(np.float32)
    s = solver_for(moved, precision=_lib.PRECISION_FP32)
    s.step(sc.dt, checkpoints[-1])
    gm = snap(s)
    s.close()
    out[f"fp32_vs_fp32_1ulp_input_at_{checkpoints[-1]}_steps"] = errors(gm, g["fp32"])[0] if len(checkpoints) > 1 \
        else None
    out["steps"] = first
    out["checkpoints"] = list(checkpoints)
    if len(checkpoints) > 1:
        out["ms_per_step"] = {"steps": f"{first + 1}-{checkpoints[-1]}", **ms_per_step}
    out["lockstep_wall_s"] = lockstep_s
    out["reference"] = "FP64 build of the same kernels (float cell arithmetic, as the FP32 build)"
    return out


def bench_adjoint(graph: bool):
    """Differentiable drop: 32,768 particles (32^3 block, r = 0.01 m), 200 steps
    at dt = 1e-3 s, fixed 2 divergence + 4 density iterations, checkpoint every
    20 steps, loss = mean |x_T - (x_0 + (0.1, 0, 0))|^2. forward =
    dfsph_adjoint_forward (the 200 steps + 11 checkpoints), backward =
    dfsph_adjoint_backward (each 20-step segment replayed once with its
    per-step records, then the reverse kernels). Device time on the solver's
    stream; the loss gradient is formed on the device between the two."""
    import torch

    from water_simulation_gb300 import scenes
    from water_simulation_gb300.solver import Solver

    sc = scenes.adjoint_drop()
    every = sc.extra["checkpoint_every"]
    stream = torch.cuda.current_stream()
    cfg = sc.config()
    cfg.use_cuda_graph = 1 if graph else 0
    s = Solver(cfg, stream=stream.cuda_stream)
    s.set_boundary(sc.boundary)
    dev = torch.device("cuda")
    x0 = torch.tensor(sc.fluid, device=dev)
    v0 = torch.tensor(sc.velocity, device=dev)
    tgt = x0 + torch.tensor(sc.extra["target_shift"], dtype=torch.float32, device=dev)
    xT, vT = torch.empty_like(x0), torch.empty_like(v0)
    gx0, gv0 = torch.empty_like(x0), torch.empty_like(v0)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    res = None
    for rep in range(2):  # the first pass allocates the checkpoints and records
        s.adjoint_set_state_device(x0.data_ptr(), v0.data_ptr(), sc.n)
        torch.cuda.synchronize()
        l0 = s.kernel_launches()
        ev[0].record(stream)
        s.adjoint_forward(sc.dt, sc.steps, every)
        ev[1].record(stream)
        l1 = s.kernel_launches()
        s.adjoint_state_device(xT.data_ptr(), vT.data_ptr())
        xbar = (2.0 / sc.n) * (xT - tgt)
        loss = ((xT - tgt) ** 2).sum(dim=1).mean()
        ev[2].record(stream)
        ge = s.adjoint_backward_device(xbar.data_ptr(), None, gx0.data_ptr(), gv0.data_ptr())
        ev[3].record(stream)
        torch.cuda.synchronize()
        l2 = s.kernel_launches()
        fwd, bwd = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
        res = {"workload": sc.name, "particles": sc.n, "steps": sc.steps, "checkpoint_every": every,
               "cuda_graph_forward": bool(graph), "forward_ms": fwd, "backward_ms": bwd,
               "backward_over_forward": bwd / fwd, "forward_launches": l1 - l0,
               "backward_launches": l2 - l1, "loss": float(loss), "grad_xsph": ge,
               "grad_v0_norm": float(gv0.norm()), "finite": bool(torch.isfinite(gv0).all())}
    s.close()
    return res


def cpu_sample(sc, seconds=10.0, max_steps=2000, threads=0):
    """The FP32 restatement of the reference step on the host cores, on a
    bounded sample: whole steps from the workload's start (after one untimed
    step) until `seconds` of CPU time have passed."""
    from oracle import oracle as O

    c = O.config_from(sc.config())
    L = O.load()
    if threads:
        L.oracle_set_threads(threads)
    cores = L.oracle_max_threads()
    o = O.Oracle(c, sc.fluid, sc.velocity, sc.boundary, precision=32)
    o.step(sc.dt, 1)  # warm the arrays
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < seconds:
        o.step(sc.dt, 1)
        steps += 1
    sec = time.perf_counter() - t0
    o.close()
    return {"value": sc.n * steps / sec, "unit": "particle-steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full steps of the {sc.n}-particle workload after 1 untimed step "
                      f"({sec:.1f} s on {cores} threads)",
            "ms_per_step": 1e3 * sec / steps}


def bench_dam_adaptive(steps=10, warmup=5):
    """The 1M dam break with the reference's default solve (DFSPHSolver::Config:
    adaptive density solve at 0.1 %, at most 100 iterations, no divergence
    solver): steps warmup+1 .. warmup+steps with CUDA events (the context's
    default plain launches: each solve stops on its own device-side decision,
    the host reads it back after every iteration as the reference does), and
    the reference's own kernels over the same steps."""
    import torch

    from water_simulation_gb300.solver import solver_for

    sc = make_scene("dam1m_adaptive")
    stream = torch.cuda.current_stream()
    s = solver_for(sc, stream=stream.cuda_stream)
    for _ in range(warmup):
        s.step(sc.dt)
    torch.cuda.synchronize()
    ms, iters = 0.0, 0
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(sc.dt)
        e1.record(stream)
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        iters += s.last_density_iters()
    s.close()
    res = {"workload": sc.name, "particles": sc.n, "steps": f"{warmup + 1}-{warmup + steps}",
           "ms_per_step": ms / steps, "density_iters_per_step": iters / steps,
           "ms_per_iteration": ms / max(iters, 1), "particle_steps_per_s": sc.n * steps / (ms * 1e-3)}
    # the same steps with use_cuda_graph: pairs of steps replay one graph whose
    # solves loop on the device (WHILE nodes), with no host read-back
    from water_simulation_gb300.solver import Solver

    cfg = sc.config()
    cfg.use_cuda_graph = 1
    g = Solver(cfg, stream=stream.cuda_stream)
    g.set_boundary(sc.boundary)
    g.set_fluid(sc.fluid, sc.velocity)
    g.step(sc.dt, warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.step(sc.dt, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    res["graph_ms_per_step"] = e0.elapsed_time(e1) / steps
    g.close()
    ref = bench_ref_cuda(sc, steps, warmup)
    res["ref_cuda"] = ref
    if "ms_per_step" in ref:
        res["speedup_vs_ref_cuda"] = ref["ms_per_step"] / (ms / steps)
    return res


def bench_puddle_adaptive(steps=50, warmup=5):
    """The settled puddle as the reference runs it (adaptive density solve at
    0.01 %, at most 100 iterations, no divergence solver): steps
    warmup+1 .. warmup+steps with CUDA events, and the reference's own kernels
    over the same steps."""
    import torch

    from water_simulation_gb300.solver import solver_for

    sc = make_scene("puddle_adaptive")
    stream = torch.cuda.current_stream()
    s = solver_for(sc, stream=stream.cuda_stream)
    for _ in range(warmup):
        s.step(sc.dt)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        s.step(sc.dt)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    s.close()
    res = {"workload": sc.name, "particles": sc.n, "steps": f"{warmup + 1}-{warmup + steps}", "ms_per_step": ms,
           "particle_steps_per_s": sc.n / (ms * 1e-3)}
    ref = bench_ref_cuda(sc, steps, warmup)
    res["ref_cuda"] = ref
    if "ms_per_step" in ref:
        res["speedup_vs_ref_cuda"] = ref["ms_per_step"] / ms
    return res


def bench_lbvh(sc, reps=20, warmup=3):
    """dfsph_lbvh_build / dfsph_lbvh_refit on the fluid positions of the
    workload (scene box = the domain), CUDA events over `reps` launches after
    `warmup`; the reference's SpatialAccel::build on the same input when its
    kernels are present, with codes, permutation, children, parents and leaf
    boxes compared."""
    import ctypes

    import torch

    from water_simulation_gb300 import _lib

    lib = _lib.load()
    n = sc.n
    dev = "cuda"
    x = torch.tensor(sc.fluid, device=dev)
    m = max(n - 1, 1)
    codes = torch.empty(n, dtype=torch.int32, device=dev)
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    left = torch.empty(m, dtype=torch.int32, device=dev)
    right = torch.empty(m, dtype=torch.int32, device=dev)
    parent = torch.empty(2 * n - 1, dtype=torch.int32, device=dev)
    boxes = torch.empty((2 * n - 1, 6), dtype=torch.float32, device=dev)
    scratch = torch.empty(m, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    st = ctypes.c_void_p(stream.cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    smin, smax = _lib.fvec3(sc.domain_min), _lib.fvec3(sc.domain_max)

    def build():
        assert lib.dfsph_lbvh_build(P(x), n, smin, smax, ctypes.c_float(0.0), P(codes), P(idx), P(left), P(right),
                                    P(parent), P(boxes), P(scratch), st) == 0

    def refit():
        assert lib.dfsph_lbvh_refit(P(x), n, ctypes.c_float(0.0), P(idx), P(left), P(right), P(parent), P(boxes),
                                    P(scratch), st) == 0

    def timed(f):
        for _ in range(warmup):
            f()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            f()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def sort():
        assert lib.dfsph_morton_sort(P(x), n, smin, smax, P(codes), P(idx), st) == 0

    sort_ms = timed(sort)
    build_ms = timed(build)
    refit_ms = timed(refit)
    build()
    torch.cuda.synchronize()
    res = {"workload": f"{sc.name} fluid positions", "particles": n, "morton_sort_ms": sort_ms,
           "build_ms": build_ms, "refit_ms": refit_ms,
           "build_particles_per_s": n / (build_ms * 1e-3), "note": "build includes the internal boxes, which the "
           "reference leaves unbuilt; refit = all boxes on the same topology"}
    from oracle import reference as R

    if not R.available():
        res["reference"] = {"unavailable": "reference kernels (oracle/_ref fatbins) not present"}
        return res
    (rc, ri, rl, rr, rp, rb), ref_ms = R.lbvh_build(sc.fluid, sc.domain_min, sc.domain_max, reps=reps)
    u = lambda t: t.cpu().numpy().view(np.uint32)  # noqa: E731
    same = (np.array_equal(u(codes), rc) and np.array_equal(u(idx), ri) and np.array_equal(u(left), rl) and
            np.array_equal(u(right), rr) and np.array_equal(u(parent)[1:], rp[1:]) and
            np.array_equal(boxes.cpu().numpy()[n - 1:], rb))
    # the reference's build stops at the leaf boxes: the like-for-like part of
    # dfsph_lbvh_build is the build without its box pass
    topo_ms = max(build_ms - refit_ms, 1e-9)
    res["topology_ms"] = topo_ms
    res["reference"] = {"build_ms": ref_ms, "speedup": ref_ms / build_ms, "speedup_topology": ref_ms / topo_ms,
                        "bit_exact": bool(same),
                        "kind": "reference kernels from its sources, sm_103a, same GPU (stream-ordered allocations "
                                "and CUB radix sort as SpatialAccel::build)"}
    return res


def bench_morton(sc, steps=20, warmup=3):
    """The step in Morton slot order (cells ranked by the Morton code of their
    coordinates, SpatialAccel's key) against the reference's x-major order, on
    the same input: ms per step (CUDA events, L2 flushed before every step)
    and the final state compared bit for bit (both orders give every particle
    the same candidates in the same sequence)."""
    import torch

    from water_simulation_gb300 import _lib
    from water_simulation_gb300.solver import Solver

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    out, final = {}, {}
    for name, order in (("cell_key", _lib.ORDER_CELL_KEY), ("morton", _lib.ORDER_MORTON)):
        cfg = sc.config()
        cfg.slot_order = order
        t0 = time.perf_counter()
        s = Solver(cfg, stream=stream.cuda_stream)
        setup_s = time.perf_counter() - t0
        s.set_boundary(sc.boundary)
        s.set_fluid(sc.fluid, sc.velocity)
        for _ in range(warmup):
            flush.zero_()
            s.step(sc.dt)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            s.step(sc.dt)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        final[name] = (s.positions(), s.velocities())
        out[name] = {"ms_per_step": ms, "particle_steps_per_s": sc.n / (ms * 1e-3), "context_setup_s": setup_s}
        s.close()
    out["morton_over_cell_key_time"] = out["morton"]["ms_per_step"] / out["cell_key"]["ms_per_step"]
    out["same_state"] = bool(np.array_equal(final["cell_key"][0], final["morton"][0]) and
                             np.array_equal(final["cell_key"][1], final["morton"][1]))
    out["steps"] = steps
    return out


def bench_ref_cuda(sc, steps, warmup=1):
    from oracle import oracle as O
    from oracle import reference as R

    if not R.available():
        return {"unavailable": "reference kernels (oracle/_ref fatbins) not present"}
    from water_simulation_gb300 import _lib
    from water_simulation_gb300.solver import Solver

    probe = Solver(sc.config())
    inv = probe.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    probe.close()
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    ref = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary)
    ref.step(sc.dt, max(warmup, 1))  # the same steps as the timed ones above (adaptive solves vary)
    ms = ref.time_steps(sc.dt, steps)
    ref.close()
    return {"value": sc.n * steps / (ms * 1e-3), "unit": "particle-steps/s", "ms_per_step": ms / steps,
            "steps": steps, "kind": "reference kernels from its sources, sm_103a, same GPU"}


def workload_config(sc, world):
    """The `config` of both arms' JSON lines (identical for the same workload)."""
    cells = 1
    for a in range(3):
        ext = np.float32(np.float32(sc.domain_max[a]) - np.float32(sc.domain_min[a]))
        cells *= int(np.ceil(ext / np.float32(2 * np.float32(sc.radius)))) + 2
    # state and grid bytes a step touches: ~96 B per fluid particle (positions,
    # velocities, scalars, indices, both buffers), 16 B per wall particle,
    # 13 B per cell (counts, starts, wall starts, wall mask)
    touched = 96 * sc.n + 16 * sc.nb + 13 * cells
    l2 = ("every step touches more than the 129 MB GPU L2 holds; the GPU arm also writes 256 MB before "
          "every timed step" if touched > 129e6 else
          "the GPU arm writes 256 MB (more than the 129 MB L2) before every timed step")
    return {"workload": sc.name, "particles": sc.n, "boundary_particles": sc.nb,
            "density_iters": sc.max_density_iters, "divergence_iters": sc.max_divergence_iters, "dt": sc.dt,
            "parallelism": f"replicas x{world}", "l2": l2}


def oracle_config(sc):
    """The oracle's configuration of a scene, built without the library (the
    values Scene.config() gives the library's dfsph_config). The stencil is
    centred with the IEEE reciprocal of the cell length, which changes no
    timing."""
    from oracle import oracle as O

    c = O.OracleConfig()
    c.rest_density = 1000.0
    c.particle_radius = sc.radius
    c.smoothing_length = np.float32(2.0 * np.float32(sc.radius))
    c.viscosity = sc.viscosity
    c.damping = sc.damping
    c.surface_tension = 0.0
    c.gravity[0], c.gravity[1], c.gravity[2] = 0.0, -9.81, 0.0
    c.max_density_iters = sc.max_density_iters
    c.max_divergence_iters = sc.max_divergence_iters
    c.eta_density = sc.eta_density
    c.eta_divergence = sc.eta_divergence
    for a in range(3):
        c.domain_min[a] = sc.domain_min[a]
        c.domain_max[a] = sc.domain_max[a]
    c.stencil_inv_cell = 0.0
    return c


def reference_arm(args, rank, world):
    """The reference arm: the reference step has no CPU implementation, so the
    arm times the FP32 restatement (oracle/) on all host cores, rank 0 only."""
    if rank != 0:
        return None
    from oracle import oracle as O

    sc = make_scene(args.workload, sampler=O.sample_aabb_boundary)
    c = oracle_config(sc)
    L = O.load()
    cores = L.oracle_max_threads()
    o = O.Oracle(c, sc.fluid, sc.velocity, sc.boundary, precision=32)
    budget_s = 150.0
    warm = 0
    tw = time.perf_counter()
    for _ in range(args.warmup):  # bounded like the timed steps
        o.step(sc.dt, 1)
        warm += 1
        if time.perf_counter() - tw > 30.0:
            break
    t0 = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        o.step(sc.dt, 1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    sec = time.perf_counter() - t0
    val = sc.n * done / sec
    return {
        "impl": "reference",
        "metric": "particle-steps/s @1M dam break" if args.workload == "dam1m" else f"particle-steps/s @{sc.name}",
        "value": val, "unit": "particle-steps/s",
        "n_gpus": world, "steps": done, "warmup": warm, "ms_per_step": 1e3 * sec / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(sc, world),
        "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{done} full steps of the {sc.n}-particle workload (bounded to {budget_s:.0f} s)"},
        "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, world = dist_setup(args)
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    sc, res = bench_ours(args, rank, world)
    hbm, hbm_src = peaks()
    cells = 1
    for d in (int(np.ceil(np.float32(np.float32(sc.domain_max[a]) - np.float32(sc.domain_min[a])) /
                          np.float32(2 * np.float32(sc.radius)))) + 2 for a in range(3)):
        cells *= d
    dom = res["dominant"]
    alg = algorithmic_bytes(dom, sc.n, res["nb_active"], cells)
    avg_ms = res["dominant_ms"] / max(res["dominant_launches"], 1)
    achieved = alg / (avg_ms * 1e-3) / 1e9 if alg else None
    traffic = NCU_TRAFFIC_PER_PARTICLE.get(dom)
    line = {
        "metric": "particle-steps/s @1M dam break" if args.workload == "dam1m" else f"particle-steps/s @{sc.name}",
        "value": res["work"] / (res["ms_total"] * 1e-3),
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": res["ms_total"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded lattice + SplitMix64 jitter, water_simulation_gb300/scenes.py)",
        "config": workload_config(sc, world),
        "run": {"threads_per_block": res["block_sizes"], "slot_order": args.slot_order},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)" if hbm_src == "measured" else "fallback",
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_ms,
                     "traffic": (traffic * sc.n) if traffic else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the 1M "
                                       "dam break, scaled by particle count",
                     "active_boundary_particles": res["nb_active"], "timed_in": res["dominant_timed_in"]},
        "issue_roofline": issue_roofline(dom, sc.n, avg_ms, res["clocks"], res["sms"]),
        "kernel_share_warmup": res["warmup_share"],
    }
    # every kernel class against the same peak (warm-up steps, per-launch
    # events; the scan class is three launches per step, the apply class
    # includes the fused last apply + integrator counted at the apply's bytes)
    kr = {}
    for k, (ms, cnt) in res["warmup_raw"].items():
        alg = algorithmic_bytes(k, sc.n, res["nb_active"], cells)
        if not alg or not cnt or ms <= 0:
            continue
        units = cnt / 3.0 if k == "grid_scan" else cnt
        gbs = alg * units / (ms * 1e-3) / 1e9
        kr[k] = {"GB/s": round(gbs, 1), "frac": round(gbs / hbm, 4)}
        # the neighbour passes against the SMs' instruction issue rate too
        ir = issue_roofline(k, sc.n, ms / cnt, res["clocks"], res["sms"])
        if ir:
            kr[k]["issue_frac"] = round(ir["frac"], 4)
    line["kernel_roofline_warmup"] = kr
    # the whole step against the same peak: compulsory bytes of one step
    # N (192 + 84 I) + 4 (C + 1) + 16 N_b,active (1 + 2 I), I = solver
    # iterations per step (x, v, rho, alpha, kappa and the grid arrays moved
    # once per pass that needs them)
    fixed = (sc.max_density_iters == 0 or sc.eta_density == 0) and (sc.max_divergence_iters == 0 or
                                                                    sc.eta_divergence == 0)
    if fixed:  # adaptive solves run a data-dependent number of iterations
        iters = sc.max_density_iters + sc.max_divergence_iters
        b_step = sc.n * (192 + 84 * iters) + 4 * (cells + 1) + 16 * res["nb_active"] * (1 + 2 * iters)
        step_gbs = b_step * args.steps * world / (res["ms_total"] * 1e-3) / 1e9
        line["step_roofline"] = {"bytes_per_step": b_step, "iterations_per_step": iters, "achieved": step_gbs,
                                 "peak": hbm, "unit": "GB/s", "frac": step_gbs / hbm}
    if "e2e" in res:
        line["e2e"] = res["e2e"]
    if "drop_in" in res:
        line["drop_in"] = res["drop_in"]
    if rank == 0 and not args.no_cpu:
        try:
            line["cpu_baseline"] = cpu_sample(sc)
        except Exception as e:  # the baseline is a report, not the product
            line["cpu_baseline"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_batch:
        try:
            line["batched"] = bench_batch(20)
        except Exception as e:
            line["batched"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_frames:
        try:
            line["frames"] = bench_frames()
        except Exception as e:
            line["frames"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_precision:
        try:
            line["precision"] = bench_precision(sc)
        except Exception as e:
            line["precision"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_adjoint:
        try:
            plain, graphed = bench_adjoint(False), bench_adjoint(True)
            line["adjoint"] = {"plain_forward": plain, "graph_forward": graphed,
                               "backward_over_forward": max(plain["backward_over_forward"],
                                                            graphed["backward_over_forward"])}
        except Exception as e:
            line["adjoint"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_puddle:
        try:
            line["puddle_adaptive"] = bench_puddle_adaptive()
        except Exception as e:
            line["puddle_adaptive"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_dam_adaptive and args.workload == "dam1m":
        try:
            line["dam1m_adaptive"] = bench_dam_adaptive()
        except Exception as e:
            line["dam1m_adaptive"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_lbvh:
        try:
            line["lbvh"] = bench_lbvh(sc)
        except Exception as e:
            line["lbvh"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_morton and args.slot_order == "cell_key":
        try:
            line["morton_order"] = bench_morton(sc)
        except Exception as e:
            line["morton_order"] = {"unavailable": str(e)[:200]}
    if rank == 0 and not args.no_ref_cuda:
        try:
            big = sc.n > 500000  # the reference's 1M step takes ~0.24 s: a bounded sample
            line["ref_cuda"] = bench_ref_cuda(sc, 3 if big else args.steps, 1 if big else args.warmup)
        except Exception as e:
            line["ref_cuda"] = {"unavailable": str(e)[:200]}
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

"""DFSPH_PRECISION_FP32_COMPENSATED: FP32 state whose position updates carry
their rounding error from step to step, checked against the FP64 build of
the same kernels; and the places where that mode's per-particle carries must
restart or stay out (new state, the autotuner's trials, the adjoint)."""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for

pytestmark = pytest.mark.gpu


def _density_rel(a, b):
    ra, rb = a.field(_lib.FIELD_DENSITY), b.field(_lib.FIELD_DENSITY)
    return float(np.max(np.abs(ra - rb) / np.abs(rb)))


def test_compensated_positions_track_the_fp64_build_over_50_steps():
    # the 128,000-particle dam break, the reference's step (4 density iterations)
    sc = scenes.dam_break(scale=1, reference_mode=True)
    ref = solver_for(sc, precision=_lib.PRECISION_FP64)
    plain = solver_for(sc, precision=_lib.PRECISION_FP32)
    comp = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    for s in (ref, plain, comp):
        s.step(sc.dt, 50)
    e_plain, e_comp = _density_rel(plain, ref), _density_rel(comp, ref)
    x_plain = np.abs(plain.positions() - ref.positions()).max()
    x_comp = np.abs(comp.positions() - ref.positions()).max()
    # the CPU oracle builds of both forms give 3.6e-5 / 6.1e-7 m (plain) and
    # 5.4e-6 / 6.7e-8 m (compensated) on this workload
    assert e_comp < 1e-4
    assert e_comp < 0.5 * e_plain
    assert x_comp < 0.5 * x_plain


def test_compensated_state_restarts_with_new_input():
    # the same input set twice gives the same trajectory: the carries of the
    # first run do not leak into the second
    sc = scenes.falling_block((12, 12, 12), seed=21, velocity_sigma=0.2)
    s = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    s.step(sc.dt, 30)
    first = s.positions().copy()
    s.set_fluid(sc.fluid, sc.velocity)
    s.step(sc.dt, 30)
    assert np.array_equal(s.positions(), first)


def test_compensated_results_do_not_depend_on_autotuning():
    sc = scenes.falling_block((16, 16, 16), seed=22, velocity_sigma=0.2)
    a = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    b = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    a.step(sc.dt, 5)
    b.step(sc.dt, 5)
    b.autotune(sc.dt, steps=2)  # trial steps from a snapshot, state restored
    a.step(sc.dt, 20)
    b.step(sc.dt, 20)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())


def test_adjoint_refuses_a_compensated_context():
    sc = scenes.falling_block((8, 8, 8), seed=23)
    s = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    with pytest.raises(_lib.DfsphError):
        s.adjoint_forward(sc.dt, 4, 2)


def test_compensated_graphs_and_device_frames_match_plain_steps():
    # the captured step and the graph-resident frame loop pass the carries
    # buffer as the plain launches do
    from water_simulation_gb300.solver import Solver

    sc = scenes.falling_block((12, 12, 12), seed=24, velocity_sigma=0.2)

    def make(graph):
        cfg = sc.config(precision=_lib.PRECISION_FP32_COMPENSATED)
        cfg.use_cuda_graph = 1 if graph else 0
        s = Solver(cfg)
        s.set_boundary(sc.boundary)
        s.set_fluid(sc.fluid, sc.velocity)
        return s

    g, p = make(True), make(False)
    g.step(sc.dt, 9)  # one counting step, then four two-step graph replays
    p.step(sc.dt, 9)
    assert np.array_equal(g.positions(), p.positions())
    assert np.array_equal(g.velocities(), p.velocities())
    # frames: substeps chosen on the device (graph) and by the host loop
    gs = g.step_frames(2)
    ps = p.step_frames(2)
    assert g.frames_on_device() and not p.frames_on_device()
    assert np.array_equal(gs, ps)
    assert np.array_equal(g.positions(), p.positions())

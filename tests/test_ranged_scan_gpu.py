"""The fluid grid build scans only the counted key range (plus the stencil
margin) and leaves the rest of cell_start stale; every export completes it.
Structure fields must still equal the oracle's bit for bit: for a small block
in a large box (most tiles skipped), across several steps, and when a particle
outside the grid forces the full range."""
import numpy as np
import pytest

from oracle import oracle as O
from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for
from test_parity_gpu import assert_structure_equal, oracle_for

pytestmark = pytest.mark.gpu


def test_small_block_in_a_large_box_keeps_exact_structure():
    # a 6^3 block in the unit box: its keys span a few percent of the cells
    sc = scenes.falling_block((6, 6, 6), seed=31, velocity_sigma=0.3)
    gpu = solver_for(sc, diagnostics=True)
    ora = oracle_for(sc, gpu)
    for k in range(4):
        gpu.step(sc.dt)
        ora.step(sc.dt)
        assert_structure_equal(gpu, ora, f"step {k}")
    # the active-wall count reads cell_start beyond the fluid's stencils
    assert gpu.active_boundary() >= 0
    assert_structure_equal(gpu, ora, "after the active-wall count")


def test_a_particle_outside_the_grid_scans_everything():
    sc = scenes.falling_block((6, 6, 6), seed=32)
    x = sc.fluid.copy()
    x[0] = [-0.5, 0.5, 0.5]  # outside the domain, so outside the grid: key = the last cell
    v = np.zeros_like(sc.velocity)
    gpu = solver_for(sc, diagnostics=True)
    gpu.set_fluid(x, v)
    ora = oracle_for(sc, gpu, x=x, v=v)
    for k in range(2):
        gpu.step(sc.dt)
        ora.step(sc.dt)
        assert_structure_equal(gpu, ora, f"step {k}")


def test_exported_cell_start_is_complete_after_graph_replays():
    sc = scenes.falling_block((8, 8, 8), seed=33, velocity_sigma=0.2)
    cfg = sc.config(diagnostics=True)
    cfg.use_cuda_graph = 1
    from water_simulation_gb300.solver import Solver

    gpu = Solver(cfg)
    gpu.set_boundary(sc.boundary)
    gpu.set_fluid(sc.fluid, sc.velocity)
    ora = oracle_for(sc, gpu)
    gpu.step(sc.dt, 5)  # one eager step, then two graph replays
    ora.step(sc.dt, 5)
    assert_structure_equal(gpu, ora, "after 5 steps")
    gpu.step(sc.dt, 4)  # replays only
    ora.step(sc.dt, 4)
    cs = gpu.field(_lib.FIELD_CELL_START)
    assert np.array_equal(cs, ora.field(O.F_CELL_START))
    assert cs[0] == 0 and cs[-1] == sc.n


def test_cell_start_after_an_adjoint_rollout_describes_the_final_state():
    # the adjoint's taped replays scan into their own copies of cell_start;
    # the context's own one, completed on export, must be the final state's
    sc = scenes.adjoint_puddle(steps=6)
    s = solver_for(sc, diagnostics=True)
    s.adjoint_set_state(sc.fluid, sc.velocity)
    s.adjoint_forward(sc.dt, 6, 2)
    xT, _ = s.adjoint_state()
    s.adjoint_backward(np.ones_like(xT) * 1e-3)
    cs = s.field(_lib.FIELD_CELL_START)
    t = solver_for(sc, diagnostics=True)
    t.set_fluid(sc.fluid, sc.velocity)
    t.step(sc.dt, 6)
    assert np.array_equal(cs, t.field(_lib.FIELD_CELL_START))

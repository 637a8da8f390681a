"""Empty and ragged inputs. A context whose fluid is empty steps as a no-op
(the reference returns before any launch when the store is empty,
solvers/dfsph/src/dfsph.cu:121-122) and keeps working when fluid arrives; a
batch whose scenes include empty ones equals its other scenes stepped alone."""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver, solver_for
from test_batch_gpu import batch_solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graph", [False, True])
def test_empty_fluid_steps_are_noops(graph):
    sc = scenes.falling_block((6, 6, 6), seed=36, velocity_sigma=0.1)
    cfg = sc.config(capacity=sc.n)
    cfg.use_cuda_graph = 1 if graph else 0
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    empty = np.zeros((0, 3), np.float32)
    s.set_fluid(empty, empty)
    s.step(sc.dt, 5)
    s.synchronize()
    assert s.positions().shape == (0, 3)
    assert s.field(_lib.FIELD_DENSITY).shape == (0,)
    subs = s.step_frames(2)
    assert (subs >= 1).all()
    # fluid arriving afterwards steps exactly as in a fresh context
    s.set_fluid(sc.fluid, sc.velocity)
    s.step(sc.dt, 4)
    t = solver_for(sc)
    t.step(sc.dt, 4)
    assert np.array_equal(s.positions(), t.positions())
    assert np.array_equal(s.velocities(), t.velocities())
    # and back to empty
    s.set_fluid(empty, empty)
    s.step(sc.dt, 3)
    assert s.positions().shape == (0, 3)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_with_empty_scenes_equals_its_scenes_alone(graph):
    scs, eps = scenes.batched_blocks(n_scenes=4, n_min=300, n_max=2000)
    for k in (1, 3):  # ragged: the second and the last scene are empty
        scs[k].fluid = np.zeros((0, 3), np.float32)
        scs[k].velocity = np.zeros((0, 3), np.float32)
    b = batch_solver(scs, eps, graph=graph)
    singles = {k: solver_for(scs[k]) for k in (0, 2)}  # each scene carries its own XSPH coefficient
    b.step(scs[0].dt, 6)
    for s in singles.values():
        s.step(scs[0].dt, 6)
    xb, vb = b.positions(), b.velocities()
    mv = b.scene_max_velocity(len(scs))
    o = 0
    for k, sc in enumerate(scs):
        if k in singles:
            assert np.array_equal(xb[o:o + sc.n], singles[k].positions()), k
            assert np.array_equal(vb[o:o + sc.n], singles[k].velocities()), k
            assert mv[k] == np.float32(singles[k].max_velocity()), k
        else:
            assert sc.n == 0 and mv[k] == 0.0, k
        o += sc.n
    assert o == b.n

"""Scene batching and CUDA-graph replay through the C ABI.

Scenes stepped together keep separate cell keys, so each scene's particles
are sorted exactly as in a context of its own and see exactly the same
neighbours in the same order: a batched step must equal the per-scene steps
bit for bit. A captured two-step CUDA graph replays the same launches, so it
must equal plain launches bit for bit too.
"""
import ctypes

import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver, solver_for

pytestmark = pytest.mark.gpu


def batch_solver(scs, eps, graph=False, steps_scene=None, precision=_lib.PRECISION_FP32):
    cfg = scs[0].config(capacity=sum(s.n for s in scs), precision=precision)
    cfg.n_scenes = len(scs)
    cfg.use_cuda_graph = 1 if graph else 0
    b = Solver(cfg)
    b.set_boundary(scs[0].boundary)
    b.set_fluid_batch([s.fluid for s in scs], [s.velocity for s in scs])
    b.set_scene_viscosity(eps)
    return b


def test_batched_scenes_equal_individual_runs():
    scs, eps = scenes.batched_blocks(n_scenes=5, n_min=300, n_max=3000)
    b = batch_solver(scs, eps)
    singles = [solver_for(s) for s in scs]
    for _ in range(6):
        b.step(scs[0].dt)
        for s in singles:
            s.step(scs[0].dt)
    xb = b.positions()
    vb = b.velocities()
    rb = b.field(_lib.FIELD_DENSITY)
    mv = b.scene_max_velocity(len(scs))
    o = 0
    for k, s in enumerate(singles):
        n = scs[k].n
        assert np.array_equal(xb[o:o + n], s.positions()), k
        assert np.array_equal(vb[o:o + n], s.velocities()), k
        assert np.array_equal(rb[o:o + n], s.field(_lib.FIELD_DENSITY)), k
        assert mv[k] == np.float32(s.max_velocity()), k
        o += n
    # the sorted order is scene-major and canonical inside each scene
    idx = b.field(_lib.FIELD_SORTED_INDEX)
    assert sorted(idx.tolist()) == list(range(b.n))
    bounds = np.cumsum([0] + [s.n for s in scs])
    for k in range(len(scs)):
        assert (idx[bounds[k]:bounds[k + 1]] >= bounds[k]).all()
        assert (idx[bounds[k]:bounds[k + 1]] < bounds[k + 1]).all()


def test_cuda_graph_replay_equals_plain_launches():
    sc = scenes.falling_block((11, 10, 9), seed=5, velocity_sigma=0.2)
    cfg_g = sc.config()
    cfg_g.use_cuda_graph = 1
    g = Solver(cfg_g)
    g.set_boundary(sc.boundary)
    g.set_fluid(sc.fluid, sc.velocity)
    p = solver_for(sc)
    g.step(sc.dt, 9)   # 1 counting step + 4 graph replays
    p.step(sc.dt, 9)
    assert np.array_equal(g.positions(), p.positions())
    assert np.array_equal(g.velocities(), p.velocities())
    assert g.max_velocity() == p.max_velocity()
    # new input invalidates the graph; a second run still matches
    g.set_fluid(sc.fluid, sc.velocity)
    p.set_fluid(sc.fluid, sc.velocity)
    g.step(sc.dt, 4)
    p.step(sc.dt, 4)
    assert np.array_equal(g.positions(), p.positions())


def test_batched_graph_equals_batched_plain():
    scs, eps = scenes.batched_blocks(n_scenes=4, n_min=500, n_max=2500, seed_base=2000)
    a = batch_solver(scs, eps, graph=True)
    b = batch_solver(scs, eps, graph=False)
    a.step(scs[0].dt, 7)
    b.step(scs[0].dt, 7)
    assert np.array_equal(a.positions(), b.positions())
    assert a.kernel_launches() == b.kernel_launches()


def test_compensated_batch_equals_compensated_scenes_alone():
    # each particle's position carry belongs to its index in the concatenated
    # arrays, so a batch compensates exactly as its scenes do alone
    scs, eps = scenes.batched_blocks(n_scenes=3, n_min=400, n_max=1500, seed_base=3000)
    b = batch_solver(scs, eps, precision=_lib.PRECISION_FP32_COMPENSATED)
    singles = [solver_for(s, precision=_lib.PRECISION_FP32_COMPENSATED) for s in scs]
    b.step(scs[0].dt, 10)
    for s in singles:
        s.step(scs[0].dt, 10)
    xb = b.positions()
    o = 0
    for k, s in enumerate(singles):
        assert np.array_equal(xb[o:o + scs[k].n], s.positions()), k
        o += scs[k].n


def test_batch_argument_errors():
    scs, eps = scenes.batched_blocks(n_scenes=3, n_min=200, n_max=400)
    b = batch_solver(scs, eps)
    with pytest.raises(_lib.DfsphError):
        b.set_fluid_batch([s.fluid for s in scs[:2]])  # wrong scene count
    with pytest.raises(_lib.DfsphError) as e:
        b.set_fluid_batch([np.zeros((10_000, 3), np.float32)] * 3)  # beyond capacity
    assert e.value.status == _lib.ERR_OUT_OF_RANGE
    single = solver_for(scs[0])
    with pytest.raises(_lib.DfsphError):
        single.set_fluid_batch([scs[0].fluid, scs[1].fluid])

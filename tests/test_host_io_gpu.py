"""Host buffers through the C ABI: page-locked arrays are read and written
in place by the import / export kernels, pageable ones go through the staging
copy. Both must give the same state and the same fields bit for bit,
including the last partial block of 256 particles and an unaligned pinned
array (which takes the staging path)."""
import ctypes

import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FIELDS = [(_lib.FIELD_POSITION, 3), (_lib.FIELD_VELOCITY, 3), (_lib.FIELD_DENSITY, 1), (_lib.FIELD_ALPHA, 1),
          (_lib.FIELD_KAPPA, 1), (_lib.FIELD_DENSITY_ADV, 1)]


def _solver(sc):
    cfg = sc.config()
    cfg.use_cuda_graph = 0
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    return s


def _ptr(a):
    return ctypes.c_void_p(a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data)


def _read(s, field, comps, pinned, offset=0):
    count = s._n_fluid * comps
    if pinned:
        buf = torch.empty(count + offset, dtype=torch.float32).pin_memory()
        view = buf[offset:]
        s._check(s._lib.dfsph_get_field(s._ctx, field, _ptr(view), count * 4, _lib.MEM_HOST))
        return view.numpy().copy()
    out = np.empty(count, dtype=np.float32)
    s._check(s._lib.dfsph_get_field(s._ctx, field, _ptr(out), count * 4, _lib.MEM_HOST))
    return out


@pytest.mark.parametrize("offset", [0, 1])
def test_pinned_and_pageable_host_io_agree(offset):
    sc = scenes.falling_block(n_side=(7, 11, 13), velocity_sigma=0.2)  # 1,001 particles: a partial last block
    runs = []
    for pinned in (False, True):
        s = _solver(sc)
        s._n_fluid = sc.n
        if pinned:
            x = torch.empty(3 * sc.n + offset, dtype=torch.float32).pin_memory()
            v = torch.empty(3 * sc.n + offset, dtype=torch.float32).pin_memory()
            x[offset:] = torch.from_numpy(sc.fluid.reshape(-1))
            v[offset:] = torch.from_numpy(sc.velocity.reshape(-1))
            xp, vp = x[offset:], v[offset:]
        else:
            xp, vp = np.ascontiguousarray(sc.fluid.reshape(-1)), np.ascontiguousarray(sc.velocity.reshape(-1))
        s._check(s._lib.dfsph_set_fluid(s._ctx, _ptr(xp), _ptr(vp), sc.n, _lib.MEM_HOST))
        for _ in range(3):
            s.step(sc.dt)
        runs.append([_read(s, f, c, pinned, offset) for f, c in FIELDS])
        s.close()
    for (f, _), a, b in zip(FIELDS, runs[0], runs[1]):
        assert np.array_equal(a, b), f
    assert np.isfinite(runs[0][0]).all()


def test_get_state_matches_the_field_reads():
    # 1,003 particles: a last partial block of 256
    sc = scenes.falling_block((17, 59, 1), seed=6, velocity_sigma=0.2)
    s = _solver(sc)
    s.set_fluid(sc.fluid, sc.velocity)
    s.step(sc.dt, 3)
    x_ref, v_ref = s.positions(), s.velocities()
    n = s.n
    # page-locked: one export kernel writes both in place
    xp = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    vp = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    s.get_state(xp.numpy(), vp.numpy())
    assert np.array_equal(xp.numpy(), x_ref)
    assert np.array_equal(vp.numpy(), v_ref)
    # pageable, and one of the two only
    xq, vq = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
    s.get_state(xq, vq)
    assert np.array_equal(xq, x_ref) and np.array_equal(vq, v_ref)
    xo = torch.zeros((n, 3), dtype=torch.float32).pin_memory()
    s.get_state(xo.numpy(), None)
    assert np.array_equal(xo.numpy(), x_ref)
    vo = np.zeros((n, 3), np.float32)
    s.get_state(None, vo)
    assert np.array_equal(vo, v_ref)
    # device memory
    xd = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    vd = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    s.get_state_ptr(xd.data_ptr(), vd.data_ptr(), _lib.MEM_DEVICE)
    torch.cuda.synchronize()
    assert np.array_equal(xd.cpu().numpy(), x_ref) and np.array_equal(vd.cpu().numpy(), v_ref)
    # a round trip through page-locked arrays continues the run bit for bit
    t = _solver(sc)
    t.set_fluid(sc.fluid, sc.velocity)
    t.step(sc.dt, 3)
    t.set_fluid(xp.numpy(), vp.numpy())
    s.step(sc.dt, 2)
    t.step(sc.dt, 2)
    assert np.array_equal(s.positions(), t.positions())


@pytest.mark.parametrize("precision", [_lib.PRECISION_FP64, _lib.PRECISION_FP32_COMPENSATED])
def test_get_state_in_the_other_precisions(precision):
    # the export converts the working type to float as dfsph_get_field does
    sc = scenes.falling_block((17, 59, 1), seed=7, velocity_sigma=0.2)
    cfg = sc.config(precision=precision)
    cfg.use_cuda_graph = 0
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    s.set_fluid(sc.fluid, sc.velocity)
    s.step(sc.dt, 3)
    x_ref, v_ref = s.positions(), s.velocities()
    xp = torch.empty((s.n, 3), dtype=torch.float32).pin_memory()
    vp = torch.empty((s.n, 3), dtype=torch.float32).pin_memory()
    s.get_state(xp.numpy(), vp.numpy())
    assert np.array_equal(xp.numpy(), x_ref) and np.array_equal(vp.numpy(), v_ref)
    xq, vq = np.empty((s.n, 3), np.float32), np.empty((s.n, 3), np.float32)
    s.get_state(xq, vq)
    assert np.array_equal(xq, x_ref) and np.array_equal(vq, v_ref)


def test_get_state_of_a_batch():
    from test_batch_gpu import batch_solver

    scs, eps = scenes.batched_blocks(n_scenes=3, n_min=300, n_max=1000)
    b = batch_solver(scs, eps)
    b.step(scs[0].dt, 3)
    x_ref, v_ref = b.positions(), b.velocities()
    xp = torch.empty((b.n, 3), dtype=torch.float32).pin_memory()
    vp = torch.empty((b.n, 3), dtype=torch.float32).pin_memory()
    b.get_state(xp.numpy(), vp.numpy())
    assert np.array_equal(xp.numpy(), x_ref) and np.array_equal(vp.numpy(), v_ref)

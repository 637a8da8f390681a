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

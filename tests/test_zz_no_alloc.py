"""The allocation-free cell-grid build (dfsph_build_cell_grid_static).

Some callers cannot let a library allocate device memory: a host callback or
graph node that must stay out of the allocator, a plugin whose host program
owns every allocation, a process with a fixed memory budget. For them the
library has a variant of the cell-grid build whose scratch is a fixed device
array compiled into the library. This test calls it through the C ABI and
checks that it returns exactly what the allocating entry point
(dfsph_build_cell_grid) returns, for two different inputs in a row (the
scratch keeps the previous call's contents, which must not leak into the
next), and that inputs beyond its stated limits are rejected. The file name
sorts last so a run that stops at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

from water_simulation_gb300 import _lib

pytestmark = pytest.mark.gpu


def _build(fn, xyz, origin, dims, cell):
    import torch

    dev = torch.device("cuda")
    n = xyz.shape[0]
    total = int(dims[0]) * int(dims[1]) * int(dims[2])
    x = torch.tensor(xyz, device=dev)
    keys = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    idx = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    cs = torch.full((total + 1,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    st = fn(ctypes.c_void_p(x.data_ptr()), n, _lib.fvec3(origin), (ctypes.c_int * 3)(*dims), ctypes.c_float(cell),
            ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(idx.data_ptr()), ctypes.c_void_p(cs.data_ptr()),
            ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return st, keys.cpu().numpy().view(np.uint32)[:n], idx.cpu().numpy().view(np.uint32)[:n], \
        cs.cpu().numpy().view(np.uint32)


def _cases():
    rng = np.random.default_rng(2024)
    a = rng.uniform(-0.05, 1.05, size=(20000, 3)).astype(np.float32)
    a[:300] = np.float32([0.5, 0.5, 0.5])  # a crowded cell
    b = rng.uniform(0.2, 0.4, size=(7000, 3)).astype(np.float32)  # different size and region
    return [(a, (-0.04, -0.04, -0.04), (28, 28, 28), 0.04), (b, (0.0, 0.0, 0.0), (52, 40, 30), 0.02)]


def test_static_build_matches_allocating_build_twice_in_a_row():
    lib = _lib.load()
    for xyz, origin, dims, cell in _cases():
        st_a, ka, ia, ca = _build(lib.dfsph_build_cell_grid, xyz, origin, dims, cell)
        st_s, ks, is_, cs = _build(lib.dfsph_build_cell_grid_static, xyz, origin, dims, cell)
        assert st_a == _lib.OK and st_s == _lib.OK
        assert np.array_equal(ka, ks)
        assert np.array_equal(ia, is_)
        assert np.array_equal(ca, cs)
        assert sorted(is_.tolist()) == list(range(xyz.shape[0]))


def test_static_build_rejects_sizes_beyond_its_limits():
    lib = _lib.load()
    xyz = np.zeros((4, 3), np.float32)
    st, *_ = _build(lib.dfsph_build_cell_grid_static, xyz, (0, 0, 0), (128, 128, 65), 0.01)
    assert st == _lib.ERR_OUT_OF_RANGE  # 1,064,960 cells > 1,048,576
    big = np.zeros((131073, 3), np.float32)
    st, *_ = _build(lib.dfsph_build_cell_grid_static, big, (0, 0, 0), (8, 8, 8), 0.1)
    assert st == _lib.ERR_OUT_OF_RANGE

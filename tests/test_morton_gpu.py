"""dfsph_morton_sort (the reference SpatialAccel's Morton order) against the
oracle restatement: codes and permutation bit-exact, including equal codes
(stability), points outside the scene box (clamped) and a flat axis."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from water_simulation_gb300 import _lib

pytestmark = pytest.mark.gpu


def gpu_morton(xyz, smin, smax):
    import torch

    n = xyz.shape[0]
    x = torch.tensor(xyz, device="cuda")
    codes = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    idx = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    st = _lib.load().dfsph_morton_sort(ctypes.c_void_p(x.data_ptr()), n, _lib.fvec3(smin), _lib.fvec3(smax),
                                       ctypes.c_void_p(codes.data_ptr()), ctypes.c_void_p(idx.data_ptr()),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    return codes.cpu().numpy().view(np.uint32)[:n], idx.cpu().numpy().view(np.uint32)[:n]


@pytest.mark.parametrize("n,seed", [(8, 0), (1, 1), (1000, 2), (300_000, 3)])
def test_morton_sort_matches_oracle(n, seed):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-0.1, 1.1, size=(n, 3)).astype(np.float32)
    if n > 100:
        xyz[: n // 4] = xyz[0]  # many equal codes
    c, i = gpu_morton(xyz, (0, 0, 0), (1, 1, 1))
    co, io = O.morton_sort(xyz, (0, 0, 0), (1, 1, 1))
    assert np.array_equal(c, co)
    assert np.array_equal(i, io)


def test_morton_sort_flat_axis():
    rng = np.random.default_rng(9)
    xyz = rng.uniform(0, 1, size=(5000, 3)).astype(np.float32)
    xyz[:, 2] = 0.5
    c, i = gpu_morton(xyz, (0, 0, 0.5), (1, 1, 0.5))
    co, io = O.morton_sort(xyz, (0, 0, 0.5), (1, 1, 0.5))
    assert np.array_equal(c, co) and np.array_equal(i, io)

"""dfsph_lbvh_build / dfsph_lbvh_refit (the reference SpatialAccel plus its
bottom-up box pass) and dfsph_cohesion_kernel against the oracle: codes,
permutation, children, parents and boxes bit-exact; a refit after the
particles moved equals the oracle's boxes on the same topology."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from water_simulation_gb300 import _lib

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def gpu_lbvh(xyz, smin, smax, radius):
    import torch

    n = xyz.shape[0]
    m = max(n - 1, 1)
    dev = "cuda"
    x = torch.tensor(xyz, device=dev)
    codes = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    idx = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    left = torch.zeros(m, dtype=torch.int32, device=dev)
    right = torch.zeros(m, dtype=torch.int32, device=dev)
    parent = torch.zeros(max(2 * n - 1, 1), dtype=torch.int32, device=dev)
    boxes = torch.zeros((max(2 * n - 1, 1), 6), dtype=torch.float32, device=dev)
    scratch = torch.zeros(m, dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    lib = _lib.load()
    assert lib.dfsph_lbvh_build(_ptr(x), n, _lib.fvec3(smin), _lib.fvec3(smax), ctypes.c_float(radius), _ptr(codes),
                                _ptr(idx), _ptr(left), _ptr(right), _ptr(parent), _ptr(boxes), _ptr(scratch),
                                ctypes.c_void_p(st)) == 0
    torch.cuda.synchronize()
    u = lambda t, k: t.cpu().numpy().view(np.uint32)[:k]  # noqa: E731
    out = (u(codes, n), u(idx, n), u(left, max(n - 1, 0)), u(right, max(n - 1, 0)), u(parent, max(2 * n - 1, 0)),
           boxes.cpu().numpy()[: max(2 * n - 1, 0)])
    return out, (x, idx, left, right, parent, boxes, scratch)


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (8, 2), (5000, 3), (400_000, 4)])
def test_lbvh_build_matches_oracle(n, seed):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-0.05, 1.05, size=(n, 3)).astype(np.float32)
    if n > 100:
        xyz[: n // 5] = xyz[1]  # equal codes
    (gc, gi, gl, gr, gp, gb), _ = gpu_lbvh(xyz, (0, 0, 0), (1, 1, 1), 0.003)
    oc, oi, ol, orr, op, ob = O.lbvh_build(xyz, (0, 0, 0), (1, 1, 1), 0.003)
    assert np.array_equal(gc, oc) and np.array_equal(gi, oi)
    assert np.array_equal(gl, ol) and np.array_equal(gr, orr) and np.array_equal(gp, op)
    assert np.array_equal(gb, ob)


def test_lbvh_refit_after_motion():
    import torch

    rng = np.random.default_rng(11)
    n = 100_000
    xyz = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    (oc, oi, *_), (x, idx, left, right, parent, boxes, scratch) = gpu_lbvh(xyz, (0, 0, 0), (1, 1, 1), 0.0)
    moved = (xyz + rng.normal(0, 0.01, size=xyz.shape)).astype(np.float32)
    x.copy_(torch.tensor(moved, device="cuda"))
    st = torch.cuda.current_stream().cuda_stream
    assert _lib.load().dfsph_lbvh_refit(_ptr(x), n, ctypes.c_float(0.001), _ptr(idx), _ptr(left), _ptr(right),
                                        _ptr(parent), _ptr(boxes), _ptr(scratch), ctypes.c_void_p(st)) == 0
    torch.cuda.synchronize()
    _, _, _, _, _, ob = O.lbvh_build(moved, (0, 0, 0), (1, 1, 1), 0.001, codes=oc, sorted_idx=oi)
    assert np.array_equal(boxes.cpu().numpy(), ob)


def test_cohesion_kernel_matches_oracle():
    import torch

    l = 0.04
    r = np.linspace(-0.01, 0.05, 20001).astype(np.float32)
    rt = torch.tensor(r, device="cuda")
    out = torch.empty_like(rt)
    assert _lib.load().dfsph_cohesion_kernel(_ptr(rt), r.size, ctypes.c_float(l), _ptr(out),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    torch.cuda.synchronize()
    ref = np.array([O.cohesion_C(float(v), float(np.float32(l))) for v in r])
    g = out.cpu().numpy().astype(np.float64)
    assert np.abs(g - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n,seed", [(1, 5), (2, 6), (9, 7), (5000, 8), (400_000, 9)])
def test_lbvh_build_matches_reference_kernels(n, seed):
    """The reference's own SpatialAccel kernels (compiled from its sources)
    under its build orchestration: codes, permutation, children, parents (the
    reference leaves the root's unwritten) and leaf boxes (radius 0) equal
    dfsph_lbvh_build's bit for bit."""
    from oracle import reference as R

    if not R.available():
        pytest.skip("reference kernels (oracle/_ref) not built")
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-0.05, 1.05, size=(n, 3)).astype(np.float32)
    if n > 100:
        xyz[: n // 5] = xyz[1]  # equal codes
    lo, hi = (0.0, -0.2, 0.1), (1.0, 1.3, 0.9)
    (gc, gi, gl, gr, gp, gb), _ = gpu_lbvh(xyz, lo, hi, 0.0)
    (rc, ri, rl, rr, rp, rb), _ = R.lbvh_build(xyz, lo, hi)
    assert np.array_equal(gi, ri)
    if n < 2:
        return
    assert np.array_equal(gc, rc)
    assert np.array_equal(gl, rl) and np.array_equal(gr, rr)
    assert np.array_equal(gp[1:], rp[1:])
    assert np.array_equal(gb[n - 1:], rb)


def test_lbvh_refit_unaligned_boxes():
    """A box array that is only 4-byte aligned takes the arrival-count refit;
    its boxes equal the oracle's as the aligned path's do."""
    import torch

    rng = np.random.default_rng(12)
    n = 50_000
    xyz = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    (oc, oi, *_), (x, idx, left, right, parent, boxes, scratch) = gpu_lbvh(xyz, (0, 0, 0), (1, 1, 1), 0.002)
    raw = torch.zeros(6 * (2 * n - 1) + 1, dtype=torch.float32, device="cuda")
    shifted = raw[1:]  # 4 bytes past an aligned base
    st = torch.cuda.current_stream().cuda_stream
    assert _lib.load().dfsph_lbvh_refit(_ptr(x), n, ctypes.c_float(0.002), _ptr(idx), _ptr(left), _ptr(right),
                                        _ptr(parent), _ptr(shifted), _ptr(scratch), ctypes.c_void_p(st)) == 0
    torch.cuda.synchronize()
    _, _, _, _, _, ob = O.lbvh_build(xyz, (0, 0, 0), (1, 1, 1), 0.002, codes=oc, sorted_idx=oi)
    assert np.array_equal(shifted.cpu().numpy().reshape(-1, 6), ob)
    assert np.array_equal(boxes.cpu().numpy(), ob)

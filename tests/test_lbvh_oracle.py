"""The LBVH restatement (SpatialAccel, core/src/spatial_accel.cu) on the CPU.

Known answers of the reference's tests/unit/test_spatial_accel.cu (8 grid
points: 8 leaves, the sorted indices a permutation; a single particle builds
without internal nodes), and an independent check of the Karras construction:
the tree must be the binary radix tree of the keys (code << 32) | slot, i.e.
every internal node splits its sorted range at the highest bit where the keys
of the range differ."""
import numpy as np
import pytest

from oracle import oracle as O

GRID8 = np.array([[0.1, 0.1, 0.1], [0.9, 0.1, 0.1], [0.1, 0.9, 0.1], [0.9, 0.9, 0.1],
                  [0.1, 0.1, 0.9], [0.9, 0.1, 0.9], [0.1, 0.9, 0.9], [0.9, 0.9, 0.9]], np.float32)


def radix_tree(codes):
    """(left, right) of the binary radix tree over keys (code << 32) | slot."""
    n = len(codes)
    keys = [(int(c) << 32) | i for i, c in enumerate(codes)]
    left = [0] * (n - 1)
    right = [0] * (n - 1)

    def prefix(a, b):
        return 64 - (keys[a] ^ keys[b]).bit_length()

    stack = [(0, n - 1, 0)]
    while stack:
        first, last, node = stack.pop()
        common = prefix(first, last)
        g = first
        while g + 1 < last and prefix(first, g + 1) > common:
            g += 1
        lc = (n - 1 + g) if g == first else g
        rc = (n - 1 + g + 1) if g + 1 == last else g + 1
        left[node], right[node] = lc, rc
        if g > first:
            stack.append((first, g, g))
        if g + 1 < last:
            stack.append((g + 1, last, g + 1))
    return np.array(left, np.uint32), np.array(right, np.uint32)


def test_reference_known_answer_grid8():
    codes, sorted_idx, left, right, parent, boxes = O.lbvh_build(GRID8, (0, 0, 0), (1, 1, 1))
    assert sorted(sorted_idx.tolist()) == list(range(8))
    assert len(left) == 7 and parent[0] == 0xFFFFFFFF
    assert np.allclose(boxes[0], [0.1, 0.1, 0.1, 0.9, 0.9, 0.9])


def test_single_particle():
    codes, sorted_idx, left, right, parent, boxes = O.lbvh_build(np.array([[0.5, 0.5, 0.5]], np.float32),
                                                                 (0, 0, 0), (1, 1, 1), 0.01)
    assert sorted_idx.tolist() == [0] and len(left) == 0 and parent.tolist() == [0xFFFFFFFF]
    assert np.allclose(boxes[0], [0.49, 0.49, 0.49, 0.51, 0.51, 0.51])


@pytest.mark.parametrize("n,seed,dups", [(2, 0, False), (57, 1, False), (1000, 2, True), (4096, 3, True)])
def test_tree_is_the_radix_tree(n, seed, dups):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    if dups:
        xyz[: n // 3] = xyz[0]  # equal codes: the slot index breaks the tie
    codes, sorted_idx, left, right, parent, boxes = O.lbvh_build(xyz, (0, 0, 0), (1, 1, 1), 0.002)
    lt, rt = radix_tree(codes)
    assert np.array_equal(left, lt) and np.array_equal(right, rt)
    # parents, reachability, and boxes that enclose their children
    for i in range(n - 1):
        assert parent[left[i]] == i and parent[right[i]] == i
        for c in (left[i], right[i]):
            assert np.all(boxes[i, :3] <= boxes[c, :3]) and np.all(boxes[i, 3:] >= boxes[c, 3:])
    seen = np.zeros(2 * n - 1, bool)
    stack = [0]
    while stack:
        v = stack.pop()
        assert not seen[v]
        seen[v] = True
        if v < n - 1:
            stack += [int(left[v]), int(right[v])]
    assert seen.all()
    lo, hi = xyz.min(0) - 0.002, xyz.max(0) + 0.002
    assert np.allclose(boxes[0, :3], lo) and np.allclose(boxes[0, 3:], hi)


def test_cohesion_kernel_shape():
    l = 0.04
    assert O.cohesion_C(0.0, l) == 0.0 and O.cohesion_C(0.05, l) == 0.0
    # negative near the centre, positive beyond l/2, continuous at l/2
    assert O.cohesion_C(0.005, l) < 0.0 < O.cohesion_C(0.03, l)
    a, b = O.cohesion_C(0.5 * l * (1 - 1e-9), l), O.cohesion_C(0.5 * l * (1 + 1e-9), l)
    assert abs(a - b) < 1e-6 * abs(b)

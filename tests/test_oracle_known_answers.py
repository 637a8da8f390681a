"""The CPU oracle against the known answers of the reference's own tests.

Each test re-expresses one case of the reference's test suite (file:line in
Qervas/water_simulation) against the oracle restatement, plus the grid and
boundary counts of the benchmark configurations computed with the reference's
make_grid / sample_aabb_boundary arithmetic.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

RHO0 = 1000.0


def cfg(r=0.01, l=None, visc=1e-3, damping=0.5, dmin=(0, 0, 0), dmax=(1, 1, 1), iters=100, eta=1e-3,
        div_iters=0):
    c = O.OracleConfig()
    c.rest_density = RHO0
    c.particle_radius = r
    c.smoothing_length = l if l is not None else 2 * r
    c.viscosity = visc
    c.damping = damping
    c.gravity[:] = [0.0, -9.81, 0.0]
    c.max_density_iters = iters
    c.max_divergence_iters = div_iters
    c.eta_density = eta
    c.eta_divergence = 1e-3
    c.domain_min[:] = list(dmin)
    c.domain_max[:] = list(dmax)
    c.stencil_inv_cell = 0.0
    return c


# tests/unit/test_sph_kernels.cu:36-41
def test_W_peak_and_support():
    l = 0.05
    assert O.W(0.0, l) > 0
    assert abs(O.W(2 * l, l)) <= 1e-6
    assert O.W(3 * l, l) == 0.0


# tests/unit/test_sph_kernels.cu:43-52
def test_W_monotone():
    l = 0.1
    prev = O.W(0.0, l)
    for i in range(1, 21):
        cur = O.W(i * 0.1 * l, l)
        assert cur <= prev + 1e-7
        prev = cur


# tests/unit/test_sph_kernels.cu:54-71
def test_gradW_zero_at_origin_and_outside_and_points_inward():
    l = 0.05
    assert O.gradW((0, 0, 0), l) == (0.0, 0.0, 0.0)
    assert O.gradW((2.5 * l, 0, 0), l)[0] == 0.0
    g = O.gradW((0.5 * l, 0, 0), l)
    assert g[0] < 0 and g[1] == 0 and g[2] == 0


def test_W_normalisation_and_gradient_consistency():
    # sigma = 1/(pi l^3): W(0) = sigma; the gradient is -dW/dr along r
    l = 0.04
    assert O.W(0.0, l, 64) == pytest.approx(1.0 / (math.pi * l ** 3), rel=1e-12)
    r, h = 0.6 * l, 1e-7
    dwdr = (O.W(r + h, l, 64) - O.W(r - h, l, 64)) / (2 * h)
    assert O.gradW((r, 0, 0), l)[0] == pytest.approx(dwdr, rel=1e-4)


# tests/unit/test_cell_grid.cu:9-47
def test_cell_grid_permutation_and_monotone_starts():
    pts = np.array([[0.25, 0.25, 0.25], [0.75, 0.25, 0.25], [0.25, 0.75, 0.25], [0.75, 0.75, 0.25],
                    [0.25, 0.25, 0.75], [0.75, 0.25, 0.75], [0.25, 0.75, 0.75], [0.75, 0.75, 0.75]], np.float32)
    keys, srt, cs = O.build_grid(pts, (0, 0, 0), (4, 4, 4), 0.5)
    assert sorted(srt.tolist()) == list(range(8))
    assert np.all(np.diff(cs.astype(np.int64)) >= 0)
    assert len(set(keys.tolist())) == 8
    # x-major key (cx*dy + cy)*dz + cz
    assert keys[1] == (1 * 4 + 0) * 4 + 0
    assert keys[4] == (0 * 4 + 0) * 4 + 1


# tests/unit/test_cell_grid.cu:49-74
def test_cell_grid_out_of_bounds_goes_to_sentinel():
    pts = np.array([[0.25, 0.25, 0.25], [99.0, 99.0, 99.0]], np.float32)
    keys, srt, cs = O.build_grid(pts, (0, 0, 0), (2, 2, 2), 0.5)
    assert cs[-1] == 1
    assert cs[0] == 0
    assert keys[1] == 8


def test_cell_grid_is_stable_and_empty_cells_point_to_next_start():
    rng = np.random.default_rng(5)
    pts = rng.uniform(-0.2, 1.2, size=(3000, 3)).astype(np.float32)
    pts[::7] = pts[3]  # many particles in one cell
    keys, srt, cs = O.build_grid(pts, (0, 0, 0), (9, 7, 5), 0.13)
    total = 9 * 7 * 5
    order = np.lexsort((np.arange(len(keys)), keys))
    assert np.array_equal(srt, order)
    sk = keys[srt]
    for c in range(total + 1):
        assert cs[c] == np.searchsorted(sk, c, side="left")


# tests/unit/test_dfsph_density.cu:16-36
def test_isolated_particle_density_is_mass_times_W0():
    c = cfg(r=0.01, l=0.04)
    o = O.Oracle(c, np.array([[0.5, 0.5, 0.5]], np.float32), precision=32)
    o.step(0.001)
    m = o.particle_mass()
    expected = m * (1.0 / (3.14159265358979323846 * 0.04 ** 3))
    assert o.field(O.F_DENSITY)[0] == pytest.approx(expected, rel=1e-4)


# tests/unit/test_dfsph_density.cu:38-79
def test_dense_pack_center_density_near_rest():
    r, s = 0.01, 0.02
    pts = np.array([[0.1 + x * s, 0.1 + y * s, 0.1 + z * s]
                    for z in range(10) for y in range(10) for x in range(10)], np.float32)
    o = O.Oracle(cfg(r=r, l=4 * r), pts, precision=32)
    o.step(0.001)
    d = o.field(O.F_DENSITY)[555]
    assert d == pytest.approx(RHO0, rel=0.30)
    assert 500 < d < 1500
    a = o.field(O.F_ALPHA)[555]
    assert a >= 0 and np.isfinite(a)


# tests/unit/test_dfsph_density.cu:81-109
def test_single_particle_falls_without_boundary():
    c = cfg(r=0.01, l=0.04, visc=0.0)
    o = O.Oracle(c, np.array([[0.5, 0.5, 0.5]], np.float32), np.zeros((1, 3), np.float32), precision=32)
    o.step(0.01, 50)
    p = o.field(O.F_POSITION)[0]
    assert p[1] < 0.5
    assert p[0] == pytest.approx(0.5, rel=0.01)
    assert p[2] == pytest.approx(0.5, rel=0.01)


# tests/unit/test_boundary_sampler.cu:7-31
def test_boundary_sampler_counts_and_faces():
    p1 = O.sample_aabb_boundary((0, 0, 0), (1, 1, 1), 0.05, 1)
    assert 2000 < len(p1) < 4000
    p2 = O.sample_aabb_boundary((0, 0, 0), (1, 1, 1), 0.05, 2)
    mi = 0.05 * 2 + 1e-3
    near = ((p2 <= mi) | (p2 >= 1 - mi)).any(axis=1)
    assert near.all()
    assert 1.5 * len(p1) < len(p2) < 2.5 * len(p1)


# tests/regression/test_settled_puddle.cu:66-117 (sanity part)
def test_boundary_mass_positive_and_single_drop():
    r = 0.012
    c = cfg(r=r, visc=0.0)
    b = O.sample_aabb_boundary((0, 0, 0), (1, 1, 1), 2 * r, 3)
    o = O.Oracle(c, np.array([[0.5, 0.05, 0.5]], np.float32), np.zeros((1, 3), np.float32), b, precision=32)
    mb = o.field(O.F_BOUNDARY_MASS)
    assert o.particle_mass() > 0
    assert mb[0] > 0 and mb[100] > 0 and mb[1000] > 0
    for _ in range(5):
        o.step(0.001)
    assert np.isfinite(o.field(O.F_POSITION)).all()


# make_grid (solvers/dfsph/src/dfsph.cu:55-65): float ceil gives 63 at 0.6/0.01
@pytest.mark.parametrize("r,dmax,dims,nb", [
    (0.01, (1, 1, 1), (52, 52, 52), 46818),
    (0.005, (1.6, 1.0, 0.6), (162, 102, 63), 193458),
    (0.0025, (1.6, 1.0, 0.6), (322, 202, 123), 766098),
])
def test_benchmark_grid_and_boundary_counts(r, dmax, dims, nb):
    c = cfg(r=r, dmax=dmax)
    origin, d = O.grid_geometry(c)
    assert d == dims
    assert origin[0] == pytest.approx(-2 * r)
    b = O.sample_aabb_boundary((0, 0, 0), dmax, 2 * r, 3)
    assert len(b) == nb


def test_fp32_and_fp64_oracles_agree_on_a_short_run():
    rng = np.random.default_rng(1)
    r = 0.02
    base = np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(6), indexing="ij"), -1).reshape(-1, 3)
    pts = (0.35 + (base + 0.5) * 2 * r + rng.uniform(-1e-3, 1e-3, base.shape)).astype(np.float32)
    c = cfg(r=r, visc=0.01, iters=4, eta=0.0)
    b = O.sample_aabb_boundary((0, 0, 0), (1, 1, 1), 2 * r, 3)
    o32 = O.Oracle(c, pts, None, b, precision=32)
    o64 = O.Oracle(c, pts, None, b, precision=64)
    for _ in range(5):
        o32.step(1e-3)
        o64.step(1e-3)
    rho32, rho64 = o32.field(O.F_DENSITY), o64.field(O.F_DENSITY)
    assert np.abs(rho32 - rho64).max() / RHO0 < 1e-4
    assert np.abs(o32.field(O.F_POSITION) - o64.field(O.F_POSITION)).max() < 1e-5
    assert o32.last_density_iters() == 4


def test_density_solver_stops_on_tolerance_from_second_iteration():
    # dfsph.cu:254-258: the error is checked from the second iteration on
    r = 0.02
    base = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    pts = (0.4 + (base + 0.5) * 2 * r).astype(np.float32)
    o = O.Oracle(cfg(r=r, iters=50, eta=1.0), pts, precision=32)
    o.step(1e-3)
    assert o.last_density_iters() == 2


def test_divergence_solver_reduces_compression_rate():
    # the reference plan's divergence solver: kappa_v from max(0, rho_dot)
    r = 0.02
    base = np.stack(np.meshgrid(np.arange(5), np.arange(5), np.arange(5), indexing="ij"), -1).reshape(-1, 3)
    pts = (0.4 + (base + 0.5) * 2 * r).astype(np.float32)
    vel = np.zeros_like(pts)
    vel[:, 1] = -0.5 * (base[:, 1] / 4.0)  # converging column
    c0 = cfg(r=r, iters=0, eta=0.0, div_iters=0, visc=0.0, damping=0.0)
    c1 = cfg(r=r, iters=0, eta=0.0, div_iters=5, visc=0.0, damping=0.0)
    o0 = O.Oracle(c0, pts, vel, precision=64)
    o1 = O.Oracle(c1, pts, vel, precision=64)
    o0.step(1e-3)
    o1.step(1e-3)
    assert o1.scalar(3) >= 1
    assert o1.scalar(5) >= 0.0
    # velocities were corrected (kappa_v > 0 somewhere)
    assert np.abs(o1.field(O.F_VELOCITY) - o0.field(O.F_VELOCITY)).max() > 0


# tests/unit/test_spatial_accel.cu:9-55 (Morton order of SpatialAccel::build)
def test_morton_order_permutation_and_known_codes():
    pts = np.array([[0.1, 0.1, 0.1], [0.9, 0.1, 0.1], [0.1, 0.9, 0.1], [0.9, 0.9, 0.1],
                    [0.1, 0.1, 0.9], [0.9, 0.1, 0.9], [0.1, 0.9, 0.9], [0.9, 0.9, 0.9]], np.float32)
    codes, idx = O.morton_sort(pts, (0, 0, 0), (1, 1, 1))
    assert sorted(idx.tolist()) == list(range(8))
    assert np.all(np.diff(codes.astype(np.int64)) >= 0)
    # x carries the highest bit of each triple: (0.9, 0.1, 0.1) sorts after (0.1, 0.9, 0.9)
    assert idx.tolist() == [0, 4, 2, 6, 1, 5, 3, 7]
    # the corner (1, 1, 1) clamps to 1023 per axis: all 30 bits set
    c, _ = O.morton_sort(np.array([[1.0, 1.0, 1.0]], np.float32), (0, 0, 0), (1, 1, 1))
    assert c[0] == (1 << 30) - 1
    c, i = O.morton_sort(np.array([[0.5, 0.5, 0.5]], np.float32), (0, 0, 0), (1, 1, 1))
    assert i.tolist() == [0]


def test_morton_order_is_stable_for_equal_codes():
    pts = np.tile(np.array([[0.3, 0.3, 0.3], [0.2, 0.2, 0.2]], np.float32), (50, 1))
    codes, idx = O.morton_sort(pts, (0, 0, 0), (1, 1, 1))
    assert idx[:50].tolist() == list(range(1, 100, 2))
    assert idx[50:].tolist() == list(range(0, 100, 2))

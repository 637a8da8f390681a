"""The step in Morton slot order (dfsph_config.slot_order = DFSPH_ORDER_MORTON)
against the step in the reference's x-major cell-key order.

The Morton variant is SpatialAccel's key (core/src/spatial_accel.cu:11-40)
applied to cell coordinates: the fluid slots are sorted by the Morton rank of
their cell instead of the x-major key (core/src/cell_grid.cu:10-30). The
stencil is still walked cell by cell in x-major order (dx, dy, then z), each
cell's particles in ascending original index, so every particle meets the same
candidates in the same sequence: with fixed iteration counts the two steps
give the same fields bit for bit. The grid fields of the Morton context hold
Morton ranks, checked here against ranks computed independently in numpy.
"""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _solver(sc, order, diagnostics=True):
    cfg = sc.config(diagnostics=diagnostics)
    cfg.slot_order = order
    s = Solver(cfg)
    if sc.nb:
        s.set_boundary(sc.boundary)
    s.set_fluid(sc.fluid, sc.velocity)
    return s


def morton_ranks(dims):
    """Rank of every x-major cell in the Morton order of (x, y, z), x highest."""
    nx, ny, nz = dims
    x, y, z = np.meshgrid(np.arange(nx, dtype=np.uint64), np.arange(ny, dtype=np.uint64),
                          np.arange(nz, dtype=np.uint64), indexing="ij")
    code = np.zeros(x.shape, np.uint64)
    for b in range(21):
        bit = np.uint64(b)
        code |= ((x >> bit) & np.uint64(1)) << np.uint64(3 * b + 2)
        code |= ((y >> bit) & np.uint64(1)) << np.uint64(3 * b + 1)
        code |= ((z >> bit) & np.uint64(1)) << np.uint64(3 * b)
    order = np.argsort(code.ravel(), kind="stable")
    rank = np.empty(order.size + 1, np.uint32)
    rank[order] = np.arange(order.size, dtype=np.uint32)
    rank[-1] = order.size
    return rank


FIELDS = [_lib.FIELD_POSITION, _lib.FIELD_VELOCITY, _lib.FIELD_DENSITY, _lib.FIELD_ALPHA, _lib.FIELD_KAPPA,
          _lib.FIELD_DENSITY_ADV, _lib.FIELD_KAPPA_V, _lib.FIELD_NBR_FLUID, _lib.FIELD_NBR_BOUNDARY,
          _lib.FIELD_NBR_SIGNATURE]


def _scene(name):
    if name == "dam":  # a column against the x = 0 wall and the floor: wall terms from the first step
        from test_divergence_gpu import small_dam

        return small_dam()
    return scenes.falling_block((14, 12, 10), seed=17, velocity_sigma=0.3)


@pytest.mark.parametrize("name,divergence", [("block", 0), ("block", 2), ("dam", 0), ("dam", 2)])
def test_morton_order_step_is_bit_identical(name, divergence):
    sc = _scene(name)
    sc.max_divergence_iters = divergence
    a = _solver(sc, _lib.ORDER_CELL_KEY)
    b = _solver(sc, _lib.ORDER_MORTON)
    rank = morton_ranks(a.dims)
    for k in range(20):
        a.step(sc.dt)
        b.step(sc.dt)
        for f in FIELDS:
            assert np.array_equal(a.field(f), b.field(f)), (k, f)
        # the Morton context's keys are the Morton ranks of the x-major keys
        assert np.array_equal(rank[a.field(_lib.FIELD_CELL_KEY)], b.field(_lib.FIELD_CELL_KEY)), k
    assert a.max_velocity() == b.max_velocity()
    if name == "dam":
        assert a.field(_lib.FIELD_NBR_BOUNDARY).max() > 0  # the walls took part
    cs = b.field(_lib.FIELD_CELL_START)
    keys = b.field(_lib.FIELD_CELL_KEY)
    order = b.field(_lib.FIELD_SORTED_INDEX)
    # slots are in Morton-rank order and cell_start indexes the ranks
    assert np.all(np.diff(keys[order].astype(np.int64)) >= 0)
    assert np.array_equal(np.searchsorted(keys[order], np.arange(cs.size), side="left"), cs)


def test_morton_order_adaptive_and_batched_scenes():
    # adaptive solves (per-pass in Morton order) stop after the same iterations
    sc = scenes.puddle()
    sc.velocity = scenes.normal(5, sc.n, 0.3)
    a = _solver(sc, _lib.ORDER_CELL_KEY, diagnostics=False)
    b = _solver(sc, _lib.ORDER_MORTON, diagnostics=False)
    for _ in range(5):
        a.step(sc.dt)
        b.step(sc.dt)
        assert a.last_density_iters() == b.last_density_iters()
        assert a.last_divergence_iters() == b.last_divergence_iters()
    assert np.abs(a.positions() - b.positions()).max() < 1e-6
    # several scenes in one context: each scene keeps its own Morton keys
    blocks, eps = scenes.batched_blocks(n_scenes=3, n_min=500, n_max=2000)
    out = []
    for order in (_lib.ORDER_CELL_KEY, _lib.ORDER_MORTON):
        cfg = blocks[0].config(capacity=sum(s.n for s in blocks))
        cfg.n_scenes = 3
        cfg.slot_order = order
        s = Solver(cfg)
        s.set_boundary(blocks[0].boundary)
        s.set_fluid_batch([x.fluid for x in blocks], [x.velocity for x in blocks])
        s.set_scene_viscosity(eps)
        s.step(1e-3, 5)
        out.append((s.positions(), s.velocities()))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_morton_order_with_compensated_positions():
    # the position carries are kept per original particle, so they follow the
    # particles through either slot order
    sc = _scene("dam")

    def make(order, precision):
        cfg = sc.config(precision=precision)
        cfg.slot_order = order
        s = Solver(cfg)
        s.set_boundary(sc.boundary)
        s.set_fluid(sc.fluid, sc.velocity)
        return s

    a = make(_lib.ORDER_CELL_KEY, _lib.PRECISION_FP32_COMPENSATED)
    b = make(_lib.ORDER_MORTON, _lib.PRECISION_FP32_COMPENSATED)
    plain = make(_lib.ORDER_CELL_KEY, _lib.PRECISION_FP32)
    for s in (a, b, plain):
        s.step(sc.dt, 20)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    assert not np.array_equal(a.positions(), plain.positions())  # the carries took part

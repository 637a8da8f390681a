"""The bounds-checked build (-DDFSPH_BOUNDS_CHECK): every neighbour run of
every pass is validated against the closing entry of its cell_start array and
counted instead of read when it falls outside. Runs the step with walls, both
solvers (fixed and adaptive), batched scenes, CUDA graphs, device frames and
the adjoint through that build, and requires zero violations. This is the GPU
half of the sanitizer plan (compute-sanitizer is not used on this pool)."""
import ctypes

import numpy as np
import pytest

from water_simulation_gb300 import _build, _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib():
    return _lib.load(_build.build(checked=True))


def _ctx(lib, cfg, sc, fluids=None):
    ctx = ctypes.c_void_p()
    assert lib.dfsph_create(ctypes.byref(cfg), 0, None, ctypes.byref(ctx)) == 0
    b = np.ascontiguousarray(sc.boundary)
    assert lib.dfsph_set_boundary(ctx, b.ctypes.data_as(ctypes.c_void_p), b.shape[0], _lib.MEM_HOST) == 0
    if fluids is None:
        f = np.ascontiguousarray(sc.fluid)
        v = np.ascontiguousarray(sc.velocity)
        assert lib.dfsph_set_fluid(ctx, f.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p),
                                   f.shape[0], _lib.MEM_HOST) == 0
    else:
        counts = np.array([x.shape[0] for x in fluids], np.uint32)
        f = np.ascontiguousarray(np.concatenate(fluids))
        assert lib.dfsph_set_fluid_batch(ctx, len(counts), counts.ctypes.data_as(ctypes.c_void_p),
                                         f.ctypes.data_as(ctypes.c_void_p), None, _lib.MEM_HOST) == 0
    return ctx


def _violations(lib, ctx):
    d = ctypes.c_double()
    assert lib.dfsph_get_scalar(ctx, _lib.SCALAR_BOUNDS_VIOLATIONS, ctypes.byref(d)) == 0
    return d.value


def test_checked_build_sees_no_out_of_range_run(checked_lib):
    lib = checked_lib
    # adaptive puddle (both solvers), with a CUDA graph: device-resident loops
    sc = scenes.puddle()
    sc.velocity = scenes.normal(3, sc.n, 0.5)
    cfg = sc.config()
    cfg.use_cuda_graph = 1
    ctx = _ctx(lib, cfg, sc)
    assert lib.dfsph_step(ctx, ctypes.c_float(1e-3), 6) == 0
    fc = _lib.DfsphFrameConfig()
    lib.dfsph_frame_config_init(ctypes.byref(fc))
    subs = (ctypes.c_uint32 * 2)()
    assert lib.dfsph_step_frames(ctx, ctypes.byref(fc), 2, subs) == 0
    assert _violations(lib, ctx) == 0
    lib.dfsph_destroy(ctx)
    # batched scenes (scene-offset keys), fixed iterations
    scs, eps = scenes.batched_blocks(n_scenes=4, n_min=2000, n_max=6000)
    cfg = scs[0].config(capacity=sum(s.n for s in scs))
    cfg.n_scenes = 4
    ctx = _ctx(lib, cfg, scs[0], [s.fluid for s in scs])
    assert lib.dfsph_step(ctx, ctypes.c_float(1e-3), 5) == 0
    assert _violations(lib, ctx) == 0
    lib.dfsph_destroy(ctx)
    # the adjoint (replayed segments with per-step cell_start records)
    sc = scenes.adjoint_puddle(steps=6)
    ctx = _ctx(lib, sc.config(), sc)
    assert lib.dfsph_adjoint_forward(ctx, ctypes.c_float(sc.dt), 6, 3) == 0
    n = sc.n
    xb = np.full((n, 3), 1e-3, np.float32)
    gx = np.empty((n, 3), np.float32)
    gv = np.empty((n, 3), np.float32)
    ge = ctypes.c_double()
    assert lib.dfsph_adjoint_backward(ctx, xb.ctypes.data_as(ctypes.c_void_p), None,
                                      gx.ctypes.data_as(ctypes.c_void_p), gv.ctypes.data_as(ctypes.c_void_p),
                                      ctypes.byref(ge), _lib.MEM_HOST) == 0
    assert np.isfinite(gv).all()
    assert _violations(lib, ctx) == 0
    lib.dfsph_destroy(ctx)


def test_normal_build_reports_no_check():
    from water_simulation_gb300.solver import solver_for

    sc = scenes.falling_block(n_side=(4, 4, 4))
    s = solver_for(sc)
    assert s.scalar(_lib.SCALAR_BOUNDS_VIOLATIONS) == -1.0

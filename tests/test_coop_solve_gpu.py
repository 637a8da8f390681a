"""Adaptive solves of small scenes run as one cooperative launch per solve
(jacobi_solve_kernel: rate pass, grid barrier, stop decision, apply pass,
grid barrier, per iteration). With per-pass profiling on, the same solves run
pass by pass (the reference's loop: the host reads the error after every
iteration, dfsph.cu:296-299). Both must give the same fields and iteration
counts bit for bit, stepped plainly and inside captured frames."""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver

pytestmark = pytest.mark.gpu

ALL_CLASSES = (1 << _lib.KERNEL_CLASSES) - 1


def _solver(sc, graph=False, damping=None, precision=_lib.PRECISION_FP32):
    cfg = sc.config()
    cfg.use_cuda_graph = 1 if graph else 0
    cfg.precision = precision
    if damping is not None:
        cfg.damping = damping
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    s.set_fluid(sc.fluid, sc.velocity)
    return s


def _run(sc, profile, steps, precision=_lib.PRECISION_FP32):
    s = _solver(sc, precision=precision)
    if profile:
        s.profile_enable(ALL_CLASSES)
    iters = []
    l0 = s.kernel_launches()
    for _ in range(steps):
        s.step(sc.dt)
        iters.append((s.last_divergence_iters(), s.last_density_iters()))
    out = (s.positions(), s.velocities(), s.field(_lib.FIELD_DENSITY), iters, s.kernel_launches() - l0)
    s.close()
    return out


@pytest.mark.parametrize("sigma,precision", [(0.0, _lib.PRECISION_FP32), (0.4, _lib.PRECISION_FP32),
                                             (0.4, _lib.PRECISION_FP64)])
def test_cooperative_solve_matches_per_pass_solve(sigma, precision):
    sc = scenes.puddle()
    if sigma:
        sc.velocity = np.random.default_rng(3).normal(0, sigma, size=sc.fluid.shape).astype(np.float32)
    x0, v0, r0, it0, l0 = _run(sc, False, 12, precision)
    x1, v1, r1, it1, l1 = _run(sc, True, 12, precision)
    assert it0 == it1
    assert sum(a + b for a, b in it0) > 3 * 12  # the solves iterate
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1) and np.array_equal(r0, r1)
    # one launch per solve instead of two per iteration
    assert l0 < l1


def test_cooperative_solve_inside_device_frames():
    sc = scenes.falling_block(n_side=(16, 16, 16), velocity_sigma=0.5)
    sc.max_density_iters, sc.max_divergence_iters = 100, 100
    sc.eta_density, sc.eta_divergence = 1e-4, 1e-3
    # damping 0: device frames evaluate e^{-d dt} on the device, the host
    # loop on the host (equal only for d = 0)
    dev = _solver(sc, graph=True, damping=0.0)
    host = _solver(sc, graph=False, damping=0.0)
    host.profile_enable(ALL_CLASSES)  # pass-by-pass solves, host-chosen substeps
    sd = dev.step_frames(2)
    sh = host.step_frames(2)
    assert dev.frames_on_device()
    assert list(sd) == list(sh)
    assert np.array_equal(dev.positions(), host.positions())
    assert np.array_equal(dev.velocities(), host.velocities())


def test_cooperative_solve_batched_scenes():
    """A batched context (4 scenes of 1,000-6,000 particles) with adaptive
    solves: one cooperative launch per solve over all scenes, equal bit for
    bit to the per-pass solve."""
    scs, eps = scenes.batched_blocks(n_scenes=4, n_min=1000, n_max=6000)

    def run(profile):
        cfg = scs[0].config(capacity=sum(s.n for s in scs))
        cfg.n_scenes = 4
        cfg.max_density_iters, cfg.max_divergence_iters = 100, 100
        cfg.eta_density, cfg.eta_divergence = 1e-4, 1e-3
        s = Solver(cfg)
        s.set_boundary(scs[0].boundary)
        s.set_fluid_batch([c.fluid for c in scs], [c.velocity for c in scs])
        s.set_scene_viscosity(eps)
        if profile:
            s.profile_enable(ALL_CLASSES)
        l0 = s.kernel_launches()
        for _ in range(8):
            s.step(scs[0].dt)
        out = (s.positions(), s.velocities(), s.last_density_iters(), s.last_divergence_iters(),
               s.kernel_launches() - l0)
        s.close()
        return out

    x0, v0, d0, g0, l0 = run(False)
    x1, v1, d1, g1, l1 = run(True)
    assert (d0, g0) == (d1, g1) and d0 >= 2
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1)
    assert l0 < l1


def test_cooperative_solve_largest_blocks():
    """27,000 particles: blocks of 224 particles (121 blocks), the largest
    cooperative shape, equal bit for bit to the per-pass solve."""
    sc = scenes.falling_block(n_side=(30, 30, 30), corner=(0.2, 0.2, 0.2), velocity_sigma=0.3)
    sc.max_density_iters, sc.max_divergence_iters = 100, 100
    sc.eta_density, sc.eta_divergence = 1e-4, 1e-3
    x0, v0, r0, it0, l0 = _run(sc, False, 6)
    x1, v1, r1, it1, l1 = _run(sc, True, 6)
    assert it0 == it1 and sum(a + b for a, b in it0) > 2 * 6
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1) and np.array_equal(r0, r1)
    assert l0 < l1


def test_cooperative_solve_fixed_iterations():
    """Fixed iteration counts (eta = 0, the reference's step): the solves of a
    small scene are cooperative launches too, equal bit for bit to the
    per-pass solve, which fuses its last apply pass with the integrator."""
    sc = scenes.puddle()
    sc.velocity = np.random.default_rng(5).normal(0, 0.3, size=sc.fluid.shape).astype(np.float32)
    sc.max_density_iters, sc.max_divergence_iters, sc.eta_density, sc.eta_divergence = 4, 2, 0.0, 0.0
    x0, v0, r0, it0, l0 = _run(sc, False, 10)
    x1, v1, r1, it1, l1 = _run(sc, True, 10)
    assert it0 == it1 == [(2, 4)] * 10
    assert np.array_equal(x0, x1) and np.array_equal(v0, v1) and np.array_equal(r0, r1)
    assert l0 < l1


@pytest.mark.parametrize("graph", [False, True])
def test_grid_barrier_wait_runs_out_and_reports_a_timeout(graph):
    """The cooperative solve's grid barrier waits a bounded time. With the test
    hook the barrier waits for two blocks that never arrive, so every wait
    runs out after the limit (20 ms here): the kernel returns, the next
    synchronising call reports DFSPH_ERR_DEVICE_TIMEOUT and the context keeps
    working once a valid state is set again. No fault, trap or endless wait."""
    import time

    sc = scenes.puddle()
    sc.max_divergence_iters, sc.eta_divergence = 4, 0.0
    sc.max_density_iters, sc.eta_density = 4, 0.0
    s = _solver(sc, graph=graph)
    ref = _solver(sc, graph=graph)
    s.set_wait_limit(0.02)
    s.test_stall_waits(2)
    t0 = time.perf_counter()
    s.step(sc.dt)
    with pytest.raises(_lib.DfsphError) as e:
        s.synchronize()
    waited = time.perf_counter() - t0
    assert e.value.status == _lib.ERR_DEVICE_TIMEOUT
    assert waited < 5.0  # two solves, each gives up after about 20 ms
    # the word was cleared: the next call is clean
    s.synchronize()
    # back to normal waits: the same steps as an untouched context, bit for bit
    s.test_stall_waits(0)
    s.set_wait_limit(1.0)
    s.set_fluid(sc.fluid, sc.velocity)
    for _ in range(3):
        s.step(sc.dt)
        ref.step(sc.dt)
    s.synchronize()
    assert np.array_equal(s.positions(), ref.positions())
    assert np.array_equal(s.velocities(), ref.velocities())
    s.close()
    ref.close()


def test_wait_limit_rejects_zero():
    sc = scenes.falling_block((4, 4, 4))
    s = _solver(sc)
    with pytest.raises(_lib.DfsphError):
        s.set_wait_limit(0.0)

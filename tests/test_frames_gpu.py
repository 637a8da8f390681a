"""CFL frames stepped on the device (dfsph_step_frames) against sim_cli's host
loop (apps/sim_cli/main.cpp:171-181): next_dt from max(max |v|, 0.5) before every
substep, until the frame's remaining time is <= 1e-6 or 64 substeps.

The device path (use_cuda_graph = 1, fixed iterations) chooses each substep in
a one-thread kernel from the max |v| the integrator left on the device and
repeats the substep with a CUDA graph WHILE node; the host path reads max |v|
back before every substep. Both paths take e^{-d dt} from the same device
function (the reference's fast-math expf, dfsph_kernels.cu:347-355), so the two
agree bit for bit with and without damping, fixed or adaptive iterations.
"""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _solver(sc, graph: bool, damping: float):
    cfg = sc.config()
    cfg.use_cuda_graph = 1 if graph else 0
    cfg.damping = damping
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    s.set_fluid(sc.fluid, sc.velocity)
    return s


@pytest.fixture(scope="module")
def block():
    # a falling block with a lively velocity field: several substeps per frame
    return scenes.falling_block(n_side=(16, 16, 16), velocity_sigma=0.5)


def test_device_frames_match_host_loop_bit_for_bit(block):
    dev = _solver(block, True, 0.0)
    host = _solver(block, False, 0.0)
    sd = dev.step_frames(4)
    sh = host.step_frames(4)
    assert dev.frames_on_device() and not host.frames_on_device()
    assert list(sd) == list(sh)
    assert sd.sum() > 4  # more than one substep per frame somewhere
    assert np.array_equal(dev.positions(), host.positions())
    assert np.array_equal(dev.velocities(), host.velocities())
    assert dev.max_velocity() == host.max_velocity()


def test_device_frames_with_damping(block):
    dev = _solver(block, True, 0.5)
    host = _solver(block, False, 0.5)
    sd = dev.step_frames(3)
    sh = host.step_frames(3)
    assert list(sd) == list(sh)
    assert np.array_equal(dev.positions(), host.positions())
    assert np.array_equal(dev.velocities(), host.velocities())
    assert dev.max_velocity() == host.max_velocity()


def test_frames_continue_across_calls_and_respect_the_cap(block):
    a = _solver(block, True, 0.5)
    b = _solver(block, True, 0.5)
    s1 = np.concatenate([a.step_frames(1), a.step_frames(1)])
    s2 = b.step_frames(2)
    assert list(s1) == list(s2)
    assert np.array_equal(a.positions(), b.positions())
    fc = a.frame_config()
    fc.max_substeps_per_frame = 2
    fc.frame_dt = 1.0  # a long frame: the cap ends it
    assert list(a.step_frames(2, fc)) == [2, 2]


def test_first_frame_uses_the_velocity_floor():
    # at rest: max |v| = 0 before the first step -> next_dt(0.5, r, 1/24) =
    # 0.4 r / 0.5 for the first substep; the substep count follows
    sc = scenes.falling_block(n_side=(8, 8, 8))
    dev = _solver(sc, True, 0.5)
    host = _solver(sc, False, 0.5)
    assert list(dev.step_frames(2)) == list(host.step_frames(2))


def test_frames_reject_bad_configs(block):
    s = _solver(block, True, 0.5)
    fc = s.frame_config()
    fc.cfl_lambda = 0.0
    with pytest.raises(_lib.DfsphError):
        s.step_frames(1, fc)


def _adaptive(graph: bool, damping: float = 0.5):
    # the settled-puddle configuration: density eta 1e-4, divergence eta 1e-3,
    # at most 100 iterations each (adaptive, the reference's solver loop)
    sc = scenes.puddle()
    sc.velocity = scenes.normal(5, sc.n, 0.3)
    cfg = sc.config()
    cfg.use_cuda_graph = 1 if graph else 0
    cfg.damping = damping
    s = Solver(cfg)
    s.set_boundary(sc.boundary)
    s.set_fluid(sc.fluid, sc.velocity)
    return s


def test_adaptive_solves_in_graphs_match_the_host_loop():
    # dfsph_step with graphs runs both adaptive solves as device-resident
    # WHILE loops; the iterations, their stopping points and the state must be
    # those of the host-driven loop, bit for bit
    dev, host = _adaptive(True), _adaptive(False)
    for _ in range(3):
        dev.step(1e-3, 4)
        host.step(1e-3, 4)
        assert dev.last_density_iters() == host.last_density_iters()
        assert dev.last_divergence_iters() == host.last_divergence_iters()
    assert dev.last_density_iters() >= 2
    assert np.array_equal(dev.positions(), host.positions())
    assert np.array_equal(dev.velocities(), host.velocities())


@pytest.mark.parametrize("damping", [0.0, 0.5])
def test_adaptive_device_frames_match_the_host_loop(damping):
    dev, host = _adaptive(True, damping), _adaptive(False, damping)
    sd = dev.step_frames(3)
    sh = host.step_frames(3)
    assert dev.frames_on_device() and not host.frames_on_device()
    assert list(sd) == list(sh)
    assert np.array_equal(dev.positions(), host.positions())
    assert np.array_equal(dev.velocities(), host.velocities())

"""The FP32 divergence solver against the FP32 oracle, through the C ABI.

The reference declares max_divergence_iters / eta_divergence and never reads
them (solvers/dfsph/include/water/solvers/dfsph.h:28,30); the solver follows
its plan (docs/superpowers/plans/2026-04-24-water-simulation-v2-phase2-dfsph-
solver.md:1856-1987): rho_dot = sum m (v_i - v_j).gradW (+ walls),
kappa_v = max(0, rho_dot) alpha / dt, the apply_kappa velocity update, and the
stop rule mean(max(0, rho_dot)) < eta_div rho0 checked after every iteration.
The oracle (oracle/dfsph_oracle.cpp, divergence_solve) restates that plan.

Every step starts from identical inputs: the GPU state is handed to a fresh
FP32 oracle, and both take the step. Bit-exact: cell keys, permutation,
cell_start, per-particle candidate counts. Tolerances: density 1e-5 of rho0;
kappa_v, kappa and rho* with the bound of tests/tolerances.py at 1e-5 of rho0
(kappa_v = max(0, dt rho_dot) alpha / dt^2 has the same form as kappa);
positions 1e-6 m; velocities 2e-4 m/s.

Adaptive iteration counts must be equal. They may differ by one only where the
solver that stopped first stopped on an error within 1e-4 (relative) of the
threshold: the two sums differ by the rounding of their FP32 terms (about
1e-5 of the threshold at these sizes), which decides ties that close.
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_parity_gpu import assert_fields_close, assert_structure_equal, oracle_for
from tolerances import pressure_field_errors
from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for

pytestmark = pytest.mark.gpu


def small_dam(nx=10, ny=20, nz=10, seed=2):
    """The dam-break tank (1.6 x 1.0 x 0.6 m, walls at spacing 2r) with a
    10 x 20 x 10 column at r = 0.01 m against the x = 0 wall, dt = 1e-3 s:
    the 128k configuration's shape at 1/64 of its particles, with its fixed
    2 divergence and 4 density iterations."""
    r = 0.01
    s = 2 * r
    lo = (3.0 * s, 3.0 * s, 0.5 * (0.6 - nz * s))
    fluid = scenes.lattice_block(lo, (nx, ny, nz), s, 0.05 * r, seed)
    dlo, dhi = (0.0, 0.0, 0.0), (1.6, 1.0, 0.6)
    return scenes.Scene(f"small_dam_{fluid.shape[0]}", r, dlo, dhi, fluid, np.zeros_like(fluid),
                        scenes.sample_aabb_boundary(dlo, dhi, s, 3), dt=1e-3, steps=20, viscosity=0.01,
                        max_density_iters=4, max_divergence_iters=2)


def kappa_v_error(gpu, ora, dt):
    kv, kvo = gpu.field(_lib.FIELD_KAPPA_V), ora.field(O.F_KAPPA_V)
    # kappa_v in the role of kappa: rho* is not involved, pass kappa_v twice
    return pressure_field_errors(kv, kv, kvo, kv, ora.field(O.F_ALPHA), dt)[1]


def test_fixed_divergence_iterations_match_the_oracle_every_step():
    sc = small_dam()
    gpu = solver_for(sc, diagnostics=True)
    worst = 0.0
    moving = False
    for k in range(20):
        x, v = gpu.positions(), gpu.velocities()
        ora = oracle_for(sc, gpu, x, v)
        gpu.step(sc.dt)
        ora.step(sc.dt)
        assert gpu.last_divergence_iters() == ora.scalar(3) == 2
        assert gpu.last_density_iters() == ora.last_density_iters() == 4
        assert_structure_equal(gpu, ora, f"step {k}")
        assert_fields_close(gpu, ora, f"step {k}", dt=sc.dt)
        e = kappa_v_error(gpu, ora, sc.dt)
        assert e < 1e-5, (k, e)
        worst = max(worst, e)
        moving = moving or float(np.abs(ora.field(O.F_KAPPA_V)).max()) > 0
        ora.close()
    assert moving  # the divergence solver did some work
    print(f"small dam, 2 divergence + 4 density iterations: kappa_v error {worst:.2e} (of alpha rho0 / dt^2)")


def _tie(err_a, thr):
    return abs(err_a - thr) <= 1e-4 * thr


def test_adaptive_divergence_and_density_stop_rules_match_the_oracle():
    """The settled-puddle configuration (eta_div 1e-3, eta_density 1e-4, at most
    100 iterations each) from a stirred start, 30 steps; per step the
    divergence and density iteration counts and the fields against the oracle
    from identical inputs."""
    sc = scenes.puddle()
    sc.velocity = scenes.normal(5, sc.n, 0.3)
    gpu = solver_for(sc, diagnostics=True)
    thr_div = float(np.float32(np.float32(sc.eta_divergence) * np.float32(1000.0)))
    thr_den = float(np.float32(np.float32(sc.eta_density) * np.float32(1000.0)))
    counts = []
    ties = 0
    for k in range(30):
        x, v = gpu.positions(), gpu.velocities()
        ora = oracle_for(sc, gpu, x, v)
        gpu.step(sc.dt)
        ora.step(sc.dt)
        gd, od = gpu.last_divergence_iters(), int(ora.scalar(3))
        gr, orr = gpu.last_density_iters(), ora.last_density_iters()
        counts.append((gd, od, gr, orr))
        for g_it, o_it, g_err, o_err, thr in ((gd, od, gpu.scalar(_lib.SCALAR_DIVERGENCE_ERROR), ora.scalar(5),
                                              thr_div),
                                             (gr, orr, gpu.scalar(_lib.SCALAR_DENSITY_ERROR), ora.scalar(4),
                                              thr_den)):
            if g_it != o_it:
                first = g_err if g_it < o_it else o_err
                assert abs(g_it - o_it) == 1 and _tie(first, thr), (k, g_it, o_it, g_err, o_err, thr)
                ties += 1
        assert_structure_equal(gpu, ora, f"step {k}")
        if (gd, gr) == (od, orr):
            assert_fields_close(gpu, ora, f"step {k}", dt=sc.dt)
            assert kappa_v_error(gpu, ora, sc.dt) < 1e-5, k
        ora.close()
    total = np.array(counts)
    # both solvers iterate beyond their minimum (1 divergence, 2 density) somewhere
    assert total[:, 0].max() > 1 and total[:, 2].max() > 2
    assert ties <= 2
    print(f"puddle adaptive: divergence iterations {total[:, 0].sum()} (oracle {total[:, 1].sum()}), density "
          f"{total[:, 2].sum()} (oracle {total[:, 3].sum()}), ties {ties}")

"""The reference's own CUDA kernels (oracle/_ref fatbins, restated host
orchestration in oracle/ref_runner.cu) against this project's CUDA step and the
CPU oracle, on identical seeded inputs with fixed iterations.

Bit-exact: cell keys, sorted permutation, cell_start of the fluid and boundary
grids. Fields: the reference is built with -use_fast_math and its XSPH pass
races (solvers/dfsph/src/dfsph_kernels.cu:327,338-340); the tolerances below
are set from that (relative density 1e-5 of rho0, boundary mass 1e-5,
positions 1e-6 m after one step).
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import reference as R
from tolerances import assert_pressure_fields_close
from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.available(), reason="reference kernels (oracle/_ref) not built here")]


def make(sc):
    gpu = solver_for(sc, diagnostics=True)
    inv = gpu.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    ref = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary if sc.nb else None)
    ora = O.Oracle(ocfg, sc.fluid, sc.velocity, sc.boundary if sc.nb else None, precision=32)
    return gpu, ref, ora


@pytest.mark.parametrize("dims,seed,visc", [((8, 8, 8), 41, 0.0), ((12, 10, 8), 42, 0.01)])
def test_reference_structure_and_fields_one_step(dims, seed, visc):
    sc = scenes.falling_block(dims, seed=seed, velocity_sigma=0.1)
    sc.viscosity = visc
    gpu, ref, ora = make(sc)
    # boundary grid + Akinci mass at construction (dfsph.cu:90-99)
    assert np.array_equal(ref.field(14), gpu.field(_lib.FIELD_BOUNDARY_SORTED_INDEX))
    assert np.array_equal(ref.field(13), gpu.field(_lib.FIELD_BOUNDARY_CELL_START))
    mb_ref = ref.field(11).astype(np.float64)
    assert np.abs(gpu.field(_lib.FIELD_BOUNDARY_MASS) - mb_ref).max() / mb_ref.max() < 1e-5
    assert np.abs(ora.field(O.F_BOUNDARY_MASS) - mb_ref).max() / mb_ref.max() < 1e-5
    ref.step(sc.dt)
    gpu.step(sc.dt)
    ora.step(sc.dt)
    for fid_ref, fid_gpu, fid_ora in ((6, _lib.FIELD_CELL_KEY, O.F_CELL_KEY),
                                      (7, _lib.FIELD_SORTED_INDEX, O.F_SORTED_INDEX),
                                      (8, _lib.FIELD_CELL_START, O.F_CELL_START)):
        r = ref.field(fid_ref)
        assert np.array_equal(r, gpu.field(fid_gpu)), fid_gpu
        assert np.array_equal(r, ora.field(fid_ora)), fid_ora
    rho_ref = ref.field(2).astype(np.float64)
    assert np.abs(gpu.field(_lib.FIELD_DENSITY) - rho_ref).max() / 1000.0 < 1e-5
    assert np.abs(ora.field(O.F_DENSITY) - rho_ref).max() / 1000.0 < 1e-5
    a_ref = ref.field(3).astype(np.float64)
    assert (np.abs(gpu.field(_lib.FIELD_ALPHA) - a_ref) / np.maximum(np.abs(a_ref), 1e-12)).max() < 1e-4
    x_ref = ref.field(0).astype(np.float64)
    assert np.abs(gpu.positions() - x_ref).max() < 1e-6
    assert np.abs(ora.field(O.F_POSITION) - x_ref).max() < 1e-6
    v_ref = ref.field(1).astype(np.float64)
    assert np.abs(gpu.velocities() - v_ref).max() < 2e-4
    assert gpu.max_velocity() == pytest.approx(ref.max_velocity(), rel=1e-4)
    assert ref.last_density_iters() == gpu.last_density_iters() == sc.max_density_iters
    # the last Jacobi iteration's kappa and rho* (dfsph_kernels.cu:226-231)
    assert_pressure_fields_close(gpu.field(_lib.FIELD_KAPPA), gpu.field(_lib.FIELD_DENSITY_ADV), ref.field(4),
                                 ref.field(5), a_ref, sc.dt, 2e-5)


def test_reference_structure_every_step_20_steps():
    sc = scenes.falling_block((10, 10, 10), seed=43, velocity_sigma=0.2)
    sc.viscosity = 0.0
    gpu = solver_for(sc, diagnostics=True)
    inv = gpu.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    for k in range(20):
        x, v = gpu.positions(), gpu.velocities()
        ref = R.ReferenceRun(ocfg, x, v, sc.boundary)
        ref.step(sc.dt)
        gpu.step(sc.dt)
        for fid_ref, fid_gpu in ((6, _lib.FIELD_CELL_KEY), (7, _lib.FIELD_SORTED_INDEX), (8, _lib.FIELD_CELL_START)):
            assert np.array_equal(ref.field(fid_ref), gpu.field(fid_gpu)), (k, fid_gpu)
        assert np.abs(gpu.positions() - ref.field(0)).max() < 1e-6
        ref.close()


def test_reference_adaptive_density_solver_iterations():
    # eta > 0: both stop when the mean error is below eta rho0, checked from iter 2
    sc = scenes.falling_block((10, 10, 10), seed=44)
    sc.max_density_iters = 30
    sc.eta_density = 1e-3
    gpu, ref, _ = make(sc)
    for _ in range(30):
        ref.step(sc.dt)
        gpu.step(sc.dt)
    assert abs(ref.last_density_iters() - gpu.last_density_iters()) <= 1
    assert np.abs(gpu.positions() - ref.field(0)).max() < 1e-4


def test_reference_run_to_run_spread_with_xsph():
    """The reference's in-place XSPH races: two identical reference runs may differ.
    Their spread bounds what velocity parity can mean; this records it."""
    sc = scenes.falling_block((10, 10, 10), seed=45, velocity_sigma=0.3)
    sc.viscosity = 0.05
    gpu, ref, _ = make(sc)
    ocfg = O.config_from(sc.config(), stencil_inv_cell=gpu.scalar(_lib.SCALAR_STENCIL_INV_CELL))
    ref2 = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary)
    for _ in range(20):
        ref.step(sc.dt)
        ref2.step(sc.dt)
        gpu.step(sc.dt)
    spread = np.abs(ref.field(1) - ref2.field(1)).max()
    diff = np.abs(gpu.velocities() - ref.field(1)).max()
    print(f"reference run-to-run velocity spread {spread:.3e}, GPU vs reference {diff:.3e}")
    assert diff < max(1e-2, 10 * spread)


def test_reference_dam_break_1m_one_step():
    """The largest configuration: the 1M-particle dam break (766,098 wall
    particles, 8.0 M cells), one reference step. Cell keys, permutation and
    cell_start of the fluid and wall grids bit for bit against the
    reference's own kernels; neighbour counts bit for bit against the oracle;
    density, positions and velocities within the one-step tolerances above."""
    sc = scenes.dam_break(scale=2, reference_mode=True)
    gpu = solver_for(sc, diagnostics=True)
    inv = gpu.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    ref = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary)
    assert np.array_equal(ref.field(14), gpu.field(_lib.FIELD_BOUNDARY_SORTED_INDEX))
    assert np.array_equal(ref.field(13), gpu.field(_lib.FIELD_BOUNDARY_CELL_START))
    ref.step(sc.dt)
    gpu.step(sc.dt)
    for fid_ref, fid_gpu in ((6, _lib.FIELD_CELL_KEY), (7, _lib.FIELD_SORTED_INDEX), (8, _lib.FIELD_CELL_START)):
        assert np.array_equal(ref.field(fid_ref), gpu.field(fid_gpu)), fid_gpu
    rho_ref = ref.field(2).astype(np.float64)
    assert np.abs(gpu.field(_lib.FIELD_DENSITY) - rho_ref).max() / 1000.0 < 1e-5
    assert np.abs(gpu.positions() - ref.field(0).astype(np.float64)).max() < 1e-6
    assert np.abs(gpu.velocities() - ref.field(1).astype(np.float64)).max() < 2e-4
    assert ref.last_density_iters() == gpu.last_density_iters() == sc.max_density_iters
    ref.close()
    # neighbour counts of the step just taken, against the oracle's
    ora = O.Oracle(ocfg, sc.fluid, sc.velocity, sc.boundary, precision=32)
    ora.step(sc.dt)
    assert np.array_equal(ora.field(O.F_NBR_FLUID), gpu.field(_lib.FIELD_NBR_FLUID))
    assert np.array_equal(ora.field(O.F_NBR_BOUNDARY), gpu.field(_lib.FIELD_NBR_BOUNDARY))


def test_reference_dam_break_128k_every_step_50_steps():
    """The dam-break configuration at 128,000 particles (193,458 wall
    particles, 4 fixed density iterations, no divergence solver: the
    reference's step), 50 steps. Before every step the GPU state is handed to
    a fresh run of the reference's own kernels, and both take the step: cell
    keys, permutation and cell_start bit for bit; density, kappa and rho* within
    2e-5 of rho0 (kappa times alpha / dt^2), positions within 2e-6 m, velocities
    within 2e-3 m/s (the reference's XSPH races), every step."""
    sc = scenes.dam_break(scale=1, reference_mode=True)
    gpu = solver_for(sc, diagnostics=True)
    inv = gpu.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    ocfg = O.config_from(sc.config(), stencil_inv_cell=inv)
    worst = np.zeros(5)
    for k in range(50):
        x, v = gpu.positions(), gpu.velocities()
        ref = R.ReferenceRun(ocfg, x, v, sc.boundary)
        ref.step(sc.dt)
        gpu.step(sc.dt)
        for fid_ref, fid_gpu in ((6, _lib.FIELD_CELL_KEY), (7, _lib.FIELD_SORTED_INDEX), (8, _lib.FIELD_CELL_START)):
            assert np.array_equal(ref.field(fid_ref), gpu.field(fid_gpu)), (k, fid_gpu)
        assert ref.last_density_iters() == gpu.last_density_iters() == 4
        e_rho = np.abs(gpu.field(_lib.FIELD_DENSITY) - ref.field(2).astype(np.float64)).max() / 1000.0
        e_x = np.abs(gpu.positions() - ref.field(0).astype(np.float64)).max()
        e_v = np.abs(gpu.velocities() - ref.field(1).astype(np.float64)).max()
        e_adv, e_kap = assert_pressure_fields_close(gpu.field(_lib.FIELD_KAPPA), gpu.field(_lib.FIELD_DENSITY_ADV),
                                                    ref.field(4), ref.field(5), ref.field(3), sc.dt, 2e-5,
                                                    f"step {k}")
        assert e_rho < 2e-5 and e_x < 2e-6 and e_v < 2e-3, (k, e_rho, e_x, e_v)
        worst = np.maximum(worst, [e_rho, e_adv, e_kap, e_x, e_v])
        ref.close()
    print("dam 128k, 50 re-fed steps against the reference's kernels: max |drho|/rho0 %.2e, rho* %.2e, "
          "kappa %.2e, |dx| %.2e m, |dv| %.2e m/s" % tuple(worst))

"""dfsph_save_state / dfsph_load_state: a run saved after k steps and resumed
in a fresh context continues exactly (the sorted order is canonical and no
physics kernel depends on the order of arrival), for FP32, FP64 and batched
scenes; mismatched files are refused."""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import Solver, solver_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [_lib.PRECISION_FP32, _lib.PRECISION_FP64,
                                       _lib.PRECISION_FP32_COMPENSATED])
def test_resume_continues_bit_for_bit(tmp_path, precision):
    sc = scenes.falling_block(n_side=(12, 12, 12), velocity_sigma=0.3)
    a = solver_for(sc, precision=precision)
    a.step(sc.dt, 5)
    path = tmp_path / "s.bin"
    a.save_state(path)
    a.step(sc.dt, 7)
    b = Solver(sc.config(precision=precision))
    b.load_state(path)
    b.step(sc.dt, 7)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())


def test_compensated_state_loads_into_other_precisions(tmp_path):
    # the position carries are the compensated form's alone: a plain FP32
    # context skips them and steps as from the same positions and velocities
    sc = scenes.falling_block(n_side=(10, 10, 10), velocity_sigma=0.3)
    a = solver_for(sc, precision=_lib.PRECISION_FP32_COMPENSATED)
    a.step(sc.dt, 5)
    path = tmp_path / "c.bin"
    a.save_state(path)
    b = Solver(sc.config(precision=_lib.PRECISION_FP32))
    b.load_state(path)
    c = solver_for(sc, precision=_lib.PRECISION_FP32)
    c.set_fluid(a.positions(), a.velocities())
    b.step(sc.dt, 3)
    c.step(sc.dt, 3)
    assert np.array_equal(b.positions(), c.positions())
    d = Solver(sc.config(precision=_lib.PRECISION_FP64))
    d.load_state(path)
    d.step(sc.dt, 1)
    assert np.isfinite(d.positions()).all()


def test_resume_batched_scenes(tmp_path):
    scs, eps = scenes.batched_blocks(n_scenes=3, n_min=2000, n_max=4000)
    cfg = scs[0].config(capacity=sum(s.n for s in scs))
    cfg.n_scenes = 3
    a = Solver(cfg)
    a.set_boundary(scs[0].boundary)
    a.set_fluid_batch([s.fluid for s in scs], [s.velocity for s in scs])
    a.step(1e-3, 3)
    a.save_state(tmp_path / "b.bin")
    a.step(1e-3, 4)
    b = Solver(cfg)
    b.load_state(tmp_path / "b.bin")
    b.step(1e-3, 4)
    assert np.array_equal(a.positions(), b.positions())


def test_load_refuses_mismatched_files(tmp_path):
    sc = scenes.falling_block(n_side=(6, 6, 6))
    a = solver_for(sc)
    a.save_state(tmp_path / "a.bin")
    (tmp_path / "junk.bin").write_bytes(b"not a state file at all, really")
    with pytest.raises(_lib.DfsphError):
        a.load_state(tmp_path / "junk.bin")
    with pytest.raises(_lib.DfsphError):
        a.load_state(tmp_path / "missing.bin")
    cfg = sc.config()
    cfg.n_scenes = 2
    b = Solver(cfg)
    with pytest.raises(_lib.DfsphError):
        b.load_state(tmp_path / "a.bin")

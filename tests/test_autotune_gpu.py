"""dfsph_autotune: picks threads per block of the neighbour passes from timed
trial steps and leaves the state as it found it. With fixed iteration counts no
result depends on the block size, so a tuned context steps bit for bit like an
untuned one."""
import numpy as np
import pytest

from water_simulation_gb300 import _lib, scenes
from water_simulation_gb300.solver import solver_for

pytestmark = pytest.mark.gpu


def test_autotune_restores_state_and_changes_no_result():
    sc = scenes.falling_block(n_side=(20, 20, 20), velocity_sigma=0.2)
    a, b = solver_for(sc), solver_for(sc)
    a.step(sc.dt, 3)
    b.step(sc.dt, 3)
    x_before = a.positions()
    chosen = a.autotune(sc.dt, 2)
    assert np.array_equal(a.positions(), x_before)
    for k in ("density_alpha", "pressure_rate", "pressure_apply", "forces_xsph"):
        assert chosen[k] in (64, 128, 256)
    assert a.block_sizes() == chosen
    a.step(sc.dt, 5)
    b.step(sc.dt, 5)
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())


def test_autotune_needs_state():
    sc = scenes.falling_block(n_side=(4, 4, 4))
    s = solver_for(sc)
    with pytest.raises(_lib.DfsphError):
        s.autotune(0.0, 1)

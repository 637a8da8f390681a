"""This project's CUDA step against the reference goldens (tests/golden/),
through the C ABI: structure bit-exact per step, fields with the tolerances of
tests/test_golden.py, and the pressure fields of the last Jacobi iteration
(kappa, rho*) with the tolerances of tests/tolerances.py: rho* within 2e-5 of
rho0, as the density (the oracle meets the goldens to 1e-6)."""
import numpy as np
import pytest

from test_golden import GOLDEN, load_case
from tolerances import assert_pressure_fields_close
from water_simulation_gb300 import _lib
from water_simulation_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", GOLDEN, ids=[p.rsplit("/", 1)[-1] for p in GOLDEN])
def test_cuda_step_matches_reference_goldens(path):
    d, c = load_case(path)
    cfg = _lib.DfsphConfig()
    _lib.load().dfsph_config_init(cfg)
    for name, _ in _lib.DfsphConfig._fields_:
        if hasattr(c, name):
            v = getattr(c, name)
            if hasattr(v, "__len__"):
                getattr(cfg, name)[:] = list(v)
            else:
                setattr(cfg, name, v)
    cfg.capacity = d["fluid"].shape[0]
    cfg.boundary_capacity = max(d["boundary"].shape[0], 1)
    cfg.record_diagnostics = 1
    s = Solver(cfg)
    assert s.scalar(_lib.SCALAR_STENCIL_INV_CELL) == float(d["cfg_stencil_inv_cell"])
    if d["boundary"].shape[0]:
        s.set_boundary(d["boundary"])
        assert np.array_equal(s.field(_lib.FIELD_BOUNDARY_SORTED_INDEX), d["boundary_sorted_index"])
        mb = d["boundary_mass"].astype(np.float64)
        assert np.abs(s.field(_lib.FIELD_BOUNDARY_MASS) - mb).max() / mb.max() < 1e-5
    s.set_fluid(d["fluid"], d["velocity0"])
    vtol = 2e-3 if float(d["cfg_viscosity"]) > 0 else 5e-4
    ptol = 2e-5
    worst = [0.0, 0.0]
    for k in range(d["position"].shape[0]):
        s.step(float(d["dt"]))
        assert np.array_equal(s.field(_lib.FIELD_CELL_KEY), d["cell_key"][k]), k
        assert np.array_equal(s.field(_lib.FIELD_SORTED_INDEX), d["sorted_index"][k]), k
        assert np.array_equal(s.field(_lib.FIELD_CELL_START), d["cell_start"][k]), k
        assert s.last_density_iters() == int(d["density_iters"][k])
        assert np.abs(s.field(_lib.FIELD_DENSITY) - d["density"][k]).max() / 1000.0 < 2e-5, k
        assert np.abs(s.positions() - d["position"][k]).max() < 2e-6, k
        assert np.abs(s.velocities() - d["velocity"][k]).max() < vtol, k
        e = assert_pressure_fields_close(s.field(_lib.FIELD_KAPPA), s.field(_lib.FIELD_DENSITY_ADV), d["kappa"][k],
                                         d["density_adv"][k], d["alpha"][k], float(d["dt"]), ptol, f"step {k}")
        worst = [max(worst[0], e[0]), max(worst[1], e[1])]
    print(f"{path.rsplit('/', 1)[-1]}: rho* {worst[0]:.2e}, kappa {worst[1]:.2e} (of rho0, alpha rho0 / dt^2)")

"""Generate the golden vectors in this directory from the reference's own kernels.

Runs on a GPU machine that has oracle/_ref/*.fatbin (the reference kernels of
solvers/dfsph/src/dfsph_kernels.cu and core/src/cell_grid.cu compiled from the
reference sources by oracle/build.py) and drives them with oracle/ref_runner.cu
(the restated DFSPHSolver / CellGrid host orchestration). The inputs are the
seeded scenes below; the outputs of every step are written as compressed npz.

    python tests/golden/make_golden.py [out_dir]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import reference as R  # noqa: E402
from water_simulation_gb300 import _lib, scenes  # noqa: E402
from water_simulation_gb300.solver import Solver  # noqa: E402


def golden_scenes():
    """(name, scene, steps) of every golden case."""
    out = []
    b = scenes.falling_block((8, 8, 8), seed=31, radius=0.02, corner=(0.3, 0.35, 0.3), velocity_sigma=0.05)
    b.viscosity = 0.0
    b.max_density_iters = 4
    out.append(("block512_noxsph", b, 10))
    b2 = scenes.falling_block((8, 8, 8), seed=32, radius=0.02, corner=(0.3, 0.35, 0.3))
    b2.viscosity = 0.01
    b2.max_density_iters = 4
    out.append(("block512_xsph", b2, 10))
    rng = np.random.default_rng(77)
    c = scenes.falling_block((4, 4, 4), seed=1, radius=0.02)
    pts = rng.uniform(-0.1, 1.1, size=(2000, 3)).astype(np.float32)
    pts[:50] = np.float32([0.5, 0.5, 0.5])
    c.fluid, c.velocity = pts, np.zeros_like(pts)
    c.viscosity = 0.0
    c.max_density_iters = 2
    out.append(("cloud2000", c, 1))
    return out


def run_case(name, sc, steps):
    cfg = sc.config()
    probe = Solver(cfg)
    inv = probe.scalar(_lib.SCALAR_STENCIL_INV_CELL)
    probe.close()
    ocfg = O.config_from(cfg, stencil_inv_cell=inv)
    ref = R.ReferenceRun(ocfg, sc.fluid, sc.velocity, sc.boundary if sc.nb else None)
    rec = {k: [] for k in ("position", "velocity", "density", "alpha", "kappa", "density_adv", "cell_key",
                           "sorted_index", "cell_start", "max_velocity", "density_iters")}
    for _ in range(steps):
        ref.step(sc.dt)
        rec["position"].append(ref.field(0))
        rec["velocity"].append(ref.field(1))
        rec["density"].append(ref.field(2))
        rec["alpha"].append(ref.field(3))
        rec["kappa"].append(ref.field(4))
        rec["density_adv"].append(ref.field(5))
        rec["cell_key"].append(ref.field(6))
        rec["sorted_index"].append(ref.field(7))
        rec["cell_start"].append(ref.field(8))
        rec["max_velocity"].append(ref.max_velocity())
        rec["density_iters"].append(ref.last_density_iters())
    arrays = {k: np.asarray(v) for k, v in rec.items()}
    cfg_vals = {f: np.asarray(getattr(ocfg, f)) for f, _ in O.OracleConfig._fields_}
    return dict(
        fluid=sc.fluid, velocity0=sc.velocity, boundary=sc.boundary, dt=np.float32(sc.dt),
        boundary_mass=ref.field(11), boundary_cell_start=ref.field(13), boundary_sorted_index=ref.field(14),
        particle_mass=np.float32(ref.particle_mass()), **{"cfg_" + k: v for k, v in cfg_vals.items()}, **arrays)


def main(out_dir=HERE):
    os.makedirs(out_dir, exist_ok=True)
    for name, sc, steps in golden_scenes():
        data = run_case(name, sc, steps)
        path = os.path.join(out_dir, f"ref_{name}.npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)

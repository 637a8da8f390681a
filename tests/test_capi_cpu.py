"""The C ABI library on a machine without a GPU: it loads, exports every entry
point include/dfsph_gb300.h declares, and its host-side pieces (defaults,
geometry, boundary sampler, argument checks) agree with the oracle. No call
here launches device work."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available
from oracle import oracle as O
from water_simulation_gb300 import _lib


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(dfsph_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert "dfsph_step" in names and "dfsph_create" in names
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert names <= set(_lib.exported_names()), names - set(_lib.exported_names())


def test_config_defaults_match_reference_config():
    # DFSPHSolver::Config (solvers/dfsph/include/water/solvers/dfsph.h:19-33)
    c = _lib.DfsphConfig()
    assert _lib.load().dfsph_config_init(ctypes.byref(c)) == 0
    assert c.rest_density == 1000.0
    assert c.particle_radius == np.float32(0.0015)
    assert c.smoothing_length == np.float32(0.003)
    assert c.viscosity == np.float32(1e-3)
    assert c.damping == np.float32(0.5)
    assert list(c.gravity) == [0.0, np.float32(-9.81), 0.0]
    assert c.max_density_iters == 100 and c.max_divergence_iters == 100
    assert c.eta_density == np.float32(1e-3) and c.eta_divergence == np.float32(1e-3)
    assert list(c.domain_min) == [0, 0, 0] and list(c.domain_max) == [1, 1, 1]


def test_frame_config_defaults_match_sim_cli():
    # TimeStepper::Config (core/include/water/core/timestep.h:10-15) and
    # sim_cli's 0.5 m/s floor and 64-substep cap (apps/sim_cli/main.cpp:172,175)
    fc = _lib.DfsphFrameConfig()
    assert _lib.load().dfsph_frame_config_init(ctypes.byref(fc)) == 0
    assert fc.frame_dt == np.float32(1 / 24) and fc.stepper_frame_dt == np.float32(1 / 24)
    assert fc.dt_max == np.float32(1 / 24) and fc.cfl_lambda == np.float32(0.4)
    assert fc.max_substeps == 16 and fc.min_velocity == np.float32(0.5) and fc.max_substeps_per_frame == 64
    lib = _lib.load()
    assert lib.dfsph_step_frames(None, ctypes.byref(fc), 1, None) == _lib.ERR_INVALID_ARGUMENT
    assert lib.dfsph_adjoint_forward(None, ctypes.c_float(1e-3), 1, 1) == _lib.ERR_INVALID_ARGUMENT
    assert lib.dfsph_adjoint_backward(None, None, None, None, None, None, 0) == _lib.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("r,dmax", [(0.01, (1, 1, 1)), (0.005, (1.6, 1.0, 0.6)), (0.0025, (1.6, 1.0, 0.6)),
                                    (0.0015, (1, 1, 1)), (0.012, (1, 1, 1))])
def test_grid_geometry_matches_oracle(r, dmax):
    lib = _lib.load()
    c = _lib.DfsphConfig()
    lib.dfsph_config_init(ctypes.byref(c))
    c.particle_radius = r
    c.smoothing_length = np.float32(2 * np.float32(r))
    c.domain_max[:] = list(dmax)
    o = (ctypes.c_float * 3)()
    d = (ctypes.c_int * 3)()
    assert lib.dfsph_grid_geometry(ctypes.byref(c), o, d) == 0
    og, dg = O.grid_geometry(O.config_from(c))
    assert tuple(d) == dg
    assert tuple(o) == og


@pytest.mark.parametrize("spacing,layers,hi", [(0.02, 3, (1, 1, 1)), (0.01, 3, (1.6, 1.0, 0.6)),
                                               (0.05, 1, (1, 1, 1)), (0.024, 3, (1, 1, 1)),
                                               (0.005, 3, (1.6, 1.0, 0.6))])
def test_boundary_sampler_bit_exact_vs_oracle(spacing, layers, hi):
    from water_simulation_gb300.scenes import sample_aabb_boundary

    a = sample_aabb_boundary((0, 0, 0), hi, spacing, layers)
    b = O.sample_aabb_boundary((0, 0, 0), hi, spacing, layers)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_boundary_sampler_rejects_bad_arguments():
    lib = _lib.load()
    lo, hi = _lib.fvec3((0, 0, 0)), _lib.fvec3((1, 1, 1))
    assert lib.dfsph_sample_aabb_boundary(lo, hi, ctypes.c_float(0.0), 3, None, 0) < 0
    assert lib.dfsph_sample_aabb_boundary(lo, hi, ctypes.c_float(0.1), -1, None, 0) < 0
    assert lib.dfsph_sample_aabb_boundary(lo, hi, ctypes.c_float(0.1), 0, None, 0) == 0


def test_create_rejects_invalid_configs_without_touching_a_device():
    lib = _lib.load()
    out = ctypes.c_void_p()
    c = _lib.DfsphConfig()
    lib.dfsph_config_init(ctypes.byref(c))
    c.smoothing_length = 0.0
    assert lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT
    assert b"smoothing_length" in lib.dfsph_last_error(None)
    lib.dfsph_config_init(ctypes.byref(c))
    c.domain_max[0] = -1.0
    assert lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT
    lib.dfsph_config_init(ctypes.byref(c))
    c.precision = 7
    assert lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT
    assert b"precision" in lib.dfsph_last_error(None)
    c.precision = _lib.PRECISION_FP32_COMPENSATED + 1
    assert lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT
    assert b"precision" in lib.dfsph_last_error(None)
    lib.dfsph_config_init(ctypes.byref(c))
    c.smoothing_length = 1e-6  # far more than 2^32 cells
    assert lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT
    assert not out.value
    assert lib.dfsph_create(None, 0, None, ctypes.byref(out)) == _lib.ERR_INVALID_ARGUMENT


def test_compensated_precision_passes_config_validation():
    lib = _lib.load()
    out = ctypes.c_void_p()
    c = _lib.DfsphConfig()
    lib.dfsph_config_init(ctypes.byref(c))
    c.precision = _lib.PRECISION_FP32_COMPENSATED
    rc = lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out))
    if rc != 0:
        assert b"precision" not in lib.dfsph_last_error(None)
    else:
        lib.dfsph_destroy(out)


def test_null_context_calls_fail_cleanly():
    lib = _lib.load()
    assert lib.dfsph_step(None, ctypes.c_float(1e-3), 1) == _lib.ERR_INVALID_ARGUMENT
    assert lib.dfsph_set_fluid(None, None, None, 0, 0) == _lib.ERR_INVALID_ARGUMENT
    d = ctypes.c_double()
    assert lib.dfsph_get_scalar(None, 0, ctypes.byref(d)) == _lib.ERR_INVALID_ARGUMENT
    lib.dfsph_destroy(None)
    assert lib.dfsph_status_string(_lib.ERR_OUT_OF_RANGE) == b"out of range"


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_create_without_device_reports_no_device():
    lib = _lib.load()
    out = ctypes.c_void_p()
    c = _lib.DfsphConfig()
    lib.dfsph_config_init(ctypes.byref(c))
    c.capacity = 10
    st = lib.dfsph_create(ctypes.byref(c), 0, None, ctypes.byref(out))
    assert st == _lib.ERR_NO_DEVICE
    assert not out.value


def test_python_wrapper_raises_on_missing_library(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        _lib.load(str(tmp_path / "nope.so"))


def header_defines():
    txt = open(os.path.join(ROOT, "include", "dfsph_gb300.h")).read()
    return {k: int(v) for k, v in re.findall(r"#define\s+(DFSPH_[A-Z0-9_]+)\s+(-?\d+)\b", txt)}


def test_binding_constants_match_the_header():
    d = header_defines()
    assert d["DFSPH_PRECISION_FP32_COMPENSATED"] == _lib.PRECISION_FP32_COMPENSATED
    checked = 0
    for name, value in d.items():
        py = name[len("DFSPH_"):]
        if hasattr(_lib, py):
            assert getattr(_lib, py) == value, name
            checked += 1
    assert checked >= 20

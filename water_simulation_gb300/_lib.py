"""ctypes binding of libdfsph_gb300.so (the C ABI of include/dfsph_gb300.h).

The library is the product path: there is no Python or CPU fallback. Loading
fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes
import os

from ._build import LIB_PATH

# status codes (include/dfsph_gb300.h)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_RANGE = 3
ERR_STATE = 4
ERR_DEVICE_TIMEOUT = 5
ERR_NONFINITE = 6
ERR_NO_DEVICE = 7
ERR_IO = 8

MEM_HOST = 0
MEM_DEVICE = 1

PRECISION_FP32 = 0
PRECISION_FP32_KAHAN = 1
PRECISION_FP64 = 2
PRECISION_FP32_COMPENSATED = 3

ORDER_CELL_KEY = 0
ORDER_MORTON = 1

FIELD_POSITION = 0
FIELD_VELOCITY = 1
FIELD_DENSITY = 2
FIELD_ALPHA = 3
FIELD_KAPPA = 4
FIELD_DENSITY_ADV = 5
FIELD_CELL_KEY = 6
FIELD_SORTED_INDEX = 7
FIELD_CELL_START = 8
FIELD_NBR_FLUID = 9
FIELD_NBR_BOUNDARY = 10
FIELD_BOUNDARY_MASS = 11
FIELD_KAPPA_V = 12
FIELD_BOUNDARY_CELL_START = 13
FIELD_BOUNDARY_SORTED_INDEX = 14
FIELD_NBR_SIGNATURE = 15

SCALAR_MAX_VELOCITY = 0
SCALAR_PARTICLE_MASS = 1
SCALAR_LAST_DENSITY_ITERS = 2
SCALAR_LAST_DIVERGENCE_ITERS = 3
SCALAR_DENSITY_ERROR = 4
SCALAR_DIVERGENCE_ERROR = 5
SCALAR_TOTAL_CELLS = 6
SCALAR_STENCIL_INV_CELL = 7
SCALAR_FLUID_COUNT = 8
SCALAR_BOUNDARY_COUNT = 9
SCALAR_KERNEL_LAUNCHES = 10
SCALAR_FLAGS = 11
SCALAR_ACTIVE_BOUNDARY = 12
SCALAR_FRAME_GRAPH = 13
SCALAR_BOUNDS_VIOLATIONS = 14
SCALAR_COOP_SOLVES = 15

KERNEL_GRID_COUNT = 0
KERNEL_GRID_SCAN = 1
KERNEL_GRID_SCATTER = 2
KERNEL_GRID_REORDER = 3
KERNEL_DENSITY_ALPHA = 4
KERNEL_PRESSURE_RATE = 5
KERNEL_PRESSURE_APPLY = 6
KERNEL_FORCES_XSPH = 7
KERNEL_ADVECT = 8
KERNEL_IO = 9
KERNEL_OTHER = 10
KERNEL_ADJOINT = 11
KERNEL_CLASSES = 12
KERNEL_NAMES = ["grid_count", "grid_scan", "grid_scatter", "grid_reorder", "density_alpha", "pressure_rate",
                "pressure_apply", "forces_xsph", "advect", "io", "other", "adjoint"]


class DfsphConfig(ctypes.Structure):
    """struct dfsph_config (include/dfsph_gb300.h)."""

    _fields_ = [
        ("rest_density", ctypes.c_float),
        ("particle_radius", ctypes.c_float),
        ("smoothing_length", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("damping", ctypes.c_float),
        ("surface_tension", ctypes.c_float),
        ("gravity", ctypes.c_float * 3),
        ("max_density_iters", ctypes.c_uint32),
        ("max_divergence_iters", ctypes.c_uint32),
        ("eta_density", ctypes.c_float),
        ("eta_divergence", ctypes.c_float),
        ("domain_min", ctypes.c_float * 3),
        ("domain_max", ctypes.c_float * 3),
        ("precision", ctypes.c_uint32),
        ("capacity", ctypes.c_uint32),
        ("boundary_capacity", ctypes.c_uint32),
        ("record_diagnostics", ctypes.c_uint32),
        ("n_scenes", ctypes.c_uint32),
        ("use_cuda_graph", ctypes.c_uint32),
        ("slot_order", ctypes.c_uint32),
    ]


class DfsphFrameConfig(ctypes.Structure):
    """struct dfsph_frame_config (include/dfsph_gb300.h)."""

    _fields_ = [
        ("frame_dt", ctypes.c_float),
        ("stepper_frame_dt", ctypes.c_float),
        ("dt_max", ctypes.c_float),
        ("cfl_lambda", ctypes.c_float),
        ("max_substeps", ctypes.c_uint32),
        ("min_velocity", ctypes.c_float),
        ("max_substeps_per_frame", ctypes.c_uint32),
    ]


# (name, restype, argtypes) of every exported entry point
_P = ctypes.c_void_p
_F = ctypes.POINTER(ctypes.c_float)
_SIGNATURES = [
    ("dfsph_config_init", ctypes.c_int, [ctypes.POINTER(DfsphConfig)]),
    ("dfsph_create", ctypes.c_int, [ctypes.POINTER(DfsphConfig), ctypes.c_int, _P, ctypes.POINTER(_P)]),
    ("dfsph_destroy", None, [_P]),
    ("dfsph_set_stream", ctypes.c_int, [_P, _P]),
    ("dfsph_set_boundary", ctypes.c_int, [_P, _P, ctypes.c_uint32, ctypes.c_int]),
    ("dfsph_set_fluid", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, ctypes.c_int]),
    ("dfsph_set_fluid_batch", ctypes.c_int, [_P, ctypes.c_uint32, _P, _P, _P, ctypes.c_int]),
    ("dfsph_set_scene_viscosity", ctypes.c_int, [_P, _F, ctypes.c_uint32]),
    ("dfsph_get_scene_max_velocity", ctypes.c_int, [_P, _F, ctypes.c_uint32]),
    ("dfsph_step", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_uint32]),
    ("dfsph_step_store", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, ctypes.c_float, _P, _P, _P, _P]),
    ("dfsph_get_field", ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_int]),
    ("dfsph_get_state", ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    ("dfsph_get_scalar", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("dfsph_synchronize", ctypes.c_int, [_P]),
    ("dfsph_set_wait_limit", ctypes.c_int, [_P, ctypes.c_uint64]),
    ("dfsph_test_stall_waits", ctypes.c_int, [_P, ctypes.c_uint32]),
    ("dfsph_profile_enable", ctypes.c_int, [_P, ctypes.c_uint32]),
    ("dfsph_profile_read", ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_uint64)]),
    ("dfsph_autotune", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32)]),
    ("dfsph_save_state", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("dfsph_load_state", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("dfsph_get_block_sizes", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    ("dfsph_frame_config_init", ctypes.c_int, [ctypes.POINTER(DfsphFrameConfig)]),
    ("dfsph_step_frames", ctypes.c_int, [_P, ctypes.POINTER(DfsphFrameConfig), ctypes.c_uint32,
                                         ctypes.POINTER(ctypes.c_uint32)]),
    ("dfsph_adjoint_set_state", ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, ctypes.c_int]),
    ("dfsph_adjoint_get_state", ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    ("dfsph_adjoint_forward", ctypes.c_int, [_P, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32]),
    ("dfsph_adjoint_backward", ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    ("dfsph_last_error", ctypes.c_char_p, [_P]),
    ("dfsph_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("dfsph_sample_aabb_boundary", ctypes.c_int64,
     [_F, _F, ctypes.c_float, ctypes.c_int, _P, ctypes.c_int64]),
    ("dfsph_grid_geometry", ctypes.c_int,
     [ctypes.POINTER(DfsphConfig), _F, ctypes.POINTER(ctypes.c_int)]),
    ("dfsph_build_cell_grid", ctypes.c_int,
     [_P, ctypes.c_uint32, _F, ctypes.POINTER(ctypes.c_int), ctypes.c_float, _P, _P, _P, _P]),
    ("dfsph_morton_sort", ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, _P, _P, _P]),
    ("dfsph_lbvh_build", ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, ctypes.c_float, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("dfsph_lbvh_refit", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_float, _P, _P, _P, _P, _P, _P, _P]),
    ("dfsph_cohesion_kernel", ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_float, _P, _P]),
    ("dfsph_build_cell_grid_static", ctypes.c_int,
     [_P, ctypes.c_uint32, _F, ctypes.POINTER(ctypes.c_int), ctypes.c_float, _P, _P, _P, _P]),
]

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load libdfsph_gb300.so; raises if it is missing (build it first)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: the CUDA library is the only implementation. "
            "Build it with water_simulation_gb300._build.build() (or __graft_entry__.build())."
        )
    lib = ctypes.CDLL(p)
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def exported_names() -> list[str]:
    return [s[0] for s in _SIGNATURES]


class DfsphError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status == OK:
        return
    lib = load()
    msg = lib.dfsph_last_error(ctx)
    msg = msg.decode() if msg else ""
    base = lib.dfsph_status_string(status).decode()
    raise DfsphError(status, f"{base}: {msg}")


def fvec3(v) -> ctypes.Array:
    return (ctypes.c_float * 3)(*[float(x) for x in v])

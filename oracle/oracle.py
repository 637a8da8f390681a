"""ctypes face of liboracle.so — TEST INFRASTRUCTURE ONLY.

The CPU restatement of the reference DFSPH step (dfsph_oracle.cpp). Only the
tests, __graft_entry__.smoke() and bench.py's baseline legs use it, as the
parity reference or as the timed CPU baseline; the product never does.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import ORACLE_LIB, build_oracle

F_POSITION, F_VELOCITY, F_DENSITY, F_ALPHA, F_KAPPA, F_DENSITY_ADV = 0, 1, 2, 3, 4, 5
F_CELL_KEY, F_SORTED_INDEX, F_CELL_START, F_NBR_FLUID, F_NBR_BOUNDARY = 6, 7, 8, 9, 10
F_BOUNDARY_MASS, F_KAPPA_V, F_BOUNDARY_CELL_START, F_BOUNDARY_SORTED_INDEX = 11, 12, 13, 14


class OracleConfig(ctypes.Structure):
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
        ("stencil_inv_cell", ctypes.c_float),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        L = ctypes.CDLL(ORACLE_LIB)
        P = ctypes.c_void_p
        F = ctypes.POINTER(ctypes.c_float)
        L.oracle_sample_aabb_boundary.restype = ctypes.c_longlong
        L.oracle_sample_aabb_boundary.argtypes = [F, F, ctypes.c_float, ctypes.c_int, P, ctypes.c_longlong]
        L.oracle_grid_geometry.argtypes = [ctypes.POINTER(OracleConfig), F, ctypes.POINTER(ctypes.c_int)]
        L.oracle_build_grid_f32.argtypes = [P, ctypes.c_uint32, F, ctypes.POINTER(ctypes.c_int), ctypes.c_float,
                                            P, P, P]
        L.oracle_W_f32.restype = ctypes.c_float
        L.oracle_W_f32.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_W_f64.restype = ctypes.c_double
        L.oracle_W_f64.argtypes = [ctypes.c_double, ctypes.c_double]
        L.oracle_gradW_f32.argtypes = [F, ctypes.c_float, F]
        L.oracle_create.restype = P
        L.oracle_create.argtypes = [ctypes.POINTER(OracleConfig), ctypes.c_int, P, P, ctypes.c_uint32, P,
                                    ctypes.c_uint32]
        L.oracle_destroy.argtypes = [P]
        L.oracle_step.argtypes = [P, ctypes.c_float, ctypes.c_uint32]
        L.oracle_get.argtypes = [P, ctypes.c_int, P]
        L.oracle_scalar.restype = ctypes.c_double
        L.oracle_scalar.argtypes = [P, ctypes.c_int]
        L.oracle_dual_create.restype = P
        L.oracle_dual_create.argtypes = [ctypes.POINTER(OracleConfig), P, P, ctypes.c_uint32, P, ctypes.c_uint32,
                                         P, P, ctypes.c_double]
        L.oracle_dual_step.argtypes = [P, ctypes.c_float, ctypes.c_uint32]
        L.oracle_dual_get.argtypes = [P, P, P, P, P]
        L.oracle_dual_destroy.argtypes = [P]
        L.oracle_lbvh_build.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_float, P, P, P, P]
        L.oracle_cohesion_C.restype = ctypes.c_double
        L.oracle_cohesion_C.argtypes = [ctypes.c_double, ctypes.c_double]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def config_from(dfsph_cfg, stencil_inv_cell: float = 0.0) -> OracleConfig:
    """An oracle config with the same values as a dfsph_config structure."""
    c = OracleConfig()
    for name, _ in OracleConfig._fields_:
        if name == "stencil_inv_cell":
            continue
        v = getattr(dfsph_cfg, name)
        if isinstance(v, ctypes.Array):
            getattr(c, name)[:] = list(v)
        else:
            setattr(c, name, v)
    c.stencil_inv_cell = stencil_inv_cell
    return c


def sample_aabb_boundary(lo, hi, spacing, n_layers=3):
    L = load()
    n = L.oracle_sample_aabb_boundary(f3(lo), f3(hi), ctypes.c_float(spacing), n_layers, None, 0)
    out = np.empty((n, 3), np.float32)
    L.oracle_sample_aabb_boundary(f3(lo), f3(hi), ctypes.c_float(spacing), n_layers,
                                  out.ctypes.data_as(ctypes.c_void_p), n)
    return out


def grid_geometry(cfg: OracleConfig):
    o = (ctypes.c_float * 3)()
    d = (ctypes.c_int * 3)()
    load().oracle_grid_geometry(ctypes.byref(cfg), o, d)
    return tuple(o), tuple(d)


def build_grid(xyz, origin, dims, cell):
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    total = int(dims[0]) * int(dims[1]) * int(dims[2])
    keys = np.empty(n, np.uint32)
    srt = np.empty(n, np.uint32)
    cs = np.empty(total + 1, np.uint32)
    load().oracle_build_grid_f32(xyz.ctypes.data_as(ctypes.c_void_p), n, f3(origin), (ctypes.c_int * 3)(*dims),
                                 ctypes.c_float(cell), keys.ctypes.data_as(ctypes.c_void_p),
                                 srt.ctypes.data_as(ctypes.c_void_p), cs.ctypes.data_as(ctypes.c_void_p))
    return keys, srt, cs


def morton_sort(xyz, smin, smax):
    L = load()
    L.oracle_morton_sort.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    codes = np.empty(n, np.uint32)
    idx = np.empty(n, np.uint32)
    L.oracle_morton_sort(xyz.ctypes.data_as(ctypes.c_void_p), n, f3(smin), f3(smax),
                         codes.ctypes.data_as(ctypes.c_void_p), idx.ctypes.data_as(ctypes.c_void_p))
    return codes, idx


def lbvh_build(xyz, smin, smax, radius=0.0, codes=None, sorted_idx=None):
    """SpatialAccel build restated: (codes, sorted, left, right, parent, boxes).
    Given codes and sorted_idx (of an earlier build), the topology is theirs and
    only the boxes follow xyz (a refit)."""
    L = load()
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    if codes is None:
        codes, sorted_idx = morton_sort(xyz, smin, smax)
    codes = np.ascontiguousarray(codes, np.uint32)
    sorted_idx = np.ascontiguousarray(sorted_idx, np.uint32)
    m = max(n - 1, 1)
    left = np.zeros(m, np.uint32)
    right = np.zeros(m, np.uint32)
    parent = np.zeros(max(2 * n - 1, 1), np.uint32)
    boxes = np.zeros((max(2 * n - 1, 1), 6), np.float32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    if n:
        L.oracle_lbvh_build(p(xyz), n, p(codes), p(sorted_idx), ctypes.c_float(radius), p(left), p(right),
                            p(parent), p(boxes))
    return codes, sorted_idx, left[: max(n - 1, 0)], right[: max(n - 1, 0)], parent[: max(2 * n - 1, 0)], \
        boxes[: max(2 * n - 1, 0)]


def cohesion_C(r, l):
    return load().oracle_cohesion_C(float(r), float(l))


def W(r, l, precision=32):
    L = load()
    return L.oracle_W_f64(r, l) if precision == 64 else L.oracle_W_f32(r, l)


def gradW(rij, l):
    out = (ctypes.c_float * 3)()
    load().oracle_gradW_f32(f3(rij), ctypes.c_float(l), out)
    return tuple(out)


class Oracle:
    """One oracle simulation (precision 32 or 64), particles in original order."""

    def __init__(self, cfg: OracleConfig, fluid, vel=None, boundary=None, precision=64, threads=0):
        L = load()
        if threads:
            L.oracle_set_threads(threads)
        self._L = L
        self.fluid = np.ascontiguousarray(fluid, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        b = np.zeros((0, 3), np.float32) if boundary is None else np.ascontiguousarray(boundary, np.float32)
        self.n = self.fluid.shape[0]
        self.nb = b.shape[0]
        self.cfg = cfg
        self._h = L.oracle_create(ctypes.byref(cfg), precision, self.fluid.ctypes.data_as(ctypes.c_void_p),
                                  None if vel is None else vel.ctypes.data_as(ctypes.c_void_p), self.n,
                                  b.ctypes.data_as(ctypes.c_void_p) if self.nb else None, self.nb)
        self.total_cells = int(L.oracle_scalar(self._h, 6))

    def close(self):
        if self._h:
            self._L.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt, n=1):
        self._L.oracle_step(self._h, ctypes.c_float(dt), n)

    def field(self, which):
        if which in (F_POSITION, F_VELOCITY):
            out = np.empty((self.n, 3), np.float64)
        elif which in (F_DENSITY, F_ALPHA, F_KAPPA, F_DENSITY_ADV, F_KAPPA_V):
            out = np.empty(self.n, np.float64)
        elif which == F_BOUNDARY_MASS:
            out = np.empty(self.nb, np.float64)
        elif which in (F_CELL_START, F_BOUNDARY_CELL_START):
            out = np.empty(self.total_cells + 1, np.uint32)
        elif which == F_BOUNDARY_SORTED_INDEX:
            out = np.empty(self.nb, np.uint32)
        else:
            out = np.empty(self.n, np.uint32)
        if out.size:
            self._L.oracle_get(self._h, which, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def scalar(self, which):
        return self._L.oracle_scalar(self._h, which)

    def max_velocity(self):
        return self.scalar(0)

    def particle_mass(self):
        return self.scalar(1)

    def last_density_iters(self):
        return int(self.scalar(2))


class DualOracle:
    """The FP64 oracle step in forward mode: values plus the exact derivative
    along one direction (dx, dv) of the initial state and d_xsph of the XSPH
    coefficient, every branch and neighbour set decided by the values. The
    reference for the GPU adjoint: <gradient, direction> = d(loss) along it."""

    def __init__(self, cfg: OracleConfig, fluid, vel, boundary, dx=None, dv=None, d_xsph=0.0, threads=0):
        L = load()
        if threads:
            L.oracle_set_threads(threads)
        self._L = L
        self.fluid = np.ascontiguousarray(fluid, np.float32).reshape(-1, 3)
        self.n = self.fluid.shape[0]
        vel = np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        b = np.ascontiguousarray(boundary, np.float32).reshape(-1, 3)
        dxa = None if dx is None else np.ascontiguousarray(dx, np.float64).reshape(-1, 3)
        dva = None if dv is None else np.ascontiguousarray(dv, np.float64).reshape(-1, 3)
        ptr = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        self._keep = (vel, b, dxa, dva)
        self._h = L.oracle_dual_create(ctypes.byref(cfg), ptr(self.fluid), ptr(vel), self.n, ptr(b), b.shape[0],
                                       ptr(dxa), ptr(dva), float(d_xsph))

    def step(self, dt, n=1):
        self._L.oracle_dual_step(self._h, ctypes.c_float(dt), n)

    def state(self):
        """(x, v, dx, dv) as (n, 3) float64 arrays."""
        out = [np.empty((self.n, 3), np.float64) for _ in range(4)]
        self._L.oracle_dual_get(self._h, *(a.ctypes.data_as(ctypes.c_void_p) for a in out))
        return tuple(out)

    def close(self):
        if self._h:
            self._L.oracle_dual_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

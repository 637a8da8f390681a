"""ctypes face of oracle/_ref/libref_runner.so — TEST INFRASTRUCTURE ONLY.

Runs the reference's own compiled DFSPH kernels (oracle/_ref/*.fatbin, built
from the reference sources by oracle/build.py) under the restated host
orchestration of oracle/ref_runner.cu. Needs a GPU and the fatbins. Used by
the tests (parity against the reference itself) and by bench.py, which times
the reference's kernels beside the product's (`ref_cuda`, `lbvh.reference`);
the product never uses it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from .oracle import OracleConfig

_lib = None


def available() -> bool:
    return _build.have_reference_fatbins()


def load():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference fatbins are missing (oracle/_ref); build them where the reference tree exists")
        path = _build.build_runner()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_create.restype = P
        L.ref_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(OracleConfig), P, P, ctypes.c_uint32, P,
                                 ctypes.c_uint32]
        L.ref_destroy.argtypes = [P]
        L.ref_step.argtypes = [P, ctypes.c_float, ctypes.c_uint32]
        L.ref_time_steps.restype = ctypes.c_double
        L.ref_time_steps.argtypes = [P, ctypes.c_float, ctypes.c_uint32]
        L.ref_get.argtypes = [P, ctypes.c_int, P]
        L.ref_scalar.restype = ctypes.c_double
        L.ref_scalar.argtypes = [P, ctypes.c_int]
        L.ref_lbvh.argtypes = [ctypes.c_char_p, P, ctypes.c_uint32, P, P, P, P, P, P, P, P, ctypes.c_uint32,
                               ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


class ReferenceRun:
    """The reference CUDA DFSPH solver on one scene (particles in original order)."""

    def __init__(self, cfg: OracleConfig, fluid, vel=None, boundary=None):
        L = load()
        self._L = L
        self.fluid = np.ascontiguousarray(fluid, np.float32).reshape(-1, 3)
        self.n = self.fluid.shape[0]
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        b = np.zeros((0, 3), np.float32) if boundary is None else np.ascontiguousarray(boundary, np.float32)
        self.nb = b.shape[0]
        self._h = L.ref_create(_build.REF_OUT.encode(), ctypes.byref(cfg),
                               self.fluid.ctypes.data_as(ctypes.c_void_p),
                               None if vel is None else vel.ctypes.data_as(ctypes.c_void_p), self.n,
                               b.ctypes.data_as(ctypes.c_void_p) if self.nb else None, self.nb)
        if not self._h:
            raise RuntimeError("reference runner: " + L.ref_last_error().decode())
        self.total_cells = int(L.ref_scalar(self._h, 6))

    def close(self):
        if self._h:
            self._L.ref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt, n=1):
        if self._L.ref_step(self._h, ctypes.c_float(dt), n) != 0:
            raise RuntimeError("reference step: " + self._L.ref_last_error().decode())

    def time_steps(self, dt, n) -> float:
        ms = self._L.ref_time_steps(self._h, ctypes.c_float(dt), n)
        if ms < 0:
            raise RuntimeError("reference step: " + self._L.ref_last_error().decode())
        return ms

    def field(self, which):
        if which in (0, 1):
            out = np.empty((self.n, 3), np.float32)
        elif which in (2, 3, 4, 5):
            out = np.empty(self.n, np.float32)
        elif which == 11:
            out = np.empty(self.nb, np.float32)
        elif which in (8, 13):
            out = np.empty(self.total_cells + 1, np.uint32)
        elif which == 14:
            out = np.empty(self.nb, np.uint32)
        else:
            out = np.empty(self.n, np.uint32)
        if out.size and self._L.ref_get(self._h, which, out.ctypes.data_as(ctypes.c_void_p)) != 0:
            raise RuntimeError("reference get: " + self._L.ref_last_error().decode())
        return out

    def max_velocity(self):
        return self._L.ref_scalar(self._h, 0)

    def particle_mass(self):
        return self._L.ref_scalar(self._h, 1)

    def last_density_iters(self):
        return int(self._L.ref_scalar(self._h, 2))


def lbvh_build(xyz, smin, smax, reps: int = 0):
    """The reference's SpatialAccel::build (core/src/spatial_accel.cu:110-179)
    on its own kernels: (codes, sorted index, left, right, parent, leaf boxes
    [n, 6]) as numpy arrays in the reference's node numbering, plus the mean
    milliseconds of `reps` further builds (0.0 when reps = 0). parent[0] (the
    root) is not written by the reference and is returned as found."""
    L = load()
    xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    codes = np.zeros(max(n, 1), np.uint32)
    idx = np.zeros(max(n, 1), np.uint32)
    left = np.zeros(max(n - 1, 1), np.uint32)
    right = np.zeros(max(n - 1, 1), np.uint32)
    parent = np.zeros(max(2 * n - 1, 1), np.uint32)
    boxes = np.zeros((max(n, 1), 6), np.float32)
    lo = np.asarray(smin, np.float32)
    hi = np.asarray(smax, np.float32)
    ms = ctypes.c_double(0.0)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    if L.ref_lbvh(_build.REF_OUT.encode(), p(xyz), n, p(lo), p(hi), p(codes), p(idx), p(left), p(right), p(parent),
                  p(boxes), reps, ctypes.byref(ms)) != 0:
        raise RuntimeError("reference lbvh: " + L.ref_last_error().decode())
    return (codes[:n], idx[:n], left[: max(n - 1, 0)], right[: max(n - 1, 0)], parent[: max(2 * n - 1, 0)],
            boxes[:n]), ms.value

"""Python face of the C ABI: one DFSPH context on one GPU.

Mirrors the reference's water::solvers::DFSPHSolver
(solvers/dfsph/include/water/solvers/dfsph.h:17-51) for tests, benchmarks and
scripting: construct from a config, give it boundary and fluid particles, call
step(dt), read fields back. All compute happens in libdfsph_gb300.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_FIELD_DTYPE = {
    _lib.FIELD_POSITION: (np.float32, 3),
    _lib.FIELD_VELOCITY: (np.float32, 3),
    _lib.FIELD_DENSITY: (np.float32, 1),
    _lib.FIELD_ALPHA: (np.float32, 1),
    _lib.FIELD_KAPPA: (np.float32, 1),
    _lib.FIELD_DENSITY_ADV: (np.float32, 1),
    _lib.FIELD_KAPPA_V: (np.float32, 1),
    _lib.FIELD_CELL_KEY: (np.uint32, 1),
    _lib.FIELD_SORTED_INDEX: (np.uint32, 1),
    _lib.FIELD_NBR_FLUID: (np.uint32, 1),
    _lib.FIELD_NBR_BOUNDARY: (np.uint32, 1),
    _lib.FIELD_NBR_SIGNATURE: (np.uint32, 1),
}


class Solver:
    def __init__(self, config: _lib.DfsphConfig, device: int = 0, stream: int | None = None):
        self._lib = _lib.load()
        self.config = config
        ptr = ctypes.c_void_p()
        st = self._lib.dfsph_create(ctypes.byref(config), device, ctypes.c_void_p(stream or 0), ctypes.byref(ptr))
        _lib.check(st, None)
        self._ctx = ptr
        origin = (ctypes.c_float * 3)()
        dims = (ctypes.c_int * 3)()
        self._lib.dfsph_grid_geometry(ctypes.byref(config), origin, dims)
        self.origin = tuple(origin)
        self.dims = tuple(dims)
        self.total_cells = dims[0] * dims[1] * dims[2]
        self.n = 0
        self.nb = 0

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.dfsph_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int) -> None:
        _lib.check(st, self._ctx)

    # -- inputs --------------------------------------------------------------
    def set_boundary(self, xyz: np.ndarray) -> None:
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        self._check(self._lib.dfsph_set_boundary(self._ctx, xyz.ctypes.data_as(ctypes.c_void_p),
                                                 xyz.shape[0], _lib.MEM_HOST))
        self.nb = xyz.shape[0]

    def set_fluid(self, xyz: np.ndarray, vel: np.ndarray | None = None) -> None:
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        vp = None
        if vel is not None:
            vel = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
            vp = vel.ctypes.data_as(ctypes.c_void_p)
        self._check(self._lib.dfsph_set_fluid(self._ctx, xyz.ctypes.data_as(ctypes.c_void_p), vp,
                                              xyz.shape[0], _lib.MEM_HOST))
        self.n = xyz.shape[0]

    def set_fluid_batch(self, fluids, velocities=None) -> None:
        """One array of positions (and velocities) per scene (n_scenes > 1)."""
        counts = np.array([f.shape[0] for f in fluids], dtype=np.uint32)
        xyz = np.ascontiguousarray(np.concatenate(fluids, axis=0), dtype=np.float32)
        vp = None
        if velocities is not None:
            vel = np.ascontiguousarray(np.concatenate(velocities, axis=0), dtype=np.float32)
            vp = vel.ctypes.data_as(ctypes.c_void_p)
        self._check(self._lib.dfsph_set_fluid_batch(self._ctx, len(counts), counts.ctypes.data_as(ctypes.c_void_p),
                                                    xyz.ctypes.data_as(ctypes.c_void_p), vp, _lib.MEM_HOST))
        self.n = int(counts.sum())
        self.scene_counts = counts

    def set_scene_viscosity(self, eps) -> None:
        e = np.ascontiguousarray(eps, dtype=np.float32)
        self._check(self._lib.dfsph_set_scene_viscosity(self._ctx, e.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                        e.size))

    def scene_max_velocity(self, n_scenes: int) -> np.ndarray:
        out = np.zeros(n_scenes, np.float32)
        self._check(self._lib.dfsph_get_scene_max_velocity(self._ctx, out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_float)), n_scenes))
        return out

    def set_fluid_device(self, xyz_ptr: int, vel_ptr: int | None, n: int) -> None:
        self._check(self._lib.dfsph_set_fluid(self._ctx, ctypes.c_void_p(xyz_ptr),
                                              ctypes.c_void_p(vel_ptr) if vel_ptr else None, n,
                                              _lib.MEM_DEVICE))
        self.n = n

    # -- stepping ----------------------------------------------------------
    def step(self, dt: float, n_steps: int = 1) -> None:
        self._check(self._lib.dfsph_step(self._ctx, ctypes.c_float(dt), n_steps))

    def step_store(self, pos_ptr: int, vel_ptr: int, n: int, dt: float, density_ptr=0, alpha_ptr=0,
                   kappa_ptr=0, density_adv_ptr=0) -> None:
        vp = lambda p: ctypes.c_void_p(p) if p else None  # noqa: E731
        self._check(self._lib.dfsph_step_store(self._ctx, vp(pos_ptr), vp(vel_ptr), n, ctypes.c_float(dt),
                                               vp(density_ptr), vp(alpha_ptr), vp(kappa_ptr),
                                               vp(density_adv_ptr)))

    def step_frames(self, n_frames: int = 1, frame_config: _lib.DfsphFrameConfig | None = None) -> np.ndarray:
        """n_frames CFL frames (sim_cli's substep loop); returns the substeps of each frame."""
        fc = frame_config or self.frame_config()
        out = np.zeros(max(n_frames, 1), dtype=np.uint32)
        self._check(self._lib.dfsph_step_frames(self._ctx, ctypes.byref(fc), n_frames,
                                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return out[:n_frames]

    def save_state(self, path: str) -> None:
        self._check(self._lib.dfsph_save_state(self._ctx, str(path).encode()))

    def load_state(self, path: str) -> None:
        """Replaces walls and fluid with a saved state (see dfsph_save_state)."""
        self._check(self._lib.dfsph_load_state(self._ctx, str(path).encode()))
        import struct
        with open(path, "rb") as f:
            head = f.read(36)
        _, _, _, n_scenes, n, nb = struct.unpack("<8sIIIII", head[:28])
        self.n, self.nb = n, nb

    def autotune(self, dt: float, steps: int = 3) -> dict:
        """Pick threads per block of the neighbour passes; returns {kernel class: threads}."""
        out = (ctypes.c_int32 * _lib.KERNEL_CLASSES)()
        self._check(self._lib.dfsph_autotune(self._ctx, ctypes.c_float(dt), steps, out))
        return {_lib.KERNEL_NAMES[k]: int(out[k]) for k in range(_lib.KERNEL_CLASSES)}

    def block_sizes(self) -> dict:
        out = (ctypes.c_int32 * _lib.KERNEL_CLASSES)()
        self._check(self._lib.dfsph_get_block_sizes(self._ctx, out))
        return {_lib.KERNEL_NAMES[k]: int(out[k]) for k in range(_lib.KERNEL_CLASSES)}

    def frame_config(self) -> _lib.DfsphFrameConfig:
        fc = _lib.DfsphFrameConfig()
        self._lib.dfsph_frame_config_init(ctypes.byref(fc))
        return fc

    def frames_on_device(self) -> bool:
        return bool(self.scalar(_lib.SCALAR_FRAME_GRAPH))

    def synchronize(self) -> None:
        self._check(self._lib.dfsph_synchronize(self._ctx))

    def set_wait_limit(self, seconds: float) -> None:
        """Time limit of every bounded device wait (the cooperative solve's
        grid barrier); a wait that runs out makes the next synchronising call
        raise DfsphError with ERR_DEVICE_TIMEOUT."""
        self._check(self._lib.dfsph_set_wait_limit(self._ctx, int(seconds * 1e9)))

    def test_stall_waits(self, missing_blocks: int) -> None:
        """Test hook: the grid barrier waits for blocks that never arrive."""
        self._check(self._lib.dfsph_test_stall_waits(self._ctx, missing_blocks))

    def set_stream(self, stream: int) -> None:
        self._check(self._lib.dfsph_set_stream(self._ctx, ctypes.c_void_p(stream)))

    # -- outputs -------------------------------------------------------------
    def field(self, which: int) -> np.ndarray:
        if which in (_lib.FIELD_CELL_START, _lib.FIELD_BOUNDARY_CELL_START):
            out = np.empty(self.total_cells + 1, dtype=np.uint32)
        elif which == _lib.FIELD_BOUNDARY_MASS:
            out = np.empty(self.nb, dtype=np.float32)
        elif which == _lib.FIELD_BOUNDARY_SORTED_INDEX:
            out = np.empty(self.nb, dtype=np.uint32)
        else:
            dt, w = _FIELD_DTYPE[which]
            out = np.empty((self.n, 3) if w == 3 else self.n, dtype=dt)
        if out.size == 0:
            return out
        self._check(self._lib.dfsph_get_field(self._ctx, which, out.ctypes.data_as(ctypes.c_void_p),
                                              out.nbytes, _lib.MEM_HOST))
        return out

    def get_state(self, pos: np.ndarray | None, vel: np.ndarray | None = None) -> None:
        """Positions and velocities into host float32 arrays of shape (n, 3)
        (either may be None) with one call; page-locked arrays are written in
        place by one kernel."""
        for a in (pos, vel):
            if a is not None and (a.dtype != np.float32 or a.size < 3 * self.n or not a.flags.c_contiguous):
                raise ValueError("pos / vel must be C-contiguous float32 arrays of at least 3n values")
        p = ctypes.c_void_p(pos.ctypes.data) if pos is not None else None
        v = ctypes.c_void_p(vel.ctypes.data) if vel is not None else None
        self._check(self._lib.dfsph_get_state(self._ctx, p, v, _lib.MEM_HOST))

    def get_state_ptr(self, pos_ptr: int, vel_ptr: int, mem: int = _lib.MEM_HOST) -> None:
        """dfsph_get_state on raw pointers (host or device memory)."""
        self._check(self._lib.dfsph_get_state(self._ctx, ctypes.c_void_p(pos_ptr or 0), ctypes.c_void_p(vel_ptr or 0),
                                              mem))

    def field_device(self, which: int, dst_ptr: int, nbytes: int) -> None:
        self._check(self._lib.dfsph_get_field(self._ctx, which, ctypes.c_void_p(dst_ptr), nbytes,
                                              _lib.MEM_DEVICE))

    def scalar(self, which: int) -> float:
        v = ctypes.c_double()
        self._check(self._lib.dfsph_get_scalar(self._ctx, which, ctypes.byref(v)))
        return v.value

    # reference accessor names (dfsph.h:40-51)
    def max_velocity(self) -> float:
        return self.scalar(_lib.SCALAR_MAX_VELOCITY)

    def particle_mass(self) -> float:
        return self.scalar(_lib.SCALAR_PARTICLE_MASS)

    def last_density_iters(self) -> int:
        return int(self.scalar(_lib.SCALAR_LAST_DENSITY_ITERS))

    def last_divergence_iters(self) -> int:
        return int(self.scalar(_lib.SCALAR_LAST_DIVERGENCE_ITERS))

    def density_at(self, i: int) -> float:
        return float(self.field(_lib.FIELD_DENSITY)[i])

    def alpha_at(self, i: int) -> float:
        return float(self.field(_lib.FIELD_ALPHA)[i])

    def boundary_mass_at(self, i: int) -> float:
        return float(self.field(_lib.FIELD_BOUNDARY_MASS)[i])

    def profile_enable(self, mask: int) -> None:
        self._check(self._lib.dfsph_profile_enable(self._ctx, mask))

    def profile_read(self, kernel_class: int):
        """(total milliseconds, launches) recorded for one kernel class."""
        t = ctypes.c_double()
        c = ctypes.c_uint64()
        self._check(self._lib.dfsph_profile_read(self._ctx, kernel_class, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def active_boundary(self) -> int:
        return int(self.scalar(_lib.SCALAR_ACTIVE_BOUNDARY))

    def kernel_launches(self) -> int:
        return int(self.scalar(_lib.SCALAR_KERNEL_LAUNCHES))

    def positions(self) -> np.ndarray:
        return self.field(_lib.FIELD_POSITION)

    def velocities(self) -> np.ndarray:
        return self.field(_lib.FIELD_VELOCITY)

    # -- differentiable rollout (arrays of the working type) -----------------
    @property
    def real_dtype(self):
        return np.float64 if self.config.precision == _lib.PRECISION_FP64 else np.float32

    def adjoint_set_state(self, pos, vel=None) -> None:
        """Host arrays (n, 3) of the working type, or device pointers (int) with n given by pos.shape."""
        pos = np.ascontiguousarray(pos, dtype=self.real_dtype).reshape(-1, 3)
        vp = None
        if vel is not None:
            vel = np.ascontiguousarray(vel, dtype=self.real_dtype).reshape(-1, 3)
            vp = vel.ctypes.data_as(ctypes.c_void_p)
        self._check(self._lib.dfsph_adjoint_set_state(self._ctx, pos.ctypes.data_as(ctypes.c_void_p), vp,
                                                      pos.shape[0], _lib.MEM_HOST))
        self.n = pos.shape[0]

    def adjoint_set_state_device(self, pos_ptr: int, vel_ptr: int | None, n: int) -> None:
        self._check(self._lib.dfsph_adjoint_set_state(self._ctx, ctypes.c_void_p(pos_ptr),
                                                      ctypes.c_void_p(vel_ptr) if vel_ptr else None, n,
                                                      _lib.MEM_DEVICE))
        self.n = n

    def adjoint_state(self):
        """(positions, velocities) as (n, 3) host arrays of the working type."""
        x = np.empty((self.n, 3), self.real_dtype)
        v = np.empty((self.n, 3), self.real_dtype)
        if self.n:
            self._check(self._lib.dfsph_adjoint_get_state(self._ctx, x.ctypes.data_as(ctypes.c_void_p),
                                                          v.ctypes.data_as(ctypes.c_void_p), _lib.MEM_HOST))
        return x, v

    def adjoint_state_device(self, pos_ptr: int, vel_ptr: int) -> None:
        vp = lambda p: ctypes.c_void_p(p) if p else None  # noqa: E731
        self._check(self._lib.dfsph_adjoint_get_state(self._ctx, vp(pos_ptr), vp(vel_ptr), _lib.MEM_DEVICE))

    def adjoint_forward(self, dt: float, n_steps: int, checkpoint_every: int = 20) -> None:
        self._check(self._lib.dfsph_adjoint_forward(self._ctx, ctypes.c_float(dt), n_steps, checkpoint_every))

    def adjoint_backward(self, pos_bar, vel_bar=None):
        """Host arrays in, (dL/dx0, dL/dv0, dL/d xsph) out."""
        xb = np.ascontiguousarray(pos_bar, dtype=self.real_dtype).reshape(-1, 3)
        vb = None if vel_bar is None else np.ascontiguousarray(vel_bar, dtype=self.real_dtype).reshape(-1, 3)
        gx = np.empty_like(xb)
        gv = np.empty_like(xb)
        ge = ctypes.c_double()
        self._check(self._lib.dfsph_adjoint_backward(
            self._ctx, xb.ctypes.data_as(ctypes.c_void_p), None if vb is None else vb.ctypes.data_as(ctypes.c_void_p),
            gx.ctypes.data_as(ctypes.c_void_p), gv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ge),
            _lib.MEM_HOST))
        return gx, gv, ge.value

    def adjoint_backward_device(self, pos_bar_ptr: int, vel_bar_ptr: int | None, pos0_bar_ptr: int,
                                vel0_bar_ptr: int) -> float:
        vp = lambda p: ctypes.c_void_p(p) if p else None  # noqa: E731
        ge = ctypes.c_double()
        self._check(self._lib.dfsph_adjoint_backward(self._ctx, vp(pos_bar_ptr), vp(vel_bar_ptr), vp(pos0_bar_ptr),
                                                     vp(vel0_bar_ptr), ctypes.byref(ge), _lib.MEM_DEVICE))
        return ge.value

    def set_xsph(self, eps: float) -> None:
        """XSPH coefficient of a one-scene context (DFSPHSolver::Config::viscosity)."""
        self.set_scene_viscosity([eps])


def solver_for(scene, precision: int = _lib.PRECISION_FP32, diagnostics: bool = False, device: int = 0,
               stream: int | None = None) -> Solver:
    """A context loaded with a Scene's boundary and fluid."""
    s = Solver(scene.config(precision=precision, diagnostics=diagnostics), device=device, stream=stream)
    if scene.nb:
        s.set_boundary(scene.boundary)
    s.set_fluid(scene.fluid, scene.velocity)
    return s

"""Host-side mirror of Flow-X's solver/sph.py over the GB300 C ABI.

``Solver`` holds what the reference keeps in its module-level ``_state``
(solver/sph.py:169-190) for one domain and exposes the same operations under
the same names:

* ``_allocate``       - solver/sph.py:350-369: particle state, predicted
                        mirrors positions, lambda zero;
* ``push_constant_values`` - solver/sph.py:433-461;
* ``_build_grid(dt)`` - solver/sph.py:482-498;
* ``_substep(dt)``    - solver/sph.py:501-514;
* ``_step(frame_dt)`` - the substep loop of solver/sph.py:517-530 (one CUDA
                        graph launch for all substeps of the frame);
* ``_apply_cached``   - solver/sph.py:700-733 (load positions/velocities,
                        predicted = positions, lambda zero, rebuild the grid);
* ``update_surface``  - the splat of solver/surface.py:201-240;
* ``read_texture`` / ``read_scalar_texture`` - solver/gpu_util.py:62-89.

Errors surface as ``FlowxError`` (a RuntimeError) with the library's message,
the way the reference's operators surface exceptions (solver/sph.py:926-933).
"""

from __future__ import annotations

import ctypes
import time
from collections import deque

import numpy as np

from . import _lib
from .config import (
    SolverConfig,
    SurfaceConfig,
    collider_binding,
    push_constant_values,
    splat_push_values,
)
from ._lib import BUF, PASS, FlowxError, Push, check

TIMING_WINDOW = 30  # solver/sph.py:103-104


def _f4(arr, n):
    a = np.ascontiguousarray(arr, dtype=np.float32)
    if a.shape != (n, 4):
        raise ValueError(f"expected ({n}, 4) float32, got {a.shape}")
    return a


class Solver:
    """One domain's PBF state on the GPU.

    exact: the reference's float expressions operation for operation
    (FLOWX_FLAG_EXACT); reference_order: every grid build orders each cell
    the way the reference's bitonic network does (FLOWX_FLAG_REFERENCE_ORDER);
    passes: "warp" or "thread" per particle for the neighbour passes, or
    "auto" (warp up to WARP_PASSES_MAX_PARTICLES particles). Results do not
    depend on `passes`.
    """

    def __init__(
        self,
        config: SolverConfig,
        positions,
        velocities=None,
        *,
        collider=None,
        collider_voxel: float = 0.0,
        max_cells: int | None = None,
        max_collider_voxels: int | None = None,
        max_surface_samples: int = 0,
        device: int = 0,
        keep_delta: bool = False,
        exact: bool = False,
        reference_order: bool = False,
        passes: str = "auto",
    ):
        self.lib = _lib.load()
        self.config = config
        self.n = int(np.asarray(positions).shape[0])
        config.particle_count = self.n
        self._ctx = ctypes.c_void_p()
        cfg = _lib.Config()
        cfg.particle_count = self.n
        cfg.max_cells = int(max_cells or config.cell_count)
        vox = 0
        if collider is not None:
            vox = int(np.asarray(collider).size)
        cfg.max_collider_voxels = int(max_collider_voxels if max_collider_voxels is not None else vox)
        cfg.max_surface_samples = int(max_surface_samples)
        cfg.device = int(device)
        self.config_device = int(device)
        if passes not in ("auto", "warp", "thread"):
            raise ValueError(f"passes must be 'auto', 'warp' or 'thread', not {passes!r}")
        cfg.flags = ((_lib.FLAG_KEEP_DELTA if keep_delta else 0) | (_lib.FLAG_EXACT if exact else 0)
                     | (_lib.FLAG_REFERENCE_ORDER if reference_order else 0)
                     | {"auto": 0, "warp": _lib.FLAG_WARP_PASSES, "thread": _lib.FLAG_THREAD_PASSES}[passes])
        check(self.lib.flowx_create(ctypes.byref(cfg), ctypes.byref(self._ctx)))
        self.collider_dims = None
        self.collider_voxel = 0.0
        self.substeps = 0
        self.timings = deque(maxlen=TIMING_WINDOW)
        self._allocate(positions, velocities)
        if collider is not None and collider_voxel > 0.0:
            self.set_collider(collider, collider_voxel)

    # ---------------------------------------------------------------- state
    def _allocate(self, positions, velocities=None):
        """solver/sph.py:350-369: positions, zero velocities, predicted =
        positions, lambda / delta / normal zero."""
        pos = _f4(positions, self.n)
        vel = np.zeros_like(pos) if velocities is None else _f4(velocities, self.n)
        zeros = np.zeros_like(pos)
        self.write("positions", pos)
        self.write("velocities", vel)
        self.write("predicted", pos)
        self.write("lambda", zeros)
        self.write("delta", zeros)
        self.write("normal", zeros)

    def _apply_cached(self, positions, velocities, dt=0.0):
        """solver/sph.py:700-733: install a stored frame and rebuild the grid."""
        pos = _f4(positions, self.n)
        self.write("positions", pos)
        self.write("velocities", _f4(velocities, self.n))
        self.write("predicted", pos)
        self.write("lambda", np.zeros_like(pos))
        self._build_grid(dt)

    def close(self):
        if self._ctx:
            self.lib.flowx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def ctx(self):
        return self._ctx

    # ------------------------------------------------------------- buffers
    def write(self, name: str, array):
        """Upload a whole buffer in the reference layout (make_texture)."""
        a = np.ascontiguousarray(array, dtype=np.float32)
        check(self.lib.flowx_upload(self._ctx, BUF[name], a.ctypes.data, a.nbytes), self._ctx)

    def read(self, name: str, count: int | None = None) -> np.ndarray:
        """Download a buffer in the reference layout (read_texture)."""
        if name in ("positions", "velocities", "lambda", "predicted", "delta", "normal"):
            out = np.empty((count or self.n, 4), np.float32)
        elif name == "keys":
            out = np.empty((count or self.config.sorted_count, 4), np.float32)
        elif name in ("cell_start", "cell_end"):
            out = np.empty(count or self.config.cell_count, np.float32)
        elif name == "surface":
            out = np.empty(int(count), np.float32)
        else:
            raise KeyError(name)
        check(self.lib.flowx_download(self._ctx, BUF[name], out.ctypes.data, out.nbytes), self._ctx)
        return out

    read_texture = read

    def read_scalar_texture(self, name: str, count: int) -> np.ndarray:
        return self.read(name, count)

    def set_collider(self, occupancy, voxel: float):
        """Install a (z, y, x) uint8 occupancy grid (collision/__init__.py:276-290)."""
        occ = np.ascontiguousarray(occupancy, dtype=np.uint8)
        dims = (ctypes.c_int32 * 3)(occ.shape[2], occ.shape[1], occ.shape[0])
        check(self.lib.flowx_set_collider(self._ctx, occ.ctypes.data, dims, float(voxel)), self._ctx)
        self.collider_dims = (occ.shape[2], occ.shape[1], occ.shape[0])
        self.collider_voxel = float(voxel)

    def voxelize(self, primitives, dims, voxel: float, origin=None):
        """Build the collider grid on the GPU from analytic shapes."""
        arr = (_lib.Primitive * max(len(primitives), 1))()
        for i, p in enumerate(primitives):
            arr[i].kind = p.kind
            arr[i].a[:] = tuple(float(v) for v in p.a)
            arr[i].b[:] = tuple(float(v) for v in p.b)
            arr[i].r = float(p.r)
        d = (ctypes.c_int32 * 3)(*dims)
        o = (ctypes.c_float * 3)(*(origin if origin is not None else self.config.lo))
        check(self.lib.flowx_voxelize(self._ctx, arr, len(primitives), d, float(voxel), o), self._ctx)
        self.collider_dims = tuple(int(v) for v in dims)
        self.collider_voxel = float(voxel)

    def voxelize_meshes(self, meshes, dims, voxel: float, origin=None):
        """Build the collider grid on the GPU from triangle meshes
        (collision/__init__.py:304-367 and the union of :225-242): each mesh a
        (vertices V x 3, triangles T x 3, matrix_world 4 x 4) triple in the
        object's local space and Blender's row-major world matrix."""
        keep = []
        arr = (_lib.Mesh * max(len(meshes), 1))()
        for i, (verts, tris, matrix) in enumerate(meshes):
            v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
            t = np.ascontiguousarray(tris, np.int32).reshape(-1, 3)
            keep += [v, t]
            arr[i].vertices = v.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
            arr[i].vertex_count = v.shape[0]
            arr[i].triangles = t.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            arr[i].triangle_count = t.shape[0]
            arr[i].matrix_world[:] = tuple(float(x) for x in np.asarray(matrix, np.float32).reshape(16))
        d = (ctypes.c_int32 * 3)(*dims)
        o = (ctypes.c_float * 3)(*(origin if origin is not None else self.config.lo))
        check(self.lib.flowx_voxelize_meshes(self._ctx, arr, len(meshes), d, float(voxel), o), self._ctx)
        self.collider_dims = tuple(int(v) for v in dims)
        self.collider_voxel = float(voxel)

    def collider_occupancy(self) -> np.ndarray:
        """The installed collider grid, (nz, ny, nx) uint8 (1 = occupied)."""
        nx, ny, nz = self.collider_dims
        out = np.empty((nz, ny, nx), np.uint8)
        check(self.lib.flowx_download_collider(self._ctx, out.ctypes.data, out.nbytes), self._ctx)
        return out

    def clear_collider(self):
        check(self.lib.flowx_set_collider(self._ctx, None, None, 0.0), self._ctx)
        self.collider_dims = None
        self.collider_voxel = 0.0

    # -------------------------------------------------------------- passes
    def push_constant_values(self, dt, sort_k=0, sort_j=0):
        ic = collider_binding(self.collider_dims, self.collider_voxel)
        return push_constant_values(self.config, dt, ic, sort_k, sort_j)

    def push(self, dt) -> Push:
        return Push.from_values(self.push_constant_values(dt))

    def _build_grid(self, dt=0.0):
        check(self.lib.flowx_build_grid(self._ctx, ctypes.byref(self.push(dt))), self._ctx)

    def _substep(self, dt):
        check(self.lib.flowx_substep(self._ctx, ctypes.byref(self.push(dt)), self.config.iterations), self._ctx)

    def step_substeps(self, dt, substeps):
        """``substeps`` substeps as one CUDA-graph launch."""
        check(
            self.lib.flowx_step(self._ctx, ctypes.byref(self.push(dt)), self.config.iterations, int(substeps)),
            self._ctx,
        )

    def _step(self, frame_dt):
        """One frame (solver/sph.py:517-545): substeps sized by substep_dt,
        timed end to end on the host like the reference."""
        started = time.perf_counter()
        substeps, dt = self.config.substep_dt(frame_dt)
        self.substeps = substeps
        self.step_substeps(dt, substeps)
        self.synchronize()
        self.timings.append((time.perf_counter() - started) * 1000.0)
        return substeps, dt

    def run_pass(self, name: str, dt):
        check(self.lib.flowx_run_pass(self._ctx, PASS[name], ctypes.byref(self.push(dt))), self._ctx)

    def update_surface(self, surface: SurfaceConfig, dt=0.0, download=True):
        """Density splat onto the surface grid (solver/surface.py:201-240)."""
        ic = collider_binding(self.collider_dims, self.collider_voxel)
        push = Push.from_values(splat_push_values(self.config, surface, dt, ic))
        if download:
            out = np.empty(surface.sample_count, np.float32)
            check(self.lib.flowx_splat(self._ctx, ctypes.byref(push), out.ctypes.data, out.nbytes), self._ctx)
            return out
        check(self.lib.flowx_splat(self._ctx, ctypes.byref(push), None, 0), self._ctx)
        return None

    def surface_mesh(self, surface: SurfaceConfig, dt=0.0, mc=None):
        """The per-frame surface (solver/surface.py:201-244): splat, then marching
        cubes on the device; returns (vertices V x 3 float64, triangles T x 3 int32)."""
        from .surface import MarchingCubes

        self.update_surface(surface, dt, download=False)
        field = ctypes.c_void_p()
        samples = ctypes.c_int64()
        check(self.lib.flowx_surface_field(self._ctx, ctypes.byref(field), ctypes.byref(samples)), self._ctx)
        mc = mc or MarchingCubes(self.config_device)
        mc.extract_device(field.value, surface.dims, surface.lo, surface.spacing, surface.iso, self.stream())
        return mc.download()

    def synchronize(self):
        check(self.lib.flowx_synchronize(self._ctx), self._ctx)

    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(self.lib.flowx_get_stream(self._ctx, ctypes.byref(s)), self._ctx)
        return s.value or 0

    def time_steps(self, dt, substeps, steps) -> float:
        ms = ctypes.c_float()
        check(
            self.lib.flowx_time_steps(
                self._ctx, ctypes.byref(self.push(dt)), self.config.iterations, int(substeps), int(steps),
                ctypes.byref(ms),
            ),
            self._ctx,
        )
        return float(ms.value)

    def profile(self, dt, substeps):
        """Per-kernel device milliseconds and launch counts over ``substeps``
        launch-by-launch substeps."""
        k = self.lib.flowx_kernel_count()
        ms = (ctypes.c_float * k)()
        n = (ctypes.c_int32 * k)()
        check(
            self.lib.flowx_profile_substeps(
                self._ctx, ctypes.byref(self.push(dt)), self.config.iterations, int(substeps), ms, n
            ),
            self._ctx,
        )
        return {
            self.lib.flowx_kernel_name(i).decode(): (float(ms[i]), int(n[i])) for i in range(k) if n[i] > 0
        }

    def stats(self):
        """Solver figures (solver/sph.py:862-886)."""
        return {
            "particles": self.n,
            "cells": self.config.cell_count,
            "substeps": self.substeps,
            "step_ms": (sum(self.timings) / len(self.timings)) if self.timings else None,
        }


def launch_count() -> int:
    return int(_lib.load().flowx_launch_count())


__all__ = ["Solver", "FlowxError", "launch_count"]

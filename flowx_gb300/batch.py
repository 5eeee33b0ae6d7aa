"""Many independent scenes stepped together (no reference counterpart).

``Batch`` packs several scenes into one context: particles, cells and
collider voxels are concatenated in scene order and each scene keeps its own
push block (parameters, dt, grid, collider), so one kernel launch per pass
serves every scene (see ``flowx_batch_*`` in include/flowx.h). Results for a
scene are the same, bit for bit, as stepping that scene alone: each scene's
particles only ever see their own scene's cells.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import BUF, Push, check
from .config import collider_binding, push_constant_values, splat_push_values
from .scenes import Scene


def scene_push(scene: Scene, dt: float | None = None) -> dict:
    ic = collider_binding(scene.collider_dims, scene.collider_voxel)
    return push_constant_values(scene.config, scene.dt if dt is None else dt, ic)


def pack_layout(scenes):
    """(particle offsets, cell offsets, voxel offsets, totals) of a list of scenes."""
    p, c, v = [0], [0], [0]
    for s in scenes:
        p.append(p[-1] + s.n)
        c.append(c[-1] + s.config.cell_count)
        v.append(v[-1] + (int(np.prod(s.collider_dims)) if s.collider_dims is not None else 0))
    return p, c, v


class Batch:
    """Several scenes in one GPU context."""

    def __init__(self, scenes, *, device=0, exact=False, max_surface_samples=0):
        self.lib = _lib.load()
        self.scenes = list(scenes)
        self.p_off, self.c_off, self.v_off = pack_layout(self.scenes)
        self.n = self.p_off[-1]
        for s in self.scenes:
            s.config.particle_count = s.n
        cfg = _lib.Config()
        cfg.particle_count = self.n
        cfg.max_cells = max(1, self.c_off[-1])
        cfg.max_collider_voxels = self.v_off[-1]
        cfg.max_surface_samples = int(max_surface_samples)
        cfg.device = int(device)
        cfg.flags = _lib.FLAG_EXACT if exact else 0
        self._ctx = ctypes.c_void_p()
        check(self.lib.flowx_create(ctypes.byref(cfg), ctypes.byref(self._ctx)))
        self.set_scenes()
        pos = np.concatenate([s.positions for s in self.scenes]).astype(np.float32)
        vel = np.concatenate([s.velocities for s in self.scenes]).astype(np.float32)
        zeros = np.zeros_like(pos)
        for name, arr in (("positions", pos), ("velocities", vel), ("predicted", pos), ("lambda", zeros),
                          ("delta", zeros), ("normal", zeros)):
            self.write(name, arr)
        for k, s in enumerate(self.scenes):
            if s.collider_dims is not None:
                self.set_collider(k, s.collider_grid(0))

    def set_scenes(self, dts=None):
        arr = (Push * len(self.scenes))()
        for k, s in enumerate(self.scenes):
            arr[k] = Push.from_values(scene_push(s, None if dts is None else dts[k]))
        check(self.lib.flowx_batch_set_scenes(self._ctx, arr, len(self.scenes)), self._ctx)

    def set_collider(self, scene: int, occupancy):
        s = self.scenes[scene]
        occ = np.ascontiguousarray(occupancy, dtype=np.uint8)
        dims = (ctypes.c_int32 * 3)(occ.shape[2], occ.shape[1], occ.shape[0])
        check(self.lib.flowx_batch_set_collider(self._ctx, scene, occ.ctypes.data, dims,
                                                float(np.float32(s.collider_voxel))), self._ctx)

    def write(self, name, array):
        a = np.ascontiguousarray(array, dtype=np.float32)
        check(self.lib.flowx_upload(self._ctx, BUF[name], a.ctypes.data, a.nbytes), self._ctx)

    def read(self, name) -> np.ndarray:
        out = np.empty((self.n, 4), np.float32)
        check(self.lib.flowx_download(self._ctx, BUF[name], out.ctypes.data, out.nbytes), self._ctx)
        return out

    def read_scene(self, name, scene: int) -> np.ndarray:
        return self.read(name)[self.p_off[scene]:self.p_off[scene + 1]]

    def build_grid(self):
        check(self.lib.flowx_batch_build_grid(self._ctx), self._ctx)

    def substep(self, iterations=4):
        check(self.lib.flowx_batch_substep(self._ctx, int(iterations)), self._ctx)

    def step(self, iterations=4, substeps=1):
        check(self.lib.flowx_batch_step(self._ctx, int(iterations), int(substeps)), self._ctx)

    def splat(self, scene: int, surface=None, dt=0.0):
        s = self.scenes[scene]
        surface = surface or s.surface
        ic = collider_binding(s.collider_dims, s.collider_voxel)
        push = Push.from_values(splat_push_values(s.config, surface, dt, ic))
        out = np.empty(surface.sample_count, np.float32)
        check(self.lib.flowx_batch_splat(self._ctx, scene, ctypes.byref(push), out.ctypes.data, out.nbytes),
              self._ctx)
        return out

    def autotune(self, iterations=4):
        k = self.lib.flowx_kernel_count()
        chosen = (ctypes.c_int32 * k)()
        check(self.lib.flowx_autotune(self._ctx, None, int(iterations), chosen), self._ctx)
        return {self.lib.flowx_kernel_name(i).decode(): int(chosen[i]) for i in range(k) if chosen[i]}

    def synchronize(self):
        check(self.lib.flowx_synchronize(self._ctx), self._ctx)

    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(self.lib.flowx_get_stream(self._ctx, ctypes.byref(s)), self._ctx)
        return s.value or 0

    def close(self):
        if self._ctx:
            self.lib.flowx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

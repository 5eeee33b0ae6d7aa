"""Disk cache of per-frame particle state in the reference's FLWXCA01 format.

Host-side mirror of Flow-X's solver/cache.py over the library's
``flowx_cache_*`` entry points (file layout and semantics in include/flowx.h
and flowx_gb300/csrc/cache.cu):

* ``FrameCache.open(path, ...)`` - solver/cache.py:284-338: reuse an existing
  file while its config hash, particle count and seed frame match the run,
  else start a fresh one holding only the header;
* ``write_frame(frame, solver)`` - :339-379: store the solver's positions and
  velocities (frames after the seed frame only; last_frame rewritten);
* ``try_load(frame, solver, dt)`` - :382-421 with solver/sph.py:700-733:
  install a cached frame (positions, velocities, predicted = positions,
  lambda zero, grid rebuilt), or return False outside the cached range or
  when the settings no longer hash to the file's config hash.

The reference's config hash fingerprints Blender objects; here the caller
supplies the 32-byte hash (``config_hash`` hashes a SolverConfig, the fps and
the collider names as a stand-in).
"""

from __future__ import annotations

import ctypes
import dataclasses
import hashlib
import os

import numpy as np

from . import _lib
from ._lib import CacheHeader, FlowxError

FORMAT_VERSION = 2


def config_hash(config, fps: float, colliders=()) -> bytes:
    """sha256 over a solver configuration's fields, the frame rate and the
    collider names (a stand-in for solver/cache.py:153-190's Blender hash)."""
    h = hashlib.sha256()
    fields = dataclasses.asdict(config) if dataclasses.is_dataclass(config) else dict(vars(config))
    for key in sorted(fields):
        h.update(f"{key}={fields[key]!r};".encode())
    h.update(f"fps={float(fps)!r};".encode())
    for name in colliders:
        h.update(f"collider={name};".encode())
    return h.digest()


class FrameCache:
    """One run's cache file."""

    def __init__(self, handle, path):
        self.lib = _lib.load()
        self._h = handle
        self.path = path

    # ---------------------------------------------------------------- open
    @classmethod
    def create(cls, path, *, particle_count, seed_frame, fps, colliders=(), config_hash_bytes=b"\0" * 32,
               flowx_version="0.1.0"):
        lib = _lib.load()
        hdr = CacheHeader()
        hdr.flowx_version = flowx_version.encode("utf-8")[:16]
        hdr.particle_count = int(particle_count)
        hdr.seed_frame = int(seed_frame)
        hdr.fps = float(fps)
        names = [n.encode("utf-8") for n in colliders]
        arr = (ctypes.c_char_p * max(len(names), 1))(*names)
        hdr.collider_count = len(names)
        hdr.collider_names = ctypes.cast(arr, ctypes.POINTER(ctypes.c_char_p))
        hdr.config_hash[:] = bytes(config_hash_bytes)[:32]
        h = ctypes.c_void_p()
        rc = lib.flowx_cache_create(os.fsencode(path), ctypes.byref(hdr), ctypes.byref(h))
        if rc != _lib.FLOWX_OK:
            raise FlowxError(rc, lib.flowx_cache_last_error(None).decode())
        return cls(h, path)

    @classmethod
    def open_existing(cls, path):
        lib = _lib.load()
        h = ctypes.c_void_p()
        rc = lib.flowx_cache_open(os.fsencode(path), ctypes.byref(h))
        if rc != _lib.FLOWX_OK:
            raise FlowxError(rc, lib.flowx_cache_last_error(None).decode())
        return cls(h, path)

    @classmethod
    def open(cls, path, *, particle_count, seed_frame, fps, colliders=(), config_hash_bytes=b"\0" * 32,
             flowx_version="0.1.0"):
        """solver/cache.py:284-338: reuse a matching file, else start afresh."""
        if os.path.exists(path):
            try:
                existing = cls.open_existing(path)
                h = existing.header()
                if (h["config_hash"] == bytes(config_hash_bytes)[:32] and h["particle_count"] == particle_count
                        and h["seed_frame"] == seed_frame):
                    return existing
                existing.close()
            except FlowxError:
                pass
        return cls.create(path, particle_count=particle_count, seed_frame=seed_frame, fps=fps, colliders=colliders,
                          config_hash_bytes=config_hash_bytes, flowx_version=flowx_version)

    def close(self):
        if self._h:
            self.lib.flowx_cache_close(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != _lib.FLOWX_OK:
            raise FlowxError(rc, self.lib.flowx_cache_last_error(self._h).decode())

    def header(self) -> dict:
        hdr = CacheHeader()
        self._check(self.lib.flowx_cache_info(self._h, ctypes.byref(hdr)))
        return {
            "format_version": FORMAT_VERSION,
            "flowx_version": bytes(hdr.flowx_version).rstrip(b"\0").decode("utf-8", "replace"),
            "particle_count": hdr.particle_count,
            "seed_frame": hdr.seed_frame,
            "last_frame": hdr.last_frame,
            "fps": hdr.fps,
            "colliders": [self.lib.flowx_cache_collider_name(self._h, i).decode("utf-8")
                          for i in range(hdr.collider_count)],
            "config_hash": bytes(hdr.config_hash),
        }

    # -------------------------------------------------------------- frames
    def write_frame(self, frame: int, solver):
        """Store the solver's state as `frame` (a no-op at or before the seed frame)."""
        self._check(self.lib.flowx_cache_write_frame(self._h, solver.ctx, int(frame)))

    def try_load(self, frame: int, solver, dt=0.0, config_hash_bytes=None) -> bool:
        """Install cached `frame` into the solver; False when it is not covered
        or (with config_hash_bytes) the file was made under other settings."""
        h = self.header()
        if not h["seed_frame"] < frame <= h["last_frame"]:
            return False
        if config_hash_bytes is not None and bytes(config_hash_bytes)[:32] != h["config_hash"]:
            return False
        self._check(self.lib.flowx_cache_load_frame(self._h, solver.ctx, int(frame),
                                                    ctypes.byref(solver.push(dt))))
        return True

    def write_frame_host(self, frame: int, positions, velocities):
        p = np.ascontiguousarray(positions, np.float32)
        v = np.ascontiguousarray(velocities, np.float32)
        self._check(self.lib.flowx_cache_write_frame_host(self._h, int(frame), p.ctypes.data, v.ctypes.data))

    def read_frame_host(self, frame: int):
        n = self.header()["particle_count"]
        p = np.empty((n, 4), np.float32)
        v = np.empty((n, 4), np.float32)
        self._check(self.lib.flowx_cache_read_frame_host(self._h, int(frame), p.ctypes.data, v.ctypes.data))
        return p, v

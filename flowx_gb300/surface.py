"""Iso-surface extraction on the GPU: solver/marching_cubes.py's ``extract``
(:191-280) over the library's ``flowx_mc_*`` entry points.

``extract(field, dims, origin, spacing, iso)`` keeps the reference's
signature and result: ``(vertices, triangles)``, the same indexed mesh the
reference builds (same vertices in the same order, same float64
coordinates, same triangles), as numpy arrays (V x 3 float64, T x 3 int32)
instead of lists of tuples. ``Solver.surface_mesh`` runs the per-frame splat
and the extraction back to back on the device, replacing the read-back of
the splat grid and the Python extraction of solver/surface.py:239-244.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import FlowxError


class MarchingCubes:
    """Device scratch and mesh buffers for repeated extractions on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        self.device = int(device)
        self._h = ctypes.c_void_p()
        self._check(self.lib.flowx_mc_create(self.device, ctypes.byref(self._h)), None)
        self.vertex_count = 0
        self.triangle_count = 0

    def _check(self, rc, handle):
        if rc != _lib.FLOWX_OK:
            msg = self.lib.flowx_mc_last_error(handle)
            raise FlowxError(rc, msg.decode() if msg else "")

    def close(self):
        if self._h:
            self.lib.flowx_mc_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def extract_device(self, field_ptr: int, dims, origin, spacing: float, iso: float, stream: int | None = None):
        """Extract from a device field (x fastest); returns (vertex_count, triangle_count)."""
        d = (ctypes.c_int32 * 3)(*(int(v) for v in dims))
        o = (ctypes.c_double * 3)(*(float(v) for v in origin))
        nv, nt = ctypes.c_int64(), ctypes.c_int64()
        rc = self.lib.flowx_mc_extract(self._h, ctypes.c_void_p(field_ptr), d, o, float(spacing), float(iso),
                                       ctypes.c_void_p(stream), ctypes.byref(nv), ctypes.byref(nt))
        self._check(rc, self._h)
        self.vertex_count, self.triangle_count = int(nv.value), int(nt.value)
        return self.vertex_count, self.triangle_count

    def download(self):
        """The last extraction as (vertices V x 3 float64, triangles T x 3 int32)."""
        v = np.empty((self.vertex_count, 3), np.float64)
        t = np.empty((self.triangle_count, 3), np.int32)
        self._check(self.lib.flowx_mc_download(self._h, v.ctypes.data, v.nbytes, t.ctypes.data, t.nbytes), self._h)
        return v, t

    def extract(self, field, dims, origin, spacing, iso):
        """solver/marching_cubes.py ``extract`` for a host or device field."""
        import torch

        nx, ny, nz = (int(v) for v in dims)
        if nx < 2 or ny < 2 or nz < 2:
            return np.zeros((0, 3), np.float64), np.zeros((0, 3), np.int32)
        f = torch.as_tensor(np.asarray(field, np.float32) if not torch.is_tensor(field) else field,
                            dtype=torch.float32, device=torch.device("cuda", self.device)).contiguous().reshape(-1)
        if f.numel() != nx * ny * nz:
            raise ValueError(f"field has {f.numel()} samples, dims ask for {nx * ny * nz}")
        stream = torch.cuda.current_stream(self.device)
        self.extract_device(f.data_ptr(), dims, origin, spacing, iso, stream.cuda_stream)
        return self.download()


_DEFAULT: MarchingCubes | None = None


def extract(field, dims, origin, spacing, iso):
    """solver/marching_cubes.py:191-280 on the GPU (device 0)."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = MarchingCubes(0)
    return _DEFAULT.extract(field, dims, origin, spacing, iso)


def case_table():
    """The library's derived 256-case table: (256 x 15 edge indices, -1 padded; 256 counts)."""
    lib = _lib.load()
    table = np.full((256, 15), -1, np.int32)
    counts = np.zeros(256, np.int32)
    buf = (ctypes.c_int32 * 15)()
    n = ctypes.c_int32()
    for c in range(256):
        rc = lib.flowx_mc_case_table(c, buf, ctypes.byref(n))
        if rc != _lib.FLOWX_OK:
            raise FlowxError(rc, "case table")
        counts[c] = n.value
        table[c, :3 * n.value] = buf[:3 * n.value]
    return table, counts

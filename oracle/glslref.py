"""Oracle (test infrastructure only): drive the reference's own GLSL passes on the CPU.

``oracle/_ref/libglslref.so`` is the reference's ``shaders/*.glsl`` compiled
unmodified as C++ (``oracle/glsl_cpu/``). This module restates the host side
that dispatches them, so a whole substep runs exactly as Flow-X issues it:

* buffers in the reference's texture layout - flat arrays wrapped at width 256,
  RGBA32F for particles and keys, R32F for cells and the splat grid
  (``solver/gpu_util.py:28-59``, ``solver/sph.py:127-152, 350-369``);
* the push-constant block packed as ``solver/sph.py:433-461``;
* ``build_grid`` = ``solver/sph.py:482-498`` (grid keys, the host-driven
  bitonic (k, j) loop, cell clear, cell ranges);
* ``substep`` = ``solver/sph.py:501-514``;
* ``splat`` = ``solver/surface.py:201-239``.

It needs the reference sources to build, so it is used where they are mounted
(fixture generation, ``tests/golden/make_golden.py``) and nowhere else.
"""

from __future__ import annotations

import ctypes
import math
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libglslref.so")
WIDTH = 256

(
    NORMAL,
    PREDICT,
    GRID_KEY,
    SORT,
    CELL_CLEAR,
    CELL_RANGE,
    LAMBDA,
    DELTA,
    APPLY_DELTA,
    VELOCITY,
    XSPH,
    FINALIZE,
    SPLAT,
) = range(13)


class Push(ctypes.Structure):
    _fields_ = [
        ("i_layout", ctypes.c_int32 * 4),
        ("i_grid", ctypes.c_int32 * 4),
        ("i_sort", ctypes.c_int32 * 4),
        ("f_lo", ctypes.c_float * 4),
        ("f_hi", ctypes.c_float * 4),
        ("f_sph", ctypes.c_float * 4),
        ("f_sim", ctypes.c_float * 4),
        ("i_collider", ctypes.c_int32 * 4),
    ]


_FP = ctypes.POINTER(ctypes.c_float)


class Images(ctypes.Structure):
    _fields_ = [
        ("positions", _FP),
        ("velocities", _FP),
        ("lambda_", _FP),
        ("predicted", _FP),
        ("delta", _FP),
        ("normal", _FP),
        ("keys", _FP),
        ("cell_start", _FP),
        ("cell_end", _FP),
        ("surface", _FP),
        ("collider", _FP),
        ("particle_rows", ctypes.c_int32),
        ("key_rows", ctypes.c_int32),
        ("cell_rows", ctypes.c_int32),
        ("surface_rows", ctypes.c_int32),
        ("collider_dims", ctypes.c_int32 * 3),
        ("width", ctypes.c_int32),
    ]


def build(ref_root=None):
    """Compile the harness from the reference checkout (oracle/glsl_cpu/Makefile);
    ``ref_root`` defaults to ``oracle.refpath.checkout()``."""
    from oracle import refpath

    ref_root = ref_root or refpath.checkout()
    subprocess.run(
        ["make", "-s", "-C", os.path.join(HERE, "glsl_cpu"), f"REF={ref_root}"],
        check=True,
    )
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        _LIB = ctypes.CDLL(LIB_PATH)
        _LIB.glslref_dispatch.argtypes = [ctypes.c_int, ctypes.POINTER(Push), ctypes.POINTER(Images), ctypes.c_int]
        _LIB.glslref_dispatch.restype = ctypes.c_int
    return _LIB


def _fbits(v):
    return struct.unpack("<i", struct.pack("<f", float(v)))[0]


def _rows(n):
    return max(1, math.ceil(n / WIDTH))


def _ptr(a):
    return a.ctypes.data_as(_FP) if a is not None else ctypes.cast(None, _FP)


class GlslRef:
    """One scene's buffers and the reference's dispatch sequence.

    Geometry and parameters are plain values (no project types), so this
    restatement stays independent of the code it checks.
    """

    def __init__(
        self,
        *,
        lo,
        hi,
        cell_size,
        cell_dims,
        h,
        mass,
        rest_density,
        relaxation,
        scorr,
        sigma,
        viscosity,
        particle_radius,
        positions,
        velocities,
        iterations=4,
        gravity=-9.81,
        damping=0.35,
        collider=None,
        collider_voxel=0.0,
    ):
        n = int(positions.shape[0])
        self.n = n
        self.s = max(2, 1 << (max(1, n) - 1).bit_length())
        self.c = int(cell_dims[0] * cell_dims[1] * cell_dims[2])
        self.lo, self.hi = tuple(lo), tuple(hi)
        self.cell_size, self.cell_dims = float(cell_size), tuple(int(d) for d in cell_dims)
        self.h, self.mass, self.rest_density, self.relaxation = h, mass, rest_density, relaxation
        self.scorr, self.sigma, self.viscosity = scorr, sigma, viscosity
        self.particle_radius, self.iterations = particle_radius, iterations
        self.gravity, self.damping = gravity, damping
        pr = _rows(n)
        self.pr, self.kr, self.cr = pr, _rows(self.s), _rows(self.c)

        def particle_buf(values=None):
            a = np.zeros((pr * WIDTH, 4), dtype=np.float32)
            if values is not None:
                a[:n] = values
            return a

        # solver/sph.py:350-369 (_allocate): predicted mirrors positions, the rest zero.
        self.positions = particle_buf(positions)
        self.velocities = particle_buf(velocities)
        self.lambda_ = particle_buf()
        self.predicted = particle_buf(positions)
        self.delta = particle_buf()
        self.normal = particle_buf()
        self.keys = np.zeros((self.kr * WIDTH, 4), dtype=np.float32)
        self.cell_start = np.zeros(self.cr * WIDTH, dtype=np.float32)
        self.cell_end = np.zeros(self.cr * WIDTH, dtype=np.float32)
        self.surface = None
        self.surface_rows = 1
        if collider is not None and collider_voxel > 0.0:
            occ = np.asarray(collider)
            self.collider = np.ascontiguousarray((occ > 0).astype(np.float32))
            self.collider_dims = (occ.shape[2], occ.shape[1], occ.shape[0])
            self.collider_voxel = float(collider_voxel)
        else:
            # solver/sph.py:408-430: a 1x1x1 empty texture and voxel size 0.
            self.collider = np.zeros(1, dtype=np.float32)
            self.collider_dims = (1, 1, 1)
            self.collider_voxel = 0.0

    # -- solver/sph.py:433-461 ------------------------------------------------
    def push(self, dt, sort_k=0, sort_j=0):
        p = Push()
        p.i_layout[:] = (self.n, WIDTH, WIDTH, self.s)
        p.i_grid[:] = (*self.cell_dims, self.c)
        p.i_sort[:] = (sort_k, sort_j, _fbits(self.scorr), _fbits(self.sigma))
        p.f_lo[:] = (*self.lo, self.cell_size)
        p.f_hi[:] = (*self.hi, self.particle_radius)
        p.f_sph[:] = (self.h, self.mass, self.rest_density, self.relaxation)
        p.f_sim[:] = (self.viscosity, dt, self.gravity, self.damping)
        if self.collider_voxel > 0.0:
            p.i_collider[:] = (*self.collider_dims, _fbits(self.collider_voxel))
        else:
            p.i_collider[:] = (1, 1, 1, 0)
        return p

    def images(self):
        im = Images()
        im.positions = _ptr(self.positions)
        im.velocities = _ptr(self.velocities)
        im.lambda_ = _ptr(self.lambda_)
        im.predicted = _ptr(self.predicted)
        im.delta = _ptr(self.delta)
        im.normal = _ptr(self.normal)
        im.keys = _ptr(self.keys)
        im.cell_start = _ptr(self.cell_start)
        im.cell_end = _ptr(self.cell_end)
        im.surface = _ptr(self.surface)
        im.collider = _ptr(self.collider)
        im.particle_rows = self.pr
        im.key_rows = self.kr
        im.cell_rows = self.cr
        im.surface_rows = self.surface_rows
        im.collider_dims[:] = self.collider_dims
        im.width = WIDTH
        return im

    def dispatch(self, pass_id, count, push):
        im = self.images()
        rc = lib().glslref_dispatch(pass_id, ctypes.byref(push), ctypes.byref(im), int(count))
        if rc != 0:
            raise RuntimeError(f"glslref_dispatch({pass_id}) failed")

    # -- solver/sph.py:482-498 ------------------------------------------------
    def build_grid(self, dt):
        n = self.s
        self.dispatch(GRID_KEY, n, self.push(dt))
        k = 2
        while k <= n:
            j = k >> 1
            while j > 0:
                self.dispatch(SORT, n, self.push(dt, k, j))
                j >>= 1
            k <<= 1
        self.dispatch(CELL_CLEAR, self.c, self.push(dt))
        self.dispatch(CELL_RANGE, n, self.push(dt))

    # -- solver/sph.py:501-514 ------------------------------------------------
    def substep(self, dt, trace=None):
        """One substep. ``trace`` (a dict) receives a copy of every buffer a pass
        writes, keyed "<pass>" (first iteration only for the loop passes)."""

        def snap(name, *bufs):
            if trace is not None and name not in trace:
                trace[name] = {b: getattr(self, b)[: self._count(b)].copy() for b in bufs}

        if self.sigma > 0.0:
            self.dispatch(NORMAL, self.n, self.push(dt))
            snap("normal", "normal")
        self.dispatch(PREDICT, self.n, self.push(dt))
        snap("predict", "velocities", "predicted")
        self.build_grid(dt)
        snap("build_grid", "keys", "cell_start", "cell_end")
        for _ in range(self.iterations):
            self.dispatch(LAMBDA, self.n, self.push(dt))
            snap("lambda", "lambda_")
            self.dispatch(DELTA, self.n, self.push(dt))
            snap("delta", "delta")
            self.dispatch(APPLY_DELTA, self.n, self.push(dt))
            snap("apply_delta", "predicted")
        self.dispatch(VELOCITY, self.n, self.push(dt))
        snap("velocity", "velocities")
        self.dispatch(XSPH, self.n, self.push(dt))
        snap("xsph", "delta")
        self.dispatch(FINALIZE, self.n, self.push(dt))
        snap("finalize", "positions", "velocities")

    def _count(self, name):
        if name == "keys":
            return self.s
        if name in ("cell_start", "cell_end"):
            return self.c
        return self.n

    # -- solver/surface.py:201-239 -------------------------------------------
    def splat(self, *, dims, spacing, kernel_radius, surface_lo, dt=0.0):
        samples = int(dims[0] * dims[1] * dims[2])
        self.surface_rows = _rows(samples)
        self.surface = np.zeros(self.surface_rows * WIDTH, dtype=np.float32)
        p = self.push(dt)
        p.i_sort[:] = (*dims, _fbits(spacing))
        p.f_sph[0] = kernel_radius
        p.f_hi[:] = (*surface_lo, 0.0)
        self.dispatch(SPLAT, samples, p)
        return self.surface[:samples].copy()

    def state(self):
        return {
            "positions": self.positions[: self.n].copy(),
            "velocities": self.velocities[: self.n].copy(),
            "lambda": self.lambda_[: self.n].copy(),
            "predicted": self.predicted[: self.n].copy(),
            "delta": self.delta[: self.n].copy(),
            "normal": self.normal[: self.n].copy(),
            "keys": self.keys[: self.s].copy(),
            "cell_start": self.cell_start[: self.c].copy(),
            "cell_end": self.cell_end[: self.c].copy(),
        }

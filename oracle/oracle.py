"""Oracle (test infrastructure only): ctypes driver for the C restatement
``oracle/pbf_oracle.c`` of the reference's PBF passes.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module; the product path never imports it.

Buffers are flat float32 arrays in the reference's layouts (see the C file's
header). ``Oracle`` mirrors the dispatch sequence of ``solver/sph.py``:
``build_grid`` (``:482-498``), ``substep`` (``:501-514``) and the splat of
``solver/surface.py:201-239``.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pbf_oracle.c")
LIB_PATH = os.path.join(HERE, "liboracle.so")

ORDER_BITONIC = 0
ORDER_STABLE = 1

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

    @classmethod
    def from_bytes(cls, raw: bytes):
        p = cls()
        ctypes.memmove(ctypes.byref(p), raw, 128)
        return p


_FP = ctypes.POINTER(ctypes.c_float)


class Buffers(ctypes.Structure):
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
        ("collider", ctypes.POINTER(ctypes.c_uint8)),
    ]


def build(force=False):
    """Compile the C restatement (gcc, OpenMP, no FP contraction)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        subprocess.run(
            [
                "gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                SRC, "-o", LIB_PATH + ".tmp", "-lm",
            ],
            check=True,
        )
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        build()
        _LIB = ctypes.CDLL(LIB_PATH)
        _LIB.oracle_pass.argtypes = [ctypes.c_int, ctypes.POINTER(Push), ctypes.POINTER(Buffers)]
        _LIB.oracle_pass.restype = ctypes.c_int
        _LIB.oracle_build_grid.argtypes = [ctypes.POINTER(Push), ctypes.POINTER(Buffers), ctypes.c_int]
        _LIB.oracle_substep.argtypes = [ctypes.POINTER(Push), ctypes.POINTER(Buffers), ctypes.c_int, ctypes.c_int]
        _LIB.oracle_set_threads.argtypes = [ctypes.c_int]
        _LIB.oracle_max_threads.restype = ctypes.c_int
    return _LIB


def set_threads(n: int):
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _p(a):
    return a.ctypes.data_as(_FP) if a is not None else ctypes.cast(None, _FP)


class Oracle:
    """One scene's state in the reference layouts, stepped on the CPU."""

    def __init__(self, push_values: dict, positions, velocities, collider=None, iterations=4):
        from_values = {k: tuple(v) for k, v in push_values.items()}
        self.values = from_values
        self.n = int(positions.shape[0])
        self.s = int(from_values["i_layout"][3])
        self.c = int(from_values["i_grid"][3])
        self.iterations = int(iterations)
        n = self.n
        self.positions = np.ascontiguousarray(positions, dtype=np.float32).copy()
        self.velocities = np.ascontiguousarray(velocities, dtype=np.float32).copy()
        self.predicted = self.positions.copy()
        self.lambda_ = np.zeros((n, 4), np.float32)
        self.delta = np.zeros((n, 4), np.float32)
        self.normal = np.zeros((n, 4), np.float32)
        self.keys = np.zeros((self.s, 4), np.float32)
        self.cell_start = np.zeros(self.c, np.float32)
        self.cell_end = np.zeros(self.c, np.float32)
        self.surface = None
        self.collider = None if collider is None else np.ascontiguousarray(collider, dtype=np.uint8)

    def push(self, dt=None, **override):
        vals = dict(self.values)
        if dt is not None:
            f_sim = list(vals["f_sim"])
            f_sim[1] = dt
            vals["f_sim"] = tuple(f_sim)
        vals.update(override)
        p = Push()
        for name, _ in Push._fields_:
            src = vals.get(name, vals.get("i_surface") if name == "i_sort" else None)
            getattr(p, name)[:] = src
        return p

    def buffers(self):
        b = Buffers()
        b.positions = _p(self.positions)
        b.velocities = _p(self.velocities)
        b.lambda_ = _p(self.lambda_)
        b.predicted = _p(self.predicted)
        b.delta = _p(self.delta)
        b.normal = _p(self.normal)
        b.keys = _p(self.keys)
        b.cell_start = _p(self.cell_start)
        b.cell_end = _p(self.cell_end)
        b.surface = _p(self.surface)
        b.collider = (
            self.collider.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
            if self.collider is not None
            else ctypes.cast(None, ctypes.POINTER(ctypes.c_uint8))
        )
        return b

    def run_pass(self, pass_id, push=None):
        p = push if push is not None else self.push()
        b = self.buffers()
        if lib().oracle_pass(int(pass_id), ctypes.byref(p), ctypes.byref(b)) != 0:
            raise RuntimeError(f"oracle pass {pass_id} failed")

    def build_grid(self, dt=0.0, order=ORDER_STABLE):
        p = self.push(dt)
        b = self.buffers()
        lib().oracle_build_grid(ctypes.byref(p), ctypes.byref(b), int(order))

    def substep(self, dt=None, order=ORDER_STABLE):
        p = self.push(dt)
        b = self.buffers()
        lib().oracle_substep(ctypes.byref(p), ctypes.byref(b), self.iterations, int(order))

    def splat(self, splat_values: dict):
        dims = splat_values["i_surface"][:3]
        samples = int(dims[0] * dims[1] * dims[2])
        self.surface = np.zeros(samples, np.float32)
        p = Push()
        for name, _ in Push._fields_:
            getattr(p, name)[:] = splat_values["i_surface"] if name == "i_sort" else splat_values[name]
        b = self.buffers()
        lib().oracle_pass(SPLAT, ctypes.byref(p), ctypes.byref(b))
        return self.surface.copy()

    def state(self):
        return {
            "positions": self.positions.copy(),
            "velocities": self.velocities.copy(),
            "lambda": self.lambda_.copy(),
            "predicted": self.predicted.copy(),
            "delta": self.delta.copy(),
            "normal": self.normal.copy(),
            "keys": self.keys.copy(),
            "cell_start": self.cell_start.copy(),
            "cell_end": self.cell_end.copy(),
        }

    def load(self, state: dict):
        for name, arr in state.items():
            attr = "lambda_" if name == "lambda" else name
            getattr(self, attr)[...] = arr

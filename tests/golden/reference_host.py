"""Import the reference's own host-side Python (solver/sph.py, solver/surface.py,
collision/__init__.py) outside Blender, for generating golden vectors.

Those modules import ``bpy``, ``gpu``, ``mathutils`` and ``bmesh`` at module
level but the functions used here (config resolution, seeding, substep size,
push-constant packing, splat-grid sizing, collider grid geometry) are plain
Python arithmetic. This installs inert stand-ins for the Blender modules and a
real 3-vector for ``mathutils.Vector``, then loads the reference package from
its checkout by path. Only ``make_golden.py`` uses it, and only where the
reference checkout is mounted.
"""

from __future__ import annotations

import importlib
import importlib.util
import sys
import types


class Vector:
    """The slice of mathutils.Vector the reference's host arithmetic uses."""

    def __init__(self, values=(0.0, 0.0, 0.0)):
        self._v = [float(v) for v in values]

    x = property(lambda self: self._v[0], lambda self, v: self._v.__setitem__(0, float(v)))
    y = property(lambda self: self._v[1], lambda self, v: self._v.__setitem__(1, float(v)))
    z = property(lambda self: self._v[2], lambda self, v: self._v.__setitem__(2, float(v)))

    def __iter__(self):
        return iter(self._v)

    def __len__(self):
        return len(self._v)

    def __getitem__(self, i):
        return self._v[i]

    def __add__(self, o):
        return Vector([a + b for a, b in zip(self._v, o)])

    def __sub__(self, o):
        return Vector([a - b for a, b in zip(self._v, o)])

    def __mul__(self, s):
        return Vector([a * s for a in self._v])

    __rmul__ = __mul__

    def __truediv__(self, s):
        return Vector([a / s for a in self._v])

    def copy(self):
        return Vector(self._v)

    def __repr__(self):
        return f"Vector({self._v})"


class _AnyModule(types.ModuleType):
    """A module whose every attribute is an inert class or callable."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        value = type(name, (), {"__init__": lambda self, *a, **k: None, "__call__": lambda self, *a, **k: None})
        setattr(self, name, value)
        return value


def _props_module():
    mod = types.ModuleType("bpy.props")
    for name in ("BoolProperty", "FloatProperty", "IntProperty", "PointerProperty", "StringProperty",
                 "EnumProperty", "CollectionProperty", "FloatVectorProperty"):
        setattr(mod, name, lambda *a, **k: None)
    return mod


def install_stubs():
    bpy = _AnyModule("bpy")
    bpy.app = _AnyModule("bpy.app")
    handlers = _AnyModule("bpy.app.handlers")
    handlers.persistent = lambda f: f
    bpy.app.handlers = handlers
    bpy.props = _props_module()
    bpy.types = _AnyModule("bpy.types")
    bpy.utils = _AnyModule("bpy.utils")
    gpu = _AnyModule("gpu")
    gpu.types = _AnyModule("gpu.types")
    gpu.shader = _AnyModule("gpu.shader")
    gpu.compute = _AnyModule("gpu.compute")
    gpu_extras = _AnyModule("gpu_extras")
    gpu_extras.batch = _AnyModule("gpu_extras.batch")
    mathutils = types.ModuleType("mathutils")
    mathutils.Vector = Vector
    mathutils.bvhtree = _AnyModule("mathutils.bvhtree")
    mods = {
        "bpy": bpy,
        "bpy.app": bpy.app,
        "bpy.app.handlers": handlers,
        "bpy.props": bpy.props,
        "bpy.types": bpy.types,
        "bpy.utils": bpy.utils,
        "gpu": gpu,
        "gpu.types": gpu.types,
        "gpu.shader": gpu.shader,
        "gpu.compute": gpu.compute,
        "gpu_extras": gpu_extras,
        "gpu_extras.batch": gpu_extras.batch,
        "mathutils": mathutils,
        "mathutils.bvhtree": mathutils.bvhtree,
        "bmesh": _AnyModule("bmesh"),
    }
    for k, v in mods.items():
        sys.modules.setdefault(k, v)


def load(ref_root="/root/reference", package="flowx_reference"):
    """Return (sph, surface, collision) modules of the reference."""
    install_stubs()
    if package not in sys.modules:
        pkg = types.ModuleType(package)
        pkg.__path__ = [ref_root]
        sys.modules[package] = pkg
    sph = importlib.import_module(f"{package}.solver.sph")
    surface = importlib.import_module(f"{package}.solver.surface")
    collision = importlib.import_module(f"{package}.collision")
    return sph, surface, collision

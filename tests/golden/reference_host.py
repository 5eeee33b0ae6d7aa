"""Import the reference's own host-side Python (solver/sph.py, solver/surface.py,
collision/__init__.py) outside Blender, for generating golden vectors.

Those modules import ``bpy``, ``gpu``, ``mathutils`` and ``bmesh`` at module
level but the functions used here (config resolution, seeding, substep size,
push-constant packing, splat-grid sizing, collider grid geometry) are plain
Python arithmetic. This installs inert stand-ins for the Blender modules and a
real 3-vector for ``mathutils.Vector``, then loads the reference package from
its checkout by path.

For the collider voxeliser (collision/__init__.py ``_rebuild_grid``,
``_point_inside``, ``_rebuild_solver_grid``) it also provides what that code
calls: ``mathutils.Matrix`` (inverse, 3x3 part, matrix @ vector),
``mathutils.bvhtree.BVHTree`` (``FromObject`` over a triangle mesh and a
nearest-hit ``ray_cast``: the Moller-Trumbore ray/triangle test in float64,
hits at t > 0 with barycentric coordinates in [0, 1] inclusive; Blender's own
BVH is compiled code that is not here), ``bpy.context`` with a depsgraph, and
``gpu.types.Buffer`` / ``GPUTexture`` that keep the data handed to them (the
union grid the reference uploads). Only the fixture scripts under
tests/golden/ use this module, and only where the reference checkout is
present.
"""

from __future__ import annotations

import importlib
import importlib.util
import os
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


def _vector_normalized(self):
    n = sum(a * a for a in self._v) ** 0.5
    return Vector([a / n for a in self._v])


Vector.normalized = _vector_normalized


class Matrix:
    """The slice of mathutils.Matrix the reference's voxeliser uses (row-major,
    3x3 or 4x4; a 4x4 matrix applied to a 3-vector treats it as a point)."""

    def __init__(self, rows):
        import numpy as np

        self._m = np.array(rows, dtype=np.float64)

    def inverted(self):
        import numpy as np

        if np.linalg.det(self._m) == 0.0:
            raise ValueError("Matrix.inverted(): matrix does not have an inverse")
        return Matrix(np.linalg.inv(self._m))

    def to_3x3(self):
        return Matrix(self._m[:3, :3])

    def __matmul__(self, v):
        import numpy as np

        a = np.array(list(v), dtype=np.float64)
        if self._m.shape == (4, 4):
            out = self._m[:3, :3] @ a + self._m[:3, 3]
        else:
            out = self._m @ a
        return Vector([float(x) for x in out])


class BVHTree:
    """Stand-in for mathutils.bvhtree.BVHTree over one triangle mesh, in the
    object's local space (as FromObject builds it)."""

    def __init__(self, vertices, triangles):
        import numpy as np

        v = np.asarray(vertices, dtype=np.float64)
        t = np.asarray(triangles, dtype=np.int64).reshape(-1, 3)
        self.v0, self.v1, self.v2 = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]

    @classmethod
    def FromObject(cls, obj, depsgraph, **_kw):
        mesh = obj.evaluated_get(depsgraph).data
        verts = [tuple(v.co) for v in mesh.vertices]
        tris = []
        for poly in mesh.polygons:
            idx = list(poly.vertices)
            for k in range(1, len(idx) - 1):  # fan
                tris.append((idx[0], idx[k], idx[k + 1]))
        return cls(verts, tris)

    def ray_cast(self, origin, direction, distance=None):
        """(location, normal, index, distance) of the nearest hit at t > 0
        along the ray, or four Nones."""
        import numpy as np

        o = np.array(list(origin), dtype=np.float64)
        d = np.array(list(direction), dtype=np.float64)
        e1 = self.v1 - self.v0
        e2 = self.v2 - self.v0
        p = np.cross(d, e2)
        det = np.einsum("ij,ij->i", e1, p)
        ok = det != 0.0
        inv = np.where(ok, 1.0 / np.where(ok, det, 1.0), 0.0)
        s = o - self.v0
        u = np.einsum("ij,ij->i", s, p) * inv
        q = np.cross(s, e1)
        w = (q @ d) * inv
        t = np.einsum("ij,ij->i", e2, q) * inv
        hit = ok & (u >= 0.0) & (w >= 0.0) & (u + w <= 1.0) & (t > 0.0)
        if distance is not None:
            hit &= t <= distance
        if not hit.any():
            return None, None, None, None
        i = int(np.argmin(np.where(hit, t, np.inf)))
        n = np.cross(e1[i], e2[i])
        n = n / np.linalg.norm(n)
        loc = o + t[i] * d
        return Vector(loc), Vector(n), i, float(t[i])


class _Buffer:
    def __init__(self, fmt, shape, values=None):
        self.format, self.shape, self.values = fmt, shape, list(values) if values is not None else None


class _Texture:
    def __init__(self, size, format=None, data=None):
        self.size, self.format, self.data = size, format, data


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
    bpy.context = types.SimpleNamespace(evaluated_depsgraph_get=lambda: types.SimpleNamespace(name="depsgraph"))
    gpu = _AnyModule("gpu")
    gpu.types = _AnyModule("gpu.types")
    gpu.types.Buffer = _Buffer
    gpu.types.GPUTexture = _Texture
    gpu.shader = _AnyModule("gpu.shader")
    gpu.compute = _AnyModule("gpu.compute")
    gpu_extras = _AnyModule("gpu_extras")
    gpu_extras.batch = _AnyModule("gpu_extras.batch")
    mathutils = types.ModuleType("mathutils")
    mathutils.Vector = Vector
    mathutils.Matrix = Matrix
    mathutils.bvhtree = types.ModuleType("mathutils.bvhtree")
    mathutils.bvhtree.BVHTree = BVHTree
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


def load(ref_root=None, package="flowx_reference"):
    """Return (sph, surface, collision) modules of the reference (``ref_root``
    defaults to ``oracle.refpath.checkout()``)."""
    if ref_root is None:
        sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
        from oracle import refpath

        ref_root = refpath.checkout()
    install_stubs()
    if package not in sys.modules:
        pkg = types.ModuleType(package)
        pkg.__path__ = [ref_root]
        sys.modules[package] = pkg
    sph = importlib.import_module(f"{package}.solver.sph")
    surface = importlib.import_module(f"{package}.solver.surface")
    collision = importlib.import_module(f"{package}.collision")
    return sph, surface, collision

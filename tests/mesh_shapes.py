"""Closed triangle meshes (outward, counterclockwise faces) and world
matrices for the collider voxeliser tests, with analytic inside tests."""

from __future__ import annotations

import math

import numpy as np


def box(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    t = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [2, 3, 7], [2, 7, 6], [1, 2, 6], [1, 6, 5], [3, 0, 4], [3, 4, 7]], np.int32)
    return v, t


def octahedron(c, r):
    cx, cy, cz = c
    v = np.array([[cx + r, cy, cz], [cx - r, cy, cz], [cx, cy + r, cz], [cx, cy - r, cz],
                  [cx, cy, cz + r], [cx, cy, cz - r]], np.float32)
    t = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]], np.int32)
    return v, t


def uv_sphere(c, r, rings=24, segments=48):
    verts = [(c[0], c[1], c[2] + r)]
    for i in range(1, rings):
        th = math.pi * i / rings
        for j in range(segments):
            ph = 2.0 * math.pi * j / segments
            verts.append((c[0] + r * math.sin(th) * math.cos(ph), c[1] + r * math.sin(th) * math.sin(ph),
                          c[2] + r * math.cos(th)))
    verts.append((c[0], c[1], c[2] - r))
    south = len(verts) - 1
    tris = []
    for j in range(segments):
        tris.append((0, 1 + j, 1 + (j + 1) % segments))
    for i in range(rings - 2):
        a0 = 1 + i * segments
        b0 = a0 + segments
        for j in range(segments):
            a, an = a0 + j, a0 + (j + 1) % segments
            b, bn = b0 + j, b0 + (j + 1) % segments
            tris.append((a, b, bn))
            tris.append((a, bn, an))
    last = 1 + (rings - 2) * segments
    for j in range(segments):
        tris.append((last + j, south, last + (j + 1) % segments))
    return np.array(verts, np.float32), np.array(tris, np.int32)


def torus(c, big, small, rings=32, segments=16):
    verts = []
    for i in range(rings):
        u = 2.0 * math.pi * i / rings
        for j in range(segments):
            v = 2.0 * math.pi * j / segments
            rr = big + small * math.cos(v)
            verts.append((c[0] + rr * math.cos(u), c[1] + rr * math.sin(u), c[2] + small * math.sin(v)))
    tris = []
    for i in range(rings):
        for j in range(segments):
            a = i * segments + j
            b = ((i + 1) % rings) * segments + j
            an = i * segments + (j + 1) % segments
            bn = ((i + 1) % rings) * segments + (j + 1) % segments
            tris.append((a, b, bn))
            tris.append((a, bn, an))
    return np.array(verts, np.float32), np.array(tris, np.int32)


def identity():
    return np.eye(4, dtype=np.float32)


def rotation(axis, angle, translate=(0.0, 0.0, 0.0), scale=1.0):
    x, y, z = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    cth, sth = math.cos(angle), math.sin(angle)
    r = np.array([[cth + x * x * (1 - cth), x * y * (1 - cth) - z * sth, x * z * (1 - cth) + y * sth],
                  [y * x * (1 - cth) + z * sth, cth + y * y * (1 - cth), y * z * (1 - cth) - x * sth],
                  [z * x * (1 - cth) - y * sth, z * y * (1 - cth) + x * sth, cth + z * z * (1 - cth)]])
    m = np.eye(4)
    m[:3, :3] = r * scale
    m[:3, 3] = translate
    return m.astype(np.float32)


def centres(dims, voxel, origin):
    nx, ny, nz = dims
    o = [float(np.float32(v)) for v in origin]
    vox = float(np.float32(voxel))
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return o[0] + (x + 0.5) * vox, o[1] + (y + 0.5) * vox, o[2] + (z + 0.5) * vox

"""Generate ``tests/golden/mc_golden.npz`` from the reference's own marching
cubes (``solver/marching_cubes.py``, pure Python, imported from the reference
checkout, which is read and never modified):

    python tests/golden/make_mc_golden.py [--ref CHECKOUT]

Contents:

* ``tri_table`` (256 x 15, -1 padded) and ``tri_count`` (256): the
  reference's derived ``TRI_TABLE``;
* for each field below, the float32 samples, the lattice (dims, origin,
  spacing, iso) and the reference's ``extract`` result on those samples as
  Python floats: ``vertices`` (V x 3 float64) and ``triangles`` (T x 3 int32).

Fields (float32; the GPU path extracts float32 splat grids):

* ``sphere``  - 0.6 - |x| on a 29^3 lattice over [-1, 1]^3, iso 0;
* ``noise``   - seeded uniform noise on a 16^3 lattice with the outer layer
  set to 0, iso 0.5: every one of the 256 corner cases, closed surface;
* ``splat``   - the 64^3 density splat of the 3,200-particle dam break after
  seeding (C oracle), iso 0.5 (the reference's default surface iso);
* ``empty``   - zeros on 8^3, iso 0.5.
"""

from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from flowx_gb300 import config as C  # noqa: E402
from flowx_gb300 import scenes  # noqa: E402
from oracle import refpath  # noqa: E402


def _fields():
    out = {}
    n = 29
    ax = np.linspace(-1.0, 1.0, n)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    out["sphere"] = ((0.6 - np.sqrt(x * x + y * y + z * z)).astype(np.float32), (n, n, n), (-1.0, -1.0, -1.0),
                     2.0 / (n - 1), 0.0)
    n = 16
    noise = np.random.default_rng(7).random((n, n, n)).astype(np.float32)
    noise[[0, -1], :, :] = 0.0
    noise[:, [0, -1], :] = 0.0
    noise[:, :, [0, -1]] = 0.0
    out["noise"] = (noise, (n, n, n), (0.0, 0.0, 0.0), 0.25, 0.5)
    from oracle import oracle as O

    sc = scenes.dam_break()
    cfg = sc.config
    o = O.Oracle(C.push_constant_values(cfg, sc.dt), sc.positions, sc.velocities, iterations=cfg.iterations)
    o.build_grid(0.0)
    surf = sc.surface
    field = o.splat(C.splat_push_values(cfg, surf, sc.dt, (1, 1, 1, 0)))
    dims = tuple(int(d) for d in surf.dims)
    out["splat"] = (field.reshape(dims[::-1]).astype(np.float32), dims, tuple(surf.lo), float(surf.spacing),
                    float(surf.iso))
    out["empty"] = (np.zeros((8, 8, 8), np.float32), (8, 8, 8), (0.0, 0.0, 0.0), 0.1, 0.5)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $FLOWX_REFERENCE)")
    args = ap.parse_args()
    args.ref = args.ref or refpath.checkout()
    sys.path.insert(0, os.path.join(args.ref, "solver"))
    import marching_cubes as mc  # the reference module

    data = {}
    table = np.full((256, 15), -1, np.int32)
    counts = np.zeros(256, np.int32)
    for c, tris in enumerate(mc.TRI_TABLE):
        counts[c] = len(tris)
        for t, tri in enumerate(tris):
            table[c, 3 * t:3 * t + 3] = tri
    data["tri_table"] = table
    data["tri_count"] = counts
    for name, (field, dims, origin, spacing, iso) in _fields().items():
        flat = [float(v) for v in field.reshape(-1)]
        verts, tris = mc.extract(flat, dims, origin, spacing, iso)
        data[f"{name}_field"] = field.reshape(-1)
        data[f"{name}_lattice"] = np.array([*dims, *origin, spacing, iso], np.float64)
        data[f"{name}_vertices"] = np.array(verts, np.float64).reshape(-1, 3)
        data[f"{name}_triangles"] = np.array(tris, np.int32).reshape(-1, 3)
        print(f"{name}: {len(verts)} vertices, {len(tris)} triangles")
    np.savez_compressed(os.path.join(HERE, "mc_golden.npz"), **data)


if __name__ == "__main__":
    main()

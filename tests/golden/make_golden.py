"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run where the reference checkout is mounted (it is read, never modified):

    python tests/golden/make_golden.py [--ref CHECKOUT]

Two kinds of fixtures:

* ``host_reference.json`` / ``seed_reference.npz`` - outputs of the
  reference's own host Python (``solver/sph.py`` ``_resolve_config``,
  ``SolverConfig.substep_dt``, ``_seed_positions``, ``push_constant_values``;
  ``solver/surface.py`` ``resolve``; ``collision/__init__.py``
  ``_domain_grid_geometry``), imported outside Blender through
  ``reference_host.py``.
* ``<scene>.npz`` - pass-by-pass traces of the reference's own GLSL passes
  (compiled for the CPU by ``oracle/glsl_cpu``) on seeded synthetic scenes:
  the state after seeding and the initial grid build, every buffer each pass
  of the first substep writes (all Jacobi iterations, in dispatch order), the
  particle state after each of the first ``substeps`` substeps, and the splat
  grid after them.
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from flowx_gb300 import config as C  # noqa: E402
from flowx_gb300 import scenes  # noqa: E402
from oracle import glslref as G  # noqa: E402
from oracle import refpath  # noqa: E402


# ---------------------------------------------------------------- host vectors
HOST_DOMAINS = [
    # lo, hi, fluid_level, smoothing_radius, rest_density, viscosity, surface_res, collider_res
    ((-1.0, -1.0, 0.0), (1.0, 1.0, 2.0), 50.0, 0.1, 1000.0, 0.1, 48, 32),
    ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 40.0, 0.1, 1000.0, 0.1, 52, 32),
    ((0.0, 0.0, 0.0), (3.0, 1.0, 0.5), 75.0, 0.05, 997.0, 0.5, 64, 48),
    ((-2.0, -0.5, 0.0), (2.0, 0.5, 1.0), 35.0, 0.02, 1000.0, 0.01, 96, 64),
    ((0.0, 0.0, 0.0), (0.3, 0.3, 0.3), 60.0, 0.04, 1200.0, 2.0, 24, 16),
]


def host_vectors(ref_root):
    import reference_host as RH

    sph, surface, collision = RH.load(ref_root)
    V = RH.Vector
    out = []
    seeds = {}
    for idx, (lo, hi, fill, h, rho, visc, sres, cres) in enumerate(HOST_DOMAINS):
        settings = types.SimpleNamespace(
            fluid_level=fill, rest_density=rho, pbf_relaxation=100.0, pbf_iterations=4, pbf_scorr_k=0.1,
            surface_tension=0.05, viscosity=visc, max_substeps=24, smoothing_radius=h,
            surface_resolution=sres, surface_iso=0.5, resolution=cres,
        )
        dom = types.SimpleNamespace(flowx_domain=settings)
        sph.world_bounds = lambda d, lo=lo, hi=hi: (V(lo), V(hi))
        collision.world_bounds = sph.world_bounds
        cfg = sph._resolve_config(dom)
        values = sph._seed_positions(cfg)
        cfg.particle_count = len(values) // 4
        cfg.sorted_count = max(2, 1 << (max(1, cfg.particle_count) - 1).bit_length())
        rec = {
            "domain": {"lo": lo, "hi": hi, "fluid_level": fill, "smoothing_radius": h, "rest_density": rho,
                       "viscosity": visc, "surface_resolution": sres, "collider_resolution": cres},
            "config": {
                "smoothing_radius": cfg.smoothing_radius, "spacing": cfg.spacing, "mass": cfg.mass,
                "cell_size": cfg.cell_size, "cell_dims": list(cfg.cell_dims), "cell_count": cfg.cell_count,
                "particle_count": cfg.particle_count, "sorted_count": cfg.sorted_count,
            },
            "substep_dt": {str(fps): list(cfg.substep_dt(1.0 / fps)) for fps in (24, 30, 60, 120)},
        }
        origin, voxel, dims = collision._domain_grid_geometry(dom)
        rec["collider_geometry"] = {"origin": list(origin), "voxel": voxel, "dims": list(dims)}
        i_collider = (*dims, C.float_bits(voxel)) if voxel > 0 else (1, 1, 1, 0)
        steps, dt = cfg.substep_dt(1.0 / 24)
        rec["push"] = {k: list(v) for k, v in sph.push_constant_values(cfg, dt, i_collider, 4, 2).items()}
        surf = surface.resolve(dom, cfg)
        rec["surface"] = {"dims": list(surf.dims), "spacing": surf.spacing, "kernel_radius": surf.kernel_radius,
                          "lo": list(surf.lo), "sample_count": surf.sample_count}
        out.append(rec)
        if cfg.particle_count <= 3000:
            seeds[f"seed{idx}"] = np.asarray(values, dtype=np.float64).reshape(-1, 4)
    with open(os.path.join(HERE, "host_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "seed_reference.npz"), **seeds)
    print("host vectors:", len(out), "domains;", ", ".join(f"{k}:{v.shape[0]}" for k, v in seeds.items()))


# ------------------------------------------------------------------ pass traces
STATE_BUFS = ("positions", "velocities", "lambda", "predicted", "delta", "normal", "keys", "cell_start", "cell_end")


def _harness(scene, col):
    c = scene.config
    return G.GlslRef(
        lo=c.lo, hi=c.hi, cell_size=c.cell_size, cell_dims=c.cell_dims, h=c.smoothing_radius, mass=c.mass,
        rest_density=c.rest_density, relaxation=c.relaxation, scorr=c.scorr_strength, sigma=c.surface_tension,
        viscosity=c.viscosity, particle_radius=c.particle_radius, positions=scene.positions,
        velocities=scene.velocities, iterations=c.iterations, collider=col, collider_voxel=scene.collider_voxel,
    )


def trace_scene(name, scene, substeps=4, splat_dims=None):
    col = scene.collider_grid(0)
    g = _harness(scene, col)
    dt = scene.dt
    g.build_grid(0.0)  # solver/sph.py:606: the seed's zero-length grid build
    rec = {}
    init = g.state()
    for b in STATE_BUFS:
        rec[f"init_{b}"] = init[b]
    order = []

    def out(pass_name, bufs):
        st = g.state()
        i = len(order)
        order.append(pass_name)
        for b in bufs:
            rec[f"p{i:02d}_{pass_name}_{b}"] = st[b]

    if g.sigma > 0.0:
        g.dispatch(G.NORMAL, g.n, g.push(dt))
        out("normal", ["normal"])
    g.dispatch(G.PREDICT, g.n, g.push(dt))
    out("predict", ["velocities", "predicted"])
    g.build_grid(dt)
    out("build_grid", ["keys", "cell_start", "cell_end"])
    for _ in range(g.iterations):
        g.dispatch(G.LAMBDA, g.n, g.push(dt))
        out("lambda", ["lambda"])
        g.dispatch(G.DELTA, g.n, g.push(dt))
        out("delta", ["delta"])
        g.dispatch(G.APPLY_DELTA, g.n, g.push(dt))
        out("apply_delta", ["predicted"])
    g.dispatch(G.VELOCITY, g.n, g.push(dt))
    out("velocity", ["velocities"])
    g.dispatch(G.XSPH, g.n, g.push(dt))
    out("xsph", ["delta"])
    g.dispatch(G.FINALIZE, g.n, g.push(dt))
    out("finalize", ["positions", "velocities"])
    st = g.state()
    for b in ("positions", "velocities", "lambda", "predicted"):
        rec[f"sub01_{b}"] = st[b]
    for k in range(2, substeps + 1):
        g.substep(dt)
        st = g.state()
        for b in ("positions", "velocities", "lambda", "predicted"):
            rec[f"sub{k:02d}_{b}"] = st[b]
    st = g.state()
    for b in ("keys", "cell_start", "cell_end", "normal"):
        rec[f"last_{b}"] = st[b]
    c = scene.config
    ic = C.collider_binding(scene.collider_dims, scene.collider_voxel)
    push = C.push_constant_values(c, dt, ic)
    meta = {
        "name": name, "n": g.n, "s": g.s, "c": g.c, "substeps": substeps, "dt": dt,
        "iterations": c.iterations, "order": order, "push": {k: list(v) for k, v in push.items()},
    }
    if col is not None:
        rec["collider"] = col
        meta["collider_dims"] = list(scene.collider_dims)
        meta["collider_voxel"] = scene.collider_voxel
    if splat_dims:
        surf = C.surface_for_dims(c, splat_dims)
        rec["splat"] = g.splat(dims=surf.dims, spacing=surf.spacing, kernel_radius=surf.kernel_radius,
                               surface_lo=surf.lo, dt=dt)
        sp = C.splat_push_values(c, surf, dt, ic)
        meta["splat_push"] = {k: list(v) for k, v in sp.items()}
    rec["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **rec)
    print(f"{name}: n={g.n} cells={g.c} passes={len(order)} -> {name}.npz "
          f"({os.path.getsize(os.path.join(HERE, name + '.npz')) // 1024} KiB)")


def pile_scene():
    """1,200 particles: a 10x10x5 lattice plus 700 particles jittered inside
    one cell (more than MAX_CELL_SCAN = 512, sph_common.glsl:27-30), a few
    seeded outside the domain (cell_coord clamping, sph_common.glsl:50-54) and
    random initial velocities."""
    lo, hi, h = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.1
    cfg = scenes.make_config(lo, hi, h)
    base = scenes.lattice(lo, cfg.spacing, (10, 10, 5), h, seed=7, offset=(0.2, 0.2, 0.0))
    rng = np.random.default_rng(8)
    pile = np.ones((700, 4), np.float32)
    pile[:, :3] = (np.array([0.55, 0.55, 0.35]) + rng.uniform(0.0, 0.1, size=(700, 3))).astype(np.float32)
    out = np.ones((12, 4), np.float32)
    out[:, :3] = rng.uniform(-0.3, 1.3, size=(12, 3)).astype(np.float32)
    pos = np.concatenate([base, pile, out])
    perm = rng.permutation(pos.shape[0])
    pos = pos[perm]
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.5, size=(pos.shape[0], 3)).astype(np.float32)
    return scenes._finish("pile", cfg, pos, 32, 1, vel=vel)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $FLOWX_REFERENCE)")
    args = ap.parse_args()
    args.ref = args.ref or refpath.checkout()
    G.build(args.ref)
    host_vectors(args.ref)
    trace_scene("dam_break", scenes.dam_break(), substeps=4, splat_dims=64)
    trace_scene("dam_break_defaults", scenes.dam_break(reference_defaults=True), substeps=1)
    trace_scene("pool_small", scenes.pool(extent=0.5, counts=(20, 20, 12)), substeps=4, splat_dims=40)
    trace_scene("pile", pile_scene(), substeps=1, splat_dims=24)


if __name__ == "__main__":
    main()

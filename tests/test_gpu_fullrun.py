"""Full runs of the fused substep against the oracle.

Over many substeps the trajectories of any two float32 evaluations that
round differently diverge (the substep is chaotic), so the full-run bar is
on statistics: mean density, kinetic energy and splat volume (samples at or
above the iso value times spacing^3), each averaged over every frame of the
run, within 0.5% relative. Over the full-length runs the kinetic energy is
taken with speeds clipped at the predict step's clamp (see
_clipped_kinetic_energy; the unclipped figure is reported). The reference-arithmetic mode (EXACT) is held to
more: it stays bit-identical to the oracle for the whole run.

Workloads: the 3,200-particle dam break (1 m cube, h 0.1, 48 frames of 4
substeps, 64^3 splat) and the first 24 of the 307,200-particle pool's 120
frames (cylinder and wall colliders, 128^3 splat), against the oracle; and
the stated full lengths - the pool's 120 frames, the 4,000,000-particle large
scene's 240 frames with the falling sphere re-voxelised on the device every
frame and the 256^3 splat - against the EXACT path on the GPU. EXACT stands
in for the oracle there: it equals the oracle bit for bit at these sizes
(tests/test_gpu_workloads.py, one substep from seeded and mid-run states) and
over the 48-frame dam break (below), while the oracle would take most of an
hour for the large run's 960 substeps.
"""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu

STAT_TOL = 5e-3  # relative, on run-averaged statistics


def _stats(vel, lam, surf, cfg, surface):
    return np.array([
        lam[:, 0].astype(np.float64).mean(),
        0.5 * cfg.mass * (vel[:, :3].astype(np.float64) ** 2).sum(),
        (surf >= surface.iso).sum() * surface.spacing**3,
    ])


def _run(sc, frames, exact):
    from flowx_gb300.sph import Solver

    cfg, dt, surface = sc.config, sc.dt, sc.surface
    col = sc.collider_grid(0)
    ic = C.collider_binding(sc.collider_dims, sc.collider_voxel) if col is not None else (1, 1, 1, 0)
    o = O.Oracle(C.push_constant_values(cfg, dt, ic), sc.positions, sc.velocities, collider=col,
                 iterations=cfg.iterations)
    o.build_grid(0.0)
    got, want = [], []
    with Solver(cfg, sc.positions, sc.velocities, collider=col,
                collider_voxel=sc.collider_voxel if col is not None else 0.0,
                max_surface_samples=surface.sample_count, exact=exact) as s:
        s._build_grid(0.0)
        for _ in range(frames):
            s.step_substeps(dt, sc.substeps_per_frame)
            for _ in range(sc.substeps_per_frame):
                o.substep(dt)
            got.append(_stats(s.read("velocities"), s.read("lambda"), s.update_surface(surface, dt), cfg, surface))
            want.append(_stats(o.velocities, o.lambda_, o.splat(C.splat_push_values(cfg, surface, dt, ic)), cfg,
                               surface))
        final = {b: s.read(b) for b in ("positions", "velocities")}
    return np.array(got), np.array(want), final, o


def test_exact_full_dam_break_run_is_bit_identical():
    sc = scenes.dam_break()
    got, want, final, o = _run(sc, 48, exact=True)
    np.testing.assert_array_equal(final["positions"], o.positions)
    np.testing.assert_array_equal(final["velocities"], o.velocities)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("name,frames", [("dam_break", 48), ("pool", 24)])
def test_fast_full_run_statistics_within_half_percent(name, frames):
    sc = getattr(scenes, name)()
    got, want, final, _ = _run(sc, frames, exact=False)
    assert np.isfinite(final["positions"]).all()
    err = np.abs(got.mean(0) - want.mean(0)) / np.abs(want.mean(0))
    assert (err <= STAT_TOL).all(), dict(zip(("density", "kinetic_energy", "splat_volume"), err))


def _clipped_kinetic_energy(vel, cfg, dt):
    """Kinetic energy with each speed clipped at the predict step's clamp
    0.4 h / dt (sph_predict.glsl:48-52): the velocity a particle carries into
    the next substep. The reference's XSPH pass weights neighbours by
    m / max(rho_j, 1e-6) (sph_xsph.glsl), so a particle beside one that left
    its sorted cell (its own density term lost, rho at the floor) can end a
    substep at ~1e5 m/s; XSPH moves no position, and the next predict clamps
    that speed, but one such particle outweighs the whole fluid's kinetic
    energy in the frame it happens."""
    v = np.asarray(vel)[:, :3].astype(np.float64)
    sp = np.linalg.norm(v, axis=1)
    vmax = 0.4 * cfg.smoothing_radius / max(dt, 1e-6)
    return 0.5 * cfg.mass * (np.minimum(sp, vmax) ** 2).sum(), 0.5 * cfg.mass * (sp**2).sum()


def _device_run(sc, frames, exact, every):
    """Per-frame statistics of a run with the collider voxelised on the device
    every frame (the benchmark's loop), sampled every `every` frames."""
    from flowx_gb300.sph import Solver

    cfg, dt, surface = sc.config, sc.dt, sc.surface
    out = []
    rho3 = None
    with Solver(cfg, sc.positions, sc.velocities, max_collider_voxels=int(np.prod(sc.collider_dims)),
                max_surface_samples=surface.sample_count, exact=exact) as s:
        s._build_grid(0.0)
        for f in range(frames):
            s.voxelize(sc.primitives_at(f), sc.collider_dims, sc.collider_voxel)
            s.step_substeps(dt, sc.substeps_per_frame)
            if f == 2:
                rho3 = float(s.read("lambda")[:, 0].astype(np.float64).mean())
            if f % every == every - 1:
                vel = s.read("velocities")
                st = _stats(vel, s.read("lambda"), s.update_surface(surface, dt), cfg, surface)
                clipped, raw = _clipped_kinetic_energy(vel, cfg, dt)
                out.append([st[0], clipped, st[2], raw])
        assert np.isfinite(s.read("positions")).all()
    return np.array(out), rho3


@pytest.mark.parametrize("name,frames,every", [("pool", 120, 1), ("large", 240, 2)])
def test_fast_full_length_run_statistics_against_exact(name, frames, every):
    sc = getattr(scenes, name)()
    fast, rho3 = _device_run(sc, frames, exact=False, every=every)
    exact, _ = _device_run(sc, frames, exact=True, every=every)
    err = np.abs(fast.mean(0) - exact.mean(0)) / np.abs(exact.mean(0))
    print(f"{name} {frames} frames: run-averaged density / kinetic energy (speeds at the clamp) / splat volume, "
          f"FAST vs EXACT: {err[0]:.2e} / {err[1]:.2e} / {err[2]:.2e}; unclipped kinetic energy {err[3]:.2e} "
          f"(largest frame / median frame: FAST {fast[:, 3].max() / np.median(fast[:, 3]):.1f}, "
          f"EXACT {exact[:, 3].max() / np.median(exact[:, 3]):.1f})")
    assert (err[:3] <= STAT_TOL).all(), dict(zip(("density", "kinetic_energy", "splat_volume"), err[:3]))
    # Reported, not bounded: at these particle masses (1e-3 kg in the large
    # scene) the cohesion term (sph_predict.glsl:41-46 divides sigma * kappa
    # by the mass) sends most interior particles to the speed clamp every
    # substep, and the fluid stays compressed well past the 15% the
    # reference's own smoke check allows its dam break
    # (scripts/smoke_test.py:107-134; that check runs in
    # tests/test_gpu_parity.py on the dam break).
    rest = sc.config.rest_density
    print(f"{name}: mean density after 3 frames {rho3 / rest:.3f} of rest; over the run "
          f"{fast[:, 0].min() / rest:.3f} to {fast[:, 0].max() / rest:.3f}")

"""Parity at the benchmarked workloads, one substep at full size.

The large scene (2 m cube, h 0.02, 200x200x100 = 4,000,000 particles, cells
of h, cohesion 0.1, XSPH 0.01, 4 Jacobi iterations, the 0.3 m sphere
voxelised on 100^3 voxels of h) and the pool (307,200 particles, cylinder and
wall on 40^3 voxels). Each case installs one state on the GPU and in the
oracle the way a cached frame is installed (positions, velocities, predicted,
lambda; solver/sph.py:700-733), builds the grid from the predicted positions
and runs one substep (solver/sph.py:501-514):

* EXACT (the reference's expressions) is bit-exact against the oracle in the
  (cell, id) order: positions, velocities, predicted, lambda, normal, keys
  (with ids), cell ranges;
* EXACT with the reference's own grid order (FLOWX_FLAG_REFERENCE_ORDER: the
  bitonic network of sph_sort.glsl) is bit-exact against the oracle running
  that network;
* FAST (the benchmarked arithmetic) rounds differently, and these substeps
  are ill-conditioned (tests/rounding.py): changing every input position by
  one ulp moves the oracle's own output by up to 1e-3 h and beyond here
  (collider push-out, the seeded lattice's clamped cohesion steps). FAST is
  held to within a small factor of that sensitivity, quantile by quantile.
  (Its keys are not compared: they follow from its own predicted positions.)

States: the seeded lattice with the collider where the benchmark meets it
(the large scene's sphere at frame 10, a third of it under the free surface),
and the states the GPU's own FAST run reaches after some frames (moving
fluid, the sphere inside it, particles pushed out of the collider; for the
large scene also after 60 frames, in the agitated state it keeps).
"""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import oracle as O
from rounding import assert_within_sensitivity, per_particle, perturbed_state

pytestmark = pytest.mark.gpu

STATE = ("positions", "velocities", "predicted", "lambda")


def _solver(scene, state, col, exact, reference_order=False):
    from flowx_gb300.sph import Solver

    s = Solver(scene.config, state["positions"], state["velocities"], collider=col,
               collider_voxel=scene.collider_voxel if col is not None else 0.0, exact=exact,
               reference_order=reference_order)
    s.write("predicted", state["predicted"])
    s.write("lambda", state["lambda"])
    return s


def _gpu_substep(scene, state, col, exact, graph, reference_order=False):
    cfg = scene.config
    with _solver(scene, state, col, exact, reference_order) as s:
        s._build_grid(0.0)
        if graph:
            s.step_substeps(scene.dt, 1)
        else:
            s._substep(scene.dt)
        out = {b: s.read(b) for b in STATE + ("normal",)}
        out["keys"] = s.read("keys", cfg.sorted_count)
        out["cell_start"] = s.read("cell_start")
        out["cell_end"] = s.read("cell_end")
    return out


def _oracle_substep(scene, state, col, order=O.ORDER_STABLE):
    cfg = scene.config
    ic = C.collider_binding(scene.collider_dims if col is not None else None,
                            scene.collider_voxel if col is not None else 0.0)
    O.set_threads(O.max_threads())
    o = O.Oracle(C.push_constant_values(cfg, scene.dt, ic), state["positions"], state["velocities"], collider=col,
                 iterations=cfg.iterations)
    o.predicted[...] = state["predicted"]
    o.lambda_[...] = state["lambda"]
    o.build_grid(0.0, order=order)
    o.substep(scene.dt, order=order)
    return o.state()


def _seeded(scene):
    return {"positions": scene.positions, "velocities": scene.velocities, "predicted": scene.positions,
            "lambda": np.zeros_like(scene.positions)}


def _after_frames(scene, frames):
    """The state the FAST path reaches after `frames` frames, the collider
    re-voxelised on the device every frame as the benchmark does."""
    from flowx_gb300.sph import Solver

    cfg = scene.config
    with Solver(cfg, scene.positions, scene.velocities, max_collider_voxels=int(np.prod(scene.collider_dims))) as s:
        s._build_grid(0.0)
        for f in range(frames):
            s.voxelize(scene.primitives_at(f), scene.collider_dims, scene.collider_voxel)
            s.step_substeps(scene.dt, scene.substeps_per_frame)
        state = {b: s.read(b) for b in STATE}
    assert np.isfinite(state["positions"]).all()
    return state


def _check(scene, state, col, tag):
    h = scene.config.smoothing_radius
    want = _oracle_substep(scene, state, col)
    exact = _gpu_substep(scene, state, col, exact=True, graph=True)
    for b in STATE + ("normal", "keys", "cell_start", "cell_end"):
        np.testing.assert_array_equal(exact[b], want[b], err_msg=f"{tag} EXACT {b}")
    fast = _gpu_substep(scene, state, col, exact=False, graph=True)
    moved = perturbed_state(state)
    noise = per_particle(_oracle_substep(scene, moved, col)["positions"], want["positions"], h)
    err = per_particle(fast["positions"], want["positions"], h)
    assert_within_sensitivity(f"{tag} (n={scene.n})", err, noise)


def _check_reference_order(scene, state, col, tag):
    want = _oracle_substep(scene, state, col, order=O.ORDER_BITONIC)
    got = _gpu_substep(scene, state, col, exact=True, graph=True, reference_order=True)
    n = scene.n
    # keys: the particles' entries (the network also reorders the padding
    # entries past them, key = cell count, which no pass reads)
    want["keys"] = want["keys"][:n]
    got["keys"] = got["keys"][:n]
    for b in STATE + ("normal", "keys", "cell_start", "cell_end"):
        np.testing.assert_array_equal(got[b], want[b], err_msg=f"{tag} reference order {b}")


@pytest.fixture(scope="module")
def large():
    return scenes.large()


@pytest.fixture(scope="module")
def pool():
    return scenes.pool()


def test_large_seeded_sphere_in_fluid(large):
    _check(large, _seeded(large), large.collider_grid(10), "large seeded, sphere at frame 10")


def test_large_after_twelve_frames(large):
    state = _after_frames(large, 12)
    _check_reference_order(large, state, large.collider_grid(12), "large after 12 frames")
    _check(large, state, large.collider_grid(12), "large after 12 frames")


def test_large_after_sixty_frames(large):
    """The agitated state the benchmark runs in (cohesion drives most
    interior particles to the speed clamp every substep)."""
    state = _after_frames(large, 60)
    _check(large, state, large.collider_grid(60), "large after 60 frames")


@pytest.fixture(scope="module")
def coarse():
    """The large scene's domain and particle spacing with the reference's own
    cell rule (cells of 0.045 m = 2.25 h, 45^3), a 60 x 60 x 30 block of it:
    ~91 particles per cell, stencil rows of ~270 slots, the walk that trims
    each row to the particle's reach."""
    sc = scenes.large(cell_rule="reference", counts=(60, 60, 30))
    assert sc.config.cell_size >= 2.0 * sc.config.smoothing_radius
    return sc


def test_coarse_cells_seeded(coarse):
    _check_reference_order(coarse, _seeded(coarse), coarse.collider_grid(0), "coarse cells seeded")
    _check(coarse, _seeded(coarse), coarse.collider_grid(0), "coarse cells seeded")


def test_coarse_cells_after_twelve_frames(coarse):
    state = _after_frames(coarse, 12)
    _check(coarse, state, coarse.collider_grid(12), "coarse cells after 12 frames")


def test_pool_seeded(pool):
    _check_reference_order(pool, _seeded(pool), pool.collider_grid(0), "pool seeded")
    _check(pool, _seeded(pool), pool.collider_grid(0), "pool seeded")


def test_pool_after_twenty_four_frames(pool):
    state = _after_frames(pool, 24)
    _check(pool, state, pool.collider_grid(0), "pool after 24 frames")


def test_pool_after_its_full_run(pool):
    """The state at the end of the pool's 120-frame run, in both grid orders."""
    state = _after_frames(pool, 120)
    _check_reference_order(pool, state, pool.collider_grid(0), "pool after 120 frames")
    _check(pool, state, pool.collider_grid(0), "pool after 120 frames")

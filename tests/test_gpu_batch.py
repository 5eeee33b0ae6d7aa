"""Batched scenes (one context, one launch per pass for all scenes) against
each scene stepped alone, and the block-size autotuner."""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mixed_scenes():
    """Scenes of different sizes, parameters, grids and colliders."""
    out = [scenes.dam_break(), scenes.pool(extent=0.5, counts=(20, 20, 12))]
    small = scenes.batched_scenes(count=4, seed=3, n_range=(800, 6000))
    out.extend(small)
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_scenes_stepped_alone(graph):
    from flowx_gb300.batch import Batch
    from flowx_gb300.sph import Solver

    sc = _mixed_scenes()
    nsub = 3
    with Batch(sc, exact=True) as b:
        b.build_grid()
        if graph:
            b.step(4, nsub)
        else:
            for _ in range(nsub):
                b.substep(4)
        got = {name: b.read(name) for name in ("positions", "velocities", "lambda", "predicted")}
    for k, s in enumerate(sc):
        lo, hi = sum(x.n for x in sc[:k]), sum(x.n for x in sc[: k + 1])
        with Solver(s.config, s.positions, s.velocities, collider=s.collider_grid(0),
                    collider_voxel=s.collider_voxel, exact=True) as one:
            one._build_grid(0.0)
            for _ in range(nsub):
                one._substep(s.dt)
            for name, arr in got.items():
                np.testing.assert_array_equal(arr[lo:hi], one.read(name), err_msg=f"scene {k} {name}")


def test_batch_beyond_the_constant_segment_table():
    """A batch reads its scenes' parameters from its slice of a constant-memory
    copy of the segment table (128 entries per device), or from the device
    table when no slice is free. 130 scenes take the device table; the same
    scenes as two batches of 65 alive at once take a slice (the first) and the
    device table (the second: 63 entries are left); the second again, after
    the first has closed, takes the slice the first released. Every one of
    these substeps is the same bit for bit (the re-associated arithmetic)."""
    from flowx_gb300.batch import Batch

    sc = scenes.batched_scenes(count=130, seed=7, n_range=(200, 600))
    nsub = 2
    names = ("positions", "velocities", "lambda")

    def run(b):
        b.build_grid()
        b.step(4, nsub)
        return {name: b.read(name) for name in names}

    with Batch(sc) as b:
        want = run(b)
    n1 = sum(x.n for x in sc[:65])
    first, second = sc[:65], sc[65:]

    def check(got, lo, tag):
        for name in names:
            np.testing.assert_array_equal(got[name], want[name][lo:lo + len(got[name])], err_msg=f"{tag} {name}")

    with Batch(first) as b1:
        check(run(b1), 0, "first (slice)")
        with Batch(second) as b2:
            check(run(b2), n1, "second (table full)")
    with Batch(second) as b3:
        check(run(b3), n1, "second (released slice)")


def test_batch_with_coarse_cells_equals_scenes_stepped_alone():
    """A batch holding a scene whose cells are coarser than its reach (the
    reference's own cell rule, 2.25 h) runs the trimmed walk for all its
    scenes (row bounds per x-row, each x-row finding its scene). Each scene's
    substeps equal the scene stepped alone, bit for bit (the reference's
    expressions), the dam break alone taking the untrimmed walk."""
    from flowx_gb300.batch import Batch
    from flowx_gb300.sph import Solver

    coarse = scenes.large(cell_rule="reference", counts=(40, 40, 20))
    assert coarse.config.cell_size >= 2.0 * coarse.config.smoothing_radius
    sc = [scenes.dam_break(), coarse]
    nsub = 2
    with Batch(sc, exact=True) as b:
        b.build_grid()
        b.step(4, nsub)
        got = {name: b.read(name) for name in ("positions", "velocities", "lambda")}
    lo = 0
    for k, s in enumerate(sc):
        col = s.collider_grid(0)
        with Solver(s.config, s.positions, s.velocities, collider=col,
                    collider_voxel=s.collider_voxel if col is not None else 0.0, exact=True) as one:
            one._build_grid(0.0)
            for _ in range(nsub):
                one._substep(s.dt)
            for name, arr in got.items():
                np.testing.assert_array_equal(arr[lo:lo + s.n], one.read(name), err_msg=f"scene {k} {name}")
        lo += s.n


def test_batch_scene_matches_oracle():
    from flowx_gb300.batch import Batch

    sc = _mixed_scenes()
    with Batch(sc, exact=True) as b:
        b.build_grid()
        b.substep(4)
        pos = b.read("positions")
    k = 1  # the pool scene (collider)
    s = sc[k]
    lo = sum(x.n for x in sc[:k])
    ic = C.collider_binding(s.collider_dims, s.collider_voxel)
    o = O.Oracle(C.push_constant_values(s.config, s.dt, ic), s.positions, s.velocities,
                 collider=s.collider_grid(0), iterations=4)
    o.build_grid(0.0)
    o.substep(s.dt)
    np.testing.assert_array_equal(pos[lo:lo + s.n], o.positions)


def test_batch_splat_matches_single_scene():
    from flowx_gb300.batch import Batch
    from flowx_gb300.sph import Solver

    sc = _mixed_scenes()
    s = sc[1]
    with Batch(sc, exact=True, max_surface_samples=max(x.surface.sample_count for x in sc)) as b:
        b.build_grid()
        b.substep(4)
        got = b.splat(1, dt=s.dt)
    with Solver(s.config, s.positions, s.velocities, collider=s.collider_grid(0), collider_voxel=s.collider_voxel,
                exact=True, max_surface_samples=s.surface.sample_count) as one:
        one._build_grid(0.0)
        one._substep(s.dt)
        want = one.update_surface(s.surface, s.dt)
    np.testing.assert_array_equal(got, want)


def test_autotune_keeps_state_and_results():
    from flowx_gb300.batch import Batch

    sc = _mixed_scenes()
    with Batch(sc, exact=True) as b:
        b.build_grid()
        b.substep(4)
        before = b.read("positions")
        chosen = b.autotune(4)
        assert chosen and all(v in (64, 128, 256, 512) for v in chosen.values())
        np.testing.assert_array_equal(b.read("positions"), before)
        b.substep(4)
        tuned = b.read("positions")
    with Batch(sc, exact=True) as ref:
        ref.build_grid()
        ref.substep(4)
        ref.substep(4)
        np.testing.assert_array_equal(ref.read("positions"), tuned)


def test_batch_rejects_single_scene_calls():
    import ctypes

    from flowx_gb300 import _lib
    from flowx_gb300.batch import Batch

    sc = _mixed_scenes()[:2]
    with Batch(sc) as b:
        push = _lib.Push.from_values(C.push_constant_values(sc[0].config, sc[0].dt))
        rc = b.lib.flowx_substep(b._ctx, ctypes.byref(push), 4)
        assert rc == 3  # FLOWX_ERR_STATE

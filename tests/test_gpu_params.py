"""A single-scene context's substep kernels read the scene's parameters from
their launch arguments, which a captured frame graph carries. A push block
whose values change between calls must therefore re-capture the graph:
graph-launched substeps with dt and then dt / 2 equal the same substeps
launched one by one (the reference's expressions, bit for bit), with the
neighbour passes one thread and one warp per particle."""

import numpy as np
import pytest

from flowx_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("passes", ["thread", "warp"])
def test_changed_parameters_recapture_the_frame_graph(passes):
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    cfg, dt = sc.config, sc.dt
    with Solver(cfg, sc.positions, sc.velocities, exact=True, passes=passes) as a:
        a._build_grid(0.0)
        a.step_substeps(dt, 2)
        a.step_substeps(0.5 * dt, 2)
        a.step_substeps(dt, 2)
        got = {b: a.read(b) for b in ("positions", "velocities", "lambda")}
    with Solver(cfg, sc.positions, sc.velocities, exact=True, passes=passes) as b:
        b._build_grid(0.0)
        for step in (dt, dt, 0.5 * dt, 0.5 * dt, dt, dt):
            b._substep(step)
        want = {k: b.read(k) for k in got}
    for k in got:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    assert not np.array_equal(got["positions"], sc.positions)

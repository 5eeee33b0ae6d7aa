"""The cached-frame path on the GPU (solver/cache.py write_frame / try_load,
solver/sph.py:700-733 _apply_cached): frames written from a running context
read back exactly, and a fresh context that loads one (positions,
velocities, predicted = positions, lambda zero, grid rebuilt) then steps
stays bit-identical to the oracle started from the same stored state."""

import numpy as np
import pytest

from flowx_gb300 import config as C
from flowx_gb300 import scenes
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_cached_frame_round_trip_and_reload_matches_oracle(tmp_path):
    from flowx_gb300.cache import FrameCache, config_hash
    from flowx_gb300.sph import Solver

    sc = scenes.dam_break()
    cfg, dt, sub = sc.config, sc.dt, sc.substeps_per_frame
    digest = config_hash(cfg, 24.0)
    path = str(tmp_path / "dam.flwxcache")
    stored = {}
    with FrameCache.open(path, particle_count=sc.n, seed_frame=0, fps=24.0, config_hash_bytes=digest) as cache:
        with Solver(cfg, sc.positions, sc.velocities, exact=True) as a:
            a._build_grid(0.0)
            for frame in range(1, 4):
                a.step_substeps(dt, sub)
                cache.write_frame(frame, a)
                stored[frame] = (a.read("positions"), a.read("velocities"))
        assert cache.header()["last_frame"] == 3
        for frame, (p, v) in stored.items():
            rp, rv = cache.read_frame_host(frame)
            np.testing.assert_array_equal(rp, p)
            np.testing.assert_array_equal(rv, v)
        with Solver(cfg, sc.positions, sc.velocities, exact=True) as b:
            assert not cache.try_load(4, b, 0.0)  # past the cached range
            assert not cache.try_load(2, b, 0.0, config_hash_bytes=b"\1" * 32)  # other settings
            assert cache.try_load(2, b, 0.0, config_hash_bytes=digest)
            np.testing.assert_array_equal(b.read("positions"), stored[2][0])
            np.testing.assert_array_equal(b.read("predicted"), stored[2][0])
            b.step_substeps(dt, sub)
            got = {k: b.read(k) for k in ("positions", "velocities", "predicted", "lambda")}
    p2, v2 = stored[2]
    o = O.Oracle(C.push_constant_values(cfg, dt), p2, v2, iterations=cfg.iterations)
    o.build_grid(0.0)
    for _ in range(sub):
        o.substep(dt)
    want = o.state()
    for k, arr in got.items():
        np.testing.assert_array_equal(arr, want[k], err_msg=k)

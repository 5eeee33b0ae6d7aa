"""Host-side packing of batched scenes (no GPU)."""

from flowx_gb300 import scenes
from flowx_gb300.batch import pack_layout, scene_push


def test_pack_layout_offsets():
    sc = scenes.batched_scenes(count=5, seed=3, n_range=(500, 3000))
    p, c, v = pack_layout(sc)
    assert p[0] == 0 and c[0] == 0 and v[0] == 0
    for k, s in enumerate(sc):
        assert p[k + 1] - p[k] == s.n
        assert c[k + 1] - c[k] == s.config.cell_count
        expect = 0 if s.collider_dims is None else s.collider_dims[0] * s.collider_dims[1] * s.collider_dims[2]
        assert v[k + 1] - v[k] == expect


def test_batched_workload_shapes():
    """The 64-scene workload: counts log-uniform in [2e3, 2e5], h from the
    h/2 lattice, 0-2 box colliders at voxel = h."""
    sc = scenes.batched_scenes()
    assert len(sc) == 64
    ns = [s.n for s in sc]
    assert min(ns) >= 1000 and max(ns) <= 260000
    for s in sc:
        assert abs(s.config.spacing * 2 - s.config.smoothing_radius) < 1e-12
        assert len(s.primitives) <= 2
        if s.primitives:
            assert abs(s.collider_voxel - s.config.smoothing_radius) < 1e-12
        push = scene_push(s)
        assert push["i_layout"][0] == s.n

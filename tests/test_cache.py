"""The disk cache writes and reads the reference's FLWXCA01 files byte for
byte (golden bytes from the reference's own header packing and frame layout,
tests/golden/make_cache_golden.py). Host-array entry points: no GPU."""

import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    from flowx_gb300 import build

    build.build()
    return np.load(os.path.join(HERE, "golden", "cache_golden.npz"))


def _create(path, z):
    from flowx_gb300.cache import FrameCache

    return FrameCache.create(path, particle_count=int(z["particle_count"]), seed_frame=int(z["seed_frame"]),
                             fps=float(z["fps"]), colliders=[str(c) for c in z["colliders"]],
                             config_hash_bytes=z["config_hash"].tobytes(), flowx_version=str(z["flowx_version"]))


def test_written_file_matches_reference_bytes(tmp_path, golden):
    z = golden
    path = str(tmp_path / "run.flwxcache")
    with _create(path, z) as c:
        c.write_frame_host(int(z["seed_frame"]), z["positions"][0], z["velocities"][0])  # seed frame: not stored
        for i, f in enumerate(z["frames"]):
            c.write_frame_host(int(f), z["positions"][i], z["velocities"][i])
            assert open(path, "rb").read() == z[f"file_after_frame_{i}"].tobytes()


def test_reference_file_reads_back(tmp_path, golden):
    from flowx_gb300._lib import FlowxError
    from flowx_gb300.cache import FrameCache

    z = golden
    path = str(tmp_path / "ref.flwxcache")
    open(path, "wb").write(z["file_after_frame_2"].tobytes())
    with FrameCache.open_existing(path) as c:
        h = c.header()
        assert h["particle_count"] == int(z["particle_count"]) and h["seed_frame"] == int(z["seed_frame"])
        assert h["last_frame"] == int(z["frames"][-1]) and h["fps"] == float(z["fps"])
        assert h["colliders"] == [str(s) for s in z["colliders"]]
        assert h["config_hash"] == z["config_hash"].tobytes() and h["flowx_version"] == str(z["flowx_version"])
        for i, f in enumerate(z["frames"]):
            p, v = c.read_frame_host(int(f))
            np.testing.assert_array_equal(p, z["positions"][i])
            np.testing.assert_array_equal(v, z["velocities"][i])
        for bad in (int(z["seed_frame"]), int(z["frames"][-1]) + 1):
            with pytest.raises(FlowxError):
                c.read_frame_host(bad)


def test_open_reuses_matching_file_and_replaces_other(tmp_path, golden):
    from flowx_gb300.cache import FrameCache

    z = golden
    path = str(tmp_path / "run.flwxcache")
    open(path, "wb").write(z["file_after_frame_2"].tobytes())
    kw = dict(particle_count=int(z["particle_count"]), seed_frame=int(z["seed_frame"]), fps=float(z["fps"]),
              colliders=[str(c) for c in z["colliders"]])
    with FrameCache.open(path, config_hash_bytes=z["config_hash"].tobytes(), **kw) as c:
        assert c.header()["last_frame"] == int(z["frames"][-1])  # reused: frames kept
    with FrameCache.open(path, config_hash_bytes=b"\1" * 32, **kw) as c:
        assert c.header()["last_frame"] == int(z["seed_frame"])  # settings changed: fresh file
    with pytest.raises(Exception):
        FrameCache.open_existing(str(tmp_path / "missing.flwxcache"))
    open(str(tmp_path / "junk"), "wb").write(b"not a cache file")
    with pytest.raises(Exception):
        FrameCache.open_existing(str(tmp_path / "junk"))

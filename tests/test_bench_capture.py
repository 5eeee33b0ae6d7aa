"""bench.py takes the dominant kernel's DRAM bytes and warp instructions from
the committed summary of an ncu capture only when that capture was taken of
the current kernel sources (the sha256 the summary records equals the digest
of flowx_gb300/csrc); otherwise the bench line reports them as null."""

import json
import os

import bench


def _tree(tmp_path, digest):
    os.symlink(os.path.join(os.path.dirname(bench.__file__), "flowx_gb300"), tmp_path / "flowx_gb300")
    prof = tmp_path / "profiles"
    prof.mkdir()
    (prof / "traffic.json").write_text(json.dumps({
        "capture": "test capture", "kernel_source_sha256": digest,
        "bytes_per_launch": {"lambda": 123}, "warp_instructions_per_launch": {"lambda": 456},
    }))
    return tmp_path


def test_capture_used_only_for_the_sources_it_was_taken_of(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(_tree(tmp_path, "0" * 64)))
    assert bench._capture_of_current_sources() is None


def test_capture_of_the_current_sources_is_used(tmp_path, monkeypatch):
    digest = bench.kernel_source_digest()  # of the repository's flowx_gb300/csrc
    monkeypatch.setattr(bench, "ROOT", str(_tree(tmp_path, digest)))
    rec = bench._capture_of_current_sources()
    assert rec["bytes_per_launch"]["lambda"] == 123
    assert rec["warp_instructions_per_launch"]["lambda"] == 456
    assert "test capture" in rec["source"]


def test_missing_summary_gives_none(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench._capture_of_current_sources() is None

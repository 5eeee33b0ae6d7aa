"""Generate ``tests/golden/cache_golden.npz``: a disk-cache file in the
reference's FLWXCA01 format, produced with the reference's own header packing
(``solver/cache.py`` ``_pack_header``, imported outside Blender through
``reference_host.py``) and its frame layout (``write_frame``, :339-379: frame
f at header_size + (f - seed_frame - 1) * frame_size, positions then
velocities as little-endian f32, the header rewritten with last_frame after
every frame). Run where the reference checkout is mounted:

    python tests/golden/make_cache_golden.py [--ref CHECKOUT]

Stored: the inputs (header fields, per-frame arrays) and the file bytes after
each frame write (checked against the reference's ``_unpack_header``).
"""

from __future__ import annotations

import argparse
import importlib
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import reference_host  # noqa: E402
from oracle import refpath  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference checkout (default: $FLOWX_REFERENCE)")
    args = ap.parse_args()
    args.ref = args.ref or refpath.checkout()
    reference_host.load(args.ref)
    cache = importlib.import_module("flowx_reference.solver.cache")

    n, seed, fps = 5, 3, 24.0
    colliders = ["Cube", "Wall.001"]
    digest = bytes(range(32))
    header = {
        "format_version": cache.FORMAT_VERSION,
        "flowx_version": "0.1.0",
        "particle_count": n,
        "seed_frame": seed,
        "last_frame": seed,
        "fps": fps,
        "colliders": colliders,
        "config_hash": digest,
        "header_size": 0,
        "frame_size": 8 * 4 * n,
    }
    packed = cache._pack_header(header)
    header["header_size"] = len(packed)
    data = bytearray(packed)
    rng = np.random.default_rng(0)
    frames = [seed + 1, seed + 2, seed + 3]
    positions = rng.normal(size=(len(frames), n, 4)).astype(np.float32)
    velocities = rng.normal(size=(len(frames), n, 4)).astype(np.float32)
    snapshots = []
    for f, pos, vel in zip(frames, positions, velocities):
        offset = header["header_size"] + (f - seed - 1) * header["frame_size"]
        body = struct.pack(f"<{n * 4}f", *pos.reshape(-1).tolist()) + struct.pack(f"<{n * 4}f",
                                                                                 *vel.reshape(-1).tolist())
        if len(data) < offset + len(body):
            data.extend(b"\0" * (offset + len(body) - len(data)))
        data[offset:offset + len(body)] = body
        header["last_frame"] = max(header["last_frame"], f)
        head = cache._pack_header(header)
        data[:len(head)] = head
        snapshots.append(bytes(data))
    parsed = cache._unpack_header(bytes(data))
    assert parsed["last_frame"] == frames[-1] and parsed["colliders"] == colliders
    np.savez_compressed(
        os.path.join(HERE, "cache_golden.npz"),
        particle_count=n, seed_frame=seed, fps=np.float32(fps), colliders=np.array(colliders),
        config_hash=np.frombuffer(digest, np.uint8), flowx_version=np.array("0.1.0"),
        frames=np.array(frames), positions=positions, velocities=velocities,
        header_size=header["header_size"], frame_size=header["frame_size"],
        **{f"file_after_frame_{i}": np.frombuffer(s, np.uint8) for i, s in enumerate(snapshots)},
    )
    print("header", header["header_size"], "bytes; file", len(data), "bytes")


if __name__ == "__main__":
    main()

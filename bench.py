#!/usr/bin/env python
"""Benchmark: PBF particle-substeps/s of the GB300 substep on the 4M-particle
large-scale workload (2 m cube, h 0.02, 200x200x100 particles, 4 Jacobi
iterations, 4 substeps per frame, a falling 0.3 m sphere collider re-voxelised
every frame on a 100^3 grid).

One step = one frame = 4 substeps over all particles (plus the frame's
collider re-voxelisation). Prints ONE JSON line on rank 0:

  value        particle-substeps/s with all state resident in HBM (CUDA events
               on the library's stream around K frames, each one CUDA-graph
               launch of 4 substeps + one device voxelisation);
  e2e          the same metric through the C ABI with host buffers: every
               frame uploads the host-voxelised collider grid from pinned
               memory and downloads all particle positions to pinned memory;
  roofline     the dominant kernel's algorithmic bytes per launch / its mean
               launch time (CUDA events, launch by launch, same state, same
               stream) against the measured HBM copy bandwidth;
  cpu_baseline the oracle's C restatement of the reference passes (OpenMP,
               all host cores) on a bounded sample of the same workload.

``--impl reference`` times the reference's algorithm on the host cores instead
(the oracle port: the reference's own GLSL passes need a graphics stack that
neither machine has), printing the same metric with "impl": "reference".

Multi-GPU: the path does not shard (one domain per scene); under torchrun each
rank runs an independent replica, the time is the max over ranks and value is
the sum of all replicas' particle-substeps ("replicas only", weak scaling).
"""

from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PBF particle-substeps/s (4M particles, 4 Jacobi iterations)"
UNIT = "particle-substeps/s"
ADJOINT_SUBSTEPS = 30  # the inverse problem's rollout

# Algorithmic bytes per particle and launch of each kernel (compulsory HBM
# traffic: every array touched once per launch, neighbour reuse served on chip;
# float4 pos/vel/pred/normal, float2 (density, lambda), u32 keys/ids/ranks, u64
# sort pairs). The neighbour passes take the per-pass figures of the
# reference's path (one row per pass: normal 44, lambda 28, delta with its
# ping-pong apply 44, velocity + XSPH + finalize 77), which also count the u32
# key each particle's slot carries; the grid-build kernels, which split that
# path's predict/sort rows differently, count their own arrays.
BYTES_PER_PARTICLE = {
    "normal": 44,
    "predict_key": 16 + 16 + 16 + 4 + 4,  # pos, vel, normal; key, rank out
    "scatter": 4 + 4 + 4 + 8,         # key, rank, id; pair out
    "permute_step": 8 + 16 + 16 + 16 + 4 + 16 + 16 + 4 + 4,  # pair, pos, vel, normal, key; pos, pred, id, key out
    "lambda": 28,
    "delta_apply": 44,
    "xsph_finalize": 77,
    "cell_sort_small": 16,            # pairs in + out
}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons,
            "samples": len(self.rows),
        }


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _max_over_ranks(value: float, world: int, device="cpu") -> float:
    """The largest of every rank's value (the replica timing rule: the job
    takes as long as its slowest rank); the value itself for one rank."""
    if world <= 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def _replica_throughput(particles: int, substeps_per_step: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job particle-substeps/s of ``world`` independent replicas that each
    advanced ``particles`` particles by ``steps`` x ``substeps_per_step``
    substeps in ``seconds`` (the max over ranks)."""
    return particles * substeps_per_step * steps * world / seconds


def _workload(args):
    from flowx_gb300 import scenes

    if args.workload == "large":
        return scenes.large(cell_rule=args.cell_rule)
    if args.workload == "pool":
        return scenes.pool(cell_rule=args.cell_rule)
    if args.workload == "dam_break":
        return scenes.dam_break(cell_rule=args.cell_rule)
    raise SystemExit(f"unknown workload {args.workload}")


def _workload_config(scene, args, extra=None):
    c = scene.config
    cfg = {
        "workload": f"{scene.name}: {scene.n} particles, h {c.smoothing_radius} m, cells {c.cell_dims} of "
                    f"{c.cell_size:.4g} m ({args.cell_rule} rule), {c.iterations} Jacobi iterations, "
                    f"{scene.substeps_per_frame} substeps/frame at dt {scene.dt:.6f} s",
        "particles": scene.n,
        "cells": c.cell_count,
        "iterations": c.iterations,
        "substeps_per_step": scene.substeps_per_frame,
        "surface_tension": c.surface_tension,
        "collider": f"{scene.collider_dims} voxels of {scene.collider_voxel} m, "
                    + ("re-voxelised every frame" if scene.animated else "static"),
        "l2": "inputs larger than L2 (particle state alone is ~10x 129 MB)",
    }
    if extra:
        cfg.update(extra)
    return cfg


def _oracle_sample(scene, target_s=10.0, max_substeps=4):
    """Time the oracle (C restatement, OpenMP, all host cores) on the
    workload's initial state: whole substeps of the full scene until
    ``target_s`` seconds have passed (at most ``max_substeps``)."""
    from flowx_gb300 import config as C
    from oracle import oracle as O

    c = dataclasses.replace(scene.config, particle_count=scene.n)
    ic = C.collider_binding(scene.collider_dims, scene.collider_voxel)
    o = O.Oracle(C.push_constant_values(c, scene.dt, ic), scene.positions, scene.velocities,
                 collider=scene.collider_grid(0), iterations=c.iterations)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    cores = O.max_threads()
    done, t0 = 0, time.perf_counter()
    while done < max_substeps:
        o.substep(scene.dt, order=O.ORDER_STABLE)
        done += 1
        if time.perf_counter() - t0 >= target_s:
            break
    elapsed = time.perf_counter() - t0
    return {
        "value": scene.n * done / elapsed,
        "unit": UNIT,
        "cores": cores,
        "kind": "port",
        "sample": f"{done} substep(s) of the full {scene.n}-particle workload from its seeded state "
                  f"({elapsed:.1f} s, oracle C restatement, OpenMP {cores} threads, stable grid order)",
        "one_core": _oracle_one_core(scene, cores),
    }


def _oracle_one_core(scene, restore_threads, corner=0.25):
    """The oracle on one host thread: one substep of the particles of the
    workload's seeded state whose x and y lie in the lowest ``corner`` of the
    domain (a full-height column of the same fluid, same cells and
    parameters), as particle-substeps/s."""
    from flowx_gb300 import config as C
    from oracle import oracle as O

    c = scene.config
    lo = np.asarray(c.lo, np.float32)
    ext = np.asarray(c.hi, np.float32) - lo
    keep = ((scene.positions[:, 0] - lo[0] < corner * ext[0]) & (scene.positions[:, 1] - lo[1] < corner * ext[1]))
    pos = np.ascontiguousarray(scene.positions[keep])
    vel = np.ascontiguousarray(scene.velocities[keep])
    n = int(pos.shape[0])
    cfg = dataclasses.replace(c, particle_count=n)
    ic = C.collider_binding(scene.collider_dims, scene.collider_voxel)
    o = O.Oracle(C.push_constant_values(cfg, scene.dt, ic), pos, vel, collider=scene.collider_grid(0),
                 iterations=c.iterations)
    o.build_grid(0.0, order=O.ORDER_STABLE)
    O.set_threads(1)
    try:
        t0 = time.perf_counter()
        o.substep(scene.dt, order=O.ORDER_STABLE)
        elapsed = time.perf_counter() - t0
    finally:
        O.set_threads(restore_threads)
    return {"value": n / elapsed, "unit": UNIT, "cores": 1,
            "sample": f"one substep of the {n} particles of the seeded state in the x, y < {corner:g} x extent "
                      f"column ({elapsed:.1f} s, oracle C restatement, one thread)"}


def _oracle_extract(field, surface, verts, tris):
    """The oracle's marching cubes (NumPy restatement of the reference's
    extract, one thread) on the frame's splat grid, timed, and whether the
    device mesh equals its mesh."""
    from oracle import mc as oracle_mc

    t0 = time.perf_counter()
    v, t = oracle_mc.extract(field, surface.dims, surface.lo, surface.spacing, surface.iso)
    elapsed = time.perf_counter() - t0
    return {"ms": elapsed * 1e3, "cores": 1, "kind": "port",
            "matches_device": bool(np.array_equal(v, verts) and np.array_equal(t, tris)),
            "sample": "one extraction of the frame's splat grid (oracle NumPy restatement of the reference's "
                      "marching cubes; the reference's own is a pure-Python loop)"}


def _mesh_voxelizer_metrics(scene, reps=5):
    """The workload's falling sphere as a triangle mesh (48 x 96 UV sphere,
    9,024 triangles) voxelised on the device onto its 100^3 collider grid
    (flowx_voxelize_meshes: the per-frame rebuild the reference does with BVH
    ray casts on the CPU), wall clock around the call and a synchronise; the
    oracle's NumPy restatement of the same rule timed once on one thread, and
    whether the grids agree."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver
    from oracle import voxelize as oracle_voxelize

    prim = scene.primitives_at(0)[0]
    verts, tris = scenes.sphere_mesh(prim.r)
    meshes = [(verts, tris, scenes.translation(*prim.a))]
    dims, voxel, origin = scene.collider_dims, scene.collider_voxel, scene.config.lo
    c = dataclasses.replace(scene.config)  # the Solver records its own particle count in its config
    with Solver(c, scene.positions[:8], None, max_cells=c.cell_count,
                max_collider_voxels=int(np.prod(dims))) as s:
        s.voxelize_meshes(meshes, dims, voxel, origin)
        s.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            s.voxelize_meshes(meshes, dims, voxel, origin)
        s.synchronize()
        gpu_ms = (time.perf_counter() - t0) / reps * 1e3
        got = s.collider_occupancy()
    t0 = time.perf_counter()
    want = oracle_voxelize.voxelize_meshes(meshes, dims, voxel, origin)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    return {"triangles": int(tris.shape[0]), "grid": list(dims), "ms": gpu_ms, "cpu_ms": cpu_ms, "cpu_cores": 1,
            "matches_oracle": bool(np.array_equal(got, want)), "occupied": int(got.sum()),
            "timing": "wall clock of Solver.voxelize_meshes (upload, two kernels), synchronised"}


def kernel_source_digest() -> str:
    """sha256 over the library's kernel sources (flowx_gb300/csrc, sorted by
    name): the build an ncu capture was taken of."""
    import hashlib

    h = hashlib.sha256()
    src = os.path.join(ROOT, "flowx_gb300", "csrc")
    for name in sorted(os.listdir(src)):
        if name.endswith((".cu", ".cuh", ".h")):
            h.update(name.encode())
            with open(os.path.join(src, name), "rb") as f:
                h.update(f.read())
    return h.hexdigest()


def _capture_of_current_sources():
    """Per-launch DRAM bytes and warp instructions of the dominant kernels
    from the committed summary of an ncu capture (profiles/traffic.json),
    used only when that capture was taken of exactly these kernel sources;
    otherwise None (the figures are then reported as null)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        rec = json.load(f)
    if rec.get("kernel_source_sha256") != kernel_source_digest():
        return None
    rec["source"] = f"profiles/traffic.json ({rec.get('capture', 'ncu capture')})"
    return rec


BATCH_BUCKETS = ((2000, 20000), (20000, 200001))


def _time_batch(scenes_, substeps, warmup):
    """Device time of ``substeps`` batched substeps (one context, one launch
    per pass for all scenes, autotuned), CUDA events on its stream."""
    import torch

    from flowx_gb300.batch import Batch

    with Batch(scenes_) as b:
        b.build_grid()
        tuned = b.autotune(4)
        for _ in range(warmup):
            b.step(4, 1)
        b.synchronize()
        stream = torch.cuda.ExternalStream(b.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(substeps):
            b.step(4, 1)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3, tuned


def _time_per_scene(scenes_, substeps, warmup, sequential):
    """The plain path per scene: each scene its own context and one-substep
    CUDA graph. sequential: scene after scene, each substep finished
    (synchronised) before the next scene's starts, so one scene runs at a
    time. Otherwise every scene's launch is issued at once and the scenes run
    concurrently on their own streams. Wall clock, synchronised at both
    ends."""
    import torch

    from flowx_gb300.sph import Solver

    solvers = [Solver(s.config, s.positions, s.velocities, collider=s.collider_grid(0),
                      collider_voxel=s.collider_voxel) for s in scenes_]
    try:
        for s, sol in zip(scenes_, solvers):
            sol._build_grid(0.0)
            for _ in range(warmup):
                sol.step_substeps(s.dt, 1)
            sol.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(substeps):
            for s, sol in zip(scenes_, solvers):
                sol.step_substeps(s.dt, 1)
                if sequential:
                    sol.synchronize()
        for sol in solvers:
            sol.synchronize()
        return time.perf_counter() - t0
    finally:
        for sol in solvers:
            sol.close()


def _batched_metrics(substeps=20, warmup=3):
    """The 64-scene batched workload (particle counts log-uniform in
    [2e3, 2e5], seed 3): one context stepping all scenes per launch, against
    the plain path run per scene sequentially (one scene at a time), over
    ``substeps`` substeps after ``warmup`` untimed ones. Also: the per-scene
    contexts issued at once on their own streams (concurrent, not a
    sequential run), and the batch against the sequential path per
    scene-size bucket."""
    from flowx_gb300 import scenes

    sc = scenes.batched_scenes()
    total = sum(s.n for s in sc)
    batched_s, tuned = _time_batch(sc, substeps, warmup)
    seq_s = _time_per_scene(sc, substeps, warmup, sequential=True)
    conc_s = _time_per_scene(sc, substeps, warmup, sequential=False)
    buckets = []
    for lo, hi in BATCH_BUCKETS:
        part = [s for s in sc if lo <= s.n < hi]
        if not part:
            continue
        n = sum(s.n for s in part)
        b_s, _ = _time_batch(part, substeps, warmup)
        q_s = _time_per_scene(part, substeps, warmup, sequential=True)
        buckets.append({"particles_range": [lo, hi - 1], "scenes": len(part), "particles": n,
                        "batched_value": n * substeps / b_s, "sequential_value": n * substeps / q_s,
                        "speedup_vs_sequential": q_s / b_s})
    batched = total * substeps / batched_s
    sequential = total * substeps / seq_s
    return {
        "scenes": len(sc),
        "particles": total,
        "substeps": substeps,
        "value": batched,
        "sequential_value": sequential,
        "unit": UNIT,
        "speedup_vs_sequential": batched / sequential,
        "target_speedup": 3.0,
        "ms_per_substep": batched_s * 1e3 / substeps,
        "sequential_ms_per_substep": seq_s * 1e3 / substeps,
        "concurrent_streams_value": total * substeps / conc_s,
        "speedup_vs_concurrent_streams": conc_s / batched_s,
        "buckets": buckets,
        "autotuned_blocks": tuned,
        "sequential": "the plain path per scene, sequentially: each scene its own context and one-substep CUDA "
                      "graph, each substep synchronised before the next scene's (wall clock)",
        "concurrent_streams": "the same contexts, every scene's substep issued before any is waited for (the "
                              "scenes' streams overlap on the GPU; wall clock)",
        "timing": "batched: CUDA events on the batch's stream",
    }


def _other_configs(frames=10, warmup=3):
    """The other plain configurations (particle-substeps/s, device-resident,
    CUDA events around ``frames`` graph-launched frames of 4 substeps after
    ``warmup``): the 3,200-particle dam break, the 307,200-particle pool with
    its colliders, and the 4M-particle workload on the reference's own cell
    rule (cells of 0.045 m = 2.25 h; its falling sphere installed at frame 0)."""
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver

    out = {}
    for name, make in (("dam_break", scenes.dam_break), ("pool", scenes.pool),
                       ("large_reference_cells", lambda: scenes.large(cell_rule="reference"))):
        sc = make()
        col = sc.collider_grid(0)
        with Solver(sc.config, sc.positions, sc.velocities, collider=col,
                    collider_voxel=sc.collider_voxel if col is not None else 0.0) as s:
            s._build_grid(0.0)
            for _ in range(warmup):
                s.step_substeps(sc.dt, sc.substeps_per_frame)
            s.synchronize()
            ms = s.time_steps(sc.dt, sc.substeps_per_frame, frames)
        out[name] = {"particles": sc.n, "value": sc.n * sc.substeps_per_frame * frames / (ms / 1e3),
                     "unit": UNIT, "ms_per_frame": ms / frames,
                     "cells": f"{sc.config.cell_dims} of {sc.config.cell_size:.4g} m"}
    return out


def _adjoint_metrics(adam_steps=200, repeats=5):
    """The differentiable workload (20,000 particles in a 1 m cube, h 0.04,
    initial velocities from a 3x3x3 control grid of 3-vectors, loss = squared
    L2 distance of the 64^3 splat after 30 substeps x 4 iterations to the
    splat of a hidden control grid). Forward and forward+adjoint wall time per
    substep through the autograd.Function (each call synchronises the
    library's stream), then ``adam_steps`` steps of the continuation method
    (InverseProblem.optimise) on the control grid, with plain Adam over the
    30 substeps and over a 3-substep rollout for comparison."""
    import torch

    from flowx_gb300 import scenes
    from flowx_gb300.adjoint import InverseProblem

    ip = InverseProblem(scenes.inverse_problem(), substeps=ADJOINT_SUBSTEPS)
    control = ip.initial.clone().requires_grad_(True)
    for _ in range(3):
        control.grad = None
        ip.loss(control).backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        with torch.no_grad():
            ip.loss(control)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(repeats):
        control.grad = None
        ip.loss(control).backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    fwd = (t1 - t0) / repeats / ADJOINT_SUBSTEPS * 1e3
    both = (t2 - t1) / repeats / ADJOINT_SUBSTEPS * 1e3
    grad_norm = float(control.grad.norm())
    t3 = time.perf_counter()
    losses, control_c = ip.optimise(steps=adam_steps, lr=0.05, method="continuation")
    adam_s = time.perf_counter() - t3
    plain, control_p = ip.optimise(steps=adam_steps, lr=0.05, method="adam")
    short = InverseProblem(scenes.inverse_problem(), substeps=3)
    short_losses, _ = short.optimise(steps=adam_steps, lr=0.05, method="adam")
    dist = lambda c: float((c - ip.hidden).norm())  # noqa: E731
    return {
        "workload": f"inverse problem: {ip.solver.n} particles, {ADJOINT_SUBSTEPS} substeps x 4 iterations, "
                    "64^3 splat, 3x3x3x3 control grid",
        "fwd_ms_per_substep": fwd,
        "fwd_adjoint_ms_per_substep": both,
        "fwd_adjoint_over_fwd": both / fwd,
        "timing": "wall clock around the autograd.Function call, synchronised at both ends",
        "control_gradient_norm": grad_norm,
        "adam": {"method": "continuation: horizon 3 -> 30 substeps over 3/4 of the steps, Adam steps kept only "
                           "when they do not raise the current horizon's loss (halved up to 6 times, else undone)",
                 "steps": adam_steps, "lr": 0.05, "loss_first": losses[0], "loss_min": min(losses),
                 "loss_min_step": int(np.argmin(losses)), "loss_last": losses[-1], "seconds": adam_s,
                 "control_distance_first": dist(ip.initial), "control_distance_last": dist(control_c)},
        "adam_plain_30_substeps": {"steps": adam_steps, "lr": 0.05, "loss_first": plain[0], "loss_last": plain[-1],
                                   "control_distance_last": dist(control_p)},
        "adam_3_substeps": {"steps": adam_steps, "lr": 0.05, "loss_first": short_losses[0],
                            "loss_last": short_losses[-1]},
    }


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores."""
    world, rank, _ = _dist()
    if rank != 0:
        return 0
    from flowx_gb300 import config as C
    from oracle import oracle as O

    oracle_build_ok = True
    try:
        O.build()
    except Exception as exc:  # pragma: no cover - depends on the host toolchain
        oracle_build_ok = False
        print(json.dumps({"impl": "reference", "unavailable": f"oracle build failed: {exc}"}))
        return 0
    scene = _workload(args)
    c = scene.config
    ic = C.collider_binding(scene.collider_dims, scene.collider_voxel)
    cores = O.max_threads()

    def timed(order, steps, warmup):
        o = O.Oracle(C.push_constant_values(c, scene.dt, ic), scene.positions, scene.velocities,
                     collider=scene.collider_grid(0), iterations=c.iterations)
        o.build_grid(0.0, order=order)
        for _ in range(warmup):
            o.substep(scene.dt, order=order)
        t0 = time.perf_counter()
        for _ in range(steps):
            o.substep(scene.dt, order=order)
        return time.perf_counter() - t0

    # value: the reference's own grid build, the bitonic network of
    # sph_sort.glsl driven as solver/sph.py:488-495 does (log2(S)(log2(S)+1)/2
    # compare-exchange passes over the padded key array); beside it the same
    # passes with the (cell, id) counting-sort order the GPU path emits.
    elapsed = timed(O.ORDER_BITONIC, args.steps, args.warmup)
    stable_steps = max(1, min(args.steps, 2))
    stable_s = timed(O.ORDER_STABLE, stable_steps, 1)
    value = scene.n * args.steps / elapsed
    sample = (f"each step is one substep of the full {scene.n}-particle workload: the oracle C restatement of "
              f"the reference passes with the reference's bitonic key sort, OpenMP {cores} threads; the "
              f"reference's own GLSL passes need a graphics stack, unavailable on this box")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": _workload_config(scene, args, {"step": "one substep (host CPU)"}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "grid_order": "bitonic (the reference's sort network; value)",
        "stable_order": {"value": scene.n * stable_steps / stable_s, "unit": UNIT, "steps": stable_steps,
                         "note": "same passes, grid sorted into (cell, id) order by a counting sort"},
        "oracle_build": oracle_build_ok,
    }
    print(json.dumps(line))
    return 0


def run_flowx(args):
    import torch

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver, launch_count

    scene = _workload(args)
    c = scene.config
    prims_by_frame = [scene.primitives_at(f) for f in range(args.warmup + args.steps + 1)]
    samples = scene.surface.sample_count
    sol = Solver(c, scene.positions, scene.velocities, max_cells=c.cell_count,
                 max_collider_voxels=int(np.prod(scene.collider_dims)) if scene.collider_dims else 0,
                 max_surface_samples=samples, device=local)
    dims = scene.collider_dims
    dt, nsub = scene.dt, scene.substeps_per_frame

    def voxelize(frame):
        if dims is not None:
            sol.voxelize(prims_by_frame[frame], dims, scene.collider_voxel)

    voxelize(0)
    sol._build_grid(0.0)
    stream = torch.cuda.ExternalStream(sol.stream(), device=local)
    frame = 0
    for _ in range(args.warmup):
        voxelize(frame)
        sol.step_substeps(dt, nsub)
        frame += 1
    sol.synchronize()

    # ---- timed region: device-resident frames ----
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sol.synchronize()
    launches0 = launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        voxelize(frame)
        sol.step_substeps(dt, nsub)
        frame += 1
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = launch_count() - launches0
    clocks.stop()
    ms = _max_over_ranks(ms, world, f"cuda:{local}")
    value = _replica_throughput(scene.n, nsub, args.steps, world, ms / 1e3)

    # ---- per-kernel times (launch by launch, same state and stream) ----
    prof = sol.profile(dt, nsub * min(args.steps, 4))
    total_prof = sum(v[0] for v in prof.values())
    kernels = {
        name: {
            "launches": n,
            "ms_per_launch": t / n,
            "share": t / total_prof if total_prof else None,
            "gbs": (BYTES_PER_PARTICLE[name] * scene.n / (t / n * 1e-3) / 1e9) if name in BYTES_PER_PARTICLE else None,
        }
        for name, (t, n) in prof.items()
    }
    dominant = max(prof, key=lambda k: prof[k][0])
    peak, peak_kind = _peaks()
    dom_bytes = BYTES_PER_PARTICLE.get(dominant, 0) * scene.n
    dom_ms = prof[dominant][0] / prof[dominant][1]
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    capture = _capture_of_current_sources()
    traffic = capture.get("bytes_per_launch", {}).get(dominant) if capture else None
    warp_inst = capture.get("warp_instructions_per_launch", {}).get(dominant) if capture else None
    lanes = capture.get("active_lanes_per_warp_instruction", {}).get(dominant) if capture else None
    roofline = {
        "bound": "hbm",
        "kernel": dominant,
        "achieved": achieved,
        "peak": peak,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": traffic,
        "traffic_source": (capture["source"] if capture else "null: no ncu capture of the current kernel sources "
                           "is committed"),
        "algorithmic_bytes_per_launch": dom_bytes,
        "ms_per_launch": dom_ms,
    }

    # ---- e2e: host buffers through the C ABI ----
    pinned_pos = torch.empty((scene.n, 4), dtype=torch.float32, pin_memory=True).numpy()
    grids = []
    if dims is not None:
        for f in range(args.steps):
            g = torch.empty(tuple(reversed(dims)), dtype=torch.uint8, pin_memory=True).numpy()
            g[...] = scene.collider_grid(frame + f)
            grids.append(g)
    import ctypes

    from flowx_gb300 import _lib

    sol.synchronize()
    t0 = time.perf_counter()
    for f in range(args.steps):
        if grids:
            g = grids[f]
            d3 = (ctypes.c_int32 * 3)(*dims)
            _lib.check(sol.lib.flowx_set_collider(sol.ctx, g.ctypes.data, d3, float(scene.collider_voxel)), sol.ctx)
        sol.step_substeps(dt, nsub)
        _lib.check(sol.lib.flowx_download(sol.ctx, _lib.BUF["positions"], pinned_pos.ctypes.data,
                                          pinned_pos.nbytes), sol.ctx)
    sol.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = _max_over_ranks(e2e_s, world, f"cuda:{local}")
    e2e = {
        "value": _replica_throughput(scene.n, nsub, args.steps, world, e2e_s),
        "unit": UNIT,
        "h2d_bytes_per_step": int(np.prod(dims)) if dims is not None else 0,
        "d2h_bytes_per_step": int(scene.n * 16),
    }

    # ---- per-frame splat (reported beside the substep metric) ----
    sol.update_surface(scene.surface, dt, download=False)
    sol.synchronize()
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    reps = 3
    for _ in range(reps):
        sol.update_surface(scene.surface, dt, download=False)
    s1.record(stream)
    s1.synchronize()
    splat_ms = s0.elapsed_time(s1) / reps
    # ---- per-frame surface mesh: splat + marching cubes on the device ----
    from flowx_gb300.surface import MarchingCubes

    mc = MarchingCubes(0)
    sol.surface_mesh(scene.surface, dt, mc)
    m0 = time.perf_counter()
    for _ in range(reps):
        verts, tris = sol.surface_mesh(scene.surface, dt, mc)
    mesh_ms = (time.perf_counter() - m0) / reps * 1e3
    surface_mesh = {"ms_per_frame": mesh_ms, "vertices": int(verts.shape[0]), "triangles": int(tris.shape[0]),
                    "samples": int(scene.surface.sample_count),
                    "timing": "wall clock of Solver.surface_mesh: splat, marching cubes and the mesh download"}
    if rank == 0 and not args.no_cpu_baseline:
        surface_mesh["cpu_extract"] = _oracle_extract(sol.update_surface(scene.surface, dt), scene.surface,
                                                      verts, tris)
    mc.close()
    finite = bool(np.isfinite(pinned_pos).all())
    sol.close()

    batched = None
    if not args.no_batched:
        batched = _batched_metrics()
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = _adjoint_metrics()
    other_configs = _other_configs() if rank == 0 and not args.no_other_configs else None
    mesh_voxelizer = None
    if rank == 0 and scene.collider_dims is not None and not args.no_other_configs:
        mesh_voxelizer = _mesh_voxelizer_metrics(scene)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = _oracle_sample(scene, target_s=args.cpu_seconds)
        except Exception as exc:  # pragma: no cover
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        clock_summary = clocks.summary()
        issue_roofline = None
        if warp_inst and clock_summary.get("sm_max_mhz"):
            # The neighbour kernels are instruction-issue-bound: their warp
            # instructions per launch (ncu, profiles/traffic.json) over the live
            # time per launch, against 4 issue slots per SM per cycle at the
            # maximum SM clock.
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            peak_issue = 4.0 * sms * clock_summary["sm_max_mhz"] * 1e6
            achieved_issue = warp_inst / (dom_ms * 1e-3)
            issue_roofline = {"kernel": dominant, "warp_instructions_per_launch": warp_inst,
                              "ms_per_launch": dom_ms, "achieved": achieved_issue, "peak": peak_issue,
                              "unit": "warp-instructions/s", "frac": achieved_issue / peak_issue,
                              "peak_basis": f"4 x {sms} SMs x {clock_summary['sm_max_mhz']:.0f} MHz",
                              "active_lanes_per_instruction": lanes}
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": _workload_config(scene, args, {"step": "one frame = 4 substeps + collider re-voxelisation",
                                                    "parallelism": f"replicas x{world}"}),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clock_summary,
            "issue_roofline": issue_roofline,
            "kernels": kernels,
            "math": "fast (re-associated float32; FLOWX_FLAG_EXACT gives the reference's expressions)",
            "batched": batched,
            "adjoint": adjoint,
            "other_configs": other_configs,
            "mesh_voxelizer": mesh_voxelizer,
            "splat_ms_per_frame": splat_ms,
            "surface_mesh": surface_mesh,
            "splat_samples": samples,
            "state_finite": finite,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["flowx", "reference"], default="flowx")
    ap.add_argument("--workload", default="large", choices=["large", "pool", "dam_break", "inverse"],
                    help="inverse (the differentiable 20,000-particle problem) is a --case workload only")
    ap.add_argument("--cell-rule", default="h", choices=["h", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-scene batched measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-substep measurement")
    ap.add_argument("--no-other-configs", action="store_true",
                    help="skip the dam-break and pool measurements (profiler launch lists of the workload alone)")
    ap.add_argument("--case", action="store_true",
                    help="untimed launch-by-launch run of --warmup frames, for profiler captures")
    ap.add_argument("--exact", action="store_true", help="with --case: the reference's float expressions")
    ap.add_argument("--mesh-collider", action="store_true",
                    help="with --case: voxelise the large scene's falling sphere from its triangle mesh every frame")
    ap.add_argument("--aux", action="store_true",
                    help="with --case: drive the kernels outside the steady-state substep once each (run_case_aux)")
    ap.add_argument("--surface", action="store_true",
                    help="with --case: then the frame's surface twice (splat and marching cubes)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("bench.py: --warmup below 3 is raised to 3", file=sys.stderr)
        args.warmup = 3
    if args.case:
        if args.aux:
            return run_case_aux(args)
        return run_case_adjoint(args) if args.workload == "inverse" else run_case(args)
    if args.workload == "inverse":
        raise SystemExit("--workload inverse is a --case workload; the bench line reports it under 'adjoint'")
    if args.impl == "reference":
        return run_reference(args)
    return run_flowx(args)


def run_case(args):
    """Untimed run for profiler captures: seed the workload, build the grid,
    run --warmup frames launch by launch (no CUDA graph, so every kernel is a
    separate launch), check the state is finite and exit."""
    import torch

    from flowx_gb300 import scenes
    from flowx_gb300.sph import Solver

    torch.cuda.set_device(0)
    scene = _workload(args)
    c = scene.config
    sol = Solver(c, scene.positions, scene.velocities, max_cells=c.cell_count,
                 max_collider_voxels=int(np.prod(scene.collider_dims)) if scene.collider_dims else 0,
                 max_surface_samples=scene.surface.sample_count if args.surface else 0, exact=args.exact)
    def voxelize(frame):
        if scene.collider_dims is None:
            return
        prims = scene.primitives_at(frame)
        if args.mesh_collider and len(prims) == 1 and prims[0].kind == 0:
            # the falling sphere from its triangle mesh (flowx_voxelize_meshes)
            verts, tris = scenes.sphere_mesh(prims[0].r)
            sol.voxelize_meshes([(verts, tris, scenes.translation(*prims[0].a))], scene.collider_dims,
                                scene.collider_voxel)
        else:
            sol.voxelize(prims, scene.collider_dims, scene.collider_voxel)

    voxelize(0)
    sol._build_grid(0.0)
    for f in range(args.warmup):
        voxelize(f)
        for _ in range(scene.substeps_per_frame):
            sol._substep(scene.dt)
    if args.surface:
        for _ in range(2):
            sol.surface_mesh(scene.surface, scene.dt)
    ok = bool(np.isfinite(sol.read("positions")).all())
    sol.close()
    print(json.dumps({"case": scene.name, "frames": args.warmup, "finite": ok}))
    return 0 if ok else 1


def run_case_aux(args):
    """Untimed run for a DRAM capture of the kernels outside the steady-state
    substep, each driven once on the 4M-particle workload: the per-pass API
    (normal, predict, lambda with its quads fill, delta, apply, velocity, XSPH,
    finalize), downloads and a keys write with their layout conversions, a
    substep with no Jacobi iteration, the reference's grid order, then the
    allocation-free grid build at its largest size (65,536 particles) and one
    3-substep forward and adjoint of the differentiable problem."""
    import ctypes

    import torch

    from flowx_gb300 import _lib, scenes
    from flowx_gb300.adjoint import InverseProblem
    from flowx_gb300.sph import Solver

    torch.cuda.set_device(0)
    sc = scenes.large()
    cfg, dt, dims = sc.config, sc.dt, sc.collider_dims
    with Solver(cfg, sc.positions, sc.velocities, exact=True, max_collider_voxels=int(np.prod(dims))) as s:
        s.voxelize(sc.primitives_at(3), dims, sc.collider_voxel)
        s._build_grid(0.0)
        for name in ("normal", "predict"):
            s.run_pass(name, dt)
        s._build_grid(dt)
        for name in ("lambda", "delta", "apply_delta", "velocity", "xsph", "finalize"):
            s.run_pass(name, dt)
        s.read("lambda")
        s.write("keys", s.read("keys", cfg.sorted_count))
        rc = s.lib.flowx_substep(s._ctx, ctypes.byref(s.push(dt)), 0)
        if rc != _lib.FLOWX_OK:
            raise RuntimeError(f"flowx_substep with no iteration: {rc}")
        ok = bool(np.isfinite(s.read("positions")).all())
    with Solver(cfg, sc.positions, sc.velocities, exact=True, reference_order=True) as s:
        s._build_grid(0.0)
        s._substep(dt)
        ok = ok and bool(np.isfinite(s.read("positions")).all())
    lib = _lib.load()
    dam = scenes.dam_break()
    n = 65536
    rng = np.random.default_rng(1)
    lo, hi = np.array(dam.config.lo), np.array(dam.config.hi)
    pts = np.zeros((n, 4), np.float32)
    pts[:, :3] = lo + rng.random((n, 3)) * (hi - lo)
    pts[:, 3] = 1.0
    with Solver(dam.config, dam.positions, dam.velocities) as s:
        push = s.push(0.0)
    push.i_layout[0] = n
    pred = torch.from_numpy(pts).to("cuda:0")
    keys = torch.zeros((n, 4), dtype=torch.float32, device="cuda:0")
    start = torch.zeros(dam.config.cell_count, dtype=torch.float32, device="cuda:0")
    end = torch.zeros(dam.config.cell_count, dtype=torch.float32, device="cuda:0")
    for _ in range(2):
        rc = lib.flowx_build_grid_static(pred.data_ptr(), n, ctypes.byref(push), keys.data_ptr(), n,
                                         start.data_ptr(), end.data_ptr(), None)
        if rc != _lib.FLOWX_OK:
            raise RuntimeError(lib.flowx_build_grid_static_error().decode())
    torch.cuda.synchronize()
    ip = InverseProblem(scenes.inverse_problem(), substeps=3)
    control = ip.initial.clone().requires_grad_(True)
    ip.loss(control).backward()
    ok = ok and bool(torch.isfinite(control.grad).all())
    print(json.dumps({"case": "auxiliary kernels", "finite": ok}))
    return 0 if ok else 1


def run_case_adjoint(args):
    """Untimed run for profiler captures of the differentiable substeps: the
    inverse problem's target forward, then one forward and one adjoint."""
    import torch

    from flowx_gb300 import scenes
    from flowx_gb300.adjoint import InverseProblem

    torch.cuda.set_device(0)
    ip = InverseProblem(scenes.inverse_problem(), substeps=ADJOINT_SUBSTEPS)
    control = ip.initial.clone().requires_grad_(True)
    loss = ip.loss(control)
    loss.backward()
    ok = bool(torch.isfinite(control.grad).all()) and bool(torch.isfinite(loss))
    print(json.dumps({"case": "inverse", "substeps": ADJOINT_SUBSTEPS, "finite": ok}))
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())

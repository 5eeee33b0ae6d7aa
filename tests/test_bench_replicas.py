"""The multi-rank path of bench.py on the CPU: two gloo ranks (127.0.0.1)
run the replica timing rule (max over ranks, whole-job throughput = every
replica's particle-substeps over that time), and the reference arm's
non-zero ranks exit at once without work."""

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        slowest = bench._max_over_ranks(10.0 + 5.0 * rank, world)  # rank 1 is the slow one
        value = bench._replica_throughput(1000, 4, 3, world, slowest)
        out.put((rank, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_and_sum_the_replicas():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    results = sorted(out.get(timeout=10) for _ in range(2))
    for rank, slowest, value in results:
        assert slowest == 15.0
        assert value == pytest.approx(1000 * 4 * 3 * 2 / 15.0)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench._max_over_ranks(7.5, 1) == 7.5
    assert bench._replica_throughput(10, 2, 3, 1, 2.0) == 30.0


def test_reference_arm_non_zero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_cpu_samples_report_their_own_workload():
    """The CPU baseline helpers on a small scene: a positive rate over the
    scene's own particle count, the threads used, and the one-thread sample
    on a column of the same fluid."""
    sys.path.insert(0, ROOT)
    import bench
    from flowx_gb300 import scenes
    from oracle import oracle as O

    O.build()
    sc = scenes.dam_break()
    sc.config.particle_count = 8  # a Solver elsewhere may have recorded its own count
    r = bench._oracle_sample(sc, target_s=0.05, max_substeps=1)
    assert r["value"] > 0 and r["cores"] >= 1 and r["kind"] == "port"
    assert f"{sc.n}-particle" in r["sample"]
    one = r["one_core"]
    assert one["cores"] == 1 and one["value"] > 0
    assert O.max_threads() == r["cores"]  # the thread count is restored

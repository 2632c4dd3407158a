"""Runs over several GPUs, host side, on CPU: world sharding of batched
worlds, the measurement's max-time / sum-units aggregation over 2 gloo ranks,
and the reference arm's rank > 0 exiting without work."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

from wrach_gb300 import replicas  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_covers_every_world_once():
    for count in (0, 1, 7, 256, 257):
        for ws in (1, 2, 3, 4, 8):
            ranges = [replicas.shard(count, r, ws) for r in range(ws)]
            assert ranges[0][0] == 0 and ranges[-1][1] == count
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(10, 2, 2)


def test_aggregate_without_a_process_group():
    assert replicas.aggregate(1.5, 10) == (1.5, 10.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=2)
    try:
        # rank r "took" 1 + r seconds for 100 * (r + 1) units
        out[rank] = replicas.aggregate(1.0 + rank, 100.0 * (rank + 1))
    finally:
        torch.distributed.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(port, out), nprocs=2, start_method="spawn")
        assert out[0] == out[1] == (2.0, 300.0)


def test_reference_arm_on_rank_1_does_no_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def _batch_rank_main(rank, port, out):
    """One rank of `bench.py --workload batch` with the GPU replaced by a CPU
    stand-in: the rank takes its worlds through bench.batch_worlds (the
    bench's own sharding) and "steps" them by counting their particles."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=2)
    try:
        lo, hi, dims, poss, vels = bench.batch_worlds(rank, 2)
        assert len(dims) == len(poss) == len(vels) == hi - lo
        sizes = [len(p) for p in poss]
        _, units = replicas.aggregate(1.0, float(sum(sizes)))
        out[rank] = (lo, hi, sizes, units)
    finally:
        torch.distributed.destroy_process_group()


def test_batch_worlds_shard_over_two_gloo_ranks():
    """Unmeasured on hardware (one GPU per run here): every one of the 256
    worlds is stepped by exactly one rank, and the ranks' units add up to
    the whole batch."""
    from wrach_gb300 import workloads
    _, all_pos, _ = workloads.batch()
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_batch_rank_main, args=(port, out), nprocs=2, start_method="spawn")
        (lo0, hi0, s0, u0), (lo1, hi1, s1, u1) = out[0], out[1]
    assert (lo0, hi0, lo1, hi1) == (0, 128, 128, 256)
    assert s0 + s1 == [len(p) for p in all_pos]
    assert u0 == u1 == float(sum(len(p) for p in all_pos))

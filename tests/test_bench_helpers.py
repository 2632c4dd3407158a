"""The benchmark's bookkeeping, on the CPU: the algorithmic bytes per launch
and the committed ncu figures its roofline lines read."""
import json
import os

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_launch_bytes_count_the_taking_part_particles():
    n, c = 1_000_000, 2_076_601
    # the Jacobi reads and writes the compacted iterate of the taking-part
    # particles only; with every particle taking part it is 20 N + 4 C
    assert bench.launch_bytes("jacobi", n, c) == 20 * n + 4 * c
    assert bench.launch_bytes("jacobi", n, c, 400_000) == 20 * 400_000 + 4 * c
    assert bench.launch_bytes("jacobi_final", n, c, 400_000) == 40 * n + 4 * c
    assert bench.launch_bytes("rebin_scan", n, c) == 12 * c
    assert bench.launch_bytes("no such kernel", n, c) == 0


def test_every_ncu_capture_names_its_frame_and_kernels():
    with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
        table = json.load(f)["workloads"]
    assert {"lattice-1M", "blobs-4M", "lattice-1M, reference physics"} <= set(table)
    for name, entry in table.items():
        assert isinstance(bench.ncu_figure(name, "frame"), int), name
        for kernel, value in entry["dram_bytes_per_launch"].items():
            assert bench.ncu_figure(name, "dram_bytes_per_launch", kernel) == value > 0
            assert bench.ncu_figure(name, "warp_instructions_per_launch", kernel) > 0
    # the workloads' own descriptions are the keys the bench looks up
    for workload in ("lattice", "blobs", "reference"):
        desc = bench._workload(workload)[0]
        assert desc["workload"] in table, workload
    assert bench.ncu_figure("no such workload", "frame") is None

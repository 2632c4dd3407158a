"""The autotuner's cache (CPU) and a small tuning run (GPU)."""
import dataclasses

import numpy as np
import pytest


def test_cache_key_and_round_trip(tmp_path):
    from wrach_gb300 import autotune, api
    cfg = api.WrachConfig(cell_size=1, mode=1, iterations=4)
    k1 = autotune.workload_key("GB300", cfg, 1, 1_000_000, 2_076_601, False)
    k2 = autotune.workload_key("GB300", cfg, 1, 1_100_000, 2_000_000, False)
    k3 = autotune.workload_key("GB300", cfg, 1, 1_000_000, 2_076_601, True)
    assert k1 == k2 and k1 != k3  # sizes are bucketed to powers of two
    path = str(tmp_path / "cache.json")
    autotune.save_cache({k1: {"choice": {"cell_size": 1, "rebin_blocks": 152, "solve_block": 256},
                              "ms": {"a": 1.0}}}, path)
    assert autotune.load_cache(path)[k1]["choice"]["rebin_blocks"] == 152
    assert autotune.load_cache(str(tmp_path / "missing.json")) == {}


@pytest.mark.gpu
def test_tune_picks_a_candidate_and_caches_it(W, tmp_path):
    from wrach_gb300 import autotune
    rng = np.random.default_rng(0)
    dims = (200.0, 120.0)
    pos = rng.uniform((0, 0), dims, size=(10000, 2)).astype(np.float32)
    vel = rng.normal(0, 1, size=pos.shape).astype(np.float32)
    cfg = W.WrachConfig(dimensions=dims, cell_size=1, mode=1, iterations=2, gravity=0.1,
                        capacity=20000)
    path = str(tmp_path / "tune.json")
    tuned, ms = autotune.tune(cfg, pos, vel, frames=4, solve_blocks=(128, 256), per_thread=(1, 3),
                              path=path)
    assert tuned.solve_block in (128, 256) and tuned.solve_per_thread in (1, 3)
    assert tuned.rebin_blocks > 0
    assert len(ms) >= 6 and all(v > 0 for v in ms.values())
    again, ms2 = autotune.tune(cfg, pos, vel, frames=4, solve_blocks=(128, 256), per_thread=(1, 3),
                               path=path)
    assert again == tuned and ms2 == ms
    # a launch shape does not change results
    odd = dataclasses.replace(cfg, solve_block=96, solve_per_thread=5)
    with W.Simulation(cfg) as a, W.Simulation(odd) as b:
        a.add_particles(pos, vel)
        b.add_particles(pos, vel)
        a.step(5)
        b.step(5)
        ra, rb = a.read_frame(), b.read_frame()
        assert np.array_equal(ra[2], rb[2]) and np.array_equal(ra[0], rb[0])

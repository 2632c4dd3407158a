"""Parity with the oracle away from the defaults: anchored viewports (negative
and fractional anchors, cell sizes 1 and 3), cell capacities from 1 to the
maximum of 16, and physics constants other than the reference's (minimum
distance, velocity cap, gravity, iteration count), in both physics modes.
Frames are compared bit for bit (table, order, positions, velocities)."""
import numpy as np
import pytest

from tests.helpers import assert_frame_equal

pytestmark = pytest.mark.gpu


def _run(W, O, cfg, pos, vel, steps):
    ph = O.Physics(cfg.mode, cfg.iterations, cfg.gravity, cfg.min_distance, cfg.max_velocity,
                   cfg.cell_capacity)
    w = O.world(cfg.dimensions[0], cfg.dimensions[1], cfg.cell_size, anchor=cfg.anchor)
    with W.Simulation(cfg) as sim:
        sim.add_particles(pos, vel)
        ref = O.pack(w, pos, vel, capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), ref, "upload")
        done = 0
        for s in steps:
            sim.step(s - done)
            ref = O.step(w, ph, ref[0], ref[1], ref[2], s - done)[:3]
            done = s
            assert_frame_equal(sim.read_frame(), ref, "after %d steps" % s)
        assert sim.flags() in (0, 1)  # at most out-of-grid (clamped) positions


def _field(seed, n, lo, hi, vel_sigma=0.6, clusters=0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(lo, hi, size=(n, 2)).astype(np.float32)
    if clusters:
        centres = rng.uniform(lo, hi, size=(clusters, 2))
        k = n // 3
        pos[:k] = (centres[rng.integers(0, clusters, k)] + rng.normal(0, 0.8, (k, 2))).astype(np.float32)
        pos[:k] = np.clip(pos[:k], lo, hi)
    vel = rng.normal(0, vel_sigma, size=(n, 2)).astype(np.float32)
    return pos, vel


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("cs", [1, 3])
def test_anchored_viewport(W, O, mode, cs):
    anchor = (-13.5, 7.25)
    dims = (70.0, 45.0)
    pos, vel = _field(21, 3000, (anchor[0] - 3, anchor[1] - 3),
                      (anchor[0] + dims[0] + 3, anchor[1] + dims[1] + 3))
    cfg = W.WrachConfig(dimensions=dims, anchor=anchor, cell_size=cs, mode=mode, iterations=4,
                        gravity=0.1 if mode else 0.0, capacity=6000)
    _run(W, O, cfg, pos, vel, [1, 5, 12])


@pytest.mark.parametrize("cap", [1, 4, 16])
def test_cell_capacity(W, O, cap):
    dims = (60.0, 40.0)
    pos, vel = _field(22, 4000, (0.0, 0.0), dims, clusters=12)
    cfg = W.WrachConfig(dimensions=dims, cell_size=1, mode=1, iterations=4, gravity=0.1,
                        cell_capacity=cap, capacity=8000)
    _run(W, O, cfg, pos, vel, [1, 4, 10])


@pytest.mark.parametrize("mode", [0, 1])
def test_other_physics_constants(W, O, mode):
    dims = (50.0, 50.0)
    pos, vel = _field(23, 3000, (0.0, 0.0), dims, vel_sigma=1.5, clusters=8)
    cfg = W.WrachConfig(dimensions=dims, cell_size=2, mode=mode, iterations=3, gravity=0.3,
                        min_distance=1.5, max_velocity=2.0, capacity=6000)
    _run(W, O, cfg, pos, vel, [1, 6, 15])


def test_read_keys_match_the_table(W, O):
    # single world and one world of a batch: each frame particle's key is the
    # cell the table places it in, cy * gx + cx
    pos, vel = _field(24, 2500, (0.0, 0.0), (40.0, 30.0))
    cfg = W.WrachConfig(dimensions=(40.0, 30.0), cell_size=1, mode=1, iterations=4, gravity=0.1,
                        capacity=5000)
    with W.Simulation(cfg) as sim:
        sim.add_particles(pos, vel)
        sim.step(3)
        p, v, table = sim.read_frame()
        keys = sim.read_keys()
        want = np.repeat(np.arange(len(table) - 2), np.diff(table[1:].astype(np.int64)))
        assert np.array_equal(keys, want.astype(np.uint32))
        w = O.world(40.0, 30.0, 1)
        oracle_keys = np.array([O.frame_key(w, float(x), float(y))[0] for x, y in p], np.uint32)
        assert np.array_equal(keys, oracle_keys)
    dims = [(30.0, 20.0), (25.0, 35.0)]
    with W.Simulation(W.WrachConfig(cell_size=1, mode=0, capacity=3000), worlds=dims) as sim:
        for k, d in enumerate(dims):
            q, u = _field(30 + k, 800, (0.0, 0.0), d)
            sim.set_particles(q, u, world=k)
        sim.step(2)
        p, v, table = sim.read_frame(world=1)
        keys = sim.read_keys(world=1)
        want = np.repeat(np.arange(len(table) - 2), np.diff(table[1:].astype(np.int64)))
        assert np.array_equal(keys, want.astype(np.uint32))

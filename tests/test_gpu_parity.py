"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Binning (cell keys, the cell-start table, the sorted order) and the physics
are compared bit for bit: both sides compute in IEEE binary32 without FMA
contraction, with correctly rounded sqrt and division, in the same order.
"""
import numpy as np
import pytest

from tests.helpers import (assert_frame_equal, frame_stats, make_sim, oracle_physics,
                           same_bits)

pytestmark = pytest.mark.gpu


def _run_both(W, O, dims, cs, pos, vel, mode, steps, iterations=4, gravity=0.0, capacity=0):
    sim = make_sim(W, dims, cs, mode, iterations, gravity, capacity)
    try:
        cap = sim.capacity()
        w = O.world(dims[0], dims[1], cs)
        ph = oracle_physics(O, mode, iterations, gravity)
        sim.add_particles(pos, vel)
        ref = O.pack(w, pos, vel, capacity=cap)
        assert_frame_equal(sim.read_frame(), ref, "upload")
        done = 0
        for target in steps:
            sim.step(target - done)
            ref = O.step(w, ph, ref[0], ref[1], ref[2], target - done)[:3]
            done = target
            assert_frame_equal(sim.read_frame(), ref, "after %d steps" % target)
        return sim.flags()
    finally:
        sim.close()


def _field(seed, n, dims, vel_sigma, outside=0.0):
    rng = np.random.default_rng(seed)
    lo = np.array([-outside, -outside])
    hi = np.array(dims, np.float64) + outside
    pos = rng.uniform(lo, hi, size=(n, 2)).astype(np.float32)
    vel = rng.normal(0, vel_sigma, size=(n, 2)).astype(np.float32)
    return pos, vel


def test_upload_binning_edge_values(W, O):
    dims, cs = (30.0, 20.0), 3
    pos, vel = _field(1, 400, dims, 0.5, outside=8.0)
    special = np.array([[0.0, 0.0], [30.0, 20.0], [-0.0, 5.0], [-1e-45, 3.0], [29.999998, 19.999998],
                        [np.nan, 1.0], [1.0, np.nan], [np.inf, 1.0], [-np.inf, 2.0], [3.0, 3.0],
                        [2.9999998, 3.0000002], [33.0, 20.9], [32.999996, 1.0], [1e30, -1e30]],
                       np.float32)
    pos = np.concatenate([pos, special])
    vel = np.concatenate([vel, np.ones_like(special)])
    sim = make_sim(W, dims, cs)
    try:
        sim.add_particles(pos, vel)
        ref = O.pack(O.world(*dims, cs), pos, vel, capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), ref, "upload")
        s = sim.settings()
        assert list(s.grid_dimensions) == [11, 7]
        assert s.particles_in_frame_count == len(ref[1])
    finally:
        sim.close()


def test_upload_empty_and_repack_store(W, O):
    dims, cs = (40.0, 40.0), 3
    a_pos, a_vel = _field(2, 300, dims, 0.3)
    b_pos, b_vel = _field(3, 200, dims, 0.3, outside=5.0)
    sim = make_sim(W, dims, cs)
    try:
        sim.add_particles(np.zeros((0, 2), np.float32), np.zeros((0, 2), np.float32))
        p, v, t = sim.read_frame()
        assert len(p) == 0 and not t.any()
        sim.add_particles(a_pos, a_vel)
        sim.step(3)
        # like the reference, a second add re-packs the whole store
        # (runners/bevy/src/state.rs:90-101): the frame restarts from it
        sim.add_particles(b_pos, b_vel)
        ref = O.pack(O.world(*dims, cs), np.concatenate([a_pos, b_pos]),
                     np.concatenate([a_vel, b_vel]), capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), ref, "repack")
    finally:
        sim.close()


def test_replacing_uploads_empty_and_refilled(W, O):
    # replacing uploads into the frame buffers directly: empty after a full
    # frame, then refilled, each followed by frames that match the oracle
    dims = (64.0, 48.0)
    pos, vel = _field(13, 2500, dims, 1.0, outside=3.0)
    sim = make_sim(W, dims, 1, 1, 4, 0.1)
    try:
        w, ph = O.world(*dims, 1), oracle_physics(O, 1, 4, 0.1)
        sim.set_particles(pos, vel)
        sim.step(3)
        empty = np.zeros((0, 2), np.float32)
        sim.set_particles(empty, empty)
        p, v, t = sim.read_frame()
        assert len(p) == 0 and not t.any()
        sim.step(2)
        assert len(sim.read_frame()[0]) == 0
        sim.set_particles(pos[:1700], vel[:1700])
        ref = O.pack(w, pos[:1700], vel[:1700], capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), ref, "refilled")
        sim.step(4)
        ref = O.step(w, ph, ref[0], ref[1], ref[2], 4)[:3]
        assert_frame_equal(sim.read_frame(), ref, "4 frames after the refill")
    finally:
        sim.close()


@pytest.mark.parametrize("seed", [0, 1])
def test_reference_mode_bit_exact(W, O, seed):
    # dense enough that cells overflow the capacity of 9 (cell.rs:79-95)
    dims, cs = (48.0, 36.0), 3
    pos, vel = _field(seed, 2500, dims, 0.6)
    pos[:300] = np.float32(7.5) + np.random.default_rng(seed).uniform(-1, 1, (300, 2)).astype(np.float32)
    _run_both(W, O, dims, cs, pos, vel, 0, [1, 2, 7, 40], capacity=4000)


def test_reference_mode_cell_size_one(W, O):
    dims = (200.0, 120.0)
    pos, vel = _field(4, 9000, dims, 1.0)
    _run_both(W, O, dims, 1, pos, vel, 0, [1, 5, 30])


@pytest.mark.parametrize("iterations", [0, 1, 2, 4])
def test_extended_mode_bit_exact(W, O, iterations):
    dims = (96.0, 64.0)
    pos, vel = _field(5, 3000, dims, 1.0)
    _run_both(W, O, dims, 1, pos, vel, 1, [1, 3, 25], iterations=iterations, gravity=0.1)


def test_extended_mode_cell_size_two(W, O):
    dims = (128.0, 96.0)
    pos, vel = _field(6, 6000, dims, 0.8)
    _run_both(W, O, dims, 2, pos, vel, 1, [1, 10], iterations=3, gravity=0.05)


def test_large_displacement_frame(W, O):
    # velocities far above the clamp: the first frame moves particles by many
    # cells at once
    dims = (64.0, 64.0)
    pos, vel = _field(7, 2000, dims, 15.0)
    flags = _run_both(W, O, dims, 1, pos, vel, 0, [1, 2, 12])
    assert flags == 0


def test_small_config_100_steps_bit_exact(W, O):
    # 16,384 particles, 512x512, N(0, 2) velocities, cell 1, gravity 0.1,
    # 4 iterations, 100 steps; bit-exact, so the kinetic energy, momentum and
    # density histogram agree exactly too
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.small()
    sim = make_sim(W, dims, 1, 1, 4, 0.1)
    try:
        w = O.world(*dims, 1)
        sim.add_particles(pos, vel)
        sim.step(100)
        gp, gv, gt = sim.read_frame()
        rt, rp, rv, _ = O.step(w, O.extended_physics(4, 0.1), *O.pack(w, pos, vel, sim.capacity()), 100)
        assert_frame_equal((gp, gv, gt), (rt, rp, rv), "100 steps")
        ke_g, mom_g, h_g = frame_stats(gp, gv, dims)
        ke_r, mom_r, h_r = frame_stats(rp, rv, dims)
        assert abs(ke_g - ke_r) <= 0.01 * abs(ke_r)
        assert np.allclose(mom_g, mom_r, rtol=0.01, atol=1e-3)
        assert np.array_equal(h_g, h_r)
    finally:
        sim.close()


def test_determinism(W):
    dims = (300.0, 200.0)
    pos, vel = _field(8, 20000, dims, 1.0)
    out = []
    for _ in range(2):
        sim = make_sim(W, dims, 1, 1, 4, 0.1)
        sim.add_particles(pos, vel)
        sim.step(37)
        out.append(sim.read_frame())
        sim.close()
    assert np.array_equal(out[0][2], out[1][2])
    assert same_bits(out[0][0], out[1][0]) and same_bits(out[0][1], out[1][1])


def test_capacity_error_keeps_state(W, O):
    sim = make_sim(W, (20.0, 20.0), 1, capacity=100)
    try:
        pos, vel = _field(9, 80, (20.0, 20.0), 0.5)
        sim.add_particles(pos, vel)
        before = sim.read_frame()
        with pytest.raises(W.CapacityError):
            sim.add_particles(*_field(10, 30, (20.0, 20.0), 0.5))
        after = sim.read_frame()
        assert np.array_equal(before[2], after[2]) and same_bits(before[0], after[0])
        # a replacing upload of more particles than the frame holds: refused
        # when more than the capacity fall inside the grid, the frame kept ...
        with pytest.raises(W.CapacityError):
            sim.set_particles(*_field(11, 130, (20.0, 20.0), 0.5))
        after = sim.read_frame()
        assert np.array_equal(before[2], after[2]) and same_bits(before[0], after[0])
        # ... and packed when no more than the capacity do
        pos, vel = _field(12, 130, (20.0, 20.0), 0.5)
        pos[:40] += np.float32(50.0)
        sim.set_particles(pos, vel)
        ref = O.pack(O.world(20.0, 20.0, 1), pos, vel, capacity=100)
        assert_frame_equal(sim.read_frame(), ref, "130 particles, 90 inside")
    finally:
        sim.close()


def test_empty_world_steps(W):
    sim = make_sim(W, (50.0, 30.0), 1, 1)
    try:
        sim.step(5)
        p, v, t = sim.read_frame()
        assert len(p) == 0 and not t.any()
        assert sim.flags() == 0
    finally:
        sim.close()


def test_batched_worlds_match_single_world_oracle(W, O):
    rng = np.random.default_rng(11)
    dims = [(37.0, 23.0), (64.0, 64.0), (5.0, 90.0), (128.0, 17.0), (1.0, 1.0)]
    counts = [300, 1500, 200, 900, 3]
    cfg = W.WrachConfig(cell_size=1, mode=1, iterations=4, gravity=0.1, capacity=2000)
    sim = W.Simulation(cfg, worlds=dims)
    try:
        refs = []
        for k, (d, n) in enumerate(zip(dims, counts)):
            pos = rng.uniform((0, 0), d, size=(n, 2)).astype(np.float32)
            vel = rng.normal(0, 1.0, size=(n, 2)).astype(np.float32)
            sim.add_particles(pos, vel, world=k)
            w = O.world(d[0], d[1], 1)
            refs.append((w, O.pack(w, pos, vel, 2000)))
        for k, (w, ref) in enumerate(refs):
            assert_frame_equal(sim.read_frame(k), ref, "world %d upload" % k)
        sim.step(9)
        ph = O.extended_physics(4, 0.1)
        for k, (w, ref) in enumerate(refs):
            want = O.step(w, ph, ref[0], ref[1], ref[2], 9)[:3]
            assert_frame_equal(sim.read_frame(k), want, "world %d after 9 steps" % k)
    finally:
        sim.close()


@pytest.mark.parametrize("cell_size", [1, 2])
def test_batch_256_worlds_checked_every_100_steps(W, O, cell_size):
    # the full batched-worlds workload: 256 worlds (sides U[128, 1024],
    # counts log-uniform in [1024, 65536], 3.85 M particles), extended
    # physics, 500 steps, at the configured cell size 1 and the tuned 2.
    # Every 100 steps the GPU state of 8 worlds (the smallest, the largest, 6
    # at random) is stepped once by the single-world oracle (the per-world
    # semantics of spatial_bin.rs:103-149, cell.rs:52-95) and the next GPU
    # frame of each (table, order, positions, velocities) must match
    from wrach_gb300 import workloads
    dims, poss, vels = workloads.batch()
    sizes = [len(p) for p in poss]
    cfg = W.WrachConfig(cell_size=cell_size, mode=1, iterations=4, gravity=0.1,
                        capacity=int(max(sizes)))
    sim = W.Simulation(cfg, worlds=dims.tolist())
    try:
        rng = np.random.default_rng(3)
        sample = sorted({int(np.argmin(sizes)), int(np.argmax(sizes))}
                        | set(int(k) for k in rng.choice(len(poss), 6, replace=False)))
        for k, (p, v) in enumerate(zip(poss, vels)):
            sim.set_particles(p, v, world=k)
        ph = O.extended_physics(4, 0.1)
        worlds = {k: O.world(float(dims[k][0]), float(dims[k][1]), cell_size) for k in sample}
        for k in sample:
            ref = O.pack(worlds[k], poss[k], vels[k], sim.capacity(k))
            assert_frame_equal(sim.read_frame(k), ref, "world %d upload" % k)
        done = 0
        while done < 500:
            sim.step(99)
            states = {k: sim.read_frame(k) for k in sample}
            sim.step(1)
            done += 100
            for k in sample:
                gp, gv, gt = states[k]
                want = O.step(worlds[k], ph, gt, gp, gv, 1)[:3]
                assert_frame_equal(sim.read_frame(k), want, "world %d step %d" % (k, done))
                assert int(gt[-1]) == sizes[k]
        assert sim.stats()["overflow"] == 0
    finally:
        sim.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_full_size_lattice_steps(W, O, mode):
    # 1,000,000 particles, 1920x1080, cell 1: the benchmark workload
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.lattice()
    _run_both(W, O, dims, 1, pos, vel, mode, [1, 2, 10], iterations=4,
              gravity=0.1 if mode else 0.0)


def test_host_round_trip_frames_at_full_size(W, O):
    """The end-to-end loop of a host application at the benchmark size:
    each frame re-uploads the host's particles (pinned arrays), steps once
    and reads the frame back into pinned arrays.  The upload copies the
    velocities beside the positions' sort and returns before its last sort
    steps end; every frame must still equal the oracle's."""
    torch = pytest.importorskip("torch")
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.lattice()
    n = len(pos)
    sim = make_sim(W, dims, 1, 1, 4, 0.1)
    try:
        cap, cells = sim.capacity(), sim.cells()
        w = O.world(dims[0], dims[1], 1)
        ph = oracle_physics(O, 1, 4, 0.1)
        h_pos = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
        h_vel = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
        o_pos = torch.empty((cap, 2), dtype=torch.float32, pin_memory=True).numpy()
        o_vel = torch.empty((cap, 2), dtype=torch.float32, pin_memory=True).numpy()
        o_idx = torch.empty(cells + 2, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        cur_pos, cur_vel = pos, vel
        for frame in range(3):
            h_pos[:len(cur_pos)] = cur_pos
            h_vel[:len(cur_vel)] = cur_vel
            sim.set_particles(h_pos[:len(cur_pos)], h_vel[:len(cur_vel)])
            # the host arrays are free once the upload returns
            h_pos[:] = np.nan
            h_vel[:] = np.nan
            sim.step(1)
            sim.read(out=(o_pos, o_vel, o_idx))
            m = int(o_idx[-1])
            table, ref_pos, ref_vel = O.pack(w, cur_pos, cur_vel, capacity=cap)
            ref = O.step(w, ph, table, ref_pos, ref_vel, 1)[:3]
            assert_frame_equal((o_pos[:m], o_vel[:m], o_idx), ref, "round trip %d" % frame)
            cur_pos, cur_vel = o_pos[:m].copy(), o_vel[:m].copy()
    finally:
        sim.close()


def test_clustered_blobs_checked_every_100_steps(W, O):
    # 4,000,000 particles in 32 blobs falling into a 4096x2048 basin, 2000
    # steps; every 100 steps the GPU's own state is stepped once by the oracle
    # and the next GPU frame (table, order, positions, velocities) must match
    from wrach_gb300 import workloads
    dims, pos, vel = workloads.blobs()
    sim = make_sim(W, dims, 1, 1, 4, 0.1)
    try:
        w = O.world(*dims, 1)
        ph = O.extended_physics(4, 0.1)
        sim.add_particles(pos, vel)
        done = 0
        while done < 2000:
            sim.step(99)
            gp, gv, gt = sim.read_frame()
            want = O.step(w, ph, gt, gp, gv, 1)[:3]
            sim.step(1)
            done += 100
            assert_frame_equal(sim.read_frame(), want, "step %d" % done)
            assert int(gt[-1]) == len(pos)
    finally:
        sim.close()


def test_few_fast_particles(W, O):
    # a quiet field with a handful of fast particles that jump several cells
    # in the first frame
    dims = (120.0, 90.0)
    pos, vel = _field(12, 5000, dims, 0.2)
    fast = np.random.default_rng(13).choice(len(pos), 60, replace=False)
    vel[fast] = np.random.default_rng(14).uniform(-6, 6, size=(60, 2)).astype(np.float32)
    sim = make_sim(W, dims, 1, 0)
    try:
        sim.add_particles(pos, vel)
        w = O.world(*dims, 1)
        ref = O.pack(w, pos, vel, sim.capacity())
        sim.step(1)
        ref = O.step(w, O.reference_physics(), *ref, 1)[:3]
        assert_frame_equal(sim.read_frame(), ref, "frame with fast particles")
        assert sim.stats()["frames"] == 1
        sim.step(5)
        ref = O.step(w, O.reference_physics(), *ref, 5)[:3]
        assert_frame_equal(sim.read_frame(), ref, "after 6 frames")
    finally:
        sim.close()


def test_many_fast_particles(W, O):
    dims = (200.0, 200.0)
    pos, vel = _field(15, 8000, dims, 5.0)
    sim = make_sim(W, dims, 1, 1, 2, 0.1)
    try:
        sim.add_particles(pos, vel)
        w = O.world(*dims, 1)
        ref = O.pack(w, pos, vel, sim.capacity())
        sim.step(2)
        ref = O.step(w, O.extended_physics(2, 0.1), *ref, 2)[:3]
        assert_frame_equal(sim.read_frame(), ref, "fast frames")
        assert sim.stats()["overflow"] == 0
    finally:
        sim.close()

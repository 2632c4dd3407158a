"""The three paths of the counting-sort rebin, bit for bit against the oracle's
stable counting sort: cells of up to 64 particles (ranked per slot), larger
cells (sorted in shared memory), and cells beyond 2048 particles (sorted in
global memory by one block).  Uploads and frames both go through the rebin."""
import numpy as np
import pytest

from tests.helpers import assert_frame_equal, make_sim, oracle_physics

pytestmark = pytest.mark.gpu


def _clustered(seed, dims, clusters, background):
    """`clusters`: [(cell x, cell y, count)], each cluster inside one cell of
    size 1; plus `background` particles spread over the box."""
    rng = np.random.default_rng(seed)
    parts = [rng.uniform((0, 0), dims, size=(background, 2))]
    for cx, cy, m in clusters:
        parts.append(np.column_stack([cx + rng.uniform(0.05, 0.95, m), cy + rng.uniform(0.05, 0.95, m)]))
    pos = np.concatenate(parts).astype(np.float32)
    order = rng.permutation(len(pos))  # uploads arrive in any order
    pos = pos[order]
    vel = rng.normal(0, 0.4, size=pos.shape).astype(np.float32)
    return pos, vel


def _run(W, O, dims, pos, vel, mode, frames, gravity=0.0):
    sim = make_sim(W, dims, 1, mode, 4, gravity, capacity=len(pos) + 16)
    try:
        w = O.world(dims[0], dims[1], 1)
        ph = oracle_physics(O, mode, 4, gravity)
        sim.add_particles(pos, vel)
        ref = O.pack(w, pos, vel, capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), ref, "upload")
        for f in range(frames):
            sim.step(1)
            ref = O.step(w, ph, ref[0], ref[1], ref[2], 1)[:3]
            assert_frame_equal(sim.read_frame(), ref, "frame %d" % (f + 1))
        return sim.stats()
    finally:
        sim.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_large_cells(W, O, mode):
    dims = (64.0, 48.0)
    pos, vel = _clustered(1, dims, [(10, 10, 2048), (20, 20, 700), (30, 30, 65), (40, 12, 64),
                                    (5, 40, 33)], 2500)
    st = _run(W, O, dims, pos, vel, mode, 4, gravity=0.1 if mode else 0.0)
    assert st["huge_cells"] == 0


def test_cell_beyond_the_shared_memory_sort(W, O):
    dims = (32.0, 24.0)
    pos, vel = _clustered(2, dims, [(8, 8, 9000), (12, 12, 2049), (16, 16, 100)], 800)
    st = _run(W, O, dims, pos, vel, 1, 2, gravity=0.1)
    assert st["huge_cells"] >= 1


def test_floor_pile(W, O):
    # the shape a long run of the extended physics reaches: most particles in
    # the bottom row of cells, a few hundred per cell
    rng = np.random.default_rng(3)
    dims = (200.0, 60.0)
    n = 60000
    pos = np.column_stack([rng.uniform(0, 200.0, n), rng.uniform(0, 0.999, n) ** 3]).astype(np.float32)
    pos = np.concatenate([pos, rng.uniform((0, 1), dims, size=(3000, 2)).astype(np.float32)])
    vel = rng.normal(0, 0.3, size=pos.shape).astype(np.float32)
    st = _run(W, O, dims, pos, vel, 1, 3, gravity=0.1)
    assert st["huge_cells"] == 0


def test_profiled_frames_match_graph_frames(W, O):
    # a profiled frame runs its launches one at a time on the frame's stream
    # (the large cells' sort included); graph frames run that sort on a
    # second stream beside the small cells' pass.  Both match the oracle.
    dims = (64.0, 48.0)
    pos, vel = _clustered(4, dims, [(10, 10, 300), (20, 20, 65), (30, 30, 64)], 2500)
    sim = make_sim(W, dims, 1, 1, 4, 0.1, capacity=len(pos) + 16)
    try:
        w = O.world(dims[0], dims[1], 1)
        ph = oracle_physics(O, 1, 4, 0.1)
        sim.add_particles(pos, vel)
        ref = O.pack(w, pos, vel, capacity=sim.capacity())
        for f in range(6):
            if f % 2 == 0:
                ms = sim.profile_frame()
                assert len(ms) == 8  # four Jacobi passes, four rebin launches
                assert all(m >= 0.0 for m in ms)
            else:
                sim.step(1)
            ref = O.step(w, ph, ref[0], ref[1], ref[2], 1)[:3]
            assert_frame_equal(sim.read_frame(), ref, "frame %d" % (f + 1))
    finally:
        sim.close()

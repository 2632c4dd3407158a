"""Viewport streaming with write-back to the store, bit for bit against the
oracle's rules: the frame is packed from the store's particles inside the
viewport (create_packed_data), a write-back makes the store its particles
outside the viewport followed by the frame, and moving the viewport writes
back and re-packs under the new anchor (walls included)."""
import numpy as np
import pytest

from tests.helpers import assert_frame_equal, make_sim, oracle_physics, same_bits

pytestmark = pytest.mark.gpu


def _field(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(lo, hi, size=(n, 2)).astype(np.float32)
    vel = rng.normal(0, 0.6, size=(n, 2)).astype(np.float32)
    return pos, vel


def _store_equal(sim, ref, what, world=0):
    gp, gv = sim.store(world)
    rp, rv = ref
    assert len(gp) == len(rp), what + ": store size %d vs %d" % (len(gp), len(rp))
    assert same_bits(gp, rp) and same_bits(gv, rv), what + ": store contents"


@pytest.mark.parametrize("mode", [0, 1])
def test_write_back_and_moving_viewport(W, O, mode):
    dims, cs = (64.0, 48.0), 1
    pos, vel = _field(1, 5000, (-40.0, -30.0), (104.0, 78.0))
    sim = make_sim(W, dims, cs, mode, 4, 0.1 if mode else 0.0, capacity=8000)
    try:
        ph = oracle_physics(O, mode, 4, 0.1 if mode else 0.0)
        w = O.world(dims[0], dims[1], cs)
        sim.add_particles(pos, vel)
        store = (pos, vel)
        _store_equal(sim, store, "after add")
        frame = O.pack(w, pos, vel, capacity=sim.capacity())
        assert_frame_equal(sim.read_frame(), frame, "upload")
        sim.step(5)
        frame = O.step(w, ph, frame[0], frame[1], frame[2], 5)[:3]
        assert_frame_equal(sim.read_frame(), frame, "5 frames")
        # write-back alone leaves the frame as it is
        sim.write_back()
        store = O.write_back(w, store[0], store[1], frame[1], frame[2])
        _store_equal(sim, store, "write-back")
        assert_frame_equal(sim.read_frame(), frame, "frame after write-back")
        for anchor in [(10.5, -7.25), (-31.0, 20.0), (0.0, 0.0)]:
            sim.set_viewport(anchor)
            store = O.write_back(w, store[0], store[1], frame[1], frame[2])
            w = O.world(dims[0], dims[1], cs, anchor=anchor)
            _store_equal(sim, store, "store at %s" % (anchor,))
            frame = O.pack(w, store[0], store[1], capacity=sim.capacity())
            assert_frame_equal(sim.read_frame(), frame, "frame at %s" % (anchor,))
            s = sim.settings()
            assert (s.view_anchor[0], s.view_anchor[1]) == anchor
            sim.step(4)
            frame = O.step(w, ph, frame[0], frame[1], frame[2], 4)[:3]
            assert_frame_equal(sim.read_frame(), frame, "4 frames at %s" % (anchor,))
    finally:
        sim.close()


def test_moving_one_world_of_a_batch(W, O):
    dims = [(40.0, 30.0), (50.0, 20.0), (30.0, 30.0)]
    cfg = W.WrachConfig(cell_size=1, mode=1, iterations=4, gravity=0.1, capacity=4000)
    fields = [_field(10 + k, 1500, (-20.0, -20.0), (d[0] + 20.0, d[1] + 20.0)) for k, d in enumerate(dims)]
    with W.Simulation(cfg, worlds=dims) as sim:
        for k, (p, v) in enumerate(fields):
            sim.set_particles(p, v, world=k)
        sim.step(3)
        before = [sim.read_frame(world=k) for k in (0, 2)]
        sim.set_viewport((7.0, -5.0), world=1)
        ph = O.extended_physics(4, 0.1)
        w1 = O.world(dims[1][0], dims[1][1], 1)
        f1 = O.pack(w1, fields[1][0], fields[1][1], capacity=sim.capacity(1))
        f1 = O.step(w1, ph, f1[0], f1[1], f1[2], 3)[:3]
        store = O.write_back(w1, fields[1][0], fields[1][1], f1[1], f1[2])
        _store_equal(sim, store, "world 1 store", world=1)
        w1 = O.world(dims[1][0], dims[1][1], 1, anchor=(7.0, -5.0))
        assert_frame_equal(sim.read_frame(world=1), O.pack(w1, store[0], store[1], capacity=sim.capacity(1)),
                           "world 1 frame")
        for k, b in zip((0, 2), before):
            a = sim.read_frame(world=k)
            assert np.array_equal(a[2], b[2]) and same_bits(a[0], b[0]) and same_bits(a[1], b[1])


def test_a_move_that_changes_the_grid_is_refused(W):
    # 10 px wide with 3 px cells: anchored at 0 the grid is 4 cells wide, at
    # 2.5 it is 5
    sim = make_sim(W, (10.0, 9.0), 3, capacity=100)
    try:
        sim.add_particles(np.array([[1.0, 1.0]], np.float32), np.zeros((1, 2), np.float32))
        with pytest.raises(W.WrachError):
            sim.set_viewport((2.5, 0.0))
        assert tuple(sim.settings().view_anchor) == (0.0, 0.0)
        sim.set_viewport((3.0, 0.0))  # a whole cell: the grid keeps its size
        assert tuple(sim.settings().view_anchor) == (3.0, 0.0)
    finally:
        sim.close()

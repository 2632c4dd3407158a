"""Failure detection without a GPU fault: a bounded device wait on a word
that nothing sets gives up after its limit and reports it, and the context
keeps working (the next frames match the oracle bit for bit).  Failures of
the host side (bad arguments, capacity) are the errors tested elsewhere."""
import numpy as np
import pytest

from tests.helpers import assert_frame_equal, make_sim, oracle_physics

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(W, O):
    dims = (50.0, 40.0)
    rng = np.random.default_rng(7)
    pos = rng.uniform((0, 0), dims, size=(1500, 2)).astype(np.float32)
    vel = rng.normal(0, 0.5, size=pos.shape).astype(np.float32)
    sim = make_sim(W, dims, 1, 1, 4, 0.1, capacity=3000)
    try:
        sim.add_particles(pos, vel)
        timed_out, waited = sim.selftest_wait(2000)
        assert timed_out and 2000 <= waited < 1_000_000
        assert sim.flags() == 0  # the probe leaves the sticky flags alone
        with pytest.raises(W.WrachError):
            sim.selftest_wait(2_000_000)  # above the 1 s cap
        w = O.world(*dims, 1)
        ref = O.pack(w, pos, vel, capacity=sim.capacity())
        sim.step(3)
        ref = O.step(w, oracle_physics(O, 1, 4, 0.1), ref[0], ref[1], ref[2], 3)[:3]
        assert_frame_equal(sim.read_frame(), ref, "frames after the probe")
    finally:
        sim.close()

"""The CUDA path against the committed golden fixtures (tests/golden/)."""
import pytest

from tests.golden import make_fixtures as F
from tests.helpers import assert_frame_equal, make_sim

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(F.CASES))
def test_cuda_matches_golden_fixture(W, name):
    meta, z = F.load(name)
    sim = make_sim(W, tuple(meta["dims"]), meta["cs"], meta["mode"], meta.get("iterations", 4),
                   meta.get("gravity", 0.0))
    try:
        sim.add_particles(z["pos_in"], z["vel_in"])
        assert_frame_equal(sim.read_frame(), (z["table_0"], z["pos_0"], z["vel_0"]), "upload")
        done = 0
        for s in meta["steps"]:
            sim.step(s - done)
            done = s
            assert_frame_equal(sim.read_frame(), (z["table_%d" % s], z["pos_%d" % s], z["vel_%d" % s]),
                               "%s after %d steps" % (name, s))
    finally:
        sim.close()

"""The headless point rasteriser against its CPU restatement, bit for bit."""
import numpy as np
import pytest

from oracle import render_oracle as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale", [1, 4])
def test_render_matches_oracle(W, scale):
    rng = np.random.default_rng(5)
    dims = (48.0, 36.0)
    pos = rng.uniform((0, 0), dims, size=(400, 2)).astype(np.float32)
    pos[:4] = [[0.0, 0.0], [48.0, 36.0], [0.2, 35.9], [24.5, 18.5]]
    with W.Simulation(W.WrachConfig(dimensions=dims, cell_size=3, capacity=1000)) as sim:
        sim.add_particles(pos, np.zeros_like(pos))
        p, _, _ = sim.read_frame()
        w, h = int(dims[0]) * scale, int(dims[1]) * scale
        img = sim.render(w, h)
        want = R.render(p, dims[0], dims[1], w, h)
        assert img.shape == (h, w)
        assert np.array_equal(img, want)
        assert img.max() == 255 and (img > 0).sum() > 0

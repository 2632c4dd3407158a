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


def test_msaa_resolves_the_union_of_covered_samples(W):
    """Two quads covering disjoint samples of one pixel: with 4x MSAA the
    pixel resolves to all four samples (white), not to the larger of the two
    particles' coverages (assets/shaders/draw.wgsl:18-40,
    runners/bevy/src/render/pipeline.rs:52-56)."""
    dims = (48.0, 36.0)
    # pixel (0, 0): samples x 0.375, 0.875, 0.125, 0.625 at y 0.125 .. 0.875;
    # the first quad spans x [-0.3, 0.5) (samples 0 and 2), the second x
    # [0.5, 1.3) (samples 1 and 3), both y [0.1, 0.9)
    pos = np.array([[0.1, 35.5], [0.9, 35.5]], np.float32)
    want = R.render(pos, dims[0], dims[1], 48, 36)
    assert want[0, 0] == 255
    assert R.render(pos[:1], dims[0], dims[1], 48, 36)[0, 0] == 127
    with W.Simulation(W.WrachConfig(dimensions=dims, cell_size=3, capacity=100)) as sim:
        sim.add_particles(pos, np.zeros_like(pos))
        p, _, _ = sim.read_frame()
        img = sim.render(48, 36)
    assert np.array_equal(img, R.render(p, dims[0], dims[1], 48, 36))
    assert img[0, 0] == 255

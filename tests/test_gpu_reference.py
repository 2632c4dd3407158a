"""The reference's GPU integration tests, restated against the CUDA library
through the WrachAPI mirror (runners/api/src/lib.rs) and the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _particles(W, coords, vel=(0.0, 0.0)):
    return [W.Particle(position=W.Vec2(*c), velocity=W.Vec2(*vel)) for c in coords]


def _four(dims, first, second):
    return [first, second, (dims[0] / 2, dims[1] / 2), (float(dims[0]), float(dims[1]))]


# runners/bevy/src/compute/03_prefix_sum.rs:150-207
def test_prefix_sum_for_small_arrays(W, O):
    dims, cs = (10, 10), 5
    api = W.WrachAPI(W.WrachConfig(dimensions=dims, cell_size=cs))
    try:
        coords = _four(dims, (0.1, 0.1), (2.0, 2.0))
        api.add_particles(_particles(W, coords))
        for _ in range(4):
            api.tick()
        gpu = api.get_simulation_state().packed_data.indices
        cpu, _, _ = O.pack(O.world(*dims, cs), np.array(coords, np.float32), np.zeros((4, 2)))
        assert cpu.tolist() == [0, 0, 2, 2, 2, 2, 3, 3, 3, 3, 4]
        assert gpu == cpu.tolist()
    finally:
        api.close()


# runners/bevy/src/compute/03_prefix_sum.rs:209-260
def test_prefix_sum_for_large_arrays(W, O):
    dims, cs = (500, 300), 6
    api = W.WrachAPI(W.WrachConfig(dimensions=dims, cell_size=cs))
    try:
        coords = _four(dims, (1.1, 1.1), (2.2, 2.2))
        api.add_particles(_particles(W, coords))
        for _ in range(4):
            api.tick()
        gpu = api.get_simulation_state().packed_data.indices
        cpu, _, _ = O.pack(O.world(*dims, cs), np.array(coords, np.float32), np.zeros((4, 2)))
        assert len(gpu) == len(cpu)
        assert gpu == cpu.tolist()
    finally:
        api.close()


# runners/bevy/src/compute/04_pack_particle_data.rs:72-140
def test_packed_data(W):
    dims, cs = (10, 10), 3
    api = W.WrachAPI(W.WrachConfig(dimensions=dims, cell_size=cs))
    try:
        api.add_particles(_particles(W, _four(dims, (0.1, 0.1), (2.5, 2.5))))
        for _ in range(4):
            api.tick()
        pos = [tuple(p) for p in api.get_simulation_state().packed_data.positions]
        f = lambda x: float(np.float32(x))
        # the reference tolerates any order inside the first cell; this
        # implementation keeps the stable order, so no sort is needed
        assert pos[0:2] == [(f(0.1), f(0.1)), (2.5, 2.5)]
        assert pos[2:4] == [(5.0, 5.0), (10.0, 10.0)]
    finally:
        api.close()


# runners/api/src/lib.rs:101-126
def test_api_returns_data(W):
    api = W.WrachAPI(W.WrachConfig(dimensions=(10, 10), cell_size=3))
    try:
        api.add_particles(_particles(W, [(5.0, 5.0)] * 3, vel=(0.5, 0.5)))
        for _ in range(5):
            api.tick()
        assert len(api.positions) == 164
        assert api.positions[0] != (0.0, 0.0)
        assert len(api.velocities) == 164
        assert api.velocities[0] != (0.0, 0.0)
    finally:
        api.close()


# shaders/physics/src/particles.rs:128-146, on the GPU
def test_pushes_particles_apart(W):
    api = W.WrachAPI(W.WrachConfig(dimensions=(10, 10), cell_size=3))
    try:
        api.add_particles(_particles(W, [(1.0, 1.0), (1.1, 1.1)]))
        api.tick()
        f = np.float32
        assert api.positions[0] == (float(f(0.69644666)), float(f(0.69644666)))
        assert api.positions[1] == (float(f(1.4035534)), float(f(1.4035534)))
    finally:
        api.close()


def test_settings_uniform_layout(W):
    import ctypes
    assert ctypes.sizeof(W._lib.WorldSettings) == 32
    api = W.WrachAPI(W.WrachConfig(dimensions=(480, 352), cell_size=3))
    try:
        s = api.get_simulation_state().shader_settings
        assert list(s.view_dimensions) == [480.0, 352.0]
        assert list(s.grid_dimensions) == [161, 118]
        assert s.cell_size == 3
    finally:
        api.close()

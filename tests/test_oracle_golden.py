"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates one test of the reference, with its expected values, and
cites it.  The reference's GPU integration tests (which need a wgpu adapter)
are restated here against the oracle and, in tests/test_gpu_reference.py,
against the CUDA library.
"""
import numpy as np

NO_VEL = np.zeros((2, 2), np.float32)


# shaders/physics/src/particles.rs:128-146 (pushes_particles_apart)
def test_pushes_particles_apart(O):
    w = O.world(10, 10, 3)
    table, pos, vel = O.pack(w, [[1.0, 1.0], [1.1, 1.1]], NO_VEL)
    po, _ = O.solve(w, O.reference_physics(), table, pos, vel)
    f = np.float32
    assert po[0].tolist() == [f(0.69644666), f(0.69644666)]
    assert po[1].tolist() == [f(1.4035534), f(1.4035534)]
    d = np.sqrt(np.sum((po[0] - po[1]) ** 2))
    assert 0.999 < d < 1.001


def test_pushes_particles_apart_with_velocity_integrates_after(O):
    # finish() integrates after pairs() (particles.rs:96-107): the pushed
    # positions plus the test's velocities, in binary32
    w = O.world(10, 10, 3)
    vel = np.array([[0.1, 0.2], [0.3, 0.4]], np.float32)
    table, pos, v = O.pack(w, [[1.0, 1.0], [1.1, 1.1]], vel)
    po, vo = O.solve(w, O.reference_physics(), table, pos, v)
    pushed = np.array([[0.69644666, 0.69644666], [1.4035534, 1.4035534]], np.float32)
    assert np.array_equal(po, pushed + vel)
    assert np.array_equal(vo, vel)


# runners/bevy/src/spatial_bin.rs:156-182
def test_cell_coords(O):
    assert (O.cell_coord(3.0, 3), O.cell_coord(3.0, 3)) == (1, 1)
    assert O.cell_coord(0.1, 3) == 0
    assert O.cell_coord(6.5, 3) == 2
    assert O.cell_coord(-3.0, 3) == -1


# runners/bevy/src/spatial_bin.rs:184-248
def test_active_cells(O):
    w = O.world(10, 10, 6)
    assert O.active_cells(w).tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    assert list(w.grid_dimensions) == [2, 2]
    w = O.world(15, 10, 6)
    assert O.active_cells(w).tolist() == [[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1]]
    assert list(w.grid_dimensions) == [3, 2]
    # viewport (3.3, 3.3, 9.0, 9.0)
    w = O.world(9.0 - 3.3, 9.0 - 3.3, 6, anchor=(3.3, 3.3))
    assert O.active_cells(w).tolist() == [[0, 0], [1, 0], [0, 1], [1, 1]]
    # viewport (-5, -5, 0, 0)
    w = O.world(5.0, 5.0, 6, anchor=(-5.0, -5.0))
    assert O.active_cells(w).tolist() == [[-1, -1], [0, -1], [-1, 0], [0, 0]]


# runners/bevy/src/particle_store.rs:143-167
def test_packed_data_one_particle_in_middle(O):
    w = O.world(6, 6, 3)
    table, pos, vel = O.pack(w, [[4.5, 4.5]], [[1.1, 2.3]])
    assert table.tolist() == [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1]
    assert pos.tolist() == [[4.5, 4.5]]
    assert np.array_equal(vel, np.array([[1.1, 2.3]], np.float32))


# runners/bevy/src/particle_store.rs:169-184
def test_packed_data_three_particles_in_middle(O):
    w = O.world(6, 6, 3)
    table, pos, vel = O.pack(w, [[3.0, 3.0]] * 3, [[1.1, 2.3]] * 3)
    assert table.tolist() == [0, 0, 0, 0, 0, 0, 3, 3, 3, 3, 3]
    assert len(pos) == 3
    assert pos[1].tolist() == [3.0, 3.0]
    assert np.array_equal(vel[1], np.array([1.1, 2.3], np.float32))


# runners/bevy/src/particle_store.rs:186-213
def test_packed_data_many_particles(O):
    w = O.world(6, 6, 3)
    table, pos, vel = O.pack(w, [[0.0, 1.0], [3.0, 3.0], [5.1, 4.3]],
                             [[0.0, 0.0], [1.2, 3.4], [0.0, 0.0]])
    assert table.tolist() == [0, 0, 1, 1, 1, 1, 3, 3, 3, 3, 3]
    assert len(pos) == 3
    assert np.array_equal(pos[2], np.array([5.1, 4.3], np.float32))
    assert np.array_equal(vel[1], np.array([1.2, 3.4], np.float32))


# runners/bevy/src/particle_store.rs:215-229
def test_packed_data_particle_offscreen(O):
    w = O.world(6, 6, 3)
    table, pos, vel = O.pack(w, [[6.1, 6.1], [9.1, 9.1]], np.zeros((2, 2)))
    assert table.tolist() == [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1]
    assert np.array_equal(pos, np.array([[6.1, 6.1]], np.float32))
    assert vel.tolist() == [[0.0, 0.0]]


# runners/bevy/src/particle_store.rs:231-234
def test_max_particles_per_frame(O):
    assert O.max_particles_per_frame(O.world(6, 6, 2)) == 74
    # runners/api/src/lib.rs:101-126 expects 164 readback entries for 10x10, cs 3
    assert O.max_particles_per_frame(O.world(10, 10, 3)) == 164


def _four_particles(dims, first, second):
    return np.array([first, second, [dims[0] / 2, dims[1] / 2], [dims[0], dims[1]]], np.float32)


# runners/bevy/src/compute/03_prefix_sum.rs:150-207 (prefix_sum_for_small_arrays)
def test_prefix_sum_small_arrays(O):
    dims, cs = (10, 10), 5
    w = O.world(*dims, cs)
    pos = _four_particles(dims, [0.1, 0.1], [2.0, 2.0])
    table, p, v = O.pack(w, pos, np.zeros_like(pos))
    assert table.tolist() == [0, 0, 2, 2, 2, 2, 3, 3, 3, 3, 4]
    t4, _, _, _ = O.step(w, O.reference_physics(), table, p, v, 4)
    assert t4.tolist() == table.tolist()


# runners/bevy/src/compute/03_prefix_sum.rs:209-260 (prefix_sum_for_large_arrays)
def test_prefix_sum_large_arrays(O):
    dims, cs = (500, 300), 6
    w = O.world(*dims, cs)
    pos = _four_particles(dims, [1.1, 1.1], [2.2, 2.2])
    table, p, v = O.pack(w, pos, np.zeros_like(pos))
    assert len(table) == w.cells + 2
    t4, _, _, _ = O.step(w, O.reference_physics(), table, p, v, 4)
    assert t4.tolist() == table.tolist()


# runners/bevy/src/compute/04_pack_particle_data.rs:72-140 (packed_data)
def test_packed_data_after_ticks(O):
    dims, cs = (10, 10), 3
    w = O.world(*dims, cs)
    pos = _four_particles(dims, [0.1, 0.1], [2.5, 2.5])
    table, p, v = O.pack(w, pos, np.zeros_like(pos))
    assert p.tolist() == np.array([[0.1, 0.1], [2.5, 2.5], [5.0, 5.0], [10.0, 10.0]],
                                  np.float32).tolist()
    _, p4, _, _ = O.step(w, O.reference_physics(), table, p, v, 4)
    first_cell = sorted(p4[0:2].tolist())
    assert first_cell == np.array([[0.1, 0.1], [2.5, 2.5]], np.float32).tolist()
    assert p4[2:4].tolist() == [[5.0, 5.0], [10.0, 10.0]]


# runners/api/src/lib.rs:101-126 (test_api_returns_data)
def test_api_returns_data(O):
    w = O.world(10, 10, 3)
    table, p, v = O.pack(w, [[5.0, 5.0]] * 3, [[0.5, 0.5]] * 3)
    _, p5, v5, _ = O.step(w, O.reference_physics(), table, p, v, 5)
    assert O.max_particles_per_frame(w) == 164
    assert p5[0].tolist() != [0.0, 0.0]
    assert v5[0].tolist() != [0.0, 0.0]

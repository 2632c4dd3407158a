"""wrach_pack_noalloc, the packing entry point for callers that cannot
allocate GPU memory (code in a host callback or a real-time loop that must
not wait on the allocator, a plugin whose host owns all device memory): its
output must equal the allocating path's (wrach_set_particles + wrach_read)
bit for bit, on consecutive calls that share its static scratch array, and
what only the device knows (particles that did not fit the output) must
reach the caller through the optional device status words.

This file is collected last on purpose: a run that stops at the first
failure has then already run every other test."""
import ctypes

import numpy as np
import pytest

from tests.helpers import same_bits

pytestmark = pytest.mark.gpu


def _inputs(seed, n, dims):
    rng = np.random.default_rng(seed)
    pos = rng.uniform((-5.0, -5.0), (dims[0] + 5.0, dims[1] + 5.0), size=(n, 2)).astype(np.float32)
    vel = rng.normal(0, 1, size=(n, 2)).astype(np.float32)
    return pos, vel


def _allocating_path(W, dims, cs, pos, vel):
    cfg = W.WrachConfig(dimensions=dims, cell_size=cs, capacity=max(len(pos), 1))
    with W.Simulation(cfg) as sim:
        sim.set_particles(pos, vel)
        want_pos, want_vel, want_idx = sim.read_frame()
        cells = sim.cells()
    return cfg, want_pos, want_vel, want_idx, cells


def _pack(W, torch, cfg, pos, vel, cells, out_capacity):
    L = W._lib.load()
    n = len(pos)
    d_pos = torch.from_numpy(pos).cuda() if n else torch.empty((1, 2), device="cuda")
    d_vel = torch.from_numpy(vel).cuda() if n else torch.empty((1, 2), device="cuda")
    out_pos = torch.full((max(out_capacity, 1), 2), -1.0, dtype=torch.float32, device="cuda")
    out_vel = torch.full((max(out_capacity, 1), 2), -1.0, dtype=torch.float32, device="cuda")
    out_idx = torch.full((cells + 2,), -1, dtype=torch.int32, device="cuda")
    status = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    c = cfg.to_c()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.wrach_pack_noalloc(ctypes.byref(c), d_pos.data_ptr() if n else None,
                              d_vel.data_ptr() if n else None, n, out_pos.data_ptr(),
                              out_vel.data_ptr(), out_capacity, out_idx.data_ptr(),
                              status.data_ptr(), stream)
    torch.cuda.synchronize()
    return (rc, out_pos.cpu().numpy(), out_vel.cpu().numpy(),
            out_idx.cpu().numpy().view(np.uint32), status.cpu().numpy().view(np.uint32))


def test_pack_noalloc_matches_the_allocating_path_twice(W):
    torch = pytest.importorskip("torch")
    for call, (dims, cs, n) in enumerate([((300.0, 200.0), 1, 50000), ((90.0, 70.0), 3, 20000)]):
        pos, vel = _inputs(100 + call, n, dims)
        cfg, want_pos, want_vel, want_idx, cells = _allocating_path(W, dims, cs, pos, vel)
        rc, out_pos, out_vel, idx, status = _pack(W, torch, cfg, pos, vel, cells, n)
        assert rc == 0
        m = int(idx[-1])
        assert np.array_equal(idx, want_idx), "call %d: table" % call
        assert m == len(want_pos)
        assert same_bits(out_pos[:m], want_pos), "call %d: positions" % call
        assert same_bits(out_vel[:m], want_vel), "call %d: velocities" % call
        assert list(status) == [0, 0], "call %d: status" % call


def test_pack_noalloc_with_no_particles(W):
    torch = pytest.importorskip("torch")
    dims = (40.0, 30.0)
    empty = np.zeros((0, 2), np.float32)
    cfg, _, _, want_idx, cells = _allocating_path(W, dims, 1, empty, empty)
    rc, _, _, idx, status = _pack(W, torch, cfg, empty, empty, cells, 0)
    assert rc == 0
    assert np.array_equal(idx, want_idx) and int(idx[-1]) == 0
    assert list(status) == [0, 0]


def test_pack_noalloc_reports_particles_past_out_capacity(W):
    torch = pytest.importorskip("torch")
    dims, n = (120.0, 80.0), 9000
    pos, vel = _inputs(7, n, dims)
    cfg, want_pos, want_vel, want_idx, cells = _allocating_path(W, dims, 1, pos, vel)
    m = len(want_pos)
    room = m - 1234
    rc, out_pos, out_vel, idx, status = _pack(W, torch, cfg, pos, vel, cells, room)
    assert rc == 0
    # the table still counts every packed particle; only the first `room` are written
    assert np.array_equal(idx, want_idx)
    assert same_bits(out_pos[:room], want_pos[:room])
    assert same_bits(out_vel[:room], want_vel[:room])
    assert status[0] & W._lib.FLAG_OVERFLOW
    assert int(status[1]) == m - room


def test_pack_noalloc_rejects_sizes_beyond_its_scratch(W):
    L = W._lib.load()
    c = W.WrachConfig(dimensions=(100.0, 100.0), cell_size=1).to_c()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.wrach_pack_noalloc(ctypes.byref(c), dummy, dummy, 131073, dummy, dummy, 131073,
                                dummy, None, None) == W._lib.WRACH_ERR_CAPACITY
    big = W.WrachConfig(dimensions=(1000.0, 1000.0), cell_size=1).to_c()
    assert L.wrach_pack_noalloc(ctypes.byref(big), dummy, dummy, 10, dummy, dummy, 10,
                                dummy, None, None) == W._lib.WRACH_ERR_CAPACITY

"""wrach_pack_noalloc, the packing entry point for callers that cannot
allocate GPU memory (code in a host callback or a real-time loop that must
not wait on the allocator, a plugin whose host owns all device memory): its
output must equal the allocating path's (wrach_set_particles + wrach_read)
bit for bit, on consecutive calls that share its static scratch array.

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


def test_pack_noalloc_matches_the_allocating_path_twice(W):
    torch = pytest.importorskip("torch")
    L = W._lib.load()
    for call, (dims, cs, n) in enumerate([((300.0, 200.0), 1, 50000), ((90.0, 70.0), 3, 20000)]):
        pos, vel = _inputs(100 + call, n, dims)
        cfg = W.WrachConfig(dimensions=dims, cell_size=cs, capacity=n)
        with W.Simulation(cfg) as sim:
            sim.set_particles(pos, vel)
            want_pos, want_vel, want_idx = sim.read_frame()
            cells = sim.cells()
        d_pos = torch.from_numpy(pos).cuda()
        d_vel = torch.from_numpy(vel).cuda()
        out_pos = torch.full((n, 2), -1.0, dtype=torch.float32, device="cuda")
        out_vel = torch.full((n, 2), -1.0, dtype=torch.float32, device="cuda")
        out_idx = torch.full((cells + 2,), -1, dtype=torch.int32, device="cuda")
        c = cfg.to_c()
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.wrach_pack_noalloc(ctypes.byref(c), d_pos.data_ptr(), d_vel.data_ptr(), n,
                                  out_pos.data_ptr(), out_vel.data_ptr(), n, out_idx.data_ptr(),
                                  stream)
        torch.cuda.synchronize()
        assert rc == 0
        idx = out_idx.cpu().numpy().view(np.uint32)
        m = int(idx[-1])
        assert np.array_equal(idx, want_idx), "call %d: table" % call
        assert m == len(want_pos)
        assert same_bits(out_pos.cpu().numpy()[:m], want_pos), "call %d: positions" % call
        assert same_bits(out_vel.cpu().numpy()[:m], want_vel), "call %d: velocities" % call


def test_pack_noalloc_rejects_sizes_beyond_its_scratch(W):
    L = W._lib.load()
    c = W.WrachConfig(dimensions=(100.0, 100.0), cell_size=1).to_c()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.wrach_pack_noalloc(ctypes.byref(c), dummy, dummy, 131073, dummy, dummy, 131073,
                                dummy, None) == W._lib.WRACH_ERR_CAPACITY
    big = W.WrachConfig(dimensions=(1000.0, 1000.0), cell_size=1).to_c()
    assert L.wrach_pack_noalloc(ctypes.byref(big), dummy, dummy, 10, dummy, dummy, 10,
                                dummy, None) == W._lib.WRACH_ERR_CAPACITY

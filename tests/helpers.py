"""Shared helpers for the parity tests: building matching oracle and CUDA
worlds and comparing their frames bit for bit."""
import numpy as np


def bits(a):
    """float32 array -> uint32 bit patterns (so NaN and -0.0 compare exactly)."""
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_bits(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(bits(a), bits(b))


def oracle_physics(O, mode, iterations=4, gravity=0.0):
    return O.reference_physics() if mode == 0 else O.extended_physics(iterations, gravity)


def make_sim(W, dims, cell_size, mode=0, iterations=4, gravity=0.0, capacity=0):
    cfg = W.WrachConfig(dimensions=dims, cell_size=cell_size, mode=mode, iterations=iterations,
                        gravity=gravity, capacity=capacity)
    return W.Simulation(cfg)


def first_mismatch(a, b):
    a, b = bits(a).reshape(len(a), -1), bits(b).reshape(len(b), -1)
    bad = np.nonzero(np.any(a != b, axis=1))[0]
    return int(bad[0]) if len(bad) else None


def assert_frame_equal(gpu, ref, what=""):
    """gpu = (pos, vel, table) trimmed; ref = (table, pos, vel)."""
    gp, gv, gt = gpu
    rt, rp, rv = ref
    assert len(gt) == len(rt), what + ": table length"
    if not np.array_equal(gt, rt):
        k = int(np.nonzero(gt != rt)[0][0])
        raise AssertionError("%s: table differs first at %d: gpu %d oracle %d" % (what, k, gt[k], rt[k]))
    assert gp.shape == rp.shape, what + ": particle count"
    if not same_bits(gp, rp):
        i = first_mismatch(gp, rp)
        raise AssertionError("%s: positions differ first at %d: gpu %r oracle %r" % (what, i, gp[i], rp[i]))
    if not same_bits(gv, rv):
        i = first_mismatch(gv, rv)
        raise AssertionError("%s: velocities differ first at %d: gpu %r oracle %r" % (what, i, gv[i], rv[i]))


def frame_stats(pos, vel, dims, bins=32):
    """Kinetic energy, momentum and a density histogram of a frame."""
    v = vel.astype(np.float64)
    ke = 0.5 * float(np.sum(v * v))
    mom = v.sum(axis=0)
    hist, _, _ = np.histogram2d(pos[:, 0], pos[:, 1], bins=bins,
                                range=[[0, dims[0]], [0, dims[1]]])
    return ke, mom, hist

"""Seeded synthetic particle fields of the benchmark shapes.

There is no public dataset for this path: the reference's published number
comes from random particles in a window (examples/youre-a-pixel.rs:13,
98-110).  Each generator returns float32 arrays built with
numpy.random.default_rng(seed).

  small      16,384 particles, positions U[0, 512)^2, velocities N(0, 2)
  lattice    1,000,000 particles on a jittered lattice filling 1920x1080 at
             about 0.48 per cell: 1334 x 750 sites (first 1,000,000 in
             row-major order), jitter U(-0.25, 0.25), velocities N(0, 1)
  blobs      4,000,000 particles in 32 Gaussian blobs (sigma 40, centres
             uniform in the box) clipped to 4096x2048, velocities N(0, 1)
  batch      256 worlds, sides U[128, 1024], particle counts log-uniform in
             [1024, 65536], positions uniform, velocities N(0, 2)
"""
import numpy as np


def _vel(rng, n, sigma):
    return rng.normal(0.0, sigma, size=(n, 2)).astype(np.float32)


def small(n=16384, side=512.0, vel_sigma=2.0, seed=0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0.0, side, size=(n, 2)).astype(np.float32)
    return (side, side), pos, _vel(rng, n, vel_sigma)


def lattice(n=1_000_000, width=1920.0, height=1080.0, sites=(1334, 750), jitter=0.25,
            vel_sigma=1.0, seed=0):
    rng = np.random.default_rng(seed)
    nx, ny = sites
    if nx * ny < n:
        raise ValueError("lattice too small for n")
    k = np.arange(n)
    ix, iy = k % nx, k // nx
    sx, sy = width / nx, height / ny
    pos = np.empty((n, 2), np.float32)
    pos[:, 0] = (ix + 0.5) * sx + rng.uniform(-jitter, jitter, n)
    pos[:, 1] = (iy + 0.5) * sy + rng.uniform(-jitter, jitter, n)
    return (width, height), pos, _vel(rng, n, vel_sigma)


def blobs(n=4_000_000, width=4096.0, height=2048.0, nblobs=32, sigma=40.0, vel_sigma=1.0,
          seed=0):
    rng = np.random.default_rng(seed)
    centres = rng.uniform((0.0, 0.0), (width, height), size=(nblobs, 2))
    which = rng.integers(0, nblobs, n)
    pos = centres[which] + rng.normal(0.0, sigma, size=(n, 2))
    pos[:, 0] = np.clip(pos[:, 0], 0.0, width)
    pos[:, 1] = np.clip(pos[:, 1], 0.0, height)
    return (width, height), pos.astype(np.float32), _vel(rng, n, vel_sigma)


def batch(nworlds=256, side=(128.0, 1024.0), count=(1024, 65536), vel_sigma=2.0, seed=0):
    """Returns (dims (nworlds, 2), [pos_w], [vel_w])."""
    rng = np.random.default_rng(seed)
    dims = rng.uniform(side[0], side[1], size=(nworlds, 2)).astype(np.float32)
    dims = np.floor(dims)
    counts = np.exp(rng.uniform(np.log(count[0]), np.log(count[1]), nworlds)).astype(np.int64)
    poss, vels = [], []
    for w in range(nworlds):
        n = int(counts[w])
        poss.append(rng.uniform((0.0, 0.0), dims[w], size=(n, 2)).astype(np.float32))
        vels.append(_vel(rng, n, vel_sigma))
    return dims.astype(np.float32), poss, vels

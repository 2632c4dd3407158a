"""Python host side of the wrach GB300 library.

Two layers over the C ABI (include/wrach.h):

* `Simulation`: numpy arrays in and out, batched worlds, device uploads.
* `WrachAPI`: the reference's public surface, name for name
  (runners/api/src/lib.rs:17-88): `WrachAPI(config)`, `tick()`,
  `read_data()`, `add_particles(particles)`, `get_simulation_state()`, and the
  `positions` / `velocities` lists of (x, y) tuples, capacity long, in cell
  order, zero-padded (runners/api/src/lib.rs:58-74).

Every call goes to the CUDA library; nothing here computes physics.
"""
import ctypes
from dataclasses import dataclass, field
from typing import List, NamedTuple, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import MODE_EXTENDED, MODE_REFERENCE


class Vec2(NamedTuple):
    x: float
    y: float


@dataclass
class Particle:
    """runners/bevy/src/state.rs:41-46."""
    position: Vec2
    velocity: Vec2


@dataclass
class WrachConfig:
    """runners/bevy/src/config_app.rs:10-36, plus the physics constants the
    reference hard-codes and the extended-mode knobs."""
    dimensions: Tuple[float, float] = (480, 352)
    boundaries_as_dimensions: bool = False  # kept for parity; unused by the physics, as in the reference
    cell_size: int = 3
    mode: int = MODE_REFERENCE
    iterations: int = 4
    gravity: float = 0.0
    min_distance: float = 1.0
    max_velocity: float = 1.0
    cell_capacity: int = 9
    capacity: int = 0
    anchor: Tuple[float, float] = (0.0, 0.0)
    device: int = 0
    rebin_blocks: int = 0
    solve_block: int = 0
    solve_per_thread: int = 0

    def to_c(self):
        c = _lib.Config()
        _lib.load().wrach_config_default(ctypes.byref(c))
        c.width, c.height = float(self.dimensions[0]), float(self.dimensions[1])
        c.anchor_x, c.anchor_y = float(self.anchor[0]), float(self.anchor[1])
        c.cell_size = int(self.cell_size)
        c.mode = int(self.mode)
        c.iterations = int(self.iterations)
        c.gravity = float(self.gravity)
        c.min_distance = float(self.min_distance)
        c.max_velocity = float(self.max_velocity)
        c.cell_capacity = int(self.cell_capacity)
        c.capacity = int(self.capacity)
        c.device = int(self.device)
        c.rebin_blocks = int(self.rebin_blocks)
        c.solve_block = int(self.solve_block)
        c.solve_per_thread = int(self.solve_per_thread)
        return c


def _f32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _u32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


class Simulation:
    """One context: a single world, or `worlds` independent worlds
    (a list of (width, height)) sharing the config's other settings."""

    def __init__(self, config: Optional[WrachConfig] = None,
                 worlds: Optional[Sequence[Tuple[float, float]]] = None):
        self.config = config or WrachConfig()
        self._L = _lib.load()
        self._ctx = ctypes.c_void_p()
        c = self.config.to_c()
        if worlds is None:
            rc = self._L.wrach_create(ctypes.byref(c), ctypes.byref(self._ctx))
        else:
            dims = np.ascontiguousarray(np.asarray(worlds, np.float32).reshape(-1, 2))
            rc = self._L.wrach_create_batch(ctypes.byref(c), dims.shape[0], _f32p(dims),
                                            ctypes.byref(self._ctx))
        if rc != _lib.WRACH_OK:
            raise _lib.WrachError(rc, "create failed")
        self.num_worlds = int(self._L.wrach_num_worlds(self._ctx))

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if self._ctx:
            self._L.wrach_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._ctx

    def _check(self, rc):
        _lib.check(rc, self._ctx)

    # -- data ---------------------------------------------------------------
    def add_particles(self, positions, velocities, world=0):
        pos = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 2))
        vel = np.ascontiguousarray(np.asarray(velocities, np.float32).reshape(-1, 2))
        if pos.shape != vel.shape:
            raise ValueError("positions and velocities differ in shape")
        self._check(self._L.wrach_add_particles(self._ctx, world, _f32p(pos), _f32p(vel),
                                                pos.shape[0]))

    def set_particles(self, positions, velocities, world=0):
        """Replace the world's particles and re-pack the frame from them."""
        pos = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 2))
        vel = np.ascontiguousarray(np.asarray(velocities, np.float32).reshape(-1, 2))
        if pos.shape != vel.shape:
            raise ValueError("positions and velocities differ in shape")
        self._check(self._L.wrach_set_particles(self._ctx, world, _f32p(pos), _f32p(vel),
                                                pos.shape[0]))

    def profile_frame(self):
        """One eager frame; the duration (ms) of each of its kernel launches."""
        buf = (ctypes.c_float * 128)()
        cnt = ctypes.c_uint32(0)
        self._check(self._L.wrach_profile_frame(self._ctx, buf, 128, ctypes.byref(cnt)))
        return [float(buf[i]) for i in range(cnt.value)]

    def add_particles_device(self, d_pos, d_vel, n, world=0):
        """Upload from device pointers (ints) of n float pairs each."""
        self._check(self._L.wrach_add_particles_device(self._ctx, world, ctypes.c_void_p(d_pos),
                                                       ctypes.c_void_p(d_vel), int(n)))

    def step(self, nsteps=1):
        self._check(self._L.wrach_step(self._ctx, int(nsteps)))

    def capacity(self, world=0):
        return int(self._L.wrach_capacity(self._ctx, world))

    def settings(self, world=0):
        s = _lib.WorldSettings()
        self._check(self._L.wrach_get_settings(self._ctx, world, ctypes.byref(s)))
        return s

    def cells(self, world=0):
        s = self.settings(world)
        return int(s.grid_dimensions[0]) * int(s.grid_dimensions[1])

    def read(self, world=0, out=None):
        """(positions, velocities, indices) of a world: capacity x 2 float32
        arrays and the cells + 2 table.  The library writes the frame's
        particles only: arrays allocated here are zero past them, `out`
        arrays keep what they held there."""
        cap = self.capacity(world)
        if out is None:
            pos = np.zeros((cap, 2), np.float32)
            vel = np.zeros((cap, 2), np.float32)
            idx = np.empty(self.cells(world) + 2, np.uint32)
        else:
            pos, vel, idx = out
        self._check(self._L.wrach_read(self._ctx, world, _f32p(pos), _f32p(vel), _u32p(idx), cap))
        return pos, vel, idx

    def read_frame(self, world=0):
        """(positions, velocities, indices) trimmed to the frame's particles."""
        pos, vel, idx = self.read(world)
        n = int(idx[-1])
        return pos[:n], vel[:n], idx

    def read_keys(self, world=0):
        """The cell key (cy * gx + cx) of each frame particle, in frame order."""
        n = int(self.settings(world).particles_in_frame_count)
        keys = np.zeros(max(n, 1), np.uint32)
        self._check(self._L.wrach_read_keys(self._ctx, world, _u32p(keys), max(n, 1)))
        return keys[:n]

    def render(self, width_px, height_px, world=0):
        """The frame drawn as the reference's draw pass does: an 8-bit image
        (height_px, width_px), row 0 at the top."""
        img = np.empty((int(height_px), int(width_px)), np.uint8)
        self._check(self._L.wrach_render(self._ctx, world, int(width_px), int(height_px),
                                         img.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return img

    def sync(self):
        self._check(self._L.wrach_sync(self._ctx))

    def flags(self):
        f = ctypes.c_uint32(0)
        self._check(self._L.wrach_flags(self._ctx, ctypes.byref(f)))
        return int(f.value)

    def stats(self):
        st = _lib.Stats()
        self._check(self._L.wrach_stats(self._ctx, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _lib.Stats._fields_ if f != "reserved"}

    def frame_metrics(self):
        """(mean penetration, max penetration, kinetic energy) of the frame."""
        a, b, c = ctypes.c_float(0), ctypes.c_float(0), ctypes.c_float(0)
        self._check(self._L.wrach_frame_metrics(self._ctx, ctypes.byref(a), ctypes.byref(b),
                                                ctypes.byref(c)))
        return float(a.value), float(b.value), float(c.value)

    # -- the learned surrogate ------------------------------------------------
    def surrogate_init(self, seed=0, max_samples=1 << 20):
        self._check(self._L.wrach_surrogate_init(self._ctx, int(seed), int(max_samples)))

    def surrogate_params(self):
        n = int(self._L.wrach_surrogate_param_count())
        out = np.empty(n, np.float32)
        self._check(self._L.wrach_surrogate_get_params(self._ctx, _f32p(out), n))
        return out

    def surrogate_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        self._check(self._L.wrach_surrogate_set_params(self._ctx, _f32p(p), p.size))

    def surrogate_features(self, d_x, rows):
        self._check(self._L.wrach_surrogate_features(self._ctx, ctypes.c_void_p(d_x), int(rows)))

    def surrogate_forward(self, d_x, n, d_y, kernel="tcgen05"):
        """Network outputs of n device feature rows into d_y; kernel
        "tcgen05" (tensor memory accumulators) or "mma" (warp-level mma.sync)."""
        fn = (self._L.wrach_surrogate_forward if kernel == "tcgen05"
              else self._L.wrach_surrogate_forward_mma)
        self._check(fn(self._ctx, ctypes.c_void_p(d_x), int(n), ctypes.c_void_p(d_y)))

    def surrogate_gradients(self, d_x, d_t, n):
        g = np.empty(int(self._L.wrach_surrogate_param_count()), np.float32)
        loss = ctypes.c_float(0)
        self._check(self._L.wrach_surrogate_gradients(self._ctx, ctypes.c_void_p(d_x),
                                                      ctypes.c_void_p(d_t), int(n), _f32p(g),
                                                      ctypes.byref(loss)))
        return g, float(loss.value)

    def surrogate_collect(self, stride=1):
        """Training rows from every stride-th taking-part particle of the
        current frame; returns the rows collected so far."""
        total = ctypes.c_uint32(0)
        self._check(self._L.wrach_surrogate_collect(self._ctx, int(stride), ctypes.byref(total)))
        return int(total.value)

    def surrogate_evaluate(self):
        """(mse of the network's correction, mse of a zero correction) on the
        current frame against the plain solver's first-iterations correction."""
        a, b = ctypes.c_float(0), ctypes.c_float(0)
        self._check(self._L.wrach_surrogate_evaluate(self._ctx, ctypes.byref(a), ctypes.byref(b)))
        return float(a.value), float(b.value)

    def surrogate_train(self, steps, batch=4096, lr=1e-3):
        loss = ctypes.c_float(0)
        self._check(self._L.wrach_surrogate_train(self._ctx, int(steps), int(batch), float(lr),
                                                  ctypes.byref(loss)))
        return float(loss.value)

    def selftest_wait(self, limit_us):
        """(timed out, microseconds waited) of a bounded device wait on a word
        that nothing sets."""
        t, us = ctypes.c_uint32(0), ctypes.c_uint32(0)
        self._check(self._L.wrach_selftest_wait(self._ctx, int(limit_us), ctypes.byref(t),
                                                ctypes.byref(us)))
        return bool(t.value), int(us.value)

    # -- viewport streaming -------------------------------------------------
    def write_back(self, world=0):
        """Write the world's frame back into its store."""
        self._check(self._L.wrach_write_back(self._ctx, world))

    def set_viewport(self, anchor, world=0):
        """Move the world's viewport to `anchor` (x, y), same size."""
        self._check(self._L.wrach_set_viewport(self._ctx, world, float(anchor[0]), float(anchor[1])))

    def store(self, world=0):
        """(positions, velocities) of the world's store, (m, 2) float32 each."""
        cnt = ctypes.c_uint32(0)
        self._check(self._L.wrach_store_size(self._ctx, world, ctypes.byref(cnt)))
        m = int(cnt.value)
        pos = np.zeros((max(m, 1), 2), np.float32)
        vel = np.zeros((max(m, 1), 2), np.float32)
        self._check(self._L.wrach_read_store(self._ctx, world, _f32p(pos), _f32p(vel), max(m, 1)))
        return pos[:m], vel[:m]

    def surrogate_correction(self, d_corr):
        """The fused kernel's correction of the current frame into the device
        buffer `d_corr` ((n, 2) float32)."""
        self._check(self._L.wrach_surrogate_correction(self._ctx, ctypes.c_void_p(int(d_corr))))

    def surrogate_step(self, nsteps=1, max_penetration=0.2, max_energy_drift=0.01):
        st = _lib.SurrogateStats()
        self._check(self._L.wrach_surrogate_step(self._ctx, int(nsteps), float(max_penetration),
                                                 float(max_energy_drift), ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _lib.SurrogateStats._fields_ if f != "reserved"}

    @property
    def kernel_launches(self):
        return int(self._L.wrach_kernel_launches(self._ctx))

    @property
    def stream(self):
        return int(self._L.wrach_stream(self._ctx) or 0)


@dataclass
class PackedData:
    """runners/bevy/src/spatial_bin.rs:20-33."""
    indices: List[int] = field(default_factory=list)
    positions: List[Vec2] = field(default_factory=list)
    velocities: List[Vec2] = field(default_factory=list)


@dataclass
class WrachState:
    """The parts of runners/bevy/src/state.rs:17-33 a caller reads."""
    config: WrachConfig
    shader_settings: _lib.WorldSettings
    packed_data: PackedData


class WrachAPI:
    """runners/api/src/lib.rs:17-88 over the CUDA library."""

    def __init__(self, config: Optional[WrachConfig] = None):
        self.config = config or WrachConfig()
        self.sim = Simulation(self.config)
        self.positions: List[Tuple[float, float]] = []
        self.velocities: List[Tuple[float, float]] = []
        self._packed = PackedData()

    @classmethod
    def new(cls, config: Optional[WrachConfig] = None):
        return cls(config)

    def tick(self):
        """One frame then the readback (runners/api/src/lib.rs:49-52)."""
        self.sim.step(1)
        self.read_data()

    def read_data(self):
        pos, vel, idx = self.sim.read()
        self._packed = PackedData(indices=idx.tolist(),
                                  positions=[Vec2(*p) for p in pos.tolist()],
                                  velocities=[Vec2(*v) for v in vel.tolist()])
        self.positions = [tuple(p) for p in pos.tolist()]
        self.velocities = [tuple(v) for v in vel.tolist()]

    def add_particles(self, particles: Sequence[Particle]):
        pos = np.array([[p.position[0], p.position[1]] for p in particles], np.float32).reshape(-1, 2)
        vel = np.array([[p.velocity[0], p.velocity[1]] for p in particles], np.float32).reshape(-1, 2)
        self.sim.add_particles(pos, vel)

    def get_simulation_state(self) -> WrachState:
        return WrachState(config=self.config, shader_settings=self.sim.settings(),
                          packed_data=self._packed)

    def close(self):
        self.sim.close()

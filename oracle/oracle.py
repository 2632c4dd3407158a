"""ctypes wrapper over the C oracle (oracle/wrach_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker that the CUDA library is compared with.
Only tests/, the smoke check and bench.py's CPU-baseline leg import it.
Arrays are numpy: positions and velocities are (n, 2) float32, tables are the
reference's C+2 u32 `indices` layout.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_u32 = ctypes.c_uint32
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i32p = ctypes.POINTER(ctypes.c_int32)


class World(ctypes.Structure):
    """The reference's 32-byte uniform (runners/bevy/src/config_shader.rs:15-29)."""
    _fields_ = [("view_dimensions", ctypes.c_float * 2),
                ("view_anchor", ctypes.c_float * 2),
                ("grid_dimensions", ctypes.c_uint32 * 2),
                ("cell_size", ctypes.c_uint32),
                ("particles_in_frame_count", ctypes.c_uint32)]

    @property
    def cells(self):
        return int(self.grid_dimensions[0]) * int(self.grid_dimensions[1])


class Physics(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_uint32),
                ("iterations", ctypes.c_uint32),
                ("gravity", ctypes.c_float),
                ("min_distance", ctypes.c_float),
                ("max_velocity", ctypes.c_float),
                ("cell_capacity", ctypes.c_uint32)]


def reference_physics():
    """Mode 0: the reference's physics constants (shaders/physics/src)."""
    return Physics(0, 1, 0.0, 1.0, 1.0, 9)


def extended_physics(iterations=4, gravity=0.1):
    """Mode 1: 3x3-cell Jacobi iterations with gravity."""
    return Physics(1, iterations, gravity, 1.0, 1.0, 9)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.wo_cell_coord.argtypes = [ctypes.c_float, _u32]
        L.wo_cell_coord.restype = ctypes.c_int32
        L.wo_world_init.argtypes = [ctypes.POINTER(World), ctypes.c_float, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_float, _u32]
        L.wo_active_cells.argtypes = [ctypes.POINTER(World), _i32p]
        L.wo_active_cells.restype = _u32
        L.wo_max_particles_per_frame.argtypes = [ctypes.POINTER(World)]
        L.wo_max_particles_per_frame.restype = _u32
        L.wo_pack.argtypes = [ctypes.POINTER(World), _u32, _f32p, _f32p, _u32, _u32p, _f32p, _f32p]
        L.wo_pack.restype = ctypes.c_int64
        L.wo_frame_key.argtypes = [ctypes.POINTER(World), ctypes.c_float, ctypes.c_float, _u32p]
        L.wo_frame_key.restype = _u32
        L.wo_solve.argtypes = [ctypes.POINTER(World), ctypes.POINTER(Physics), _u32p,
                               _f32p, _f32p, _f32p, _f32p]
        L.wo_solve_f64.argtypes = [ctypes.POINTER(World), ctypes.POINTER(Physics), _u32p,
                                   _f64p, _f64p, _f64p, _f64p]
        L.wo_rebin.argtypes = [ctypes.POINTER(World), _u32, _f32p, _f32p, _u32p, _u32p, _f32p, _f32p]
        L.wo_rebin.restype = _u32
        L.wo_step.argtypes = [ctypes.POINTER(World), ctypes.POINTER(Physics), _u32, _u32p, _f32p, _f32p]
        L.wo_step.restype = _u32
        L.wo_num_threads.restype = ctypes.c_int
        L.wo_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def world(width, height, cell_size=3, anchor=(0.0, 0.0)):
    w = World()
    lib().wo_world_init(ctypes.byref(w), float(width), float(height),
                        float(anchor[0]), float(anchor[1]), int(cell_size))
    return w


def cell_coord(x, cell_size):
    return int(lib().wo_cell_coord(float(x), int(cell_size)))


def active_cells(w):
    n = lib().wo_active_cells(ctypes.byref(w), None)
    out = np.zeros((n, 2), np.int32)
    lib().wo_active_cells(ctypes.byref(w), _p(out, _i32p))
    return out


def max_particles_per_frame(w):
    return int(lib().wo_max_particles_per_frame(ctypes.byref(w)))


def pack(w, pos, vel, capacity=None):
    """create_packed_data: returns (table, pos, vel) of the packed frame."""
    pos, vel = _f32(pos).reshape(-1, 2), _f32(vel).reshape(-1, 2)
    n = pos.shape[0]
    if capacity is None:
        capacity = max(n, 1)
    table = np.zeros(w.cells + 2, np.uint32)
    op = np.zeros((max(n, 1), 2), np.float32)
    ov = np.zeros((max(n, 1), 2), np.float32)
    cnt = lib().wo_pack(ctypes.byref(w), n, _p(pos, _f32p), _p(vel, _f32p), int(capacity),
                        _p(table, _u32p), _p(op, _f32p), _p(ov, _f32p))
    if cnt < 0:
        raise ValueError("more particles than the frame capacity")
    return table, op[:cnt].copy(), ov[:cnt].copy()


def frame_key(w, x, y):
    flags = ctypes.c_uint32(0)
    k = lib().wo_frame_key(ctypes.byref(w), float(x), float(y), ctypes.byref(flags))
    return int(k), int(flags.value)


def solve(w, ph, table, pos, vel):
    """The solve half of a frame: outputs in the input (binned) order."""
    table = np.ascontiguousarray(table, np.uint32)
    pos, vel = _f32(pos).reshape(-1, 2), _f32(vel).reshape(-1, 2)
    po, vo = np.empty_like(pos), np.empty_like(vel)
    lib().wo_solve(ctypes.byref(w), ctypes.byref(ph), _p(table, _u32p), _p(pos, _f32p),
                   _p(vel, _f32p), _p(po, _f32p), _p(vo, _f32p))
    return po, vo


def solve_f64(w, ph, table, pos, vel):
    table = np.ascontiguousarray(table, np.uint32)
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 2)
    vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 2)
    po, vo = np.empty_like(pos), np.empty_like(vel)
    lib().wo_solve_f64(ctypes.byref(w), ctypes.byref(ph), _p(table, _u32p), _p(pos, _f64p),
                       _p(vel, _f64p), _p(po, _f64p), _p(vo, _f64p))
    return po, vo


def rebin(w, pos_out, vel_out):
    """Count + scan + stable pack: returns (keys, table, pos, vel, flags)."""
    pos_out, vel_out = _f32(pos_out).reshape(-1, 2), _f32(vel_out).reshape(-1, 2)
    n = pos_out.shape[0]
    keys = np.zeros(max(n, 1), np.uint32)
    table = np.zeros(w.cells + 2, np.uint32)
    pi, vi = np.empty_like(pos_out), np.empty_like(vel_out)
    flags = lib().wo_rebin(ctypes.byref(w), n, _p(pos_out, _f32p), _p(vel_out, _f32p),
                           _p(keys, _u32p), _p(table, _u32p), _p(pi, _f32p), _p(vi, _f32p))
    return keys[:n], table, pi, vi, int(flags)


def step(w, ph, table, pos, vel, nsteps=1):
    """`nsteps` frames from a binned state; returns (table, pos, vel, flags)."""
    table = np.array(table, np.uint32, copy=True)
    pos = np.array(pos, np.float32, copy=True).reshape(-1, 2)
    vel = np.array(vel, np.float32, copy=True).reshape(-1, 2)
    flags = lib().wo_step(ctypes.byref(w), ctypes.byref(ph), int(nsteps), _p(table, _u32p),
                          _p(pos, _f32p), _p(vel, _f32p))
    return table, pos, vel, int(flags)


def num_threads():
    return int(lib().wo_num_threads())


def set_num_threads(n):
    lib().wo_set_num_threads(int(n))


# -- viewport streaming (no reference implementation: the write-back is a TODO
#    in runners/bevy/src/particle_store.rs:71-85; these are the rules the CUDA
#    path states, restated here for its tests) --------------------------------

def inside_viewport(w, pos):
    """Mask of the particles whose cell (div_euclid, as create_packed_data:
    spatial_bin.rs:48-64, 103-149) lies in the viewport's grid."""
    pos = _f32(pos).reshape(-1, 2)
    cs = int(w.cell_size)
    blx, bly = cell_coord(w.view_anchor[0], cs), cell_coord(w.view_anchor[1], cs)
    gx, gy = int(w.grid_dimensions[0]), int(w.grid_dimensions[1])
    out = np.zeros(len(pos), bool)
    for k, (x, y) in enumerate(pos):
        cx, cy = cell_coord(float(x), cs) - blx, cell_coord(float(y), cs) - bly
        out[k] = 0 <= cx < gx and 0 <= cy < gy
    return out


def write_back(w, store_pos, store_vel, frame_pos, frame_vel):
    """The store after writing the frame back: its particles outside the
    viewport (store order), then the frame's particles (frame order)."""
    keep = ~inside_viewport(w, store_pos)
    return (np.concatenate([_f32(store_pos).reshape(-1, 2)[keep], _f32(frame_pos).reshape(-1, 2)]),
            np.concatenate([_f32(store_vel).reshape(-1, 2)[keep], _f32(frame_vel).reshape(-1, 2)]))


"""ctypes binding of the C ABI declared in include/wrach.h.

Loads wrach_gb300/_build/libwrach_gb300.so and fails loudly when it is
missing: there is no CPU fallback on the product path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwrach_gb300.so")

WRACH_OK = 0
WRACH_ERR_INVALID_ARGUMENT = 1
WRACH_ERR_CAPACITY = 2
WRACH_ERR_CUDA = 3
WRACH_ERR_OUT_OF_MEMORY = 4
WRACH_ERR_DEVICE = 5
WRACH_ERR_UNSUPPORTED = 6

MODE_REFERENCE = 0
MODE_EXTENDED = 1

FLAG_OUT_OF_GRID = 1
FLAG_NAN = 2
FLAG_TIMEOUT = 4
FLAG_OVERFLOW = 8

ERROR_NAMES = {
    1: "invalid argument", 2: "capacity exceeded", 3: "CUDA error",
    4: "out of device memory", 5: "device check failed", 6: "unsupported",
}


class WrachError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "error"), code, message))
        self.code = code


class CapacityError(WrachError):
    pass


class WorldSettings(ctypes.Structure):
    """The reference's 32-byte uniform (runners/bevy/src/config_shader.rs:15-29)."""
    _fields_ = [("view_dimensions", ctypes.c_float * 2),
                ("view_anchor", ctypes.c_float * 2),
                ("grid_dimensions", ctypes.c_uint32 * 2),
                ("cell_size", ctypes.c_uint32),
                ("particles_in_frame_count", ctypes.c_uint32)]


class Config(ctypes.Structure):
    _fields_ = [("width", ctypes.c_float),
                ("height", ctypes.c_float),
                ("anchor_x", ctypes.c_float),
                ("anchor_y", ctypes.c_float),
                ("cell_size", ctypes.c_uint32),
                ("mode", ctypes.c_uint32),
                ("iterations", ctypes.c_uint32),
                ("gravity", ctypes.c_float),
                ("min_distance", ctypes.c_float),
                ("max_velocity", ctypes.c_float),
                ("cell_capacity", ctypes.c_uint32),
                ("capacity", ctypes.c_uint32),
                ("device", ctypes.c_int32),
                ("rebin_blocks", ctypes.c_uint32),
                ("solve_block", ctypes.c_uint32),
                ("solve_per_thread", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32 * 4)]


class Stats(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("frames", ctypes.c_uint32),
                ("overflow", ctypes.c_uint32), ("rebin_blocks", ctypes.c_uint32),
                ("tiles", ctypes.c_uint32), ("particles", ctypes.c_uint32),
                ("cells", ctypes.c_uint32), ("huge_cells", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32 * 8)]


class SurrogateStats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_uint32), ("fallbacks", ctypes.c_uint32),
                ("mean_penetration", ctypes.c_float), ("max_penetration", ctypes.c_float),
                ("max_energy_drift", ctypes.c_float), ("calibrations", ctypes.c_uint32),
                ("reference_penetration", ctypes.c_float), ("reserved", ctypes.c_uint32 * 9)]


# name -> (restype, argtypes); every symbol include/wrach.h declares
_P = ctypes.c_void_p
_F = ctypes.POINTER(ctypes.c_float)
_U = ctypes.POINTER(ctypes.c_uint32)
SIGNATURES = {
    "wrach_config_default": (ctypes.c_int, [ctypes.POINTER(Config)]),
    "wrach_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "wrach_create_batch": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_uint32, _F,
                                          ctypes.POINTER(_P)]),
    "wrach_destroy": (ctypes.c_int, [_P]),
    "wrach_add_particles": (ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, ctypes.c_uint32]),
    "wrach_set_particles": (ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, ctypes.c_uint32]),
    "wrach_profile_frame": (ctypes.c_int, [_P, _F, ctypes.c_uint32, _U]),
    "wrach_add_particles_device": (ctypes.c_int, [_P, ctypes.c_uint32, _P, _P, ctypes.c_uint32]),
    "wrach_pack_noalloc": (ctypes.c_int, [ctypes.POINTER(Config), _P, _P, ctypes.c_uint32, _P, _P,
                                          ctypes.c_uint32, _P, _P, _P]),
    "wrach_step": (ctypes.c_int, [_P, ctypes.c_uint32]),
    "wrach_read": (ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, _U, ctypes.c_uint32]),
    "wrach_tick": (ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, _U, ctypes.c_uint32]),
    "wrach_render": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.POINTER(ctypes.c_uint8)]),
    "wrach_get_settings": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.POINTER(WorldSettings)]),
    "wrach_max_particles_per_frame": (ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32]),
    "wrach_capacity": (ctypes.c_uint32, [_P, ctypes.c_uint32]),
    "wrach_num_worlds": (ctypes.c_uint32, [_P]),
    "wrach_sync": (ctypes.c_int, [_P]),
    "wrach_flags": (ctypes.c_int, [_P, _U]),
    "wrach_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "wrach_last_error": (ctypes.c_char_p, [_P]),
    "wrach_kernel_launches": (ctypes.c_uint64, [_P]),
    "wrach_stream": (ctypes.c_void_p, [_P]),
    "wrach_surrogate_param_count": (ctypes.c_uint32, []),
    "wrach_surrogate_init": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32]),
    "wrach_surrogate_get_params": (ctypes.c_int, [_P, _F, ctypes.c_uint32]),
    "wrach_surrogate_set_params": (ctypes.c_int, [_P, _F, ctypes.c_uint32]),
    "wrach_surrogate_features": (ctypes.c_int, [_P, _P, ctypes.c_uint32]),
    "wrach_surrogate_forward": (ctypes.c_int, [_P, _P, ctypes.c_uint32, _P]),
    "wrach_surrogate_forward_mma": (ctypes.c_int, [_P, _P, ctypes.c_uint32, _P]),
    "wrach_surrogate_gradients": (ctypes.c_int, [_P, _P, _P, ctypes.c_uint32, _F, _F]),
    "wrach_surrogate_collect": (ctypes.c_int, [_P, ctypes.c_uint32, _U]),
    "wrach_surrogate_evaluate": (ctypes.c_int, [_P, _F, _F]),
    "wrach_frame_metrics": (ctypes.c_int, [_P, _F, _F, _F]),
    "wrach_surrogate_correction": (ctypes.c_int, [_P, _P]),
    "wrach_write_back": (ctypes.c_int, [_P, ctypes.c_uint32]),
    "wrach_read_keys": (ctypes.c_int, [_P, ctypes.c_uint32, _U, ctypes.c_uint32]),
    "wrach_selftest_wait": (ctypes.c_int, [_P, ctypes.c_uint32, _U, _U]),
    "wrach_set_viewport": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_float, ctypes.c_float]),
    "wrach_store_size": (ctypes.c_int, [_P, ctypes.c_uint32, _U]),
    "wrach_read_store": (ctypes.c_int, [_P, ctypes.c_uint32, _F, _F, ctypes.c_uint32]),
    "wrach_surrogate_train": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _F]),
    "wrach_surrogate_step": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                            ctypes.POINTER(SurrogateStats)]),
}

_lib = None


def load():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "wrach_gb300: the CUDA library %s is missing; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` "
            "(there is no CPU fallback)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, ctx=None):
    if rc == WRACH_OK:
        return
    msg = ""
    if ctx:
        raw = load().wrach_last_error(ctx)
        msg = raw.decode() if raw else ""
    cls = CapacityError if rc == WRACH_ERR_CAPACITY else WrachError
    raise cls(rc, msg)

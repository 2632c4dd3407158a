"""wrach_gb300: wrach's per-frame particle physics step as hand-written CUDA
for GB300 (sm_103a) behind a C ABI (include/wrach.h).

`build()` compiles the library in-tree; `Simulation` and `WrachAPI` drive it.
"""
from ._lib import (FLAG_NAN, FLAG_OUT_OF_GRID, FLAG_TIMEOUT,
                   MODE_EXTENDED, MODE_REFERENCE, CapacityError, WrachError)
from .api import (PackedData, Particle, Simulation, Vec2, WrachAPI, WrachConfig,
                  WrachState)
from .build import build

__all__ = [
    "build", "Simulation", "WrachAPI", "WrachConfig", "WrachState", "PackedData",
    "Particle", "Vec2", "WrachError", "CapacityError", "MODE_REFERENCE", "MODE_EXTENDED",
    "FLAG_OUT_OF_GRID", "FLAG_NAN", "FLAG_TIMEOUT",
]

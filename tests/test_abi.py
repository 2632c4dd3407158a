"""The C ABI library builds, loads and exports every symbol include/wrach.h
declares.  No compute calls: these run without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(wrach_[a-z0-9_]+)\s*\(", text))
    return names


def test_header_declares_the_boundary():
    names = declared_symbols()
    for must in ("wrach_create", "wrach_add_particles", "wrach_step", "wrach_read",
                 "wrach_destroy", "wrach_last_error", "wrach_sync"):
        assert must in names


def test_library_exports_every_declared_symbol(W):
    lib = ctypes.CDLL(W._lib.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_declared_symbol(W):
    assert declared_symbols() <= set(W._lib.SIGNATURES)


def test_struct_layouts(W):
    assert ctypes.sizeof(W._lib.WorldSettings) == 32
    assert ctypes.sizeof(W._lib.Config) == 80


def test_config_default_matches_reference(W):
    c = W._lib.Config()
    assert W._lib.load().wrach_config_default(ctypes.byref(c)) == 0
    # runners/bevy/src/config_app.rs:23-36 and the shader constants
    assert (c.width, c.height, c.cell_size) == (480.0, 352.0, 3)
    assert (c.min_distance, c.max_velocity, c.cell_capacity) == (1.0, 1.0, 9)


def test_max_particles_per_frame(W):
    L = W._lib.load()
    assert L.wrach_max_particles_per_frame(16, 2) == 74    # 6x6 at cs 2: particle_store.rs:231-234
    assert L.wrach_max_particles_per_frame(16, 3) == 164   # api/src/lib.rs:101-126


def test_null_arguments_are_rejected(W):
    L = W._lib.load()
    assert L.wrach_create(None, None) == W._lib.WRACH_ERR_INVALID_ARGUMENT
    assert L.wrach_step(None, 1) == W._lib.WRACH_ERR_INVALID_ARGUMENT
    assert L.wrach_destroy(None) == W._lib.WRACH_ERR_INVALID_ARGUMENT


def test_missing_library_fails_loudly(W, monkeypatch):
    monkeypatch.setattr(W._lib, "_lib", None)
    monkeypatch.setattr(W._lib, "LIB_PATH", "/nonexistent/libwrach_gb300.so")
    with pytest.raises(ImportError):
        W._lib.load()


def test_grid_width_division_constants():
    # cell (x, y) = (c - y * gx, (c * m) >> s) with m = floor(2^(31+l)/gx) + 1,
    # s = 31 + l, l = ceil(log2 gx): exact for every c < 2^31 (the kernels'
    # cell indices stay below 2^31)
    import random
    rng = random.Random(0)
    for gx in list(range(1, 3000)) + [1921, 4097, 65535, 65536, 1 << 20, 99991]:
        l = 0
        while (1 << l) < gx:
            l += 1
        m, s = (1 << (31 + l)) // gx + 1, 31 + l
        assert m < 2 ** 32
        for x in [0, 1, gx - 1, gx, gx + 1, 2 ** 31 - 1] + [rng.randrange(2 ** 31) for _ in range(50)]:
            assert (x * m) >> s == x // gx


def test_rust_binding_mirrors_the_header():
    # bindings/rust/src/lib.rs declares the same config fields in the same
    # order as the header's WrachConfig (ctypes mirror), and only functions
    # the header declares
    import wrach_gb300._lib as L
    src = open(os.path.join(ROOT, "bindings", "rust", "src", "lib.rs")).read()
    block = src[src.index("pub struct WrachConfigC {"):]
    block = block[:block.index("}")]
    rust_fields = re.findall(r"pub (\w+):", block)
    assert rust_fields == [f for f, _ in L.Config._fields_]
    externs = set(re.findall(r"fn (wrach_\w+)\(", src))
    assert externs and externs <= declared_symbols()

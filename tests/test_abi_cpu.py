"""The C-ABI library loads and exports every entry point include/ffnoml_gb300.h declares (no GPU work)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ffnoml_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(ffno_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from ffnoml_gb300 import _native, build
    if not os.path.exists(_native.LIB_PATH):
        build.build()
    return ctypes.CDLL(_native.LIB_PATH)


def test_header_declares_entry_points():
    names = declared()
    assert len(names) >= 29
    assert "ffno_xform" in names and "ffno_gn_bwd_apply" in names and "ffno_head_fwd" in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    from ffnoml_gb300 import _native
    assert set(declared()) <= set(_native.exported_symbols())


def test_version(lib):
    lib.ffno_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.ffno_version()


def _has_pointer(argtypes):
    return any(a is ctypes.c_void_p or hasattr(a, "_type_") and issubclass(a, ctypes._Pointer) for a in argtypes)


def test_null_pointers_are_refused_before_any_device_work(lib):
    """Every entry point with pointer arguments returns FFNO_EINVAL (1) for null pointers, before any CUDA call, so
    this runs without a GPU; the optional pointers (base, zp, hg, head_out, ...) are never the only ones given."""
    from ffnoml_gb300 import _native
    filler = {ctypes.c_int: 64, ctypes.c_long: 4096, ctypes.c_float: 1.0, ctypes.c_double: 1.0}
    checked = 0
    for name, argtypes in _native.PROTOTYPES.items():
        if not _has_pointer(argtypes):
            continue
        fn = getattr(lib, name)
        fn.argtypes, fn.restype = argtypes, ctypes.c_int
        args = [None if a not in filler else filler[a] for a in argtypes]
        assert fn(*args) == 1, name
        checked += 1
    assert checked >= 55


def test_invalid_sizes_are_refused_before_any_device_work(lib):
    lib.ffno_tc_set_prefetch_tiles.argtypes = [ctypes.c_int]
    assert lib.ffno_tc_set_prefetch_tiles(-1) == 1 and lib.ffno_tc_set_prefetch_tiles(5) == 1
    lib.ffno_copy2d.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p, ctypes.c_long, ctypes.c_long,
                                ctypes.c_long, ctypes.c_void_p]
    buf = ctypes.create_string_buffer(64)
    assert lib.ffno_copy2d(buf, 8, buf, 16, 16, 2, None) == 1      # destination pitch below the row width
    assert lib.ffno_copy2d(buf, 16, buf, 16, 16, 0, None) == 0     # nothing to copy: no CUDA call

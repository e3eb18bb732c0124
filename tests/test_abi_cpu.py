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

"""The C-ABI library builds, loads and exports every declared entry point
(no GPU needed: nothing here calls into the device)."""
import ctypes as C

from clear_gb300 import _lib
from clear_gb300.build import build


def test_library_exports_declared_symbols():
    build()
    L = _lib.load()
    names = _lib.declared_symbols()
    assert "clr_lbvh_build" in names and "clr_trace_closest" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_error_string_without_gpu():
    build()
    L = _lib.load()
    L.clr_last_error_string.restype = C.c_char_p
    assert isinstance(L.clr_last_error_string(), bytes)

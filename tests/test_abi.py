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


def test_sort_workspace_size_without_gpu():
    """The sorted-order ray queries' scratch size: at least the sort's 16 bytes
    per ray, growing with the ray count; NULL output is an argument error."""
    build()
    L = _lib.load()
    sizes = []
    for n in (0, 1, 4096, 4097, 1 << 20):
        b = C.c_uint64(0)
        assert L.clr_trace_sort_workspace_bytes(C.c_uint32(n), C.byref(b)) == 0
        assert b.value >= 16 * n
        sizes.append(b.value)
    assert sizes == sorted(sizes)
    assert L.clr_trace_sort_workspace_bytes(C.c_uint32(10), None) != 0

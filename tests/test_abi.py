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


def test_python_constants_match_the_header():
    """Every flag and size the Python mirror passes across the C ABI has the
    value the header defines."""
    import os
    import re

    from clear_gb300 import batch, render

    hdr = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                            "clear_cuda.h")).read()
    defs = {m.group(1): int(m.group(2), 0) for m in re.finditer(r"^#define (CLR_\w+)\s+(0x[0-9a-fA-F]+|\d+)u?\b", hdr,
                                                                 re.M)}
    pairs = {"CLR_DEVERR_SORT_TIMEOUT": _lib.DEVERR_SORT_TIMEOUT, "CLR_DEVERR_STACK": _lib.DEVERR_STACK,
             "CLR_DEVERR_REFIT": _lib.DEVERR_REFIT, "CLR_DEVERR_QUEUE": _lib.DEVERR_QUEUE,
             "CLR_DEVERR_INPUT": _lib.DEVERR_INPUT, "CLR_NODE_BYTES": _lib.NODE_BYTES,
             "CLR_TRI_BYTES": _lib.TRI_BYTES, "CLR_REF_NODE_BYTES": _lib.REF_NODE_BYTES,
             "CLR_SCENE_ALPHA": render.SCENE_ALPHA, "CLR_RENDER_ORDERED": render.RENDER_ORDERED,
             "CLR_RENDER_WAVEFRONT": render.RENDER_WAVEFRONT, "CLR_ADJOINT_RETRACE": render.ADJOINT_RETRACE,
             "CLR_TAPE_WORDS": render.TAPE_WORDS, "CLR_TAPE_VISIBLE": render.TAPE_VISIBLE,
             "CLR_BATCH_GRAPH": batch.BATCH_GRAPH}
    for name, value in pairs.items():
        assert defs.get(name) == value, (name, defs.get(name), value)

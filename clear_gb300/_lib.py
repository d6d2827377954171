"""ctypes binding of ``libclear_gb300.so`` (the C ABI of include/clear_cuda.h).

The library is the only compute path: if it is missing or cannot be loaded,
``lib()`` raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libclear_gb300.so"
HEADER = PKG.parent / "include" / "clear_cuda.h"

CLR_OK = 0
DEVERR_SORT_TIMEOUT = 0x1
DEVERR_STACK = 0x2
DEVERR_REFIT = 0x4
DEVERR_QUEUE = 0x8
DEVERR_INPUT = 0x10
NODE_BYTES = 64
TRI_BYTES = 48
REF_NODE_BYTES = 48


class ClrBvh(C.Structure):
    _fields_ = [("num_tris", C.c_uint32), ("bits_per_dim", C.c_uint32), ("nodes", C.c_void_p),
                ("tris", C.c_void_p), ("root_box", C.c_void_p)]


class ClrAdjointParams(C.Structure):
    _fields_ = [("param_tex", C.c_void_p), ("param_kind", C.c_void_p), ("num_params", C.c_uint32),
                ("grad_params", C.c_void_p), ("env_tex", C.c_uint32), ("grad_env", C.c_void_p),
                ("tape", C.c_void_p), ("tape_capacity", C.c_uint32), ("tape_count", C.c_void_p)]


class ClrObjGroup(C.Structure):
    _fields_ = [("first_face", C.c_uint32), ("num_faces", C.c_uint32), ("format", C.c_uint32),
                ("smooth", C.c_uint32), ("name", C.c_uint32), ("material", C.c_uint32)]


class ClrObjMaterial(C.Structure):
    _fields_ = [("Kd", C.c_float * 3), ("Ks", C.c_float * 3), ("Ka", C.c_float * 3), ("Ns", C.c_float),
                ("Ni", C.c_float), ("name", C.c_uint32), ("map_Kd", C.c_uint32), ("map_Ks", C.c_uint32),
                ("map_Ka", C.c_uint32)]


class ClrObjCounts(C.Structure):
    _fields_ = [(k, C.c_uint32) for k in ("num_positions", "num_uvs", "num_normals", "num_faces", "num_groups",
                                          "num_materials", "num_skipped", "string_bytes")]


OBJ_VTN, OBJ_VN, OBJ_VT, OBJ_V, OBJ_NONE = range(5)

_lib = None


class ClrError(RuntimeError):
    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def declared_symbols() -> list[str]:
    """Entry points declared in include/clear_cuda.h."""
    txt = HEADER.read_text()
    return re.findall(r"CLR_API\s+(?:const\s+)?\w+\s*\*?\s*(clr_\w+)\s*\(", txt)


def load(path: Path | None = None) -> C.CDLL:
    """Load the library without touching the GPU (ctypes only)."""
    p = Path(path or os.environ.get("CLEAR_GB300_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is not built; run clear_gb300/build.py (or __graft_entry__.build())")
    return C.CDLL(str(p))


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = load()
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        L.clr_last_error_string.restype = C.c_char_p
        sig = {
            "clr_lbvh_create": [u32, C.POINTER(vp)],
            "clr_lbvh_destroy": [vp],
            "clr_lbvh_build": [vp, vp, vp, vp, vp, u32, u32, C.POINTER(ClrBvh), vp],
            "clr_lbvh_build_host": [vp, vp, vp, vp, vp, u32, u32, u32, C.POINTER(ClrBvh), vp, vp],
            "clr_lbvh_host_copy_after": [vp, vp],
            "clr_lbvh_host_copy_wait": [vp],
            "clr_lbvh_build_noalloc": [vp, vp, vp, vp, u32, u32, C.POINTER(ClrBvh), vp],
            "clr_lbvh_build_batched": [vp, vp, vp, vp, vp, C.POINTER(u32), u32, u32, u32, vp, vp, vp, vp],
            "clr_lbvh_export_reference": [vp, C.POINTER(ClrBvh), vp, vp, vp, vp, vp, vp],
            "clr_trace_closest": [C.POINTER(ClrBvh), vp, u32, vp, vp, vp],
            "clr_trace_closest_ordered": [C.POINTER(ClrBvh), vp, u32, vp, vp, vp],
            "clr_trace_shadow": [C.POINTER(ClrBvh), vp, u32, vp, vp],
            "clr_trace_sort_workspace_bytes": [u32, C.POINTER(C.c_uint64)],
            "clr_trace_closest_sorted": [C.POINTER(ClrBvh), vp, u32, vp, vp, vp, C.c_uint64, vp],
            "clr_trace_shadow_sorted": [C.POINTER(ClrBvh), vp, u32, vp, vp, C.c_uint64, vp],
            "clr_device_status": [C.POINTER(u32), i32],
            "clr_trace_replays": [C.POINTER(C.c_uint64), i32],
            "clr_debug_set_wait_limits": [u32, u32],
            "clr_debug_set_tma_gather": [i32],
            "clr_debug_lookback_stall": [vp, vp, u32, vp],
            "clr_lbvh_set_profiling": [vp, i32],
            "clr_render": [vp, u32, u32, vp, vp, u32, u32, u32, vp],
            "clr_render_counted": [vp, u32, u32, vp, vp, u32, u32, u32, vp, vp],
            "clr_render_workspace_bytes": [u32, u32, C.POINTER(C.c_uint64)],
            "clr_render_wavefront": [vp, u32, u32, vp, vp, u32, u32, u32, vp, C.c_uint64, vp],
            "clr_render_wavefront_rows": [vp, u32, u32, u32, u32, vp, vp, u32, u32, u32, vp, C.c_uint64, vp],
            "clr_render_adjoint_workspace_bytes": [u32, u32, u32, C.POINTER(C.c_uint64)],
            "clr_render_adjoint": [vp, u32, u32, vp, vp, u32, u32, u32, C.POINTER(ClrAdjointParams), vp,
                                   C.c_uint64, vp],
            "clr_batch_create": [vp, C.POINTER(u32), C.POINTER(u32), u32, vp, C.POINTER(vp)],
            "clr_batch_destroy": [vp],
            "clr_batch_set_config": [vp, vp],
            "clr_batch_get_config": [vp, vp],
            "clr_batch_pixels": [vp, C.POINTER(u32)],
            "clr_batch_render": [vp, vp, vp, u32, u32, u32, vp],
            "clr_postprocess_ldr": [vp, u32, u32, u32, vp, vp],
            "clr_postprocess_scales": [vp, u32, u32, u32, vp, vp],
            "clr_bvh_visualize": [vp, u32, u32, vp, vp, vp],
            "clr_trace_closest_counted": [C.POINTER(ClrBvh), vp, u32, vp, vp, vp],
            "clr_env_distribution_update": [vp, u32, vp, u32, u32, u32, vp, vp],
            "clr_lbvh_pass_times": [vp, C.POINTER(C.c_float), C.POINTER(C.c_char_p), i32, C.POINTER(i32)],
            "clr_obj_parse": [C.c_char_p, C.POINTER(vp)],
            "clr_obj_counts_of": [vp, C.POINTER(ClrObjCounts)],
            "clr_obj_data": [vp, *([C.POINTER(vp)] * 7)],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = i32
        L.clr_obj_free.argtypes = [vp]
        L.clr_obj_free.restype = None
        _lib = L
    return _lib


def check(fn: str, rc: int) -> None:
    if rc != CLR_OK:
        msg = lib().clr_last_error_string().decode(errors="replace")
        raise ClrError(fn, rc, msg)


def call(fn: str, *args) -> None:
    check(fn, getattr(lib(), fn)(*args))


def device_status(clear: bool = True) -> int:
    v = C.c_uint32(0)
    call("clr_device_status", C.byref(v), 1 if clear else 0)
    return v.value

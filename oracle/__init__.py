"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; the shipped library never does.

``lbvh_build`` / ``trace_closest`` / ``trace_shadow`` / ``midbvh_build`` wrap
the C restatement in ``oracle/lbvh_oracle.c``; ``ref_*`` wrap the reference's
own CPU code compiled in place (``oracle/_ref``), present only where the
reference checkout was available at build time.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import build_oracle, build_ref

HERE = Path(__file__).resolve().parent

INODE_DTYPE = np.dtype([("min", "<f4", 4), ("max", "<f4", 4), ("isChild", "u1", 2), ("pad0", "u1", 2),
                        ("c", "<u4", 2), ("pad1", "u1", 4)])
LNODE_DTYPE = np.dtype([("min", "<f4", 4), ("max", "<f4", 4), ("objIdx", "<u4"), ("pad", "u1", 12)])
BVHNODE_DTYPE = np.dtype([("min", "<f4", 4), ("max", "<f4", 4), ("children", "<u4", 2), ("pad", "<u4", 2)])
assert INODE_DTYPE.itemsize == 48 and LNODE_DTYPE.itemsize == 48 and BVHNODE_DTYPE.itemsize == 48

_lib = None
_ref_lbvh = None
_ref_mid = None
_ref_scene = None
_ref_kbump = {}


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build_oracle()))
        _lib.orc_lbvh_build.restype = C.c_int
        _lib.orc_lbvh_build_mt.restype = C.c_int
        _lib.orc_trace_closest.restype = C.c_int
        _lib.orc_trace_shadow.restype = C.c_int
        _lib.orc_midbvh_build.restype = C.c_int64
        _lib.orc_trace_closest_mid.restype = C.c_int
        _lib.orc_morton_key.restype = C.c_uint64
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.uint32)


class OracleBVH:
    """Reference-layout LBVH produced by the restatement."""

    def __init__(self, inodes, lnodes, parents, sorted_idx, q, scene_box, bits):
        self.inodes, self.lnodes, self.parents = inodes, lnodes, parents
        self.sorted_idx, self.q, self.scene_box, self.bits = sorted_idx, q, scene_box, bits

    def keys(self):
        """3b-bit Morton keys of the triangles in sorted order (uint64)."""
        return morton_keys(self.q[self.sorted_idx], self.bits)


def morton_keys(q, bits):
    q = np.asarray(q, dtype=np.uint64)
    k = np.zeros(q.shape[0], dtype=np.uint64)
    for b in range(bits):
        d = ((q[:, 0] >> np.uint64(b)) & np.uint64(1)) | (((q[:, 1] >> np.uint64(b)) & np.uint64(1)) << np.uint64(1)) \
            | (((q[:, 2] >> np.uint64(b)) & np.uint64(1)) << np.uint64(2))
        k |= d << np.uint64(3 * b)
    return k


def lbvh_build(vx, vy, vz, tri, n, bits=10) -> OracleBVH:
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    inodes = np.zeros(max(n - 1, 0), dtype=INODE_DTYPE)
    lnodes = np.zeros(n, dtype=LNODE_DTYPE)
    parents = np.zeros(max(2 * n - 1, 0), dtype=np.uint32)
    sidx = np.zeros(n, dtype=np.uint32)
    q = np.zeros((n, 3), dtype=np.uint32)
    box = np.zeros(6, dtype=np.float32)
    rc = lib().orc_lbvh_build(_p(vx), _p(vy), _p(vz), _p(tri), C.c_uint32(n), C.c_uint32(bits), _p(inodes),
                              _p(lnodes), _p(parents), _p(sidx), _p(q), _p(box))
    if rc != 0:
        raise RuntimeError(f"orc_lbvh_build failed: {rc}")
    return OracleBVH(inodes, lnodes, parents, sidx, q, box, bits)


def lbvh_build_mt(vx, vy, vz, tri, n, bits=10, threads=0) -> OracleBVH:
    """lbvh_build on all host cores (threads <= 0) or `threads`; identical
    outputs (the per-triangle quantised coordinates are not returned)."""
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    inodes = np.zeros(max(n - 1, 0), dtype=INODE_DTYPE)
    lnodes = np.zeros(n, dtype=LNODE_DTYPE)
    parents = np.zeros(max(2 * n - 1, 0), dtype=np.uint32)
    sidx = np.zeros(n, dtype=np.uint32)
    box = np.zeros(6, dtype=np.float32)
    rc = lib().orc_lbvh_build_mt(_p(vx), _p(vy), _p(vz), _p(tri), C.c_uint32(n), C.c_uint32(bits), _p(inodes),
                                 _p(lnodes), _p(parents), _p(sidx), _p(box), C.c_int(int(threads)))
    if rc != 0:
        raise RuntimeError(f"orc_lbvh_build_mt failed: {rc}")
    return OracleBVH(inodes, lnodes, parents, sidx, None, box, bits)


def trace_closest(vx, vy, vz, tri, bvh: OracleBVH, rays, stats=False):
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    rays = _f32(rays).reshape(-1, 8)
    nr = rays.shape[0]
    ids = np.zeros(nr, dtype=np.uint32)
    ts = np.zeros(nr, dtype=np.float32)
    # per ray: internal nodes popped, internal boxes accepted, leaf box tests,
    # leaf boxes accepted (= triangle tests)
    st = np.zeros((nr, 4), dtype=np.uint32) if stats else None
    rc = lib().orc_trace_closest(_p(vx), _p(vy), _p(vz), _p(tri), _p(bvh.inodes), _p(bvh.lnodes),
                                 C.c_uint32(len(bvh.lnodes)), _p(rays), C.c_uint32(nr), _p(ids), _p(ts), _p(st))
    if rc != 0:
        raise RuntimeError(f"orc_trace_closest failed: {rc}")
    return (ids, ts, st) if stats else (ids, ts)


def trace_shadow(vx, vy, vz, tri, bvh: OracleBVH, rays):
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    rays = _f32(rays).reshape(-1, 8)
    nr = rays.shape[0]
    occ = np.zeros(nr, dtype=np.uint8)
    rc = lib().orc_trace_shadow(_p(vx), _p(vy), _p(vz), _p(tri), _p(bvh.inodes), _p(bvh.lnodes),
                                C.c_uint32(len(bvh.lnodes)), _p(rays), C.c_uint32(nr), _p(occ))
    if rc != 0:
        raise RuntimeError(f"orc_trace_shadow failed: {rc}")
    return occ


def midbvh_build(vx, vy, vz, tri, n):
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    nodes = np.zeros(max(2 * n - 1, 1), dtype=BVHNODE_DTYPE)
    cnt = lib().orc_midbvh_build(_p(vx), _p(vy), _p(vz), _p(tri), C.c_uint32(n), _p(nodes))
    if cnt < 0:
        raise RuntimeError("orc_midbvh_build failed")
    return nodes[:cnt]


def trace_closest_mid(vx, vy, vz, tri, nodes, n, rays):
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    rays = _f32(rays).reshape(-1, 8)
    nr = rays.shape[0]
    ids = np.zeros(nr, dtype=np.uint32)
    ts = np.zeros(nr, dtype=np.float32)
    rc = lib().orc_trace_closest_mid(_p(vx), _p(vy), _p(vz), _p(tri), _p(nodes), C.c_uint32(n), _p(rays),
                                     C.c_uint32(nr), _p(ids), _p(ts))
    if rc != 0:
        raise RuntimeError(f"orc_trace_closest_mid failed: {rc}")
    return ids, ts


# --------------------------------------------------------------- reference


def ref_available() -> bool:
    return bool(build_ref())


def _ref(name):
    global _ref_lbvh, _ref_mid, _ref_scene, _ref_kbump
    libs = {p.name: p for p in build_ref()}
    if not libs:
        raise RuntimeError("reference checkout not available; oracle/_ref not built")
    if name == "scene":
        if _ref_scene is None:
            L = C.CDLL(str(libs["libref_scene.so"]))
            L.ref_scene_new.restype = C.c_void_p
            L.ref_scene_free.argtypes = [C.c_void_p]
            L.ref_scene_exec.argtypes = [C.c_void_p, C.c_char_p]
            L.ref_scene_exec.restype = C.c_int
            L.ref_scene_blob.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
            L.ref_scene_blob.restype = C.c_uint64
            L.ref_scene_names.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_uint64]
            L.ref_scene_names.restype = C.c_uint64
            L.ref_save_bmp.argtypes = [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32]
            L.ref_save_bmp.restype = None
            L.ref_scene_next_model_id.argtypes = [C.c_void_p]
            L.ref_scene_next_model_id.restype = C.c_int64
            _ref_scene = L
        return _ref_scene
    if name == "lbvh":
        if _ref_lbvh is None:
            _ref_lbvh = C.CDLL(str(libs["libref_lbvh.so"]))
        return _ref_lbvh
    if name in ("lbvh_kbump", "lbvh_kbump_ulp"):
        if name not in _ref_kbump:
            _ref_kbump[name] = C.CDLL(str(libs[f"lib{name.replace('lbvh', 'ref_lbvh')}.so"]))
        return _ref_kbump[name]
    if _ref_mid is None:
        _ref_mid = C.CDLL(str(libs["libref_mid.so"]))
        _ref_mid.ref_midbvh_build.restype = C.c_int64
    return _ref_mid


def verts16(vx, vy, vz):
    """float3 vertex array with the 16-byte stride of cl_float3."""
    v = np.zeros((len(vx), 4), dtype=np.float32)
    v[:, 0], v[:, 1], v[:, 2] = vx, vy, vz
    return v


FACE_DTYPE = np.dtype([("p", "<u4", 3), ("vn", "<u4", 3), ("vt", "<u4", 3), ("uv", "<u4", 3),
                       ("alphaTexPtr", "<u4"), ("matPtr", "<u2"), ("lightPtr", "<u2")])
assert FACE_DTYPE.itemsize == 56


def faces_from_tri(tri, n):
    f = np.zeros(n, dtype=FACE_DTYPE)
    f["p"] = np.asarray(tri, dtype=np.uint32).reshape(n, 3) if tri is not None else np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    f["vn"] = f["vt"] = f["uv"] = 0xFFFFFFFF
    f["alphaTexPtr"] = 0xFFFFFFFF
    f["matPtr"] = 0
    f["lightPtr"] = 0xFFFF
    return f


def ref_trace_closest_lbvh(vx, vy, vz, tri, n, bvh: OracleBVH, rays):
    v = verts16(vx, vy, vz)
    faces = faces_from_tri(tri, n)
    rays = _f32(rays).reshape(-1, 8)
    nr = rays.shape[0]
    ids = np.zeros(nr, dtype=np.uint32)
    ts = np.zeros(nr, dtype=np.float32)
    _ref("lbvh").ref_trace_closest_lbvh(_p(v), _p(faces), _p(bvh.inodes), _p(bvh.lnodes), _p(rays),
                                        C.c_uint32(nr), _p(ids), _p(ts))
    return ids, ts


def ref_midbvh_build(vx, vy, vz, tri, n):
    v = verts16(vx, vy, vz)
    tri = _u32(tri) if tri is not None else np.arange(3 * n, dtype=np.uint32)
    nodes = np.zeros(max(2 * n - 1, 1), dtype=BVHNODE_DTYPE)
    cnt = _ref("mid").ref_midbvh_build(_p(v), _p(tri), C.c_uint32(n), _p(nodes))
    return nodes[:cnt]


def ref_trace_closest_mid(vx, vy, vz, tri, n, nodes, rays):
    v = verts16(vx, vy, vz)
    faces = faces_from_tri(tri, n)
    rays = _f32(rays).reshape(-1, 8)
    nr = rays.shape[0]
    ids = np.zeros(nr, dtype=np.uint32)
    ts = np.zeros(nr, dtype=np.float32)
    _ref("mid").ref_trace_closest_mid(_p(v), _p(faces), _p(nodes), _p(rays), C.c_uint32(nr), _p(ids), _p(ts))
    return ids, ts


def ref_bvh_visualizer(scene_blobs: dict, inodes, lnodes, pixels, width, height):
    """sim::bvh_visualizer over the whole image; pixels (f32[W*H*4]) are
    updated in place."""
    b = scene_blobs
    rs = np.zeros(4 * width * height, dtype=np.uint32)
    _ref("lbvh").ref_bvh_visualizer(_p(b["vertices"]), _p(b["normals"]), _p(b["tangents"]), _p(b["uvs"]),
                                    _p(b["faces"]), _p(b["lights"]), _p(b["materials"]), _p(b["textures"]),
                                    _p(b["others"]), _p(inodes), _p(lnodes), _p(rs), _p(pixels),
                                    C.c_uint32(width), C.c_uint32(height))


def ref_render(scene_blobs: dict, inodes, lnodes, rand_states, pixels, width, height, y0, y1, spp,
               bump_as_kernel: bool = False, max_depth: int = 100, perturb_math: bool = False):
    """sim::pathtracing over rows [y0, y1); rand_states (u32[4*W*H]) and
    pixels (f32[W*H*4]) are updated in place.  bump_as_kernel: the build of
    the renderer whose bump frame follows the OpenCL kernel and whose depth
    cap is max_depth (libref_lbvh_kbump, see build_oracle.build_ref_kernel_bump);
    perturb_math: that build with the transcendentals one ulp off on an eighth
    of the inputs."""
    b = scene_blobs
    if max_depth != 100 or perturb_math:
        bump_as_kernel = True
    L = _ref(("lbvh_kbump_ulp" if perturb_math else "lbvh_kbump") if bump_as_kernel else "lbvh")
    if bump_as_kernel:
        L.ref_set_max_depth(C.c_uint32(max_depth))
    L.ref_render(_p(b["vertices"]), _p(b["normals"]), _p(b["tangents"]), _p(b["uvs"]),
                            _p(b["faces"]), _p(b["lights"]), _p(b["materials"]), _p(b["textures"]),
                            _p(b["others"]), _p(inodes), _p(lnodes), _p(rand_states), _p(pixels),
                            C.c_uint32(width), C.c_uint32(height), C.c_uint32(y0), C.c_uint32(y1),
                            C.c_uint32(spp))


SCENE_BLOBS = ("vertices", "normals", "tangents", "uvs", "faces", "lights", "materials", "textures", "others",
               "light_powers")
SCENE_NAMES = ("materials", "light_props", "textures", "others", "tex_files")


class RefScene:
    """The reference's Scene + MaterialCreator + loadModel driven by a command
    script (oracle/ref_scene.cpp lists the commands).  Note the reference's
    MaterialCreator is a process-wide singleton and its .obj model counter a
    process-wide static: ``next_model_id`` says which number the next load
    gets."""

    def __init__(self):
        self.L = _ref("scene")
        self.h = self.L.ref_scene_new()

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_scene_free(self.h)
            self.h = None

    def exec(self, script: str) -> int:
        n = self.L.ref_scene_exec(self.h, script.encode())
        if n < 0:
            raise ValueError(f"unknown command on line {-n}: {script.splitlines()[-n - 1]!r}")
        return n

    def blob(self, name: str) -> bytes:
        p = C.c_void_p()
        n = self.L.ref_scene_blob(self.h, SCENE_BLOBS.index(name), C.byref(p))
        return C.string_at(p, n) if n else b""

    def names(self, name: str) -> dict:
        which = SCENE_NAMES.index(name)
        n = self.L.ref_scene_names(self.h, which, None, 0)
        buf = C.create_string_buffer(n)
        self.L.ref_scene_names(self.h, which, buf, n)
        out = {}
        for line in buf.raw[:n].decode().splitlines():
            k, v = line.rsplit("\t", 1)
            out[k] = int(v)
        return out

    @property
    def next_model_id(self) -> int:
        return int(self.L.ref_scene_next_model_id(self.h))


def ref_save_bmp(path: str, pixels: np.ndarray, width: int, height: int) -> None:
    """The reference's saveBMP (BMPExporter.cpp) writing `pixels`."""
    px = np.ascontiguousarray(pixels, dtype=np.uint8)
    _ref("scene").ref_save_bmp(str(path).encode(), px.ctypes.data, width, height)


def ref_cl_lbvh_build(vx, vy, vz, tri, n, bits=10) -> OracleBVH:
    """The reference's own LBVH kernels (lbvh_construction.cl,
    generic_kernels.cl) run on the CPU in the order of LBVHBuilder::perform
    (oracle/ref_lbvh_cl.cpp); n >= 2."""
    libs = {p.name: p for p in build_ref()}
    if "libref_lbvh_cl.so" not in libs:
        raise RuntimeError("reference checkout not available; oracle/_ref not built")
    L = C.CDLL(str(libs["libref_lbvh_cl.so"]))
    vx, vy, vz, tri = _f32(vx), _f32(vy), _f32(vz), _u32(tri)
    inodes = np.zeros(n - 1, dtype=INODE_DTYPE)
    lnodes = np.zeros(n, dtype=LNODE_DTYPE)
    parents = np.zeros(2 * n - 1, dtype=np.uint32)
    sidx = np.zeros(n, dtype=np.uint32)
    q = np.zeros((n, 4), dtype=np.uint32)
    box = np.zeros(6, dtype=np.float32)
    rc = L.ref_cl_lbvh_build(_p(vx), _p(vy), _p(vz), _p(tri), C.c_uint32(n), C.c_uint32(bits), _p(inodes),
                             _p(lnodes), _p(parents), _p(sidx), _p(q), _p(box))
    if rc != 0:
        raise RuntimeError(f"ref_cl_lbvh_build failed: {rc}")
    return OracleBVH(inodes, lnodes, parents, sidx, np.ascontiguousarray(q[:, :3]), box, bits)


def ref_cl_postprocess(accum, width: int, height: int, spp: int) -> np.ndarray:
    """The reference's own `clear`, `scaling` and `toneMapping` kernels
    (post_processing.cl) run on the CPU: the BMP pixel array, padding zero."""
    libs = {p.name: p for p in build_ref()}
    if "libref_post_cl.so" not in libs:
        raise RuntimeError("reference checkout not available; oracle/_ref not built")
    L = C.CDLL(str(libs["libref_post_cl.so"]))
    a = np.ascontiguousarray(np.asarray(accum, dtype=np.float32).reshape(width * height, 4))
    out = np.zeros(height * (3 * width + width % 4), dtype=np.uint8)
    L.ref_cl_postprocess(_p(a), C.c_uint32(width), C.c_uint32(height), C.c_uint32(spp), _p(out))
    return out

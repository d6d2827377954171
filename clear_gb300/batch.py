"""Many scenes in one pass: segmented LBVH build + one batched wavefront.

``BatchRenderer(scenes)`` uploads the scenes' blobs into one buffer per blob
kind, builds every scene's LBVH with one segmented build
(``clr_lbvh_build_batched``) and renders all images with one wavefront over a
pool of path slots (``clr_batch_render``; with ``graph=True`` the whole frame
loop is one CUDA graph launch).  ``per_scene_loop`` is the plain form the
batched one replaces: a standalone build and a wavefront render per scene.
Both give bit-identical images (same per-pixel random streams, same
arithmetic).

``random_scene`` makes the batched workload's scenes: the LBVH benchmark's
random-triangle distribution (``workloads.triangle_soup``) with a Lambertian
and a coated material and one quad light.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib, lbvh
from . import scene as S
from . import workloads as W
from .render import RENDER_ORDERED, ClrScene, DeviceScene, scene_flags
from .scenes import pixel_seeds

BATCH_GRAPH = 0x2
BLOB_KEYS = ("vertices", "normals", "tangents", "uvs", "faces", "lights", "materials", "textures", "others")
RESOLUTIONS = (128, 256, 384, 512)


class ClrBatchConfig(C.Structure):
    _fields_ = [("trace_block", C.c_uint32), ("shade_block", C.c_uint32), ("pool_slots", C.c_uint32),
                ("reserved", C.c_uint32)]


def random_scene(n_tris: int, width: int, height: int, seed: int) -> S.Scene:
    """n_tris random triangles in the unit cube (half Lambertian, half an
    Ashikhmin coat over a diffuse base), a 0.5 x 0.5 quad light above the
    cube facing down, a pinhole camera in front."""
    rng = np.random.default_rng(seed)
    sc = S.Scene()
    mc = sc.mc
    a = rng.uniform(0.2, 0.9, size=3)
    mc.float3_constant_texture("R", *map(float, a))
    mc.float_constant_texture("sigma0", 0.0)
    mc.matte_material("lambert", None, "R", "sigma0")
    mc.float3_constant_texture("Rs", 0.04, 0.04, 0.04)
    mc.float3_constant_texture("Rd", *map(float, rng.uniform(0.2, 0.9, size=3)))
    mc.float_constant_texture("n", float(rng.uniform(20.0, 200.0)))
    mc.ashikhmin_material("coated", None, "Rs", "Rd", "n", "n")
    mc.float3_constant_texture("M", 12.0 * math.pi, 12.0 * math.pi, 12.0 * math.pi)
    mc.diffuse_light_property("light", "M")
    vx, vy, vz = W.triangle_soup(n_tris, seed=seed)
    v = np.stack([vx, vy, vz], axis=1).reshape(n_tris, 3, 3)
    half = n_tris // 2
    for mat, part in (("lambert", v[:half]), ("coated", v[half:])):
        if len(part):
            sc.add_mesh(part.reshape(-1, 3), np.arange(3 * len(part)).reshape(-1, 3), sc.mat_ref[mat])
    sc.begin_object()
    for x, z in ((0.25, 0.25), (0.75, 0.25), (0.75, 0.75), (0.25, 0.75)):
        sc.add_vertex(x, 1.3, z)
    sc.add_face((0, 1, 2), sc.mat_ref["lambert"], light=sc.light_ref["light"])
    sc.add_face((0, 2, 3), sc.mat_ref["lambert"], light=sc.light_ref["light"])
    sc.end_object()
    cam = S.look_at((0.5, 0.55, 2.6), (0.5, 0.5, 0.5), (0, 1, 0))
    sc.set_camera(width, height, cam, fov_y_deg=40.0)
    sc.build()
    return sc


def batch_workload(num_scenes: int = 512, seed: int = 7, min_tris: int = 1000, max_tris: int = 200_000):
    """Triangle counts log-uniform in [min_tris, max_tris] and square
    resolutions drawn from RESOLUTIONS, seeded."""
    rng = np.random.default_rng(seed)
    tris = np.exp(rng.uniform(math.log(min_tris), math.log(max_tris), size=num_scenes)).astype(np.int64)
    res = rng.choice(RESOLUTIONS, size=num_scenes)
    return [(int(n), int(r), int(r), seed * 100003 + i) for i, (n, r) in enumerate(zip(tris, res))]


def _concat(arrays, align=256):
    """Byte-concatenate numpy arrays at `align`-byte offsets."""
    offs, total = [], 0
    for a in arrays:
        offs.append(total)
        total += (a.nbytes + align - 1) // align * align
    buf = np.zeros(max(total, align), dtype=np.uint8)
    for a, o in zip(arrays, offs):
        buf[o:o + a.nbytes] = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    return buf, offs


class BatchRenderer:
    def __init__(self, scenes: list[S.Scene], device="cuda", bits_per_dim: int = 10, radix_bits: int = 8,
                 config: dict | None = None):
        self.device = torch.device(device)
        self.scenes = scenes
        self.sizes = [(sc.width, sc.height) for sc in scenes]
        blobs = [sc.blobs() for sc in scenes]
        self.num_faces = [len(sc.faces) for sc in scenes]
        self.t, self.boff = {}, {}
        for k in BLOB_KEYS:
            buf, offs = _concat([b[k] for b in blobs])
            self.t[k] = torch.from_numpy(buf).to(self.device)
            self.boff[k] = offs
        # geometry for the segmented build: concatenated SoA, global indices
        vxs, vys, vzs, tris, base = [], [], [], [], 0
        for sc in scenes:
            vx, vy, vz, tri = sc.soa()
            vxs.append(vx)
            vys.append(vy)
            vzs.append(vz)
            tris.append(tri.astype(np.int64) + base)
            base += len(vx)
        self.soa = tuple(torch.from_numpy(np.concatenate(a)).to(self.device) for a in (vxs, vys, vzs))
        self.tri = torch.from_numpy(np.concatenate(tris).astype(np.int32)).to(self.device)
        self.offsets = np.concatenate([[0], np.cumsum(self.num_faces)]).astype(np.int64).tolist()
        self.bits = bits_per_dim
        self.radix_bits = radix_bits
        self.builder = lbvh.LBVHBuilder(self.offsets[-1], self.device)
        self.bvh = self.build()
        self._bvh_c = [self.bvh.scene(s) for s in range(len(scenes))]
        arr = (ClrScene * len(scenes))()
        for s in range(len(scenes)):
            p = {k: self.t[k].data_ptr() + self.boff[k][s] for k in BLOB_KEYS}
            arr[s] = ClrScene(p["vertices"], p["normals"], p["tangents"], p["uvs"], p["faces"], p["lights"],
                              p["materials"], p["textures"], p["others"], C.pointer(self._bvh_c[s].c),
                              scene_flags(blobs[s]))
        self._arr = arr
        w = (C.c_uint32 * len(scenes))(*[wh[0] for wh in self.sizes])
        h = (C.c_uint32 * len(scenes))(*[wh[1] for wh in self.sizes])
        cfg = self._cfg(config)
        handle = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("clr_batch_create", arr, w, h, C.c_uint32(len(scenes)), C.byref(cfg), C.byref(handle))
        self._h = handle
        self.total_pixels = sum(a * b for a, b in self.sizes)
        self.pix0 = np.concatenate([[0], np.cumsum([a * b for a, b in self.sizes])]).astype(np.int64).tolist()

    @staticmethod
    def _cfg(config: dict | None) -> ClrBatchConfig:
        c = config or {}
        return ClrBatchConfig(int(c.get("trace_block", 0)), int(c.get("shade_block", 0)),
                              int(c.get("pool_slots", 0)), 0)

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().clr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, radix_bits: int | None = None) -> lbvh.BatchBVH:
        """The segmented build of every scene (into fresh buffers)."""
        return self.builder.perform_batched(self.soa, self.tri, self.offsets, self.bits,
                                            radix_bits or self.radix_bits)

    def rebuild_into_current(self, radix_bits: int | None = None) -> None:
        """Re-run the segmented build into the buffers the batch renders from."""
        offs = (C.c_uint32 * len(self.offsets))(*self.offsets)
        with torch.cuda.device(self.device):
            _lib.call("clr_lbvh_build_batched", self.builder._h, C.c_void_p(self.soa[0].data_ptr()),
                      C.c_void_p(self.soa[1].data_ptr()), C.c_void_p(self.soa[2].data_ptr()),
                      C.c_void_p(self.tri.data_ptr()), offs, C.c_uint32(len(self.offsets) - 1), C.c_uint32(self.bits),
                      C.c_uint32(radix_bits or self.radix_bits), C.c_void_p(self.bvh.nodes.data_ptr()),
                      C.c_void_p(self.bvh.tris.data_ptr()), C.c_void_p(self.bvh.root_boxes.data_ptr()),
                      C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))

    def config(self) -> dict:
        c = ClrBatchConfig()
        _lib.call("clr_batch_get_config", self._h, C.byref(c))
        return {"trace_block": c.trace_block, "shade_block": c.shade_block, "pool_slots": c.pool_slots}

    def set_config(self, config: dict) -> None:
        cfg = self._cfg(config)
        with torch.cuda.device(self.device):
            _lib.call("clr_batch_set_config", self._h, C.byref(cfg))

    def new_frame(self):
        """Per-pixel seeds of every scene (seed = pixel index + 1 within its
        scene) and a zeroed accumulation buffer, concatenated."""
        seeds = np.concatenate([pixel_seeds(w, h) for w, h in self.sizes])
        rng = torch.from_numpy(seeds.view(np.int32)).to(self.device)
        pix = torch.zeros((self.total_pixels, 4), dtype=torch.float32, device=self.device)
        return rng, pix

    def render(self, rng: torch.Tensor, pix: torch.Tensor, spp: int, max_depth: int = 5, ordered: bool = True,
               graph: bool = True) -> None:
        flags = (RENDER_ORDERED if ordered else 0) | (BATCH_GRAPH if graph else 0)
        with torch.cuda.device(self.device):
            _lib.call("clr_batch_render", self._h, C.c_void_p(rng.data_ptr()), C.c_void_p(pix.data_ptr()),
                      C.c_uint32(spp), C.c_uint32(max_depth), C.c_uint32(flags),
                      C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))

    def image(self, pix: torch.Tensor, s: int) -> torch.Tensor:
        return pix[self.pix0[s]:self.pix0[s + 1]]


class PerSceneLoop:
    """The plain form: each scene uploaded on its own, built with a
    standalone LBVH build and rendered with its own wavefront call."""

    def __init__(self, scenes: list[S.Scene], device="cuda", bits_per_dim: int = 10):
        self.device = torch.device(device)
        self.ds = [DeviceScene(sc, self.device, bits_per_dim) for sc in scenes]
        self.bits = bits_per_dim

    def build_all(self) -> None:
        for d in self.ds:
            d.bvh = d.builder.perform(d.soa, d.tri, d.num_faces, self.bits, out=d.bvh)

    def new_frame(self):
        rngs, pixs = zip(*[d.new_frame() for d in self.ds])
        return list(rngs), list(pixs)

    def render(self, rngs, pixs, spp: int, max_depth: int = 5, ordered: bool = True) -> None:
        for d, r, p in zip(self.ds, rngs, pixs):
            d.render(r, p, spp, max_depth=max_depth, ordered=ordered, wavefront=True)

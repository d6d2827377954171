"""Host-side mirror of the reference's LBVH builder and ray queries.

``LBVHBuilder(num_faces).perform(vertices, faces, num_faces, bits)`` follows
``LBVHBuilder::LBVHBuilder`` / ``LBVHBuilder::perform``
(OpenCL_PathTracer/LBVHBuilder.h:70-74): the builder owns a scratch pool that
grows on demand, the caller owns inputs and outputs.  ``trace_closest`` and
``trace_shadow`` replace ``rayIntersection`` (OpenCL/bvh_traversal.cl:182-215)
for batches of rays.

Device memory and streams come from PyTorch; all compute runs in
``libclear_gb300.so`` through its C ABI.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import ClrBvh, call


def _ptr(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _f32(t: torch.Tensor, device) -> torch.Tensor:
    t = t.to(device=device, dtype=torch.float32)
    return t.contiguous()


class BVH:
    """A built BVH: child-box nodes, leaf-ordered triangle records, root box."""

    def __init__(self, num_tris: int, device):
        self.device = torch.device(device)
        n = int(num_tris)
        self.nodes = torch.empty(max(n - 1, 1) * _lib.NODE_BYTES, dtype=torch.uint8, device=self.device)
        self.tris = torch.empty(max(n, 1) * _lib.TRI_BYTES, dtype=torch.uint8, device=self.device)
        self.root_box = torch.zeros(8, dtype=torch.float32, device=self.device)
        self.c = ClrBvh(n, 0, self.nodes.data_ptr(), self.tris.data_ptr(), self.root_box.data_ptr())

    @property
    def num_tris(self) -> int:
        return self.c.num_tris

    @property
    def bits_per_dim(self) -> int:
        return self.c.bits_per_dim


class BatchBVH:
    """The BVHs of a segmented build: shared node / record buffers, one
    root box per scene; ``scene(s)`` is scene s's BVH (a view)."""

    def __init__(self, offsets: list[int], bits: int, device):
        self.device = torch.device(device)
        self.offsets = offsets
        total = offsets[-1]
        self.nodes = torch.empty(max(total, 1) * _lib.NODE_BYTES, dtype=torch.uint8, device=self.device)
        self.tris = torch.empty(max(total, 1) * _lib.TRI_BYTES, dtype=torch.uint8, device=self.device)
        self.root_boxes = torch.zeros((len(offsets) - 1, 8), dtype=torch.float32, device=self.device)
        self.bits = bits

    def __len__(self) -> int:
        return len(self.offsets) - 1

    def scene(self, s: int) -> BVH:
        o, n = self.offsets[s], self.offsets[s + 1] - self.offsets[s]
        b = BVH.__new__(BVH)
        b.device = self.device
        b.nodes = self.nodes[o * _lib.NODE_BYTES:(o + max(n - 1, 1)) * _lib.NODE_BYTES]
        b.tris = self.tris[o * _lib.TRI_BYTES:(o + n) * _lib.TRI_BYTES]
        b.root_box = self.root_boxes[s]
        b.c = ClrBvh(n, self.bits, b.nodes.data_ptr(), b.tris.data_ptr(), b.root_box.data_ptr())
        b._owner = self
        return b


class LBVHBuilder:
    def __init__(self, num_faces: int, device="cuda"):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise RuntimeError("LBVHBuilder needs a CUDA device; there is no CPU path")
        with torch.cuda.device(self.device):
            h = C.c_void_p()
            call("clr_lbvh_create", C.c_uint32(max(int(num_faces), 1)), C.byref(h))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.lib().clr_lbvh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def perform(self, vertices, faces, num_faces: int, num_bits_per_dim: int = 10,
                out: BVH | None = None) -> BVH:
        """Build the LBVH on the current stream.  vertices = (vx, vy, vz)
        float32 tensors; faces = (num_faces, 3) integer tensor of vertex
        indices, or None for an unindexed soup (vertex k of triangle t at
        3t+k).  A builder's builds share its scratch pool: builds on other
        streams must wait for this one (separate builders do not)."""
        vx, vy, vz = (_f32(v, self.device) for v in vertices)
        tri = None
        if faces is not None:
            tri = faces.to(device=self.device, dtype=torch.int32).contiguous()
        n = int(num_faces)
        bvh = out if out is not None and out.num_tris == n else BVH(n, self.device)
        with torch.cuda.device(self.device):
            call("clr_lbvh_build", self._h, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(tri), C.c_uint32(n),
                 C.c_uint32(int(num_bits_per_dim)), C.byref(bvh.c), _stream(self.device))
        bvh._inputs = (vx, vy, vz, tri)  # keep alive until the stream has consumed them
        return bvh

    def perform_host(self, vertices, faces, num_faces: int, num_bits_per_dim: int = 10,
                     out: BVH | None = None, root_host: torch.Tensor | None = None) -> BVH:
        """Upload and build from HOST arrays (clr_lbvh_build_host): vertices =
        (vx, vy, vz) contiguous float32 CPU tensors (page-locked for the copy
        to overlap the previous build), faces = (num_faces, 3) int32 CPU
        tensor or None for a soup.  root_host (8 float32, CPU) receives the
        root record.  Keep the host tensors unchanged until host_copy_wait()
        or a synchronisation of the stream."""
        vs = []
        for v in vertices:
            if v.device.type != "cpu" or v.dtype != torch.float32 or not v.is_contiguous():
                raise ValueError("perform_host takes contiguous float32 CPU tensors")
            vs.append(v)
        nv = int(vs[0].numel())
        if any(int(v.numel()) != nv for v in vs):
            raise ValueError("vx, vy, vz differ in length")
        tri = None
        if faces is not None:
            if faces.device.type != "cpu" or faces.dtype != torch.int32 or not faces.is_contiguous():
                raise ValueError("faces must be a contiguous int32 CPU tensor")
            tri = faces
        if root_host is not None and (root_host.device.type != "cpu" or root_host.dtype != torch.float32
                                      or root_host.numel() < 8):
            raise ValueError("root_host must be a float32 CPU tensor of 8 elements")
        n = int(num_faces)
        bvh = out if out is not None and out.num_tris == n else BVH(n, self.device)
        with torch.cuda.device(self.device):
            call("clr_lbvh_build_host", self._h, _ptr(vs[0]), _ptr(vs[1]), _ptr(vs[2]), _ptr(tri), C.c_uint32(nv),
                 C.c_uint32(n), C.c_uint32(int(num_bits_per_dim)), C.byref(bvh.c), _ptr(root_host),
                 _stream(self.device))
        return bvh

    def host_copy_after_stream(self) -> None:
        """Later perform_host copies start after the work queued on the
        current stream so far."""
        with torch.cuda.device(self.device):
            call("clr_lbvh_host_copy_after", self._h, _stream(self.device))

    def host_copy_wait(self) -> None:
        """Block until every perform_host copy issued so far is done."""
        call("clr_lbvh_host_copy_wait", self._h)

    def perform_batched(self, vertices, faces, scene_offsets, num_bits_per_dim: int = 10,
                        radix_bits: int = 8) -> "BatchBVH":
        """Build one LBVH per scene in one segmented pass.  vertices and faces
        are concatenated over the scenes (faces index the concatenated
        vertices, or None for a soup); scene_offsets (host sequence of
        num_scenes + 1 ints, from 0) delimits each scene's triangles."""
        vx, vy, vz = (_f32(v, self.device) for v in vertices)
        tri = None
        if faces is not None:
            tri = faces.to(device=self.device, dtype=torch.int32).contiguous()
        offs = (C.c_uint32 * len(scene_offsets))(*[int(o) for o in scene_offsets])
        b = BatchBVH([int(o) for o in scene_offsets], int(num_bits_per_dim), self.device)
        with torch.cuda.device(self.device):
            call("clr_lbvh_build_batched", self._h, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(tri), offs,
                 C.c_uint32(len(scene_offsets) - 1), C.c_uint32(int(num_bits_per_dim)), C.c_uint32(int(radix_bits)),
                 _ptr(b.nodes), _ptr(b.tris), _ptr(b.root_boxes), _stream(self.device))
        b._inputs = (vx, vy, vz, tri)
        return b

    def set_profiling(self, enable: bool) -> None:
        call("clr_lbvh_set_profiling", self._h, 1 if enable else 0)

    def pass_times(self) -> list[tuple[str, float]]:
        """(kernel, ms) of the last build; needs set_profiling(True)."""
        ms = (C.c_float * 16)()
        names = (C.c_char_p * 16)()
        cnt = C.c_int(0)
        call("clr_lbvh_pass_times", self._h, ms, names, 16, C.byref(cnt))
        return [(names[i].decode(), float(ms[i])) for i in range(cnt.value)]

    def export_reference(self, bvh: BVH) -> dict:
        """The last build in the reference's 48-byte node layouts plus the
        sorted triangle order and Morton keys (for parity checks)."""
        n = bvh.num_tris
        dev = self.device
        out = {
            "inodes": torch.zeros(max(n - 1, 0) * _lib.REF_NODE_BYTES, dtype=torch.uint8, device=dev),
            "lnodes": torch.zeros(n * _lib.REF_NODE_BYTES, dtype=torch.uint8, device=dev),
            "parents": torch.zeros(max(2 * n - 1, 0), dtype=torch.int32, device=dev),
            "sorted_idx": torch.zeros(n, dtype=torch.int32, device=dev),
            "keys": torch.zeros(n, dtype=torch.int64, device=dev),
        }
        with torch.cuda.device(dev):
            call("clr_lbvh_export_reference", self._h, C.byref(bvh.c),
                 _ptr(out["inodes"]) if n > 1 else None, _ptr(out["lnodes"]) if n else None,
                 _ptr(out["parents"]) if n else None, _ptr(out["sorted_idx"]) if n else None,
                 _ptr(out["keys"]) if n else None, _stream(dev))
        return out


def _rays(rays: torch.Tensor, device) -> torch.Tensor:
    r = rays.to(device=device, dtype=torch.float32).contiguous().view(-1, 8)
    return r


def _sort_workspace(m: int, device) -> tuple[torch.Tensor, int]:
    """A 256-byte aligned scratch buffer for the sorted-order searches (torch's
    caching allocator keeps it between calls)."""
    n = C.c_uint64(0)
    call("clr_trace_sort_workspace_bytes", C.c_uint32(m), C.byref(n))
    ws = torch.empty(int(n.value) + 256, dtype=torch.uint8, device=device)
    off = (-ws.data_ptr()) % 256
    return ws, off


def trace_closest(bvh: BVH, rays: torch.Tensor, hit_id: torch.Tensor | None = None,
                  hit_t: torch.Tensor | None = None, ordered: bool = True, sort: bool = False):
    """Closest hit for rays packed {ox,oy,oz,tmax,dx,dy,dz,0}.  Returns
    (hit_id int32 [-1 = miss], hit_t float32), the reference's answer in every
    form: ordered=True (default) visits the nearer child first and replays in
    the reference's order the rays whose answer could depend on the order;
    ordered=False searches every ray in the reference's order; sort=True (with
    ordered) first sorts the rays by origin (clr_trace_closest_sorted)."""
    r = _rays(rays, bvh.device)
    m = r.shape[0]
    if hit_id is None:
        hit_id = torch.empty(m, dtype=torch.int32, device=bvh.device)
    if hit_t is None:
        hit_t = torch.empty(m, dtype=torch.float32, device=bvh.device)
    with torch.cuda.device(bvh.device):
        if sort:
            if not ordered:
                raise ValueError("sort=True searches nearer-first (ordered=True)")
            ws, off = _sort_workspace(m, bvh.device)
            call("clr_trace_closest_sorted", C.byref(bvh.c), _ptr(r), C.c_uint32(m), _ptr(hit_id), _ptr(hit_t),
                 C.c_void_p(ws.data_ptr() + off), C.c_uint64(ws.numel() - off), _stream(bvh.device))
        else:
            call("clr_trace_closest_ordered" if ordered else "clr_trace_closest", C.byref(bvh.c), _ptr(r),
                 C.c_uint32(m), _ptr(hit_id), _ptr(hit_t), _stream(bvh.device))
    return hit_id, hit_t


def trace_replays(clear: bool = True) -> int:
    """Rays the nearer-first closest-hit query searched again in the
    reference's order, summed over its launches since the last clear."""
    v = C.c_uint64(0)
    call("clr_trace_replays", C.byref(v), 1 if clear else 0)
    return int(v.value)


def trace_shadow(bvh: BVH, rays: torch.Tensor, occluded: torch.Tensor | None = None, sort: bool = False):
    """Any-hit query: 1 where a triangle is hit at 0 <= t <= tmax; sort=True
    searches the rays in origin order (clr_trace_shadow_sorted)."""
    r = _rays(rays, bvh.device)
    m = r.shape[0]
    if occluded is None:
        occluded = torch.empty(m, dtype=torch.uint8, device=bvh.device)
    with torch.cuda.device(bvh.device):
        if sort:
            ws, off = _sort_workspace(m, bvh.device)
            call("clr_trace_shadow_sorted", C.byref(bvh.c), _ptr(r), C.c_uint32(m), _ptr(occluded),
                 C.c_void_p(ws.data_ptr() + off), C.c_uint64(ws.numel() - off), _stream(bvh.device))
        else:
            call("clr_trace_shadow", C.byref(bvh.c), _ptr(r), C.c_uint32(m), _ptr(occluded), _stream(bvh.device))
    return occluded


def trace_closest_counted(bvh: BVH, rays: torch.Tensor):
    """Closest hit in the reference's order with per-ray visiting counts:
    returns (hit_id int32, counts int32 (n, 2): internal boxes accepted = nodes
    loaded, leaf boxes accepted = triangles tested)."""
    r = _rays(rays, bvh.device)
    m = r.shape[0]
    hit_id = torch.empty(m, dtype=torch.int32, device=bvh.device)
    counts = torch.empty((m, 2), dtype=torch.int32, device=bvh.device)
    with torch.cuda.device(bvh.device):
        call("clr_trace_closest_counted", C.byref(bvh.c), _ptr(r), C.c_uint32(m), _ptr(hit_id), _ptr(counts),
             _stream(bvh.device))
    return hit_id, counts

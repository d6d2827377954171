"""Host side of the path tracer: uploads a scene's blobs, builds its LBVH and
calls ``clr_render`` (the counterpart of enqueueing the reference's
``pathtracing`` kernel per tile and sample, main.cpp:477-494)."""
from __future__ import annotations

import contextlib
import ctypes as C

import numpy as np
import torch

from . import _lib, lbvh
from .scene import FACE_DTYPE, NONE32, Scene, zenith_weights
from .scenes import pixel_seeds

RENDER_ORDERED = 0x1
ADJOINT_RETRACE = 0x4
RENDER_WAVEFRONT = 0x2  # clr_render: the wavefront form on the library's own workspace
NO_TEX = 0xFFFFFFFF
TAPE_WORDS = 32
TAPE_VISIBLE = 0x100


class ClrScene(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p), ("uvs", C.c_void_p),
                ("faces", C.c_void_p), ("lights", C.c_void_p), ("materials", C.c_void_p),
                ("textures", C.c_void_p), ("others", C.c_void_p), ("bvh", C.POINTER(_lib.ClrBvh)),
                ("flags", C.c_uint32)]

SCENE_ALPHA = 0x1  # CLR_SCENE_ALPHA


def scene_flags(blobs: dict) -> int:
    """CLR_SCENE_* of a scene's blobs: CLR_SCENE_ALPHA when some face has an
    alpha texture."""
    faces = np.asarray(blobs["faces"]).view(FACE_DTYPE)
    return SCENE_ALPHA if bool((faces["alphaTexPtr"] != NONE32).any()) else 0


def _dev(a: np.ndarray, device) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).to(device)


class DeviceScene:
    """A scene resident on the GPU with its LBVH."""

    def __init__(self, scene: Scene, device="cuda", bits_per_dim: int = 10):
        self.device = torch.device(device)
        b = scene.blobs()
        self.blobs = b
        self.env_dist = getattr(scene, "env_dist", None)
        self.width, self.height = scene.width, scene.height
        self.t = {k: _dev(b[k], self.device) for k in ("vertices", "normals", "tangents", "uvs", "faces", "lights",
                                                        "materials", "textures", "others")}
        vx, vy, vz, tri = scene.soa()
        self.num_faces = len(scene.faces)
        self.builder = lbvh.LBVHBuilder(self.num_faces, self.device)
        self.soa = tuple(torch.from_numpy(a).to(self.device) for a in (vx, vy, vz))
        self.tri = torch.from_numpy(tri.astype(np.int32)).to(self.device)
        self.bvh = self.builder.perform(self.soa, self.tri, self.num_faces, bits_per_dim)
        p = lambda k: self.t[k].data_ptr()  # noqa: E731
        self._ws_last_use = None  # torch.cuda.Event recorded after each workspace use
        self.c = ClrScene(p("vertices"), p("normals"), p("tangents"), p("uvs"), p("faces"), p("lights"),
                          p("materials"), p("textures"), p("others"), C.pointer(self.bvh.c), scene_flags(b))

    def new_frame(self):
        """Fresh per-pixel RNG states (seed = pixel index + 1) and a zeroed
        accumulation buffer."""
        w, h = self.width, self.height
        rng = torch.from_numpy(pixel_seeds(w, h).view(np.int32)).to(self.device)
        pix = torch.zeros((w * h, 4), dtype=torch.float32, device=self.device)
        return rng, pix

    def render(self, rng: torch.Tensor, pix: torch.Tensor, spp: int, max_depth: int = 100,
               ordered: bool = True, wavefront: bool = True, rows: tuple[int, int] | None = None) -> None:
        """Adds `spp` samples per pixel to `pix`.  wavefront=True (the
        default) runs the extend/shade/shadow kernel split, wavefront=False
        the megakernel (clr_render); the results are identical.
        rows=(y0, y1) renders those image rows only (wavefront form): `rng`
        and `pix` then hold just those rows."""
        cur = torch.cuda.current_stream(self.device)
        stream = C.c_void_p(cur.cuda_stream)
        flags = C.c_uint32(RENDER_ORDERED if ordered else 0)
        if rows is not None:
            y0, y1 = rows
            if rng.numel() < 4 * self.width * (y1 - y0) or pix.numel() < 4 * self.width * (y1 - y0):
                raise ValueError("rng / pix hold fewer than the band's pixels")
            with torch.cuda.device(self.device), self._workspace_turn(cur, self.workspace()) as ws:
                _lib.call("clr_render_wavefront_rows", C.byref(self.c), C.c_uint32(self.width), C.c_uint32(self.height),
                          C.c_uint32(y0), C.c_uint32(y1 - y0), C.c_void_p(rng.data_ptr()), C.c_void_p(pix.data_ptr()),
                          C.c_uint32(spp), C.c_uint32(max_depth), flags, C.c_void_p(ws.data_ptr()),
                          C.c_uint64(ws.numel()), stream)
            return
        args = (C.byref(self.c), C.c_uint32(self.width), C.c_uint32(self.height), C.c_void_p(rng.data_ptr()),
                C.c_void_p(pix.data_ptr()), C.c_uint32(spp), C.c_uint32(max_depth), flags)
        with torch.cuda.device(self.device):
            if not wavefront:
                _lib.call("clr_render", *args, stream)
                return
            with self._workspace_turn(cur, self.workspace()) as ws:
                _lib.call("clr_render_wavefront", *args, C.c_void_p(ws.data_ptr()), C.c_uint64(ws.numel()), stream)

    def render_counted(self, rng: torch.Tensor, pix: torch.Tensor, spp: int, max_depth: int = 100,
                       ordered: bool = True) -> dict:
        """clr_render (megakernel) that also counts what the paths visit:
        closest-hit and shadow rays, BVH nodes loaded, triangles tested,
        surface hits shaded.  Same image and RNG updates as render()."""
        counts = torch.zeros(5, dtype=torch.int64, device=self.device)
        stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        with torch.cuda.device(self.device):
            _lib.call("clr_render_counted", C.byref(self.c), C.c_uint32(self.width), C.c_uint32(self.height),
                      C.c_void_p(rng.data_ptr()), C.c_void_p(pix.data_ptr()), C.c_uint32(spp), C.c_uint32(max_depth),
                      C.c_uint32(RENDER_ORDERED if ordered else 0), C.c_void_p(counts.data_ptr()), stream)
        c = [int(v) for v in counts.cpu().tolist()]
        return {"rays": c[0], "shadow_rays": c[1], "nodes": c[2], "tris": c[3], "hits": c[4],
                "samples": self.width * self.height * int(spp)}

    def render_adjoint(self, rng: torch.Tensor, dloss: torch.Tensor, spp: int, max_depth: int,
                       param_tex: torch.Tensor, param_kind: torch.Tensor, grad: torch.Tensor,
                       env_tex: int | None = None, grad_env: torch.Tensor | None = None,
                       tape: torch.Tensor | None = None, tape_count: torch.Tensor | None = None,
                       ordered: bool = True, retrace: bool = False) -> None:
        """Adds sum_p dloss[p] . dAccum[p]/dtheta to `grad` (K x 4 float32) and
        `grad_env` (texels x 4) for the samples clr_render_wavefront would
        take from the same `rng` (advanced in place).  param_tex (int32) /
        param_kind (uint8) list the differentiated constant textures by their
        textures-blob offsets.  `tape` (records x 32 int32) with `tape_count`
        (1 int32, zeroed by the caller) records the replayed paths.
        retrace=True traces every replayed ray again (CLR_ADJOINT_RETRACE)
        instead of taking the primal pass's hits for the first 8 vertices."""
        K = int(param_tex.numel())
        p = _lib.ClrAdjointParams(
            param_tex.data_ptr() if K else None, param_kind.data_ptr() if K else None, K,
            grad.data_ptr() if K else None, NO_TEX if env_tex is None else int(env_tex),
            grad_env.data_ptr() if grad_env is not None else None,
            tape.data_ptr() if tape is not None else None, int(tape.shape[0]) if tape is not None else 0,
            tape_count.data_ptr() if tape_count is not None else None)
        cur = torch.cuda.current_stream(self.device)
        stream = C.c_void_p(cur.cuda_stream)
        with torch.cuda.device(self.device), self._workspace_turn(cur, self.adjoint_workspace(K)) as ws:
            _lib.call("clr_render_adjoint", C.byref(self.c), C.c_uint32(self.width), C.c_uint32(self.height),
                      C.c_void_p(rng.data_ptr()), C.c_void_p(dloss.data_ptr()), C.c_uint32(spp),
                      C.c_uint32(max_depth),
                      C.c_uint32((RENDER_ORDERED if ordered else 0) | (ADJOINT_RETRACE if retrace else 0)), C.byref(p),
                      C.c_void_p(ws.data_ptr()), C.c_uint64(ws.numel()), stream)

    def adjoint_workspace(self, num_params: int) -> torch.Tensor:
        n = C.c_uint64(0)
        _lib.call("clr_render_adjoint_workspace_bytes", C.c_uint32(self.width), C.c_uint32(self.height),
                  C.c_uint32(num_params), C.byref(n))
        cur = getattr(self, "_aws", None)
        if cur is None or cur.numel() < int(n.value):
            buf = torch.empty(int(n.value) + 256, dtype=torch.uint8, device=self.device)
            off = (-buf.data_ptr()) % 256
            self._aws = buf[off:off + int(n.value)]
        return self._aws

    def visualize_bvh(self, pix: torch.Tensor | None = None):
        """The reference's BVH visualiser image (the hit material's base colour
        plus 0.025 per accepted BVH box, one centred ray per pixel) added to
        `pix`, and the per-pixel box counts.  Returns (pix, visits)."""
        n = self.width * self.height
        if pix is None:
            pix = torch.zeros((n, 4), dtype=torch.float32, device=self.device)
        visits = torch.zeros(n, dtype=torch.int32, device=self.device)
        with torch.cuda.device(self.device):
            _lib.call("clr_bvh_visualize", C.byref(self.c), C.c_uint32(self.width), C.c_uint32(self.height),
                      C.c_void_p(pix.data_ptr()), C.c_void_p(visits.data_ptr()),
                      C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        return pix, visits

    def env_row_weights(self) -> torch.Tensor:
        """The zenith correction of each environment row as the scene encoder
        computes it (scene.zenith_weights), on the device (computed once)."""
        if getattr(self, "_env_weights", None) is None:
            self._env_weights = torch.from_numpy(zenith_weights(self.env_dist["height"])).to(self.device)
        return self._env_weights

    def update_env_distribution(self, row_weight: torch.Tensor | None = None, encoder_weights: bool = True) -> None:
        """Rebuilds the environment light's importance distribution on the
        device from the environment texels now in the textures blob (after an
        optimisation step changed them).  With encoder_weights the row weights
        are the scene encoder's, so the result equals re-encoding the scene."""
        if self.env_dist is None:
            raise ValueError("the scene has no image-based environment light")
        if row_weight is None and encoder_weights:
            row_weight = self.env_row_weights()
        d = self.env_dist
        with torch.cuda.device(self.device):
            _lib.call("clr_env_distribution_update", C.c_void_p(self.t["others"].data_ptr()),
                      C.c_uint32(d["dist_offset"]), C.c_void_p(self.t["textures"].data_ptr()),
                      C.c_uint32(d["tex_offset"]), C.c_uint32(d["height"]), C.c_uint32(d["width"]),
                      C.c_void_p(row_weight.data_ptr()) if row_weight is not None else None,
                      C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))

    @contextlib.contextmanager
    def _workspace_turn(self, stream: torch.cuda.Stream, ws: torch.Tensor):
        """Orders the uses of this scene's workspaces across streams: the
        call on `stream` starts after the last call that used a workspace of
        this scene (on whatever stream) has finished on the GPU, and the next
        call waits for this one.  Renders on two streams thus take turns
        instead of sharing the wavefront queues at the same time."""
        if self._ws_last_use is None:
            self._ws_last_use = torch.cuda.Event()
        else:
            stream.wait_event(self._ws_last_use)
        ws.record_stream(stream)
        try:
            yield ws
        finally:
            self._ws_last_use.record(stream)

    def workspace(self) -> torch.Tensor:
        if getattr(self, "_ws", None) is None:
            n = C.c_uint64(0)
            _lib.call("clr_render_workspace_bytes", C.c_uint32(self.width), C.c_uint32(self.height), C.byref(n))
            self._ws = torch.empty(int(n.value) + 256, dtype=torch.uint8, device=self.device)
            off = (-self._ws.data_ptr()) % 256
            self._ws = self._ws[off:off + int(n.value)]
        return self._ws

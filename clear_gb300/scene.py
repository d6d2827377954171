"""Scene description: the reference's byte-blob scene format, built on the host.

Mirrors ``Scene`` (OpenCL_PathTracer/Scene.h:29-295, Scene.cpp:12-42) and
``MaterialCreator`` (OpenCL_PathTracer/CreateFunctions.hpp:16-101,
CreateFunctions.cpp:18-505).  The blobs (materials, textures, "other
resources") have the reference's byte layout, read by the reference's render
kernel (OpenCL/pathtracer.cl:25-46) and by this project's CUDA path tracer
alike, so one encoder serves both.

Deliberate differences from the reference's host code, each a defect there:
  * The 2D environment distribution stores the marginal (row) distribution's
    PDF/CDF offsets relative to its embedded ContinuousConsts1D, which is the
    base the kernel adds them to (distribution.cl:296, 326); the reference
    stores them relative to the enclosing 2D head (CreateFunctions.cpp:309-310),
    8 bytes off.
  * The light-power PMF has numItems entries; the reference's loop writes one
    past the end (Scene.h:281-284).
  * The 2D environment distribution maps a black row (zero mass) to zero PDF
    and CDF values; the reference multiplies them by 1/0 and stores NaN.
  * createFloatCheckerBoardTexture tags its texture ColorProcedural as the
    reference does (CreateFunctions.cpp:117), so evaluateFloatTexture reads 0
    from it, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import math
import struct

import numpy as np

FACE_DTYPE = np.dtype([("p", "<u4", 3), ("vn", "<u4", 3), ("vt", "<u4", 3), ("uv", "<u4", 3),
                       ("alphaTexPtr", "<u4"), ("matPtr", "<u2"), ("lightPtr", "<u2")])
NONE32 = 0xFFFFFFFF
NONE16 = 0xFFFF

# TextureType (TextureStructures.hpp)
TEX_COLOR_CONSTANT, TEX_RGB8, TEX_RGBA8, TEX_RGBA16F, TEX_COLOR_PROCEDURAL, TEX_GRAY8, \
    TEX_FLOAT_CONSTANT, TEX_FLOAT_IMAGE, TEX_FLOAT_PROCEDURAL = range(9)
PROC_CHECKER, PROC_CHECKER_BUMP = 0, 1
FRESNEL_NOOP, FRESNEL_CONDUCTOR, FRESNEL_DIELECTRIC = 0, 1, 2
# MatElem (MaterialStructures.hpp)
ME_DIFFUSE, ME_SPEC_R, ME_SPEC_T, ME_NEWWARD, ME_ASH_S, ME_ASH_D = range(6)
LP_DIFFUSE = 0
ENV_IMAGE = 0


class Blob:
    """Growable byte vector with the alignment rules of CLUtil::addDataAligned
    / fillZerosAligned / align (CommonSources/clUtility.cpp:554-571)."""

    def __init__(self, initial: bytes = b""):
        self.b = bytearray(initial)

    def __len__(self):
        return len(self.b)

    def align(self, a: int) -> int:
        pad = (-len(self.b)) % a
        self.b.extend(b"\0" * pad)
        return len(self.b)

    def add(self, data: bytes, a: int) -> int:
        self.align(a)
        off = len(self.b)
        self.b.extend(data)
        return off

    def zeros(self, n: int, a: int) -> int:
        return self.add(b"\0" * n, a)

    def put(self, off: int, data: bytes):
        self.b[off:off + len(data)] = data

    def array(self) -> np.ndarray:
        out = np.zeros(max(len(self.b), 16), dtype=np.uint8)
        out[: len(self.b)] = np.frombuffer(bytes(self.b), dtype=np.uint8)
        return out


def _f3(x, y, z) -> bytes:
    return struct.pack("<4f", x, y, z, 0.0)


# ---------------------------------------------------------------- matrices
# 4x4 float32 matrices m[row, col] with the reference's arithmetic
# (LinearAlgebra/Matrix4f.hpp, LinearAlgebra.cpp:47-98): every product and sum
# is rounded to float in the order written there (sums left to right, no
# fused multiply-add), so that vertices and normals placed by a transform are
# the reference's bit for bit.  The blobs store them column-major, as the
# kernels read them (matrix.cl reads s048c as the first row).

_F = np.float32


_libm_handle = None


def _libm():
    """The C library's float functions (cosf, sinf, sqrtf), which the
    reference's host code calls."""
    global _libm_handle
    if _libm_handle is None:
        L = C.CDLL(ctypes.util.find_library("m"))
        for fn in ("cosf", "sinf", "sqrtf"):
            getattr(L, fn).argtypes = [C.c_float]
            getattr(L, fn).restype = C.c_float
        _libm_handle = L
    return _libm_handle


def identity():
    return np.eye(4, dtype=np.float32)


def translate(x, y, z):
    m = identity()
    m[:3, 3] = (_F(x), _F(y), _F(z))
    return m


def scale(x, y, z):
    m = identity()
    m[0, 0], m[1, 1], m[2, 2] = _F(x), _F(y), _F(z)
    return m


def rotate(angle, ax, ay, az):
    """RotateMatrix (LinearAlgebra.cpp:73-98): `angle` in radians, rounded to
    float as the reference's parameter is; cosf/sinf of the C library."""
    L = _libm()
    rx, ry, rz = _F(ax), _F(ay), _F(az)
    length = _F(L.sqrtf(float(rx * rx + ry * ry + rz * rz)))
    rx, ry, rz = rx / length, ry / length, rz / length
    a = float(_F(angle))
    c, s = _F(L.cosf(a)), _F(L.sinf(a))
    omc = _F(1) - c
    m = identity()
    m[0, 0] = rx * rx * omc + c
    m[1, 0] = rx * ry * omc + rz * s
    m[2, 0] = rz * rx * omc - ry * s
    m[0, 1] = rx * ry * omc - rz * s
    m[1, 1] = ry * ry * omc + c
    m[2, 1] = ry * rz * omc + rx * s
    m[0, 2] = rz * rx * omc + ry * s
    m[1, 2] = ry * rz * omc - rx * s
    m[2, 2] = rz * rz * omc + c
    return m


def mul(*ms):
    """Product of matrices left to right, each entry dot(row, column) summed
    left to right in float (Matrix4f::operator*, Matrix4f.hpp:193-213)."""
    out = np.asarray(ms[0], dtype=np.float32)
    for m in ms[1:]:
        m = np.asarray(m, dtype=np.float32)
        out = ((out[:, 0:1] * m[0:1, :] + out[:, 1:2] * m[1:2, :]) + out[:, 2:3] * m[2:3, :]) + \
            out[:, 3:4] * m[3:4, :]
    return out


def invert(m):
    """Matrix4f::Invert (Matrix4f.hpp:81-163): Gauss-Jordan elimination with
    full pivoting on the transposed matrix, in float; NaNs for a singular
    matrix."""
    inv = [[_F(m[j, i]) for j in range(4)] for i in range(4)]  # inverse[i][j] = m_ji
    col_idx, row_idx, piv = [0] * 4, [0] * 4, [-1] * 4
    icol = irow = 0
    for i in range(4):
        best = _F(0)
        for j in range(4):
            if piv[j] != 0:
                for k in range(4):
                    if piv[k] == -1:
                        v = abs(inv[j][k])
                        if v > best:
                            best, irow, icol = v, j, k
                    elif piv[k] > 0:
                        return np.asarray(m, dtype=np.float32).copy()
        piv[icol] += 1
        if irow != icol:
            inv[irow], inv[icol] = inv[icol], inv[irow]
        row_idx[i], col_idx[i] = irow, icol
        pivot = inv[icol][icol]
        if pivot == 0:
            return np.full((4, 4), np.nan, dtype=np.float32)
        one_over = _F(1) / pivot
        inv[icol][icol] = _F(1)
        inv[icol] = [x * one_over for x in inv[icol]]
        for j in range(4):
            if j != icol:
                f = inv[j][icol]
                inv[j][icol] = _F(0)
                inv[j] = [inv[j][k] - inv[icol][k] * f for k in range(4)]
    for i in range(3, -1, -1):
        ir, ic = row_idx[i], col_idx[i]
        for j in range(4):
            inv[j][ir], inv[j][ic] = inv[j][ic], inv[j][ir]
    out = np.empty((4, 4), dtype=np.float32)
    for c in range(4):
        for r in range(4):
            out[r, c] = inv[c][r]
    return out


def transform_points(m, p):
    """Matrix4f * Point3f (Matrix4f.hpp:247-256) for each row of p (n, 3)."""
    m = np.asarray(m, dtype=np.float32)
    p = np.asarray(p, dtype=np.float32).reshape(-1, 3)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    r = [((m[i, 0] * x + m[i, 1] * y) + m[i, 2] * z) + m[i, 3] for i in range(4)]
    nw = r[3]
    out = np.stack(r[:3], axis=1)
    keep = nw == _F(1)
    return np.where(keep[:, None], out, out / np.where(keep, _F(1), nw)[:, None])


def transform_vectors(m, v):
    """Matrix4f * Vector3f (Matrix4f.hpp:231-235): the upper 3x3 block."""
    m = np.asarray(m, dtype=np.float32)
    v = np.asarray(v, dtype=np.float32).reshape(-1, 3)
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    return np.stack([(m[i, 0] * x + m[i, 1] * y) + m[i, 2] * z for i in range(3)], axis=1)


def look_at(eye, target, up):
    """Camera-to-world transform of a camera at `eye` looking at `target`;
    the camera looks down its local -z axis."""
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = s, u, -f, eye
    return m


def _colmajor(m) -> bytes:
    return np.asarray(m, dtype=np.float32).T.reshape(-1).tobytes()


# --------------------------------------------------- environment rows

def zenith_weights(h: int) -> np.ndarray:
    """Row weights of the environment distribution, as
    CreateFunctions.cpp:275 computes them: cosf((float)(M_PI * (double)a))
    with a = 0.5f - (i + 0.5f) / h in float, through the C library's cosf."""
    cosf = _libm().cosf
    i = np.arange(h, dtype=np.float32)
    a = (np.float32(0.5) - (i + np.float32(0.5)) / np.float32(h)).astype(np.float32)
    arg = (math.pi * a.astype(np.float64)).astype(np.float32)
    return np.array([cosf(float(x)) for x in arg], dtype=np.float32)


# ------------------------------------------------------------------- scene


class _Rows:
    """Append-only table built from single rows or whole arrays."""

    def __init__(self, dtype, width=None):
        self.dtype, self.width = dtype, width
        self.parts, self.pending, self.n = [], [], 0

    def __len__(self):
        return self.n

    def _flush(self):
        if self.pending:
            a = np.array(self.pending, dtype=self.dtype)
            self.parts.append(a.reshape(-1, self.width) if self.width else a)
            self.pending = []

    def append(self, row):
        self.pending.append(row)
        self.n += 1

    def extend(self, arr):
        self._flush()
        arr = np.asarray(arr, dtype=self.dtype)
        self.parts.append(arr.reshape(-1, self.width) if self.width else arr)
        self.n += len(self.parts[-1])

    def array(self):
        self._flush()
        if not self.parts:
            shape = (0, self.width) if self.width else (0,)
            return np.zeros(shape, dtype=self.dtype)
        if len(self.parts) > 1:
            self.parts = [np.concatenate(self.parts)]
        return self.parts[0]


class _NameMap(dict):
    """Name -> blob offset with the reference's std::map::insert semantics
    (Scene.h:117-140): registering a name again keeps the first offset (the
    second record is still written to the blob)."""

    def __setitem__(self, key, value):
        if key not in self:
            super().__setitem__(key, value)


class Scene:
    def __init__(self):
        self.vertices = _Rows(np.float64, 3)
        self.normals = _Rows(np.float64, 3)
        self.tangents = _Rows(np.float64, 3)
        self.uvs = _Rows(np.float64, 2)
        self.faces = _Rows(FACE_DTYPE)
        self.light_infos: list = []   # (atInfinity, reference)
        self.light_powers: list = []
        self.materials = Blob()
        self.textures = Blob()
        self.others = Blob(b"\0" * 12)  # offsets of camera, environment, light distribution
        self.mat_ref, self.light_ref, self.tex_ref, self.other_ref = _NameMap(), _NameMap(), _NameMap(), _NameMap()
        self.tex_files = _NameMap()  # image file -> texture offset (texFilesDatabase)
        self.models: set = set()     # loaded model files (modelDatabase)
        self.local_to_world = [identity()]
        self._base = None
        self.mc = MaterialCreator(self)

    # Scene.h:62-81 -------------------------------------------------------
    def push(self, m=None):
        """Matrix4fStack::push, then `*= m` (Matrix4fStack.hpp:28-47)."""
        top = self.local_to_world[-1]
        self.local_to_world.append(mul(top, m) if m is not None else top.copy())

    def apply(self, m):
        """Matrix4fStack `*= m`: the top becomes top * m."""
        self.local_to_world[-1] = mul(self.local_to_world[-1], m)

    def pop(self):
        if len(self.local_to_world) > 1:
            self.local_to_world.pop()
        else:
            self.local_to_world[0] = identity()

    def add_vertex(self, x, y, z):
        self.vertices.append(transform_points(self.local_to_world[-1], [x, y, z])[0])

    def add_normal(self, x, y, z):
        self.normals.append(transform_vectors(invert(self.local_to_world[-1]).T, [x, y, z])[0])

    def add_tangent(self, x, y, z):
        self.tangents.append(transform_vectors(self.local_to_world[-1], [x, y, z])[0])

    def add_uv(self, u, v):
        self.uvs.append((u, v))

    def begin_object(self):
        self._base = (len(self.vertices), len(self.normals), len(self.tangents), len(self.uvs))

    def end_object(self):
        self._base = None

    def add_mesh(self, verts, tris, mat, uvs=None, normals=None, light=NONE16):
        """Bulk form of add_vertex/add_uv/add_normal/add_face for a whole
        mesh: verts (n,3) in object space (transformed by the current
        matrix), tris (m,3) object-relative vertex indices; uvs and normals,
        if given, are per vertex and indexed like the vertices."""
        m4 = self.local_to_world[-1]
        bv, bn, bu = len(self.vertices), len(self.normals), len(self.uvs)
        self.vertices.extend(transform_points(m4, verts))
        tris = np.asarray(tris, dtype=np.int64)
        f = np.zeros(len(tris), dtype=FACE_DTYPE)
        f["p"] = tris + bv
        f["vn"] = f["vt"] = f["uv"] = NONE32
        if normals is not None:
            self.normals.extend(transform_vectors(invert(m4).T, normals))
            f["vn"] = tris + bn
        if uvs is not None:
            self.uvs.extend(np.asarray(uvs, dtype=np.float64))
            f["uv"] = tris + bu
        f["alphaTexPtr"] = NONE32
        f["matPtr"] = mat
        f["lightPtr"] = light
        base_f = len(self.faces)
        self.faces.extend(f)
        if light != NONE16:
            for i in range(len(tris)):
                self.light_infos.append((0, base_f + i))
                self.light_powers.append(1.0)

    def add_face(self, p, mat, light=NONE16, uv=None, vn=None, vt=None, alpha_tex=NONE32):
        """Scene::addFace (Scene.h:82-116): indices are object-relative
        between begin_object/end_object; an emissive face registers a light of
        power 1."""
        bv, bn, bt, bu = self._base or (0, 0, 0, 0)
        f = np.zeros((), dtype=FACE_DTYPE)
        f["p"] = [i + bv for i in p]
        f["vn"] = [i + bn for i in vn] if vn is not None else [NONE32] * 3
        f["vt"] = [i + bt for i in vt] if vt is not None else [NONE32] * 3
        f["uv"] = [i + bu for i in uv] if uv is not None else [NONE32] * 3
        f["alphaTexPtr"] = alpha_tex
        f["matPtr"] = mat
        f["lightPtr"] = light
        self.faces.append(f)
        if light != NONE16:
            self.light_infos.append((0, len(self.faces) - 1))
            self.light_powers.append(1.0)

    # bulk forms of the four calls above, for whole arrays ------------------
    def add_vertices(self, p):
        """add_vertex for each row of p (n, 3)."""
        self.vertices.extend(transform_points(self.local_to_world[-1], p))

    def add_normals(self, n):
        """add_normal for each row of n (n, 3)."""
        self.normals.extend(transform_vectors(invert(self.local_to_world[-1]).T, n))

    def add_uvs(self, uv):
        self.uvs.extend(np.asarray(uv, dtype=np.float64).reshape(-1, 2))

    def add_faces(self, p, mat, light=NONE16, uv=None, vn=None, alpha_tex=NONE32):
        """add_face for each row of p (m, 3) (uv, vn likewise, or None), with
        one material, light and alpha texture for all of them."""
        bv, bn, bt, bu = self._base or (0, 0, 0, 0)
        p = np.asarray(p, dtype=np.int64).reshape(-1, 3)
        f = np.zeros(len(p), dtype=FACE_DTYPE)
        f["p"] = p + bv
        f["vn"] = np.asarray(vn, dtype=np.int64).reshape(-1, 3) + bn if vn is not None else NONE32
        f["vt"] = NONE32
        f["uv"] = np.asarray(uv, dtype=np.int64).reshape(-1, 3) + bu if uv is not None else NONE32
        f["alphaTexPtr"] = alpha_tex
        f["matPtr"] = mat
        f["lightPtr"] = light
        first = len(self.faces)
        self.faces.extend(f)
        if light != NONE16:
            self.light_infos.extend((0, first + i) for i in range(len(p)))
            self.light_powers.extend([1.0] * len(p))

    # Scene.h:140-152 -----------------------------------------------------
    def set_camera(self, width, height, cam_to_world, fov_y_deg=30.0, lens_radius=0.0, focus_dist=1.0):
        """PerspectiveInfo blob (main.cpp:52-90, camera.cl:28-35); the camera
        looks down its local -z axis."""
        aspect = width / height
        t = math.tan(math.radians(fov_y_deg) / 2)
        near, far = 1.0, 100.0
        clip_to_cam = np.linalg.inv(np.array([[1 / (aspect * t), 0, 0, 0], [0, 1 / t, 0, 0],
                                              [0, 0, -(far + near) / (far - near), -2 * far * near / (far - near)],
                                              [0, 0, -1, 0]]))
        raster_to_screen = np.array([[2.0 / width, 0, 0, -1], [0, -2.0 / height, 0, 1], [0, 0, 2, -1],
                                     [0, 0, 0, 1]])
        raster_to_cam = clip_to_cam @ raster_to_screen
        blob = bytearray(256)
        struct.pack_into("<II", blob, 0, width, height)
        blob[64:128] = _colmajor(cam_to_world)
        struct.pack_into("<B3xfff", blob, 128, 0, aspect * t * t, lens_radius, focus_dist)
        blob[192:256] = _colmajor(raster_to_cam)
        self.other_ref["Camera"] = self.others.add(bytes(blob), 64)
        self.width, self.height = width, height

    def set_environment(self, light_prop_name):
        self.other_ref["Environment"] = self.others.add(struct.pack("<I", self.light_ref[light_prop_name]), 4)
        self.light_infos.append((1, NONE32))
        self.light_powers.append(1.0)

    def calc_light_power_distribution(self):
        """Discrete1D over light powers (Scene.h:268-292)."""
        head = self.others.zeros(16, 4)
        p = np.asarray(self.light_powers, dtype=np.float32)
        cdf = np.zeros(len(p) + 1, dtype=np.float32)
        for i in range(1, len(cdf)):
            cdf[i] = np.float32(cdf[i - 1] + p[i - 1])
        total = cdf[-1]
        cdf = (cdf / total).astype(np.float32)
        pmf = (p / total).astype(np.float32)
        o_cdf = self.others.add(cdf.tobytes(), 4)
        o_pmf = self.others.add(pmf.tobytes(), 4)
        self.others.put(head, struct.pack("<B3xIii", 0, len(p), o_pmf - head, o_cdf - head))
        self.other_ref["LightPowerDistribution"] = head

    def build(self):
        """Scene::build (Scene.cpp:12-42) without the CPU BVH (the LBVH is
        built on the device)."""
        if "Environment" not in self.other_ref:
            self.mc.begin_light_property("Dark")
            self.mc.end_light_property()
            self.other_ref["Environment"] = self.others.add(struct.pack("<I", self.light_ref["Dark"]), 4)
        self.calc_light_power_distribution()
        self.others.put(0, struct.pack("<III", self.other_ref["Camera"], self.other_ref["Environment"],
                                       self.other_ref["LightPowerDistribution"]))

    def blobs(self) -> dict:
        def f4(v):
            a = np.zeros((max(len(v), 1), 4), dtype=np.float32)
            if len(v):
                a[: len(v), :3] = v.array().astype(np.float32)
            return a

        uv = np.zeros((max(len(self.uvs), 1), 2), dtype=np.float32)
        if len(self.uvs):
            uv[: len(self.uvs)] = self.uvs.array().astype(np.float32)
        lights = np.zeros((max(len(self.light_infos), 1), 2), dtype=np.uint32)
        for i, (inf, ref) in enumerate(self.light_infos):
            lights[i] = (inf, ref)
        return {"vertices": f4(self.vertices), "normals": f4(self.normals), "tangents": f4(self.tangents),
                "uvs": uv, "faces": self.faces.array(), "lights": lights,
                "materials": self.materials.array(), "textures": self.textures.array(),
                "others": self.others.array(), "num_lights": len(self.light_infos)}

    def soa(self):
        """Vertex SoA + triangle index array for the LBVH build."""
        v = self.vertices.array().astype(np.float32)
        f = self.faces.array()
        return (np.ascontiguousarray(v[:, 0]), np.ascontiguousarray(v[:, 1]), np.ascontiguousarray(v[:, 2]),
                np.ascontiguousarray(f["p"].reshape(-1)))


class MaterialCreator:
    """CreateFunctions.cpp:18-505 -- writes textures, materials, light
    properties and the structures they point to into the scene blobs."""

    def __init__(self, scene: Scene):
        self.s = scene
        self.num_bxdfs = 0
        self.num_eedfs = 0

    # textures ------------------------------------------------------------
    def float3_constant_texture(self, name, r, g, b):
        self.s.tex_ref[name] = self.s.textures.add(struct.pack("<B15x", TEX_COLOR_CONSTANT) + _f3(r, g, b), 16)

    def float_constant_texture(self, name, v):
        self.s.tex_ref[name] = self.s.textures.add(struct.pack("<B3xf", TEX_FLOAT_CONSTANT, v), 4)

    def image_texture(self, name, data: np.ndarray, kind: str):
        """kind: 'rgb8' (H,W,3 uint8), 'rgba8' (H,W,4 uint8), 'rgba16f'
        (H,W,4 float16), 'gray8' (H,W uint8), 'float' (H,W float32)."""
        t = self.s.textures
        h, w = data.shape[:2]
        head = t.zeros(16, 4)
        img = t.align(128)
        if kind == "rgb8":
            # 4 bytes per texel, the fourth 0xFF, as the reference's PNG reader
            # stores RGB (ImageLoader.cpp:161-162, png_set_filler)
            px = np.full((h, w, 4), 0xFF, dtype=np.uint8)
            px[..., :3] = data
            t.b.extend(px.tobytes())
            tt = TEX_RGB8
        elif kind == "rgba8":
            t.b.extend(np.ascontiguousarray(data, dtype=np.uint8).tobytes())
            tt = TEX_RGBA8
        elif kind == "rgba16f":
            t.b.extend(np.ascontiguousarray(data, dtype=np.float16).tobytes())
            tt = TEX_RGBA16F
        elif kind == "gray8":
            t.b.extend(np.ascontiguousarray(data, dtype=np.uint8).tobytes())
            tt = TEX_GRAY8
        elif kind == "float":
            t.b.extend(np.ascontiguousarray(data, dtype=np.float32).tobytes())
            tt = TEX_FLOAT_IMAGE
        else:
            raise ValueError(kind)
        t.put(head, struct.pack("<B3xIIi", tt, w, h, img - head))
        self.s.tex_ref[name] = head
        return head

    def normal_map_texture(self, name, rgb8: np.ndarray):
        self.image_texture(name, rgb8, "rgb8")

    def float3_checkerboard_texture(self, name, c0, c1):
        self.s.tex_ref[name] = self.s.textures.add(
            struct.pack("<BB14x", TEX_COLOR_PROCEDURAL, PROC_CHECKER) + _f3(*c0) + _f3(*c1), 16)

    def float3_checkerboard_bump_texture(self, name, width=0.01, reverse=False):
        self.s.tex_ref[name] = self.s.textures.add(
            struct.pack("<BB2xfB3x", TEX_COLOR_PROCEDURAL, PROC_CHECKER_BUMP, width, int(reverse)), 4)

    def float_checkerboard_texture(self, name, v0, v1):
        self.s.tex_ref[name] = self.s.textures.add(
            struct.pack("<BB2xff", TEX_COLOR_PROCEDURAL, PROC_CHECKER, v0, v1), 4)

    # fresnel (other resources) -------------------------------------------
    def fresnel_noop(self, name):
        self.s.other_ref[name] = self.s.others.add(struct.pack("<B", FRESNEL_NOOP), 1)

    def fresnel_conductor(self, name, eta, k):
        self.s.other_ref[name] = self.s.others.add(struct.pack("<B15x", FRESNEL_CONDUCTOR) + _f3(*eta) + _f3(*k), 16)

    def fresnel_dielectric(self, name, eta_ext, eta_int):
        self.s.other_ref[name] = self.s.others.add(struct.pack("<B3xff", FRESNEL_DIELECTRIC, eta_ext, eta_int), 4)

    # environment distribution --------------------------------------------
    def continuous_consts_2d_h(self, name, rgb: np.ndarray, zenith_correction=True):
        """ContinuousConsts2D_H over an equirectangular image, one stratum
        per texel, rows weighted by sin(theta) (CreateFunctions.cpp:246-349)."""
        o = self.s.others
        h, w = rgb.shape[:2]
        head = o.zeros(36, 4)
        p_pdf = o.zeros(4 * h, 4)
        p_cdf = o.zeros(4 * (h + 1), 4)
        children = o.zeros(28 * h, 4)
        c_pdfs = o.zeros(4 * w * h, 4)
        c_cdfs = o.zeros(4 * (w + 1) * h, 4)
        rgb = np.asarray(rgb, dtype=np.float32)
        lum = (np.float32(0.2126) * rgb[..., 0] + np.float32(0.7152) * rgb[..., 1] +
               np.float32(0.0722) * rgb[..., 2]).astype(np.float32)
        # averageLuminance (CreateFunctions.cpp:159-244) of a one-texel stratum:
        # the texel is added once per corner of the stratum, weight 1 each, and
        # the sum divided by the stratum's area, 1
        lum = ((lum + lum) + lum) + lum
        width_c = np.float32(1.0) / np.float32(w)
        corr = zenith_weights(h) if zenith_correction else np.ones(h, dtype=np.float32)
        pdf = (lum * corr[:, None]).astype(np.float32)
        # running sums in float32, left to right, as the reference's loop
        cdf = np.zeros((h, w + 1), dtype=np.float32)
        cdf[:, 1:] = np.cumsum((pdf * width_c).astype(np.float32), axis=1, dtype=np.float32)
        row_mass = cdf[:, w].copy()
        with np.errstate(divide="ignore"):
            norm = np.where(row_mass > 0, np.float32(1.0) / row_mass, np.float32(0)).astype(np.float32)
        pdf = (pdf * norm[:, None]).astype(np.float32)
        cdf[:, 1:] = (cdf[:, 1:] * norm[:, None]).astype(np.float32)
        for i in range(h):
            ch = children + 28 * i
            o.put(ch, struct.pack("<B3xIfffii", 1, w, 0.0, 1.0, float(width_c),
                                  c_pdfs + 4 * w * i - ch, c_cdfs + 4 * (w + 1) * i - ch))
        o.put(c_pdfs, pdf.tobytes())
        o.put(c_cdfs, cdf.tobytes())
        width_p = np.float32(1.0) / np.float32(h)
        pcdf = np.zeros(h + 1, dtype=np.float32)
        pcdf[1:] = np.cumsum((row_mass * width_p).astype(np.float32), dtype=np.float32)
        norm = np.float32(1.0) / pcdf[h]
        ppdf = (row_mass * norm).astype(np.float32)
        pcdf[1:] = (pcdf[1:] * norm).astype(np.float32)
        o.put(p_pdf, ppdf.tobytes())
        o.put(p_cdf, pcdf.tobytes())
        parent = head + 8  # the embedded ContinuousConsts1D the kernel offsets from
        o.put(head, struct.pack("<B3xi", 2, children - head) +
              struct.pack("<B3xIfffii", 1, h, 0.0, 1.0, float(width_p), p_pdf - parent, p_cdf - parent))
        self.s.other_ref[name] = head

    # materials -----------------------------------------------------------
    def begin_material(self, name, bump=None):
        m = self.s.materials
        self.num_bxdfs = 0
        self.mat_head = m.add(b"\0", 1)
        assert self.mat_head % 4 == 0, "MaterialInfo must start 4-byte aligned"
        self.s.mat_ref[name] = self.mat_head
        m.add(struct.pack("<B", bump is not None), 1)
        m.add(struct.pack("<I", self.s.tex_ref[bump] if bump is not None else 0), 4)

    def end_material(self):
        assert self.num_bxdfs > 0
        self.s.materials.b[self.mat_head] = self.num_bxdfs

    def _elem(self, data: bytes):
        self.num_bxdfs += 1
        self.s.materials.align(4)
        self.s.materials.b.extend(data)

    def diffuse_elem(self, R, sigma):
        self._elem(struct.pack("<B3xII", ME_DIFFUSE, self.s.tex_ref[R], self.s.tex_ref[sigma]))

    def specular_r_elem(self, R, fresnel):
        self._elem(struct.pack("<B3xII", ME_SPEC_R, self.s.tex_ref[R], self.s.other_ref[fresnel]))

    def specular_t_elem(self, T, eta_ext, eta_int, mat_name):
        fname = "internalFresnelDielectric_" + mat_name
        self.fresnel_dielectric(fname, eta_ext, eta_int)
        self._elem(struct.pack("<B3xIffI", ME_SPEC_T, self.s.tex_ref[T], eta_ext, eta_int, self.s.other_ref[fname]))

    def newward_elem(self, R, ax, ay):
        self._elem(struct.pack("<B3xIII", ME_NEWWARD, self.s.tex_ref[R], self.s.tex_ref[ax], self.s.tex_ref[ay]))

    def ashikhmin_s_elem(self, Rs, nu, nv):
        self._elem(struct.pack("<B3xIII", ME_ASH_S, self.s.tex_ref[Rs], self.s.tex_ref[nu], self.s.tex_ref[nv]))

    def ashikhmin_d_elem(self, Rd, Rs):
        self._elem(struct.pack("<B3xII", ME_ASH_D, self.s.tex_ref[Rs], self.s.tex_ref[Rd]))

    def matte_material(self, name, bump, R, sigma):
        self.begin_material(name, bump)
        self.diffuse_elem(R, sigma)
        self.end_material()

    def glass_material(self, name, bump, R, T, eta_ext, eta_int):
        self.begin_material(name, bump)
        fname = "GlassInternalFresnelDielectric_" + name
        self.fresnel_dielectric(fname, eta_ext, eta_int)
        self.specular_r_elem(R, fname)
        self.specular_t_elem(T, eta_ext, eta_int, name)
        self.end_material()

    def metal_material(self, name, bump, R, eta, k):
        self.begin_material(name, bump)
        fname = "MetalInternalFresnelConductor_" + name
        self.fresnel_conductor(fname, eta, k)
        self.specular_r_elem(R, fname)
        self.end_material()

    def newward_material(self, name, bump, R, ax, ay):
        self.begin_material(name, bump)
        self.newward_elem(R, ax, ay)
        self.end_material()

    def ashikhmin_material(self, name, bump, Rs, Rd, nu, nv):
        self.begin_material(name, bump)
        self.ashikhmin_s_elem(Rs, nu, nv)
        self.ashikhmin_d_elem(Rd, Rs)
        self.end_material()

    # light properties ----------------------------------------------------
    def begin_light_property(self, name):
        self.num_eedfs = 0
        self.lit_head = self.s.materials.add(b"\0", 1)
        self.s.light_ref[name] = self.lit_head

    def end_light_property(self):
        self.s.materials.b[self.lit_head] = self.num_eedfs

    def diffuse_light_property(self, name, M):
        self.begin_light_property(name)
        self.num_eedfs += 1
        self.s.materials.align(4)
        self.s.materials.b.extend(struct.pack("<B3xI", LP_DIFFUSE, self.s.tex_ref[M]))
        self.end_light_property()

    def image_based_env_light_property(self, name, radiance_tex, rgb: np.ndarray, multiplier=1.0):
        """rgb: the texture's texels as float (H,W,3) for the importance
        distribution (the reference reads the same texels as half floats)."""
        dname = "InternalDistribution2D_" + radiance_tex
        self.continuous_consts_2d_h(dname, rgb, True)
        h, w = np.asarray(rgb).shape[:2]
        # where the device rebuild of this distribution finds its inputs
        self.s.env_dist = {"dist_offset": self.s.other_ref[dname], "tex_offset": self.s.tex_ref[radiance_tex],
                           "width": w, "height": h}
        self.begin_light_property(name)
        self.num_eedfs += 1
        self.s.materials.align(4)
        self.s.materials.b.extend(struct.pack("<B3xIfI", ENV_IMAGE, self.s.tex_ref[radiance_tex], multiplier,
                                              self.s.other_ref[dname]))
        self.end_light_property()

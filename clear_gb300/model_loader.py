"""Wavefront .obj models into a scene: ``loadModel`` / ``OBJ::load``
(ModelLoader.cpp:155-495, 495-508) over the native parser ``clr_obj_parse``
(csrc/obj_parse.cpp, which states the line rules).

What a load adds to the scene, in the reference's order:

* per .mtl material, named ``"%05u_<name>"`` with the model number (the
  reference's process-wide ``OBJ::objID``, ModelLoader.cpp:32, 404-405):
  ``Ni == 1`` gives a matte material over ``<name>_Kd`` (the ``map_Kd`` image,
  else the constant ``Kd``) and a zero ``<name>_Kd_sigma``; any other ``Ni``
  gives a glass material with constant 0.95 reflectance and transmittance
  and ``eta_ext = Ni, eta_int = 1`` (ModelLoader.cpp:407-432);
* all positions, uvs and normals of the file, then per group its faces, with
  the group's material (a ``usemtl`` name the .mtl does not define takes the
  first material), no light, and the ``<name>_Kd`` image as alpha texture
  when it has an alpha channel (ModelLoader.cpp:434-485).  ``mat_override``
  / ``light_override`` replace the material and light of every face.

Image files go through ``image_reader(path) -> (array, kind)`` with ``kind``
as ``MaterialCreator.image_texture`` takes it.  The reference decodes PNG
with libpng and EXR with OpenEXR, which are not part of this build; the
default reader, ``read_image``, decodes binary netpbm (PGM, PPM, PAM) and
``.npy`` arrays.  An image file is decoded once per scene
(``Scene.tex_files``), as the reference's texture-file database does.

Differences from the reference, all where its behaviour is undefined or
silently wrong: a file with no ``o`` line loads (the reference dereferences a
null object); the extension is the text after the LAST dot (the reference
takes the first, so ``./dir/a.obj`` fails there); a missing file raises
instead of printing; a material offset that does not fit the face record's
16-bit material field raises instead of wrapping.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .scene import NONE16, NONE32, TEX_RGBA8, TEX_RGBA16F, Scene

_next_model_id = 0  # OBJ::objID: numbers the models this process loads


@dataclass
class ObjModel:
    """One parsed .obj with its .mtl materials (see ``clr_obj_parse``)."""
    positions: np.ndarray          # (P, 3) float32
    uvs: np.ndarray                # (U, 2) float32, v already flipped
    normals: np.ndarray            # (N, 3) float32
    faces: np.ndarray              # (F, 9) uint32: p0..2, uv0..2, n0..2
    groups: list = field(default_factory=list)     # dicts: first_face, num_faces, format, smooth, name, material
    materials: list = field(default_factory=list)  # dicts: name, Kd, Ks, Ka, Ns, Ni, map_Kd, map_Ks, map_Ka
    skipped: int = 0


def parse_obj(path: str | os.PathLike) -> ObjModel:
    L = _lib.lib()
    h = C.c_void_p()
    _lib.call("clr_obj_parse", os.fsencode(path), C.byref(h))
    try:
        n = _lib.ClrObjCounts()
        _lib.call("clr_obj_counts_of", h, C.byref(n))
        ptrs = [C.c_void_p() for _ in range(7)]
        _lib.call("clr_obj_data", h, *(C.byref(p) for p in ptrs))
        pos, uv, nrm, fc, grp, mat, strs = ptrs

        def arr(p, count, width, dtype):
            if count == 0:
                return np.zeros((0, width), dtype=dtype)
            nbytes = count * width * np.dtype(dtype).itemsize
            return np.frombuffer(C.string_at(p, nbytes), dtype=dtype).reshape(count, width).copy()

        table = C.string_at(strs, n.string_bytes) if n.string_bytes else b"\0"

        def text(off):
            return table[off:table.index(b"\0", off)].decode("utf-8", errors="surrogateescape")

        groups = []
        if n.num_groups:
            for g in (_lib.ClrObjGroup * n.num_groups).from_address(grp.value):
                groups.append({"first_face": g.first_face, "num_faces": g.num_faces, "format": g.format,
                               "smooth": g.smooth, "name": text(g.name), "material": text(g.material)})
        materials = []
        if n.num_materials:
            for m in (_lib.ClrObjMaterial * n.num_materials).from_address(mat.value):
                materials.append({"name": text(m.name), "Kd": tuple(m.Kd), "Ks": tuple(m.Ks), "Ka": tuple(m.Ka),
                                  "Ns": m.Ns, "Ni": m.Ni, "map_Kd": text(m.map_Kd), "map_Ks": text(m.map_Ks),
                                  "map_Ka": text(m.map_Ka)})
        return ObjModel(arr(pos, n.num_positions, 3, np.float32), arr(uv, n.num_uvs, 2, np.float32),
                        arr(nrm, n.num_normals, 3, np.float32), arr(fc, n.num_faces, 9, np.uint32), groups,
                        materials, n.num_skipped)
    finally:
        L.clr_obj_free(h)


# ------------------------------------------------------------------ images


def _pnm_tokens(data: bytes, pos: int):
    while True:
        while pos < len(data) and (data[pos:pos + 1].isspace() or data[pos] == ord("#")):
            if data[pos] == ord("#"):
                pos = data.index(b"\n", pos) if b"\n" in data[pos:] else len(data)
            else:
                pos += 1
        start = pos
        while pos < len(data) and not data[pos:pos + 1].isspace() and data[pos] != ord("#"):
            pos += 1
        if start == pos:
            return
        yield data[start:pos].decode("ascii"), pos


def read_image(path: str) -> tuple[np.ndarray, str]:
    """Binary PGM (gray8), PPM (rgb8), PAM with 1, 3 or 4 channels, all 8-bit;
    .npy arrays of uint8 (h, w[, 3|4]), float16 (h, w, 4) -> rgba16f, or
    float32 (h, w) -> float."""
    if str(path).endswith(".npy"):
        a = np.load(path)
        if a.dtype == np.float16 and a.ndim == 3 and a.shape[2] == 4:
            return a, "rgba16f"
        if a.dtype == np.float32 and a.ndim == 2:
            return a, "float"
        if a.dtype == np.uint8:
            kind = {2: "gray8"}.get(a.ndim) or {3: "rgb8", 4: "rgba8"}.get(a.shape[2])
            if kind:
                return a, kind
        raise ValueError(f"{path}: unsupported array {a.dtype} {a.shape}")
    data = open(path, "rb").read()
    magic = data[:2]
    hdr = {}
    if magic in (b"P5", b"P6"):
        it = _pnm_tokens(data, 2)
        (w, _), (h, _), (maxval, pos) = next(it), next(it), next(it)
        hdr = {"WIDTH": w, "HEIGHT": h, "MAXVAL": maxval, "DEPTH": "1" if magic == b"P5" else "3"}
    elif magic == b"P7":
        it = _pnm_tokens(data, 2)
        for key, pos in it:
            if key == "ENDHDR":
                break
            hdr[key], pos = next(it)
    else:
        raise ValueError(f"{path}: not a binary netpbm image or .npy array (PNG/EXR decoding is not built in; "
                         "pass image_reader=)")
    w, h, depth = int(hdr["WIDTH"]), int(hdr["HEIGHT"]), int(hdr["DEPTH"])
    if int(hdr["MAXVAL"]) != 255 or depth not in (1, 3, 4):
        raise ValueError(f"{path}: only 8-bit images with 1, 3 or 4 channels are read")
    px = np.frombuffer(data, dtype=np.uint8, count=w * h * depth, offset=pos + 1)
    if depth == 1:
        return px.reshape(h, w).copy(), "gray8"
    return px.reshape(h, w, depth).copy(), "rgb8" if depth == 3 else "rgba8"


# ------------------------------------------------------------------ loading


def _image_texture(scene: Scene, name: str, path: str, image_reader) -> None:
    """MaterialCreator::createImageTexture (CreateFunctions.cpp:38-70)."""
    if path in scene.tex_files:
        scene.tex_ref[name] = scene.tex_files[path]
        return
    data, kind = image_reader(path)
    scene.tex_files[path] = scene.mc.image_texture(name, data, kind)


def _u16(v: int, what: str) -> int:
    if not 0 <= v <= 0xFFFF:
        raise ValueError(f"{what} {v} does not fit the face record's 16-bit field")
    return v


def load_model(file_name: str | os.PathLike, scene: Scene, mat_override: int | None = None,
               light_override: int | None = None, image_reader=read_image, model_id: int | None = None) -> int:
    """loadModel (ModelLoader.cpp:495-508) for .obj files: adds the model to
    `scene` and returns its model number (the material-name prefix).
    Raises on a missing file or an extension other than .obj."""
    global _next_model_id
    path = os.fspath(file_name)
    if os.path.splitext(path)[1] != ".obj":
        raise ValueError(f"{path}: only .obj models are read")
    obj = parse_obj(path)
    num = _next_model_id if model_id is None else model_id
    prefix = f"{num:05d}_"
    mc = scene.mc
    for m in obj.materials:
        name = prefix + m["name"]
        if np.float32(m["Ni"]) == np.float32(1.0):
            kd = name + "_Kd"
            if m["map_Kd"]:
                _image_texture(scene, kd, m["map_Kd"], image_reader)
            else:
                mc.float3_constant_texture(kd, *m["Kd"])
            mc.float_constant_texture(name + "_Kd_sigma", 0.0)
            mc.matte_material(name, None, kd, name + "_Kd_sigma")
        else:
            mc.float3_constant_texture(name + "_Reflectance", 0.95, 0.95, 0.95)
            mc.float3_constant_texture(name + "_Transmittance", 0.95, 0.95, 0.95)
            mc.glass_material(name, None, name + "_Reflectance", name + "_Transmittance", m["Ni"], 1.0)

    first_index = {}
    for i, m in enumerate(obj.materials):
        first_index.setdefault(m["name"], i)
    if not obj.materials and mat_override is None and any(g["num_faces"] for g in obj.groups):
        raise ValueError(f"{path}: faces but no materials (no .mtl material and no mat_override)")

    scene.begin_object()
    scene.add_vertices(obj.positions)
    scene.add_uvs(obj.uvs)
    scene.add_normals(obj.normals)
    light = NONE16 if light_override is None else _u16(light_override, "light offset")
    for g in obj.groups:
        if g["num_faces"] == 0:
            continue
        alpha = NONE32
        mat = None
        if obj.materials:
            m = obj.materials[first_index.get(g["material"], 0)]
            mat_name = prefix + m["name"]
            if np.float32(m["Ni"]) == np.float32(1.0) and m["map_Kd"]:
                head = scene.tex_ref[mat_name + "_Kd"]
                if scene.textures.b[head] in (TEX_RGBA8, TEX_RGBA16F):
                    alpha = head
            if mat_override is None:
                mat = scene.mat_ref[mat_name]
        mat = _u16(mat if mat_override is None else mat_override, "material offset")
        f = obj.faces[g["first_face"]:g["first_face"] + g["num_faces"]].astype(np.int64)
        fmt = g["format"]
        uv = f[:, 3:6] if fmt in (_lib.OBJ_VTN, _lib.OBJ_VT) else None
        vn = f[:, 6:9] if fmt in (_lib.OBJ_VTN, _lib.OBJ_VN) else None
        scene.add_faces(f[:, 0:3], mat, light, uv=uv, vn=vn, alpha_tex=alpha)
    scene.end_object()
    scene.models.add(path)
    if model_id is None:
        _next_model_id += 1
    return num


__all__ = ["ObjModel", "parse_obj", "read_image", "load_model"]

"""The scene encoders (clear_gb300/scene.py) and the .obj loader
(clear_gb300/model_loader.py over csrc/obj_parse.cpp) against the reference's
own Scene / MaterialCreator / loadModel: the command scripts of
tests/golden/make_golden_scene.py replayed through this package give the same
blobs and name maps, byte for byte, as the golden fixtures the reference
produced (and as the reference itself, where its checkout is present).

One difference is intended and adjusted for: the 2D environment
distribution's parent PDF/CDF offsets are stored relative to the embedded 1D
record the kernels add them to, 8 bytes after the reference's base.
"""
import ctypes
import json
import os
import struct
import sys

import numpy as np
import pytest

import oracle
from clear_gb300 import _lib, model_loader
from clear_gb300 import scene as S
from clear_gb300.scene import Scene

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_scene as G  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "scene_blobs.npz"))
_libc = ctypes.CDLL(None)
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
_libc.strtof.restype = ctypes.c_float


def F(text) -> np.float32:
    """A number of a script as the reference's harness reads it (strtof)."""
    return np.float32(_libc.strtof(str(text).encode(), None))


def _texels(s: Scene, name: str) -> np.ndarray:
    head = s.tex_ref[name]
    _, w, h, rel = struct.unpack_from("<B3xIIi", s.textures.b, head)
    px = np.frombuffer(bytes(s.textures.b[head + rel:head + rel + 8 * w * h]), dtype=np.float16)
    return px.reshape(h, w, 4)[..., :3].astype(np.float32)


def run_ours(script: str, objdir: str, model_ids) -> tuple[Scene, list]:
    """Replays a command script (oracle/ref_scene.cpp's commands) through
    this package; returns the scene and the 2D distributions it created."""
    s, ids, dists = Scene(), iter(model_ids), []
    mc = s.mc
    bump = lambda x: None if x == "-" else x  # noqa: E731
    for line in script.strip().splitlines():
        a = line.replace("<obj>", objdir).split()
        c, v = a[0], [F(x) if x.lstrip("-").replace(".", "", 1).isdigit() else x for x in a[1:]]
        if c == "f3tex":
            mc.float3_constant_texture(a[1], *v[1:4])
        elif c == "ftex":
            mc.float_constant_texture(a[1], v[1])
        elif c == "imgtex":
            model_loader._image_texture(s, a[1], a[2], model_loader.read_image)
        elif c == "nrmtex":
            mc.normal_map_texture(a[1], model_loader.read_image(a[2])[0])
        elif c == "checker3":
            mc.float3_checkerboard_texture(a[1], v[1:4], v[4:7])
        elif c == "checkerbump":
            mc.float3_checkerboard_bump_texture(a[1], v[1], a[3] != "0")
        elif c == "checker1":
            mc.float_checkerboard_texture(a[1], v[1], v[2])
        elif c == "fresnel_noop":
            mc.fresnel_noop(a[1])
        elif c == "fresnel_cond":
            mc.fresnel_conductor(a[1], v[1:4], v[4:7])
        elif c == "fresnel_diel":
            mc.fresnel_dielectric(a[1], v[1], v[2])
        elif c == "matte":
            mc.matte_material(a[1], bump(a[2]), a[3], a[4])
        elif c == "glass":
            mc.glass_material(a[1], bump(a[2]), a[3], a[4], v[4], v[5])
        elif c == "metal":
            mc.metal_material(a[1], bump(a[2]), a[3], v[3:6], v[6:9])
        elif c == "newward":
            mc.newward_material(a[1], bump(a[2]), a[3], a[4], a[5])
        elif c == "ashikhmin":
            mc.ashikhmin_material(a[1], bump(a[2]), a[3], a[4], a[5], a[6])
        elif c == "diffuse_light":
            mc.diffuse_light_property(a[1], a[2])
        elif c == "ibl_light":
            mc.image_based_env_light_property(a[1], a[2], _texels(s, a[2]), v[2])
            dists.append("InternalDistribution2D_" + a[2])
        elif c == "cc2d":
            mc.continuous_consts_2d_h(a[1], _texels(s, a[2]), a[3] != "0")
            dists.append(a[1])
        elif c == "vertex":
            s.add_vertex(*v)
        elif c == "normal":
            s.add_normal(*v)
        elif c == "uv":
            s.add_uv(*v)
        elif c == "light_dist":
            s.calc_light_power_distribution()
        elif c == "push":
            s.push()
        elif c == "pop":
            s.pop()
        elif c == "translate":
            s.apply(S.translate(*v))
        elif c == "scale":
            s.apply(S.scale(*v))
        elif c == "rotate":
            s.apply(S.rotate(*v))
        elif c == "obj":
            model_loader.load_model(a[1], s, None, None, model_id=next(ids))
        elif c == "objn":
            mat = None if a[2] == "-" else s.mat_ref[a[2]]
            light = None if a[3] == "-" else s.light_ref[a[3]]
            model_loader.load_model(a[1], s, mat, light, model_id=next(ids))
        else:
            raise ValueError(line)
    return s, dists


def ours_blobs(s: Scene) -> dict:
    def f4(rows):
        a = rows.array().astype(np.float32)
        out = np.zeros((len(a), 4), dtype=np.float32)
        out[:, :a.shape[1]] = a
        return out.view(np.uint8).reshape(-1)

    lights = b"".join(struct.pack("<B3xI", inf, ref) for inf, ref in s.light_infos)
    return {"vertices": f4(s.vertices), "normals": f4(s.normals), "tangents": f4(s.tangents),
            "uvs": s.uvs.array().astype(np.float32).view(np.uint8).reshape(-1),
            "faces": s.faces.array().view(np.uint8).reshape(-1), "lights": np.frombuffer(lights, np.uint8),
            "materials": np.frombuffer(bytes(s.materials.b), np.uint8),
            "textures": np.frombuffer(bytes(s.textures.b), np.uint8),
            "others": np.frombuffer(bytes(s.others.b), np.uint8),
            "light_powers": np.array(s.light_powers, dtype=np.float32).view(np.uint8)}


def ours_names(s: Scene, objdir: str) -> dict:
    def clean(d):
        return {k.replace(objdir, "<obj>"): int(v) for k, v in d.items()}

    return {"materials": clean(s.mat_ref), "light_props": clean(s.light_ref), "textures": clean(s.tex_ref),
            "others": clean(s.other_ref), "tex_files": clean(s.tex_files)}


def compare(s: Scene, dists, ref_blobs: dict, ref_names: dict, objdir: str) -> None:
    ours = ours_blobs(s)
    names = ours_names(s, objdir)
    assert names == ref_names
    for k in ("vertices", "normals", "uvs"):  # float equality: +0 and -0 compare equal
        a, b = ours[k].view(np.float32), ref_blobs[k].view(np.float32)
        assert a.shape == b.shape and np.array_equal(a, b), k
    ref_others = ref_blobs["others"].copy()
    for name in dists:  # the parent's offsets are relative to the embedded 1D record
        head = names["others"][name]
        for off in (head + 28, head + 32):
            v = struct.unpack_from("<i", ref_others, off)[0]
            struct.pack_into("<i", ref_others, off, v - 8)
    ref = dict(ref_blobs, others=ref_others)
    for k in ("tangents", "faces", "lights", "materials", "textures", "others", "light_powers"):
        assert ours[k].tobytes() == ref[k].tobytes(), k


def golden(name: str):
    blobs = {k: GOLDEN[f"{name}/{k}"] for k in oracle.SCENE_BLOBS}
    return blobs, json.loads(str(GOLDEN[f"{name}/names"])), GOLDEN[f"{name}/model_ids"].tolist()


@pytest.mark.parametrize("name", list(G.SCRIPTS))
def test_encoders_and_loader_match_reference_golden(name):
    blobs, names, ids = golden(name)
    s, dists = run_ours(G.SCRIPTS[name], G.OBJ_DIR, ids)
    compare(s, dists, blobs, names, G.OBJ_DIR)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not available")
@pytest.mark.parametrize("name", list(G.SCRIPTS))
def test_encoders_and_loader_match_reference_live(name, tmp_path):
    """The same against the reference built here, on assets written afresh
    to another directory (paths and model numbers differ from the golden)."""
    G.write_assets(str(tmp_path))
    blobs, names, ids = G.run_reference(G.SCRIPTS[name], str(tmp_path))
    s, dists = run_ours(G.SCRIPTS[name], str(tmp_path), ids)
    compare(s, dists, blobs, names, str(tmp_path))


# ------------------------------------------------------------- the parser


def test_parser_reads_the_reference_line_rules():
    m = model_loader.parse_obj(os.path.join(G.OBJ_DIR, "scene1.obj"))
    assert len(m.positions) == 10 and len(m.uvs) == 6 and len(m.normals) == 4
    assert m.positions[8].tolist() == [9, 9, 9] and m.positions[9].tolist() == [1, 2, 3]  # stripped ' ' / 't'
    assert m.uvs[4].tolist() == [0.25, np.float32(1.0) - np.float32(0.75)]  # 1 - v
    # groups: runs of f lines with the g / s / usemtl state at their first line
    got = [(g["name"], g["material"], g["smooth"], g["format"], g["num_faces"]) for g in m.groups]
    assert got == [("walls", "red", 0, _lib.OBJ_VTN, 3), ("walls", "textured", 0, _lib.OBJ_VTN, 1),
                   ("top", "alpha", 1, _lib.OBJ_VN, 2), ("top", "alpha", 1, _lib.OBJ_VN, 1),
                   ("top", "glass", 1, _lib.OBJ_VTN, 1), ("top", "nothere", 1, _lib.OBJ_VTN, 1),
                   ("top", "bumpy", 3, _lib.OBJ_VTN, 1), ("top", "bumpy", 3, _lib.OBJ_VTN, 1)]
    assert m.skipped == 0
    # a quad keeps its first three corners; indices are 0-based p, uv, n
    assert m.faces[2].tolist() == [0, 1, 4, 0, 1, 2, 1, 1, 2]
    # forward reference to vertices 9 and 10 (defined later in the file)
    assert m.faces[6].tolist()[:3] == [8, 9, 5] and m.faces[6].tolist()[3:6] == [0xFFFFFFFF] * 3
    mats = {x["name"]: x for x in m.materials}
    assert list(mats) == ["red", "textured", "alpha", "glass", "two", "bumpy"]
    assert mats["red"]["Kd"] == tuple(F(x) for x in ("0.63", "0.065", "0.05")) and mats["red"]["Ni"] == 1.0
    assert mats["alpha"]["Kd"] == (0.0, 0.0, 0.0)  # its Kd line is tab-indented
    assert mats["two"]["Kd"] == (0.0, 0.0, 0.0)    # fewer than three numbers
    assert mats["glass"]["Ni"] == F(1.5) and mats["red"]["Ns"] == 100.0  # Ns is not read
    assert mats["bumpy"]["map_Kd"].endswith("/tex_rgb.ppm")  # map_bump sets the Kd map


def test_parser_defines_what_the_reference_leaves_undefined(tmp_path):
    p = tmp_path / "loose.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1\n"  # no `o`; a vertex with a missing component
                 "f 1 2 3\n"            # v-only format
                 "f -3 -2 -1\n"         # relative indices
                 "f 1 2 99\n"           # index past the list: skipped
                 "f 1/1 2/1 3/1\n"      # v/t line in a v-only run: skipped
                 "\n"
                 "f 1/1 2/1 3/1\n"      # a new run in v/t format, uv 1 never defined: skipped
                 "vn 0 0 1\n"
                 "f 1//1 2//1 3//1 4//1\n")
    m = model_loader.parse_obj(p)
    assert m.positions[3].tolist() == [1, 1, 0]
    assert [g["format"] for g in m.groups] == [_lib.OBJ_V, _lib.OBJ_VT, _lib.OBJ_VN]
    assert m.faces[:, :3].tolist() == [[0, 1, 2], [1, 2, 3], [0, 1, 2]]
    assert m.faces[0, 3:].tolist() == [0xFFFFFFFF] * 6
    assert m.skipped == 3 and m.materials == []


def test_parser_and_loader_errors(tmp_path):
    with pytest.raises(_lib.ClrError):
        model_loader.parse_obj(tmp_path / "missing.obj")
    p = tmp_path / "nomat.obj"
    p.write_text("o a\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    with pytest.raises(ValueError):  # faces but no material to give them
        model_loader.load_model(p, Scene())
    s = Scene()
    s.mc.float3_constant_texture("R", 0.5, 0.5, 0.5)
    s.mc.float_constant_texture("z", 0.0)
    s.mc.matte_material("m", None, "R", "z")
    model_loader.load_model(p, s, mat_override=s.mat_ref["m"], model_id=7)
    assert s.faces.array()["matPtr"].tolist() == [s.mat_ref["m"]] and s.faces.array()["p"].tolist() == [[0, 1, 2]]
    with pytest.raises(ValueError):
        model_loader.load_model(p, s, mat_override=1 << 16)
    with pytest.raises(ValueError):
        model_loader.load_model(tmp_path / "x.ply", s)
    (tmp_path / "t.png").write_bytes(b"\x89PNG")
    with pytest.raises(ValueError):
        model_loader.read_image(str(tmp_path / "t.png"))


def test_model_numbers_count_up():
    s = Scene()
    path = os.path.join(G.OBJ_DIR, "scene2.obj")
    a = model_loader.load_model(path, s)
    b = model_loader.load_model(path, s)
    assert b == a + 1 and f"{a:05d}_plain" in s.mat_ref and f"{b:05d}_plain" in s.mat_ref
    assert path in s.models

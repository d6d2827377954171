"""Golden scene blobs from the reference's own scene encoders and .obj loader.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_scene.py

Writes the synthetic test assets under tests/golden/obj/ (two .obj/.mtl
pairs that exercise the reference's parsing rules, netpbm textures and an
RGBA16F environment map as .npy) and scene_blobs.npz: for each command script
of SCRIPTS (the commands are listed in oracle/ref_scene.cpp) the blobs and
name maps that the reference's Scene / MaterialCreator / loadModel produce,
and the model numbers its .obj loads used.  ``<obj>`` in a script stands for
the asset directory; file paths in the name maps are stored with that prefix.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OBJ_DIR = os.path.join(HERE, "obj")
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

SCENE1_OBJ = """# synthetic model: objects, groups, v/t/n and v//n faces, a quad, a
# tab-indented face (ignored), a CR line end, forward references, a usemtl
# name the library does not define, and lines with stripped leading bytes
mtllib scene1.mtl
o first
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 0.5 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
vn 0 0 -1
vn 0.6 0.8 0
g walls
usemtl red\r
s off
f 1/1/1 2/2/1 3/3/1
f 1/1/1 3/3/1 4/4/1
f 1/1/2 2/2/2 5/3/3 4/4/3
\tf 1/1/1 2/2/1 3/3/1
usemtl textured
f 2/2/1 3/3/1 5/4/3
g top
s 1
usemtl alpha
f 3//1 4//2 5//3
f 5//3 4//2 1//1
o second
f 9//4 10//4 6//4
v 2 0 0
v 3 0 0
v 3 1 0
vn 0 1 0
vt 0.25 0.75
usemtl glass
f 6/5/4 7/5/4 8/5/4
usemtl nothere
f 8/5/4 7/5/4 6/5/4
g
usemtl bumpy
s 3
f 6/5/4 8/5/4 7/5/4
  v 9 9 9
tv 1 2 3
vt 0.5 0.25
f 9/6/4 10/6/4 8/6/4"""

SCENE1_MTL = """# materials: constant and image diffuse, RGBA alpha map, glass, a Kd
# with two numbers, a tab-indented statement (ignored), map_bump
newmtl red
Kd 0.63 0.065 0.05
Ks 0.1 0.1 0.1
Ns 50
Ni 1.0
newmtl textured
Kd 0.5 0.5 0.5
map_Kd tex_rgb.ppm
newmtl alpha
map_Kd tex_rgba.pam
\tKd 0.9 0.9 0.9
newmtl glass
Ni 1.5
Kd 1 1 1
newmtl two
Kd 0.2 0.4
newmtl bumpy
map_Kd tex_gray.pgm
map_bump tex_rgb.ppm
"""

SCENE2_OBJ = """mtllib scene2.mtl
o tri
v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0
vn 0 0 1
f 1//1 2//1 3//1
f 2//1 4//1 3//1
"""

SCENE2_MTL = "newmtl plain\nKd 0.25 0.5 0.75\n"

SCRIPTS = {
    "materials": """f3tex R 0.625 0.0625 0.046875
f3tex Rs 0.03125 0.03125 0.03125
ftex sigma 0.25
ftex rough 0.1875
ftex nu 40
checker3 chk 0.125 0.25 0.375 0.75 0.875 0.9375
checkerbump bump 0.015625 1
checker1 chk1 0.25 0.75
fresnel_noop fn
fresnel_cond fc 0.15625 0.375 1.5 3.9375 2.625 1.9375
fresnel_diel fd 1 1.5
matte m1 - R sigma
matte m2 bump R sigma
glass g1 - R Rs 1 1.5
metal met - R 0.15625 0.375 1.5 3.9375 2.625 1.9375
newward nw - R rough rough
ashikhmin ash - Rs R nu nu
f3tex Le 10 10 10
diffuse_light light Le
vertex 0.5 -1.25 2
normal 0 0 1
uv 0.25 0.75
""",
    "images": """imgtex rgb <obj>/tex_rgb.ppm
imgtex rgba <obj>/tex_rgba.pam
imgtex gray <obj>/tex_gray.pgm
imgtex rgb_again <obj>/tex_rgb.ppm
nrmtex nrm <obj>/tex_rgb.ppm
imgtex env <obj>/env.npy
cc2d dist_flat env 0
cc2d dist_zenith env 1
ibl_light sky env 2.5
""",
    "obj": """obj <obj>/scene1.obj - -
obj <obj>/scene2.obj - -
""",
    "transforms": """push
translate 0.25 -0.5 1.5
rotate 0.52359879 0 1 0
scale 0.25 0.5 0.25
vertex 1 2 3
vertex -0 0.1 -7.25
normal 0 0 1
normal 0.6 0.8 0
push
rotate -0.9424778 0.3 1 0.2
translate 1 0 0
scale 1 -2 0.5
obj <obj>/scene1.obj - -
pop
pop
pop
vertex 1 2 3
normal 0.6 0.8 0
""",
    "obj_override": """f3tex Le 4 4 4
diffuse_light lamp Le
ftex s0 0
f3tex R 0.5 0.5 0.5
matte base - R s0
objn <obj>/scene2.obj base lamp
light_dist
""",
}


def write_assets(d: str = OBJ_DIR) -> None:
    os.makedirs(d, exist_ok=True)
    for name, text in (("scene1.obj", SCENE1_OBJ), ("scene1.mtl", SCENE1_MTL), ("scene2.obj", SCENE2_OBJ),
                       ("scene2.mtl", SCENE2_MTL)):
        with open(os.path.join(d, name), "wb") as f:
            f.write(text.encode())
    rng = np.random.default_rng(7)
    rgb = rng.integers(0, 256, size=(3, 4, 3), dtype=np.uint8)
    with open(os.path.join(d, "tex_rgb.ppm"), "wb") as f:
        f.write(b"P6\n# test texture\n4 3\n255\n" + rgb.tobytes())
    rgba = rng.integers(0, 256, size=(2, 2, 4), dtype=np.uint8)
    with open(os.path.join(d, "tex_rgba.pam"), "wb") as f:
        f.write(b"P7\nWIDTH 2\nHEIGHT 2\nDEPTH 4\nMAXVAL 255\nTUPLTYPE RGB_ALPHA\nENDHDR\n" + rgba.tobytes())
    gray = rng.integers(0, 256, size=(2, 3), dtype=np.uint8)
    with open(os.path.join(d, "tex_gray.pgm"), "wb") as f:
        f.write(b"P5 3 2 255\n" + gray.tobytes())
    env = np.ones((16, 32, 4), dtype=np.float16)
    env[..., :3] = rng.uniform(0.05, 8.0, size=(16, 32, 3)).astype(np.float16)
    np.save(os.path.join(d, "env.npy"), env)


def run_reference(script: str, objdir: str = OBJ_DIR):
    """Blobs, name maps and model numbers of `script` run through the
    reference (oracle.RefScene)."""
    import oracle

    r = oracle.RefScene()
    ids = []
    for line in script.strip().splitlines():
        if line.split()[0] in ("obj", "objn"):
            ids.append(r.next_model_id)
        r.exec(line.replace("<obj>", objdir))
    blobs = {k: np.frombuffer(r.blob(k), dtype=np.uint8).copy() for k in oracle.SCENE_BLOBS}
    names = {k: {n.replace(objdir, "<obj>"): v for n, v in r.names(k).items()} for k in oracle.SCENE_NAMES}
    return blobs, names, ids


def main() -> None:
    write_assets()
    out = {}
    for name, script in SCRIPTS.items():
        blobs, names, ids = run_reference(script)
        for k, v in blobs.items():
            out[f"{name}/{k}"] = v
        out[f"{name}/names"] = np.array(json.dumps(names))
        out[f"{name}/model_ids"] = np.array(ids, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "scene_blobs.npz"), **out)
    print("wrote", os.path.join(HERE, "scene_blobs.npz"), "and", OBJ_DIR)


if __name__ == "__main__":
    main()

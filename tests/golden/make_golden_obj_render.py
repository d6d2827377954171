"""Golden image of a scene loaded from .obj files, from the reference's own
CPU renderer.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_obj_render.py

Writes tests/golden/obj_render/ (room.obj / room.mtl: three walls and a floor
in three matte materials; sphere.obj: a UV sphere with uvs and normals in a
glass material; lamp.obj: a quad loaded with a material and a light
override) and render_obj.npz: ``sim::pathtracing``
(OpenCL_PathTracer/Equivalent/sim_pathtracer.hpp, depth cap 100) over the
oracle-built LBVH of the scene ``build_scene`` makes from those files with
clear_gb300.model_loader, per-pixel XORShift128 streams seeded with pixel
index + 1.  A SHA-256 of the scene blobs pins the encoding.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ASSETS = os.path.join(HERE, "obj_render")
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

W = H = 64
SPP = 32


def _fmt(x: float) -> str:
    return f"{x:.6f}".rstrip("0").rstrip(".") if x != 0 else "0"


def write_assets(d: str = ASSETS) -> None:
    os.makedirs(d, exist_ok=True)
    room = ["mtllib room.mtl", "o room"]
    quads = {  # material: corners (counter-clockwise seen from inside), normal
        "white": [((-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)), (0, 1, 0)],
        "back": [((-1, 0, -1), (-1, 1, -1), (1, 1, -1), (1, 0, -1)), (0, 0, 1)],
        "red": [((-1, 0, 1), (-1, 1, 1), (-1, 1, -1), (-1, 0, -1)), (1, 0, 0)],
        "green": [((1, 0, -1), (1, 1, -1), (1, 1, 1), (1, 0, 1)), (-1, 0, 0)],
    }
    for k, (corners, nrm) in enumerate(quads.values()):
        room += [f"v {' '.join(_fmt(c) for c in p)}" for p in corners]
        room.append(f"vn {' '.join(_fmt(c) for c in nrm)}")
    for k, name in enumerate(quads):
        b = 4 * k + 1
        room += [f"g {name}", f"usemtl {'white' if name == 'back' else name}",
                 f"f {b}//{k + 1} {b + 1}//{k + 1} {b + 2}//{k + 1}",
                 f"f {b}//{k + 1} {b + 2}//{k + 1} {b + 3}//{k + 1}"]
    mtl = ["newmtl white", "Kd 0.75 0.75 0.75", "newmtl red", "Kd 0.63 0.065 0.05",
           "newmtl green", "Kd 0.14 0.45 0.091", "newmtl glass", "Ni 1.5"]
    nu, nv, r, c = 16, 8, 0.3, (0.0, 0.35, -0.1)
    sph = ["mtllib room.mtl", "o sphere"]
    for j in range(nv + 1):
        th = math.pi * j / nv
        for i in range(nu + 1):
            ph = 2 * math.pi * i / nu
            n = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            sph.append(f"v {_fmt(c[0] + r * n[0])} {_fmt(c[1] + r * n[1])} {_fmt(c[2] + r * n[2])}")
            sph.append(f"vt {_fmt(i / nu)} {_fmt(j / nv)}")
            sph.append(f"vn {_fmt(n[0])} {_fmt(n[1])} {_fmt(n[2])}")
    sph.append("usemtl glass")
    for j in range(nv):
        for i in range(nu):
            a, b = j * (nu + 1) + i + 1, j * (nu + 1) + i + 2
            cc, dd = a + nu + 1, b + nu + 1
            if j > 0:
                sph.append(f"f {a}/{a}/{a} {b}/{b}/{b} {dd}/{dd}/{dd}")
            if j < nv - 1:
                sph.append(f"f {a}/{a}/{a} {dd}/{dd}/{dd} {cc}/{cc}/{cc}")
    lamp = ["o lamp", "v -0.25 0.99 -0.25", "v 0.25 0.99 -0.25", "v 0.25 0.99 0.25", "v -0.25 0.99 0.25",
            "vn 0 -1 0", "f 1//1 3//1 2//1", "f 1//1 4//1 3//1"]
    for name, lines in (("room.obj", room), ("room.mtl", mtl), ("sphere.obj", sph), ("lamp.obj", lamp)):
        with open(os.path.join(d, name), "w") as fh:
            fh.write("\n".join(lines) + "\n")


def build_scene(d: str = ASSETS, width: int = W, height: int = H):
    from clear_gb300 import model_loader
    from clear_gb300 import scene as S

    sc = S.Scene()
    mc = sc.mc
    model_loader.load_model(os.path.join(d, "room.obj"), sc, model_id=0)
    model_loader.load_model(os.path.join(d, "sphere.obj"), sc, model_id=1)
    mc.float3_constant_texture("M_lamp", 12.0 * math.pi, 12.0 * math.pi, 12.0 * math.pi)
    mc.diffuse_light_property("lamp", "M_lamp")
    model_loader.load_model(os.path.join(d, "lamp.obj"), sc, mat_override=sc.mat_ref["00000_white"],
                            light_override=sc.light_ref["lamp"], model_id=2)
    sc.set_camera(width, height, S.look_at((0.0, 0.5, 2.4), (0.0, 0.45, 0.0), (0, 1, 0)), fov_y_deg=40.0)
    sc.build()
    return sc


def main() -> None:
    import oracle
    from clear_gb300 import scenes
    from make_golden_render import blob_hash

    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    write_assets()
    sc = build_scene()
    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    rng = scenes.pixel_seeds(W, H)
    pix = np.zeros((W * H, 4), dtype=np.float32)
    oracle.ref_render(b, ob.inodes, ob.lnodes, rng, pix, W, H, 0, H, SPP)
    np.savez_compressed(os.path.join(HERE, "render_obj.npz"), width=W, height=H, spp=SPP, image=pix[:, :3].copy(),
                        hash=blob_hash(b))
    print("wrote render_obj.npz", float(pix[:, :3].mean()), len(sc.faces), "triangles")


if __name__ == "__main__":
    main()

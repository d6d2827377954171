"""Golden image of a scene holding every material and texture kind, from the
reference's own CPU renderer.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_zoo.py

Writes render_zoo.npz: ``sim::pathtracing`` (OpenCL_PathTracer/Equivalent/
sim_pathtracer.hpp, depth cap 100) over the oracle-built LBVH of the scene
``build_scene`` makes, per-pixel XORShift128 streams seeded with pixel index
+ 1.  The scene: a floor with a colour checkerboard and the checkerboard bump
texture, eight spheres -- a conductor, a dielectric, Ward with a float-image
roughness, Ashikhmin over an RGB8 image, Lambertian with an RGB8 normal map,
Lambertian with an RGBA8 image, Oren-Nayar with a Gray8 roughness image and
Oren-Nayar with the float checkerboard as roughness -- a quad light, an
RGBA16F environment map and a thin-lens camera.  A SHA-256 of the blobs pins
the encoding.

The renderer is the reference's CPU renderer with the one line where it
departs from the reference's OpenCL kernel put back as the kernel has it: the
bump frame's rotation axis is normalised (OpenCL/reflection.cl:210;
Equivalent/sim_reflection.hpp omits it), oracle/_ref/libref_lbvh_kbump.so.

The reference's MaterialCreator tags the float checkerboard as a colour
procedural texture, which its float-texture evaluation does not handle: it
reads 0 (as a Ward roughness that gives NaN; as an Oren-Nayar sigma, a
Lambertian surface).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

W = H = 64
SPP = 32


def build_scene(width: int = W, height: int = H):
    from clear_gb300 import scenes
    from clear_gb300 import scene as S

    rng = np.random.default_rng(21)
    sc = S.Scene()
    mc = sc.mc
    # textures
    mc.float3_checkerboard_texture("floor_R", (0.8, 0.8, 0.75), (0.2, 0.25, 0.3))
    mc.float3_checkerboard_bump_texture("floor_bump", 0.02, False)
    mc.image_texture("ward_ax", rng.uniform(0.1, 0.4, size=(8, 8)).astype(np.float32), "float")
    mc.float_constant_texture("ward_ay", 0.15)
    mc.float_checkerboard_texture("sigma_checker", 0.1, 0.5)
    mc.image_texture("rgb_img", rng.integers(0, 256, size=(16, 16, 3), dtype=np.uint8), "rgb8")
    mc.image_texture("rgba_img", rng.integers(0, 256, size=(16, 16, 4), dtype=np.uint8), "rgba8")
    mc.image_texture("gray_sigma", rng.integers(0, 256, size=(8, 8), dtype=np.uint8), "gray8")
    mc.normal_map_texture("nmap", scenes.normal_map(32, 5))
    mc.float3_constant_texture("white", 0.75, 0.75, 0.75)
    mc.float3_constant_texture("gold", 0.95, 0.8, 0.45)
    mc.float3_constant_texture("one", 1.0, 1.0, 1.0)
    mc.float3_constant_texture("coat_rs", 0.04, 0.04, 0.04)
    mc.float_constant_texture("coat_n", 60.0)
    mc.float_constant_texture("sigma0", 0.0)
    mc.float_constant_texture("sigma3", 0.3)
    # materials
    mc.matte_material("floor", "floor_bump", "floor_R", "sigma0")
    mc.metal_material("metal", None, "gold", (0.2, 0.9, 1.1), (3.9, 2.4, 2.2))
    mc.glass_material("glass", None, "one", "one", 1.0, 1.5)
    mc.newward_material("ward", None, "white", "ward_ax", "ward_ay")
    mc.ashikhmin_material("coat", None, "coat_rs", "rgb_img", "coat_n", "coat_n")
    mc.matte_material("bumped", "nmap", "white", "sigma0")
    mc.matte_material("rgba", None, "rgba_img", "sigma3")
    mc.matte_material("on_gray", None, "white", "gray_sigma")
    mc.matte_material("on_float", None, "gold", "sigma_checker")
    mc.matte_material("lamp", None, "white", "sigma0")  # the lamp has no uvs: no textures on it
    mc.float3_constant_texture("M_light", 6.0 * math.pi, 6.0 * math.pi, 6.0 * math.pi)
    mc.diffuse_light_property("light", "M_light")
    # floor y = 0 over [-2, 2]^2, uvs tiled 4x
    sc.begin_object()
    for x, z in ((-2.0, -2.0), (2.0, -2.0), (2.0, 2.0), (-2.0, 2.0)):
        sc.add_vertex(x, 0.0, z)
        sc.add_uv((x + 2.0), (z + 2.0))
    sc.add_face((0, 2, 1), sc.mat_ref["floor"], uv=(0, 2, 1))
    sc.add_face((0, 3, 2), sc.mat_ref["floor"], uv=(0, 3, 2))
    sc.end_object()
    names = ("metal", "glass", "ward", "coat", "bumped", "rgba", "on_gray", "on_float")
    for k, name in enumerate(names):
        x = -1.2 + 0.8 * (k % 4)
        z = -0.5 + 0.9 * (k // 4)
        scenes._uv_sphere(sc, sc.mat_ref[name], (x, 0.3, z), 0.3, seg=24, rings=12)
    # quad light above, facing down
    sc.begin_object()
    for x, z in ((-0.5, -0.5), (0.5, -0.5), (0.5, 0.5), (-0.5, 0.5)):
        sc.add_vertex(x, 2.5, z)
    sc.add_face((0, 1, 2), sc.mat_ref["lamp"], light=sc.light_ref["light"])
    sc.add_face((0, 2, 3), sc.mat_ref["lamp"], light=sc.light_ref["light"])
    sc.end_object()
    env = np.exp(rng.normal(0.0, 0.7, size=(8, 16, 3))).astype(np.float32) * 0.4
    rgba = np.ones((8, 16, 4), dtype=np.float16)
    rgba[..., :3] = env.astype(np.float16)
    mc.image_texture("env", rgba, "rgba16f")
    mc.image_based_env_light_property("IBL", "env", rgba[..., :3].astype(np.float32), 1.0)
    sc.set_environment("IBL")
    sc.set_camera(width, height, S.look_at((0.0, 1.6, 3.2), (0.0, 0.3, 0.0), (0, 1, 0)), fov_y_deg=45.0,
                  lens_radius=0.02, focus_dist=3.3)
    sc.build()
    return sc


def main() -> None:
    import oracle
    from clear_gb300 import scenes
    from make_golden_render import blob_hash

    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    sc = build_scene()
    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    pix = np.zeros((W * H, 4), dtype=np.float32)
    oracle.ref_render(b, ob.inodes, ob.lnodes, scenes.pixel_seeds(W, H), pix, W, H, 0, H, SPP, bump_as_kernel=True)
    np.savez_compressed(os.path.join(HERE, "render_zoo.npz"), width=W, height=H, spp=SPP, image=pix[:, :3].copy(),
                        hash=blob_hash(b))
    print("wrote render_zoo.npz", float(pix[:, :3].mean()), len(sc.faces), "triangles")


if __name__ == "__main__":
    main()

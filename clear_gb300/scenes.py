"""Procedural benchmark scenes in the reference's scene format.

``cornell_box()`` is the small path-tracing workload: a unit-cube room with
five walls (red left, green right, white floor/ceiling/back; open front),
two boxes rotated 15 and -18 degrees about y, a 32x16 UV sphere with a
two-layer coat-over-diffuse material, and a 0.25 x 0.25 quad light under the
ceiling with radiance 15.  The coat uses the reference's own layered material
(createAshikhminMaterial: AshikhminS specular lobe over AshikhminD diffuse,
CreateFunctions.cpp:457-462) with Rs = 0.04 (IOR 1.5 at normal incidence) and
Phong exponent 2/roughness^2 - 2 (roughness 0.1).  Optionally a small
equirectangular environment map adds fill light.
"""
from __future__ import annotations

import math

import numpy as np

from . import scene as S


def _box(sc: S.Scene, mat, center, size, angle_deg):
    m = S.translate(*center) @ S.rotate(math.radians(angle_deg), 0, 1, 0) @ S.scale(*size)
    sc.push(m)
    sc.begin_object()
    for x in (-0.5, 0.5):
        for y in (-0.5, 0.5):
            for z in (-0.5, 0.5):
                sc.add_vertex(x, y, z)
    # vertex index = 4*ix + 2*iy + iz; faces wound counter-clockwise seen from outside
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    for a, b, c, d in quads:
        sc.add_face((a, b, c), mat)
        sc.add_face((a, c, d), mat)
    sc.end_object()
    sc.pop()


def _uv_sphere(sc: S.Scene, mat, center, radius, seg=32, rings=16):
    sc.begin_object()
    for j in range(rings + 1):
        th = math.pi * j / rings
        for i in range(seg + 1):
            ph = 2 * math.pi * i / seg
            n = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            sc.add_vertex(center[0] + radius * n[0], center[1] + radius * n[1], center[2] + radius * n[2])
            sc.add_normal(*n)
            sc.add_uv(i / seg, j / rings)
    row = seg + 1
    for j in range(rings):
        for i in range(seg):
            a, b, c, d = j * row + i, j * row + i + 1, (j + 1) * row + i, (j + 1) * row + i + 1
            if j != 0:
                sc.add_face((a, b, c), mat, uv=(a, b, c), vn=(a, b, c))
            if j != rings - 1:
                sc.add_face((b, d, c), mat, uv=(b, d, c), vn=(b, d, c))
    sc.end_object()


def cornell_box(width=256, height=256, env: np.ndarray | None = None, env_multiplier=1.0,
                albedos=None, roughness=0.1) -> S.Scene:
    sc = S.Scene()
    mc = sc.mc
    alb = albedos or {"red": (0.63, 0.06, 0.06), "green": (0.14, 0.45, 0.09), "white": (0.73, 0.73, 0.73),
                      "base": (0.8, 0.8, 0.8)}
    for k, v in alb.items():
        mc.float3_constant_texture("R_" + k, *v)
    mc.float_constant_texture("sigma0", 0.0)
    for k in ("red", "green", "white"):
        mc.matte_material("mat_" + k, None, "R_" + k, "sigma0")
    # coat over diffuse (AshikhminS + AshikhminD)
    n_exp = 2.0 / (roughness * roughness) - 2.0
    mc.float3_constant_texture("Rs_coat", 0.04, 0.04, 0.04)
    mc.float_constant_texture("n_coat", n_exp)
    mc.ashikhmin_material("mat_coat", None, "Rs_coat", "R_base", "n_coat", "n_coat")
    mc.float3_constant_texture("M_light", 15.0 * math.pi, 15.0 * math.pi, 15.0 * math.pi)
    mc.diffuse_light_property("light", "M_light")
    mat = {k: sc.mat_ref["mat_" + k] for k in ("red", "green", "white", "coat")}
    # room: floor y=0, ceiling y=1, back z=0, left x=0, right x=1; inward normals
    sc.begin_object()
    for x in (0.0, 1.0):
        for y in (0.0, 1.0):
            for z in (0.0, 1.0):
                sc.add_vertex(x, y, z)
    V = lambda x, y, z: 4 * x + 2 * y + z  # noqa: E731
    walls = [
        ((V(0, 0, 0), V(1, 0, 0), V(1, 0, 1), V(0, 0, 1)), "white"),  # floor, normal +y
        ((V(0, 1, 0), V(0, 1, 1), V(1, 1, 1), V(1, 1, 0)), "white"),  # ceiling, normal -y
        ((V(0, 0, 0), V(0, 1, 0), V(1, 1, 0), V(1, 0, 0)), "white"),  # back, normal +z
        ((V(0, 0, 0), V(0, 0, 1), V(0, 1, 1), V(0, 1, 0)), "red"),    # left, normal +x
        ((V(1, 0, 0), V(1, 1, 0), V(1, 1, 1), V(1, 0, 1)), "green"),  # right, normal -x
    ]
    for (a, b, c, d), m in walls:
        sc.add_face((a, b, c), mat[m])
        sc.add_face((a, c, d), mat[m])
    sc.end_object()
    # light quad under the ceiling, facing down
    sc.begin_object()
    for x, z in ((0.375, 0.375), (0.625, 0.375), (0.625, 0.625), (0.375, 0.625)):
        sc.add_vertex(x, 0.999, z)
    sc.add_face((0, 1, 2), mat["white"], light=sc.light_ref["light"])
    sc.add_face((0, 2, 3), mat["white"], light=sc.light_ref["light"])
    sc.end_object()
    _box(sc, mat["white"], (0.72, 0.3, 0.33), (0.27, 0.6, 0.27), -18.0)
    _box(sc, mat["white"], (0.70, 0.14, 0.76), (0.25, 0.28, 0.25), 15.0)
    _uv_sphere(sc, mat["coat"], (0.3, 0.25, 0.6), 0.2)
    if env is not None:
        h, w = env.shape[:2]
        rgba = np.ones((h, w, 4), dtype=np.float16)
        rgba[..., :3] = env.astype(np.float16)
        mc.image_texture("env", rgba, "rgba16f")
        mc.image_based_env_light_property("IBL", "env", rgba[..., :3].astype(np.float32), env_multiplier)
        sc.set_environment("IBL")
    cam = S.look_at((0.5, 0.5, 2.35), (0.5, 0.5, 0.0), (0, 1, 0))
    sc.set_camera(width, height, cam, fov_y_deg=38.0)
    sc.build()
    return sc


def pixel_seeds(width: int, height: int) -> np.ndarray:
    """Per-pixel XORShift128 states, seed = pixel index + 1, expanded as the
    reference does (main.cpp:101-104): s = 1812433253*(s ^ (s >> 30)) + k."""
    s = np.arange(1, width * height + 1, dtype=np.uint64)
    out = np.zeros((width * height, 4), dtype=np.uint32)
    m = np.uint64(0xFFFFFFFF)
    for k in range(4):
        s = (np.uint64(1812433253) * (s ^ (s >> np.uint64(30))) + np.uint64(k)) & m
        out[:, k] = s.astype(np.uint32)
    return out

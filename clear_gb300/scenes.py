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
    m = S.mul(S.translate(*center), S.rotate(math.radians(angle_deg), 0, 1, 0), S.scale(*size))
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


# Differentiable Cornell box: 8 materials, each with one colour (albedo) and
# one float (roughness) constant texture.  Kinds: "matte" = Oren-Nayar
# diffuse (roughness = sigma), "plastic" = diffuse + Ward coat (roughness =
# ax = ay, coat colour 0.04), "ashikhmin" = Ashikhmin-Shirley coat over a
# diffuse base (roughness = the exponent nu = nv, coat colour 0.04).
ADJ_MATERIALS = [  # (surface, kind, albedo, roughness)
    ("left", "matte", (0.63, 0.06, 0.06), 0.3),
    ("right", "matte", (0.14, 0.45, 0.09), 0.3),
    ("floor", "plastic", (0.73, 0.73, 0.73), 0.15),
    ("ceiling", "matte", (0.75, 0.75, 0.75), 0.2),
    ("back", "matte", (0.70, 0.70, 0.68), 0.25),
    ("tall", "plastic", (0.60, 0.55, 0.50), 0.2),
    ("short", "matte", (0.50, 0.60, 0.70), 0.3),
    ("sphere", "ashikhmin", (0.80, 0.70, 0.30), 40.0),
]


def adjoint_env(w=64, h=32, seed=3) -> np.ndarray:
    """A seeded equirectangular fill-light map (h, w, 3) float32: a sky
    gradient times smooth noise."""
    v = (np.arange(h, dtype=np.float32) + 0.5) / h
    sky = np.stack([0.5 + 0.3 * (1 - v), 0.6 + 0.3 * (1 - v), 0.8 + 0.2 * (1 - v)], axis=-1)
    n = value_noise((h, w), 3, seed)
    return (sky[:, None, :] * (0.6 + 0.4 * n[..., None])).astype(np.float32)


def cornell_adjoint(width=512, height=512, albedo=None, roughness=None, env=None, env_multiplier=1.0):
    """The Cornell box with its 8 surfaces as separate parameterised
    materials and an image-based environment seen through the open front.
    Returns (scene, info): info["albedo_tex"] / info["rough_tex"] hold the
    textures-blob offsets of the 8 albedo (colour) and roughness (float)
    textures, info["env_tex"] that of the environment image (RGBA16F)."""
    sc = S.Scene()
    mc = sc.mc
    albedo = np.asarray(albedo if albedo is not None else [m[2] for m in ADJ_MATERIALS], dtype=np.float32)
    roughness = np.asarray(roughness if roughness is not None else [m[3] for m in ADJ_MATERIALS], dtype=np.float32)
    env = adjoint_env() if env is None else np.asarray(env, dtype=np.float32)
    mc.float3_constant_texture("coat_Rs", 0.04, 0.04, 0.04)
    mc.float_constant_texture("sigma0", 0.0)
    mat, alb_tex, rough_tex = {}, [], []
    for i, (name, kind, _, _) in enumerate(ADJ_MATERIALS):
        mc.float3_constant_texture("A_" + name, *map(float, albedo[i]))
        mc.float_constant_texture("r_" + name, float(roughness[i]))
        alb_tex.append(sc.tex_ref["A_" + name])
        rough_tex.append(sc.tex_ref["r_" + name])
        if kind == "matte":
            mc.matte_material("m_" + name, None, "A_" + name, "r_" + name)
        elif kind == "plastic":
            mc.begin_material("m_" + name)
            mc.diffuse_elem("A_" + name, "sigma0")
            mc.newward_elem("coat_Rs", "r_" + name, "r_" + name)
            mc.end_material()
        else:
            mc.ashikhmin_material("m_" + name, None, "coat_Rs", "A_" + name, "r_" + name, "r_" + name)
        mat[name] = sc.mat_ref["m_" + name]
    mc.float3_constant_texture("M_light", 15.0 * math.pi, 15.0 * math.pi, 15.0 * math.pi)
    mc.diffuse_light_property("light", "M_light")
    sc.begin_object()
    for x in (0.0, 1.0):
        for y in (0.0, 1.0):
            for z in (0.0, 1.0):
                sc.add_vertex(x, y, z)
    V = lambda x, y, z: 4 * x + 2 * y + z  # noqa: E731
    walls = [
        ((V(0, 0, 0), V(1, 0, 0), V(1, 0, 1), V(0, 0, 1)), "floor"),
        ((V(0, 1, 0), V(0, 1, 1), V(1, 1, 1), V(1, 1, 0)), "ceiling"),
        ((V(0, 0, 0), V(0, 1, 0), V(1, 1, 0), V(1, 0, 0)), "back"),
        ((V(0, 0, 0), V(0, 0, 1), V(0, 1, 1), V(0, 1, 0)), "left"),
        ((V(1, 0, 0), V(1, 1, 0), V(1, 1, 1), V(1, 0, 1)), "right"),
    ]
    for (a, b, c, d), m in walls:
        sc.add_face((a, b, c), mat[m])
        sc.add_face((a, c, d), mat[m])
    sc.end_object()
    sc.begin_object()
    for x, z in ((0.375, 0.375), (0.625, 0.375), (0.625, 0.625), (0.375, 0.625)):
        sc.add_vertex(x, 0.999, z)
    sc.add_face((0, 1, 2), mat["ceiling"], light=sc.light_ref["light"])
    sc.add_face((0, 2, 3), mat["ceiling"], light=sc.light_ref["light"])
    sc.end_object()
    _box(sc, mat["tall"], (0.72, 0.3, 0.33), (0.27, 0.6, 0.27), -18.0)
    _box(sc, mat["short"], (0.70, 0.14, 0.76), (0.25, 0.28, 0.25), 15.0)
    _uv_sphere(sc, mat["sphere"], (0.3, 0.25, 0.6), 0.2)
    h, w = env.shape[:2]
    rgba = np.ones((h, w, 4), dtype=np.float16)
    rgba[..., :3] = env.astype(np.float16)
    mc.image_texture("env", rgba, "rgba16f")
    mc.image_based_env_light_property("IBL", "env", rgba[..., :3].astype(np.float32), env_multiplier)
    sc.set_environment("IBL")
    cam = S.look_at((0.5, 0.5, 2.35), (0.5, 0.5, 0.0), (0, 1, 0))
    sc.set_camera(width, height, cam, fov_y_deg=38.0)
    sc.build()
    info = {"albedo_tex": alb_tex, "rough_tex": rough_tex, "env_tex": sc.tex_ref["env"], "env_shape": (h, w),
            "albedo": albedo, "roughness": roughness, "env": rgba[..., :3].astype(np.float32)}
    return sc, info


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


# ------------------------------------------------------------- large scene


def value_noise(shape, octaves, seed, base_cells=4):
    """Seeded fractal value noise on [0,1]^2 sampled on a (h, w) grid:
    `octaves` lattices of random values, each twice as fine and half as
    strong, smoothstep-interpolated; result in roughly [-1, 1]."""
    rng = np.random.default_rng(seed)
    h, w = shape
    y = np.linspace(0.0, 1.0, h)[:, None]
    x = np.linspace(0.0, 1.0, w)[None, :]
    out = np.zeros((h, w))
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        lat = rng.uniform(-1.0, 1.0, size=(cells + 1, cells + 1))
        fx, fy = x * cells, y * cells
        ix, iy = np.minimum(fx.astype(int), cells - 1), np.minimum(fy.astype(int), cells - 1)
        tx, ty = fx - ix, fy - iy
        sx, sy = tx * tx * (3 - 2 * tx), ty * ty * (3 - 2 * ty)
        v00, v10 = lat[iy, ix], lat[iy, ix + 1]
        v01, v11 = lat[iy + 1, ix], lat[iy + 1, ix + 1]
        out += amp * ((v00 * (1 - sx) + v10 * sx) * (1 - sy) + (v01 * (1 - sx) + v11 * sx) * sy)
        total += amp
        amp *= 0.5
    return out / total


def normal_map(size, seed):
    """RGB8 tangent-space normal map from seeded noise heights."""
    hgt = value_noise((size, size), 5, seed, base_cells=8) * 2.0
    gy, gx = np.gradient(hgt, 1.0 / size)
    n = np.stack([-gx * 0.02, -gy * 0.02, np.ones_like(hgt)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.clip((n * 0.5 + 0.5) * 255.0 + 0.5, 0, 255).astype(np.uint8)


def sky_map(w, h, seed, sun_dir=(0.4, 0.6, -0.5), sun_peak=5e3, sun_sigma_deg=1.0):
    """Equirectangular fp32 RGB sky: lognormal(0, 1) radiance plus a Gaussian
    sun spot (peak `sun_peak`, sigma `sun_sigma_deg`)."""
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(0.0, 1.0, size=(h, w, 3)))
    v = (np.arange(h) + 0.5) / h
    u = (np.arange(w) + 0.5) / w
    theta = (v * np.pi)[:, None]
    phi = (u * 2 * np.pi)[None, :]
    # direction of texel (u, v) as the kernels map it (light.cl:165-168)
    d = np.stack([-np.sin(phi) * np.sin(theta), np.cos(theta) * np.ones_like(phi), np.cos(phi) * np.sin(theta)], -1)
    s = np.asarray(sun_dir, dtype=np.float64)
    s /= np.linalg.norm(s)
    ang = np.arccos(np.clip(d @ s, -1.0, 1.0))
    sig = math.radians(sun_sigma_deg)
    img += (sun_peak * np.exp(-0.5 * (ang / sig) ** 2))[..., None]
    return img.astype(np.float32)


def _sphere_mesh(seg, rings):
    th = np.pi * np.arange(rings + 1) / rings
    ph = 2 * np.pi * np.arange(seg + 1) / seg
    n = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :], np.cos(th)[:, None] * np.ones_like(ph)[None, :],
                  np.sin(th)[:, None] * np.sin(ph)[None, :]], -1).reshape(-1, 3)
    uv = np.stack(np.meshgrid(np.arange(seg + 1) / seg, np.arange(rings + 1) / rings), -1).reshape(-1, 2)
    row = seg + 1
    tris = []
    for j in range(rings):
        for i in range(seg):
            a, b, c, d = j * row + i, j * row + i + 1, (j + 1) * row + i, (j + 1) * row + i + 1
            if j != 0:
                tris.append((a, b, c))
            if j != rings - 1:
                tris.append((b, d, c))
    return n, uv, np.array(tris, dtype=np.int64)


def terrain_scene(width=1920, height=1080, grid=1024, n_spheres=256, env_w=1024, env_h=512, seed=7,
                  aperture=0.02, focus=1.5) -> S.Scene:
    """Large path-tracing scene: a grid x grid heightfield (2 triangles per
    cell) displaced by 6-octave value noise (amplitude 0.15), 256 UV spheres
    (24 x 12) with log-uniform radii 0.005-0.05 resting on it, 8 materials
    drawn from {Lambertian, Lambertian + coat, rough conductor, dielectric}
    with albedo U[0.05, 0.9] and roughness U[0.02, 0.6}, one 512 x 512 RGB8
    normal map per material, lit only by an equirectangular sky (stored as
    RGBA16F, the reference's environment texture format), thin-lens camera."""
    rng = np.random.default_rng(seed)
    sc = S.Scene()
    mc = sc.mc
    # materials
    kinds = rng.integers(0, 4, size=8)
    mats = []
    for m in range(8):
        alb = rng.uniform(0.05, 0.9, size=3)
        rough = float(rng.uniform(0.02, 0.6))
        mc.normal_map_texture(f"bump{m}", normal_map(512, seed * 100 + m))
        mc.float3_constant_texture(f"alb{m}", *alb)
        name = f"mat{m}"
        if kinds[m] == 0:
            mc.float_constant_texture(f"sig{m}", 0.0)
            mc.matte_material(name, f"bump{m}", f"alb{m}", f"sig{m}")
        elif kinds[m] == 1:
            mc.float3_constant_texture(f"rs{m}", 0.04, 0.04, 0.04)
            mc.float_constant_texture(f"n{m}", 2.0 / (rough * rough) - 2.0)
            mc.ashikhmin_material(name, f"bump{m}", f"rs{m}", f"alb{m}", f"n{m}", f"n{m}")
        elif kinds[m] == 2:
            mc.float_constant_texture(f"r{m}", rough)
            mc.newward_material(name, f"bump{m}", f"alb{m}", f"r{m}", f"r{m}")
        else:
            mc.float3_constant_texture(f"one{m}", 1.0, 1.0, 1.0)
            mc.glass_material(name, f"bump{m}", f"one{m}", f"one{m}", 1.0, 1.5)
        mats.append(sc.mat_ref[name])
    # heightfield over [0,1]^2 in xz, uv tiled 4x
    hgt = 0.15 * value_noise((grid + 1, grid + 1), 6, seed)
    xs = np.linspace(0.0, 1.0, grid + 1)
    X, Z = np.meshgrid(xs, xs)
    verts = np.stack([X, hgt, Z], -1).reshape(-1, 3)
    uvs = np.stack([X * 4.0, Z * 4.0], -1).reshape(-1, 2)
    i = np.arange(grid)
    a = (i[:, None] * (grid + 1) + i[None, :]).reshape(-1)
    b, c, d = a + 1, a + (grid + 1), a + (grid + 1) + 1
    tris = np.concatenate([np.stack([a, c, b], -1), np.stack([b, c, d], -1)])
    sc.add_mesh(verts, tris, mats[0], uvs=uvs)
    # spheres resting on the terrain
    n_unit, uv_unit, t_unit = _sphere_mesh(24, 12)
    for k in range(n_spheres):
        r = float(np.exp(rng.uniform(np.log(0.005), np.log(0.05))))
        px, pz = rng.uniform(0.05, 0.95, size=2)
        gx, gz = int(round(px * grid)), int(round(pz * grid))
        cy = float(hgt[gz, gx]) + r
        sc.add_mesh(n_unit * r + np.array([px, cy, pz]), t_unit, mats[int(rng.integers(0, 8))], uvs=uv_unit,
                    normals=n_unit)
    # sky
    sky = sky_map(env_w, env_h, seed + 1)
    rgba = np.ones((env_h, env_w, 4), dtype=np.float16)
    rgba[..., :3] = sky.astype(np.float16)
    mc.image_texture("sky", rgba, "rgba16f")
    mc.image_based_env_light_property("IBL", "sky", rgba[..., :3].astype(np.float32), 1.0)
    sc.set_environment("IBL")
    cam = S.look_at((0.5, 0.45, 1.45), (0.5, 0.05, 0.35), (0, 1, 0))
    sc.set_camera(width, height, cam, fov_y_deg=40.0, lens_radius=aperture, focus_dist=focus)
    sc.build()
    return sc

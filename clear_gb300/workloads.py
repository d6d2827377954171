"""Seeded synthetic inputs for the LBVH build and traversal benchmarks.

No dataset is involved: the random-triangle soup and query rays below stand in
for the scenes the reference loads from disk (its .obj/.exr assets are not
shipped with it).

``triangle_soup(n)``: centroids uniform in [0,1]^3; each vertex is centroid +
uniform unit direction x edge length, edge length ~ Exp(mean 0.5 * n^(-1/3));
vertices are fp32 SoA, unindexed (vertex k of triangle t at 3t+k).

``closest_rays(m)``: origins uniform in [-0.1,1.1]^3, directions uniform on
the sphere, tmax = inf.  ``shadow_rays(m)``: segments between two uniform
points of [0,1]^3, direction normalised, tmax = segment length.

Rays are packed as 8 fp32 per ray {ox, oy, oz, tmax, dx, dy, dz, 0}.
"""
from __future__ import annotations

import numpy as np


def _unit_dirs(rng, m):
    d = rng.standard_normal((m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return d


def triangle_soup(n: int, seed: int = 1):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    ell = rng.exponential(0.5 * n ** (-1.0 / 3.0), size=(n, 3))
    v = c[:, None, :] + _unit_dirs(rng, 3 * n).reshape(n, 3, 3) * ell[:, :, None]
    v = v.reshape(3 * n, 3).astype(np.float32)
    return np.ascontiguousarray(v[:, 0]), np.ascontiguousarray(v[:, 1]), np.ascontiguousarray(v[:, 2])


def pack_rays(org, dirs, tmax):
    m = org.shape[0]
    r = np.zeros((m, 8), dtype=np.float32)
    r[:, 0:3] = org
    r[:, 3] = tmax
    r[:, 4:7] = dirs
    return r


def closest_rays(m: int, seed: int = 2):
    rng = np.random.default_rng(seed)
    org = rng.uniform(-0.1, 1.1, size=(m, 3))
    return pack_rays(org.astype(np.float32), _unit_dirs(rng, m).astype(np.float32), np.inf)


def shadow_rays(m: int, seed: int = 3):
    rng = np.random.default_rng(seed)
    a = rng.random((m, 3))
    b = rng.random((m, 3))
    d = b - a
    L = np.linalg.norm(d, axis=1)
    L = np.maximum(L, 1e-12)
    d = d / L[:, None]
    return pack_rays(a.astype(np.float32), d.astype(np.float32), L.astype(np.float32))


def write_grid_obj(directory: str, n: int = 708) -> str:
    """Writes ``grid.obj`` and ``grid.mtl`` into `directory`: an n x n
    heightfield (2 (n-1)^2 triangles; n = 708 gives about 1 M and 93 MB) with
    one uv and one normal per vertex, faces in v/t/n form, one material.
    Returns the .obj path."""
    import os

    xs = np.linspace(0.0, 1.0, n)
    x, z = np.meshgrid(xs, xs)
    y = 0.1 * np.sin(7.0 * x) * np.cos(5.0 * z)
    path = os.path.join(directory, "grid.obj")
    with open(path, "w") as fh:
        fh.write("mtllib grid.mtl\no grid\n")
        fh.write("".join(f"v {a:.6f} {b:.6f} {c:.6f}\n" for a, b, c in zip(x.ravel(), y.ravel(), z.ravel())))
        fh.write("".join(f"vt {a:.6f} {c:.6f}\n" for a, c in zip(x.ravel(), z.ravel())))
        fh.write("vn 0 1 0\n" * (n * n))
        fh.write("usemtl white\n")
        j, i = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
        a = (j * n + i + 1).ravel()
        fh.write("".join(f"f {p}/{p}/{p} {q}/{q}/{q} {r}/{r}/{r}\nf {r}/{r}/{r} {q}/{q}/{q} {s}/{s}/{s}\n"
                         for p, q, r, s in zip(a, a + n, a + 1, a + n + 1)))
    with open(os.path.join(directory, "grid.mtl"), "w") as fh:
        fh.write("newmtl white\nKd 0.7 0.7 0.7\n")
    return path

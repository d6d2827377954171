"""Golden images of the path tracer from the reference's own CPU code.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_render.py

render_cornell.npz -- the Cornell-box scene of clear_gb300/scenes.py rendered
by the reference's ``sim::pathtracing`` (OpenCL_PathTracer/Equivalent/
sim_pathtracer.hpp, depth cap 100 as hard-coded there) with per-pixel
XORShift128 streams seeded with pixel index + 1, over the oracle-built LBVH;
once without and once with a small environment map.  A SHA-256 of the scene
blobs pins the scene encoding the images were made from.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from clear_gb300 import scenes  # noqa: E402

W = H = 64
SPP = 32


def env_map():
    rng = np.random.default_rng(4)
    return np.exp(rng.normal(0.0, 1.0, size=(8, 16, 3))).astype(np.float32) * 0.5


def blob_hash(b: dict) -> str:
    h = hashlib.sha256()
    for k in ("vertices", "normals", "tangents", "uvs", "faces", "lights", "materials", "textures", "others"):
        h.update(np.ascontiguousarray(b[k]).tobytes())
    return h.hexdigest()


def render(env):
    sc = scenes.cornell_box(W, H, env=env)
    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    rng = scenes.pixel_seeds(W, H)
    pix = np.zeros((W * H, 4), dtype=np.float32)
    oracle.ref_render(b, ob.inodes, ob.lnodes, rng, pix, W, H, 0, H, SPP)
    return pix[:, :3].copy(), blob_hash(b)


def main():
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    img0, h0 = render(None)
    img1, h1 = render(env_map())
    np.savez_compressed(os.path.join(HERE, "render_cornell.npz"), width=W, height=H, spp=SPP,
                        plain=img0, plain_hash=h0, env=img1, env_hash=h1)
    print("wrote render_cornell.npz", img0.mean(), img1.mean())


if __name__ == "__main__":
    main()

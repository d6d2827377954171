"""Golden BVH-visualiser images from the reference's own CPU code.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_vis.py

bvh_vis.npz -- ``sim::bvh_visualizer`` (OpenCL_PathTracer/Equivalent/
sim_bvh_visualizer.hpp, the CPU form of OpenCL/bvh_visualizer.cl) over the
oracle-built LBVH of three scenes of clear_gb300: the Cornell box (96 x 96),
the differentiable Cornell box with Ward and Ashikhmin materials and an
environment (64 x 64), and one random-triangle scene of the batched workload
(2000 triangles, 64 x 64).  A SHA-256 of each scene's blobs pins the encoding.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from clear_gb300 import batch, scenes  # noqa: E402
from make_golden_render import blob_hash  # noqa: E402


def vis_scenes():
    return {"cornell": scenes.cornell_box(96, 96), "adjoint": scenes.cornell_adjoint(64, 64)[0],
            "random": batch.random_scene(2000, 64, 64, 17)}


def visualize(sc):
    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    pix = np.zeros((sc.width * sc.height, 4), dtype=np.float32)
    oracle.ref_bvh_visualizer(b, ob.inodes, ob.lnodes, pix, sc.width, sc.height)
    return pix[:, :3].copy(), blob_hash(b)


def main():
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    out = {}
    for name, sc in vis_scenes().items():
        img, h = visualize(sc)
        out[name] = img
        out[name + "_hash"] = h
        print(name, img.shape, float(img.mean()))
    np.savez_compressed(os.path.join(HERE, "bvh_vis.npz"), **out)


if __name__ == "__main__":
    main()

"""Generate the golden fixtures of tests/golden from the reference's own CPU code.

Run where the reference checkout is available (it is compiled in place by
oracle/build_oracle.py into oracle/_ref):

    python tests/golden/make_golden.py

lbvh_traversal.npz -- small seeded triangle soups, closest-hit query rays, and
the hit ids / t that the reference's ``sim::rayIntersection``
(OpenCL_PathTracer/Equivalent/sim_bvh_traversal.hpp) returns when it walks the
oracle-built LBVH; plus the reference's CPU midpoint BVH
(OpenCL_PathTracer/BVH.hpp) over the same soup and the hits its own traversal
returns over that BVH.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from clear_gb300 import workloads as W  # noqa: E402

CASES = [(2, 11), (3, 12), (17, 13), (300, 14), (5000, 15)]
NRAYS = 512


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    out = {}
    for n, seed in CASES:
        vx, vy, vz = W.triangle_soup(n, seed=seed)
        rays = W.closest_rays(NRAYS, seed=seed + 100)
        bvh = oracle.lbvh_build(vx, vy, vz, None, n, 10)
        ids, ts = oracle.ref_trace_closest_lbvh(vx, vy, vz, None, n, bvh, rays)
        mid = oracle.ref_midbvh_build(vx, vy, vz, None, n)
        mids, mts = oracle.ref_trace_closest_mid(vx, vy, vz, None, n, mid, rays)
        p = f"n{n}_"
        out.update({p + "vx": vx, p + "vy": vy, p + "vz": vz, p + "rays": rays,
                    p + "ref_lbvh_ids": ids, p + "ref_lbvh_t": ts,
                    p + "ref_mid_min": mid["min"][:, :3].copy(), p + "ref_mid_max": mid["max"][:, :3].copy(),
                    p + "ref_mid_children": mid["children"].copy(),
                    p + "ref_mid_ids": mids, p + "ref_mid_t": mts})
    out["cases"] = np.array([c[0] for c in CASES], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "lbvh_traversal.npz"), **out)
    print("wrote", os.path.join(HERE, "lbvh_traversal.npz"))


if __name__ == "__main__":
    main()

"""Golden LBVH builds from the reference's own OpenCL kernels run on the CPU.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_build.py

lbvh_build_ref.npz -- for each case of CASES, the outputs of
``oracle.ref_cl_lbvh_build`` (lbvh_construction.cl and generic_kernels.cl in
the launch order of LBVHBuilder::perform): SHA-256 digests of the sorted
indices, Morton codes, internal and leaf nodes, parents and scene box, and the
arrays themselves for the small cases.  The inputs are regenerated by
``case_inputs`` (seeded), so the fixture holds no geometry.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from clear_gb300 import workloads as W  # noqa: E402

# name -> (kind, triangles, bits per axis, seed)
CASES = {
    "soup_2": ("soup", 2, 10, 11),
    "soup_3": ("soup", 3, 10, 12),
    "soup_64": ("soup", 64, 10, 13),
    "soup_65": ("soup", 65, 10, 14),
    "soup_1000": ("soup", 1000, 10, 15),
    "soup_4097": ("soup", 4097, 10, 16),
    "soup_3000_b20": ("soup", 3000, 20, 17),
    "soup_777_b4": ("soup", 777, 4, 18),
    "indexed_dups_600": ("dups", 600, 10, 19),
}
FULL_MAX = 100  # cases up to this many triangles also store the arrays


def case_inputs(kind: str, n: int, seed: int):
    """(vx, vy, vz, tri or None).  "dups": an indexed mesh in which every
    triangle appears three times (equal Morton keys, the index tie rule of
    the Karras search) over shared, permuted vertices."""
    if kind == "soup":
        vx, vy, vz = W.triangle_soup(n, seed=seed)
        return vx, vy, vz, None
    rng = np.random.default_rng(seed)
    base = n // 3
    vx, vy, vz = W.triangle_soup(base, seed=seed)
    perm = rng.permutation(3 * base)
    inv = np.argsort(perm).astype(np.uint32)
    tri = np.concatenate([inv.reshape(base, 3)] * 3)[rng.permutation(3 * base)]
    return vx[perm], vy[perm], vz[perm], np.ascontiguousarray(tri.reshape(-1))


def outputs(bvh) -> dict:
    return {"sorted_idx": np.ascontiguousarray(bvh.sorted_idx, dtype=np.uint32),
            "q": np.ascontiguousarray(bvh.q, dtype=np.uint32),
            "inodes": np.ascontiguousarray(bvh.inodes).view(np.uint8).reshape(-1),
            "lnodes": np.ascontiguousarray(bvh.lnodes).view(np.uint8).reshape(-1),
            "parents": np.ascontiguousarray(bvh.parents, dtype=np.uint32),
            "scene_box": np.ascontiguousarray(bvh.scene_box, dtype=np.float32)}


def canonical(name: str, arr: np.ndarray, n: int) -> np.ndarray:
    """The bytes the reference defines: internal nodes and leaves without
    their padding, parents without the root's entry (never written)."""
    import oracle

    def raw(x):
        return np.ascontiguousarray(x).view(np.uint8).reshape(-1)

    if name == "inodes":
        a = arr.view(oracle.INODE_DTYPE)
        return np.concatenate([raw(a["min"][:, :3]), raw(a["max"][:, :3]), raw(a["isChild"]), raw(a["c"])])
    if name == "lnodes":
        a = arr.view(oracle.LNODE_DTYPE)
        return np.concatenate([raw(a["min"][:, :3]), raw(a["max"][:, :3]), raw(a["objIdx"])])
    if name == "parents":
        keep = np.ones(len(arr), dtype=bool)
        keep[n] = False
        return arr[keep]
    return arr


def digest(name: str, arr: np.ndarray, n: int) -> str:
    return hashlib.sha256(np.ascontiguousarray(canonical(name, arr, n)).tobytes()).hexdigest()


def main() -> None:
    import oracle

    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    out = {}
    for name, (kind, n, bits, seed) in CASES.items():
        vx, vy, vz, tri = case_inputs(kind, n, seed)
        ref = outputs(oracle.ref_cl_lbvh_build(vx, vy, vz, tri, n, bits))
        for k, a in ref.items():
            out[f"{name}/{k}_sha256"] = np.array(digest(k, a, n))
            if n <= FULL_MAX:
                out[f"{name}/{k}"] = a
    np.savez_compressed(os.path.join(HERE, "lbvh_build_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "lbvh_build_ref.npz"))


if __name__ == "__main__":
    main()

"""CPU tests of the oracle: pinned to the reference's own code and properties.

The reference has no tests or golden vectors of its own; the fixtures in
tests/golden come from its CPU code (OpenCL_PathTracer/Equivalent and BVH.hpp)
compiled in place -- see tests/golden/make_golden.py -- and from its LBVH
construction kernels run on the CPU (tests/golden/make_golden_build.py).
"""
import os
import sys

import numpy as np
import pytest

import oracle
from clear_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lbvh_traversal.npz")
BUILD_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "lbvh_build_ref.npz")
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden_build as GB  # noqa: E402
MISS = 0xFFFFFFFF


def test_golden_traversal_matches_reference_sim():
    g = np.load(GOLDEN)
    for n in g["cases"]:
        p = f"n{n}_"
        vx, vy, vz, rays = g[p + "vx"], g[p + "vy"], g[p + "vz"], g[p + "rays"]
        bvh = oracle.lbvh_build(vx, vy, vz, None, int(n), 10)
        ids, ts = oracle.trace_closest(vx, vy, vz, None, bvh, rays)
        ref_ids = g[p + "ref_lbvh_ids"]
        # the reference truncates face ids to ushort; all cases have n < 65536
        np.testing.assert_array_equal(ids, ref_ids)
        hit = ref_ids != MISS
        np.testing.assert_array_equal(ts[hit], g[p + "ref_lbvh_t"][hit])


def test_golden_midpoint_bvh_matches_reference():
    g = np.load(GOLDEN)
    for n in g["cases"]:
        p = f"n{n}_"
        vx, vy, vz, rays = g[p + "vx"], g[p + "vy"], g[p + "vz"], g[p + "rays"]
        nodes = oracle.midbvh_build(vx, vy, vz, None, int(n))
        np.testing.assert_array_equal(nodes["children"], g[p + "ref_mid_children"])
        np.testing.assert_array_equal(nodes["min"][:, :3], g[p + "ref_mid_min"])
        np.testing.assert_array_equal(nodes["max"][:, :3], g[p + "ref_mid_max"])
        ids, ts = oracle.trace_closest_mid(vx, vy, vz, None, nodes, int(n), rays)
        np.testing.assert_array_equal(ids, g[p + "ref_mid_ids"])
        # both reference BVHs find the same closest triangle
        np.testing.assert_array_equal(ids, g[p + "ref_lbvh_ids"])


def check_tree(bvh: oracle.OracleBVH, n: int):
    """Structural properties of a Karras radix tree with refitted boxes."""
    inodes, lnodes, parents = bvh.inodes, bvh.lnodes, bvh.parents
    assert sorted(bvh.sorted_idx.tolist()) == list(range(n))
    if n < 2:
        return
    seen_leaf = np.zeros(n, dtype=np.int64)
    seen_inner = np.zeros(n - 1, dtype=np.int64)
    stack = [0]
    seen_inner[0] = 1
    while stack:
        i = stack.pop()
        for c in range(2):
            child = int(inodes["c"][i, c])
            if inodes["isChild"][i, c]:
                seen_leaf[child] += 1
                assert parents[child] == i
                box_min, box_max = lnodes["min"][child, :3], lnodes["max"][child, :3]
            else:
                seen_inner[child] += 1
                assert parents[n + child] == i
                stack.append(child)
                box_min, box_max = inodes["min"][child, :3], inodes["max"][child, :3]
            assert (inodes["min"][i, :3] <= box_min).all() and (inodes["max"][i, :3] >= box_max).all()
    assert (seen_leaf == 1).all() and (seen_inner == 1).all()
    np.testing.assert_array_equal(inodes["min"][0, :3], bvh.scene_box[:3])
    np.testing.assert_array_equal(inodes["max"][0, :3], bvh.scene_box[3:])
    np.testing.assert_array_equal(lnodes["objIdx"], bvh.sorted_idx)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 65, 1000, 20000])
@pytest.mark.parametrize("bits", [10, 20])
def test_oracle_tree_properties(n, bits):
    vx, vy, vz = W.triangle_soup(n, seed=n + bits)
    bvh = oracle.lbvh_build(vx, vy, vz, None, n, bits)
    keys = bvh.keys()
    assert (np.diff(keys.astype(np.float64)) >= 0).all() or (keys[1:] >= keys[:-1]).all()
    # stable: equal keys keep input order
    order = np.argsort(oracle.morton_keys(bvh.q, bits), kind="stable")
    np.testing.assert_array_equal(order, bvh.sorted_idx)
    check_tree(bvh, n)


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 65537])
@pytest.mark.parametrize("bits", [10, 20])
@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parallel_oracle_build_equals_serial(n, bits, threads):
    """The data-parallel build (the CPU baseline of the benchmark) gives the
    serial restatement's nodes, parents, order and scene box byte for byte,
    on unindexed and indexed inputs, whatever the thread count."""
    vx, vy, vz = W.triangle_soup(n, seed=n + 7 * bits)
    tris = [None]
    if n > 2:
        tris.append(np.random.default_rng(n).permutation(3 * n).astype(np.uint32))
    for tri in tris:
        a = oracle.lbvh_build(vx, vy, vz, tri, n, bits)
        b = oracle.lbvh_build_mt(vx, vy, vz, tri, n, bits, threads)
        for k in ("inodes", "lnodes", "parents", "sorted_idx", "scene_box"):
            np.testing.assert_array_equal(getattr(a, k).view(np.uint8), getattr(b, k).view(np.uint8), err_msg=k)


def test_oracle_duplicate_keys_and_planar_scene():
    # many triangles with identical centres (equal keys) and a zero-extent z
    # axis (0/0 quantises to 0): the index extension of the Karras search and
    # the stable sort must still give a valid tree.
    n = 257
    rng = np.random.default_rng(7)
    c = np.repeat(rng.random((17, 2)), 16, axis=0)[:n]
    c = np.concatenate([c, rng.random((n - len(c), 2))])
    v = np.zeros((n, 3, 3), dtype=np.float32)
    v[:, :, :2] = c[:, None, :] + np.array([[0, 0], [0.01, 0], [0, 0.01]], dtype=np.float32)
    v = v.reshape(-1, 3)
    bvh = oracle.lbvh_build(v[:, 0], v[:, 1], v[:, 2], None, n, 10)
    assert (bvh.q[:, 2] == 0).all()
    check_tree(bvh, n)


def test_oracle_indexed_matches_unindexed():
    n = 500
    vx, vy, vz = W.triangle_soup(n, seed=3)
    # share vertices through an index buffer: dedupe nothing, just permute
    perm = np.random.default_rng(1).permutation(3 * n).astype(np.uint32)
    inv = np.argsort(perm).astype(np.uint32)
    tri = inv  # vertex 3t+k of the soup lives at index inv[3t+k] of the permuted arrays
    b0 = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    b1 = oracle.lbvh_build(vx[perm], vy[perm], vz[perm], tri, n, 10)
    np.testing.assert_array_equal(b0.sorted_idx, b1.sorted_idx)
    np.testing.assert_array_equal(b0.inodes["c"], b1.inodes["c"])


def test_known_triangle_hit():
    # unit right triangle in z=1, ray straight down from z=3: t = 2
    vx = np.array([0, 1, 0, 5, 6, 5], dtype=np.float32)
    vy = np.array([0, 0, 1, 5, 5, 6], dtype=np.float32)
    vz = np.array([1, 1, 1, 2, 2, 2], dtype=np.float32)
    bvh = oracle.lbvh_build(vx, vy, vz, None, 2, 10)
    rays = W.pack_rays(np.array([[0.25, 0.25, 3.0], [0.9, 0.9, 3.0]], dtype=np.float32),
                       np.array([[0, 0, -1.0], [0, 0, -1.0]], dtype=np.float32), np.inf)
    ids, ts = oracle.trace_closest(vx, vy, vz, None, bvh, rays)
    assert ids[0] == 0 and ts[0] == np.float32(2.0)
    assert ids[1] == MISS
    occ = oracle.trace_shadow(vx, vy, vz, None, bvh, W.pack_rays(rays[:, :3], rays[:, 4:7], 1.5))
    assert occ.tolist() == [0, 0]
    occ = oracle.trace_shadow(vx, vy, vz, None, bvh, W.pack_rays(rays[:, :3], rays[:, 4:7], 2.0))
    assert occ.tolist() == [1, 0]


def test_shadow_agrees_with_closest_hit():
    n = 20000
    vx, vy, vz = W.triangle_soup(n, seed=5)
    bvh = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    rays = W.shadow_rays(4000, seed=6)
    occ = oracle.trace_shadow(vx, vy, vz, None, bvh, rays)
    ids, ts = oracle.trace_closest(vx, vy, vz, None, bvh, W.pack_rays(rays[:, :3], rays[:, 4:7], np.inf))
    np.testing.assert_array_equal(occ.astype(bool), ts <= rays[:, 3])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("n,seed", [(9, 1), (1234, 2), (40000, 3)])
def test_live_pin_against_reference(n, seed):
    vx, vy, vz = W.triangle_soup(n, seed=seed)
    bvh = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    rays = W.closest_rays(3000, seed=seed + 9)
    ids, ts = oracle.trace_closest(vx, vy, vz, None, bvh, rays)
    rids, rts = oracle.ref_trace_closest_lbvh(vx, vy, vz, None, n, bvh, rays)
    np.testing.assert_array_equal(ids, rids)
    np.testing.assert_array_equal(ts[rids != MISS], rts[rids != MISS])


@pytest.mark.parametrize("case", list(GB.CASES))
def test_oracle_build_matches_reference_kernels_golden(case):
    """The restated build equals the reference's own kernels
    (lbvh_construction.cl, generic_kernels.cl, run on the CPU): Morton codes,
    sorted order, internal and leaf nodes, parents, scene box -- digests of
    every output, and the arrays themselves for the small cases."""
    g = np.load(BUILD_GOLDEN)
    kind, n, bits, seed = GB.CASES[case]
    vx, vy, vz, tri = GB.case_inputs(kind, n, seed)
    got = GB.outputs(oracle.lbvh_build(vx, vy, vz, tri, n, bits))
    for k, a in got.items():
        if f"{case}/{k}" in g.files:
            assert np.array_equal(GB.canonical(k, a, n), GB.canonical(k, g[f"{case}/{k}"], n)), k
        assert GB.digest(k, a, n) == str(g[f"{case}/{k}_sha256"]), k


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not present")
@pytest.mark.parametrize("n,bits,seed", [(2, 10, 1), (129, 10, 2), (2500, 10, 3), (1500, 21, 4), (600, 1, 5)])
def test_oracle_build_matches_reference_kernels_live(n, bits, seed):
    vx, vy, vz = W.triangle_soup(n, seed=seed)
    ref = GB.outputs(oracle.ref_cl_lbvh_build(vx, vy, vz, None, n, bits))
    got = GB.outputs(oracle.lbvh_build(vx, vy, vz, None, n, bits))
    for k in ref:
        assert np.array_equal(GB.canonical(k, got[k], n), GB.canonical(k, ref[k], n)), k
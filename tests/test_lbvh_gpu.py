"""GPU parity of the LBVH build and the traversal kernels against the oracle.

Integer outputs (sorted order, keys, topology, parents, leaf objects, hit ids)
must be bit-exact; boxes and hit distances are compared with float equality
(the kernels use the reference's operations in the reference's order, so they
are expected to be identical; +0 and -0 compare equal).
"""
import numpy as np
import pytest
import torch

import oracle
from clear_gb300 import _lib, lbvh
from clear_gb300 import workloads as W

MISS = 0xFFFFFFFF

pytestmark = pytest.mark.gpu


def gpu_build(cuda, vx, vy, vz, tri, n, bits):
    b = lbvh.LBVHBuilder(max(n, 1), cuda)
    v = tuple(torch.from_numpy(np.asarray(a)).to(cuda) for a in (vx, vy, vz))
    t = None if tri is None else torch.from_numpy(np.asarray(tri, dtype=np.int32)).to(cuda)
    bvh = b.perform(v, t, n, bits)
    ref = {k: x.cpu().numpy() for k, x in b.export_reference(bvh).items()}
    torch.cuda.synchronize()
    return b, bvh, ref


def assert_build_equal(ref, ob: oracle.OracleBVH, n):
    np.testing.assert_array_equal(ref["sorted_idx"].view(np.uint32), ob.sorted_idx)
    np.testing.assert_array_equal(ref["keys"].view(np.uint64), ob.keys())
    ln = ref["lnodes"].view(oracle.LNODE_DTYPE)
    np.testing.assert_array_equal(ln["objIdx"], ob.lnodes["objIdx"])
    assert (ln["min"][:, :3] == ob.lnodes["min"][:, :3]).all()
    assert (ln["max"][:, :3] == ob.lnodes["max"][:, :3]).all()
    if n >= 2:
        inn = ref["inodes"].view(oracle.INODE_DTYPE)
        np.testing.assert_array_equal(inn["c"], ob.inodes["c"])
        np.testing.assert_array_equal(inn["isChild"], ob.inodes["isChild"])
        assert (inn["min"][:, :3] == ob.inodes["min"][:, :3]).all()
        assert (inn["max"][:, :3] == ob.inodes["max"][:, :3]).all()
        par = ref["parents"].view(np.uint32)
        keep = np.ones(2 * n - 1, dtype=bool)
        keep[n] = False  # the root has no parent (unwritten in the reference)
        np.testing.assert_array_equal(par[keep], ob.parents[keep])


def no_device_errors():
    assert _lib.device_status(clear=True) == 0


@pytest.mark.parametrize("bits", [10, 20])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 63, 64, 65, 1000, 2047, 2048, 2049, 4095, 4096, 4097, 65543, 300001])
def test_build_parity(cuda, n, bits):
    vx, vy, vz = W.triangle_soup(n, seed=1000 + n)
    b, bvh, ref = gpu_build(cuda, vx, vy, vz, None, n, bits)
    ob = oracle.lbvh_build(vx, vy, vz, None, n, bits)
    assert_build_equal(ref, ob, n)
    rb = bvh.root_box.cpu().numpy()
    assert (rb[:3] == ob.scene_box[:3]).all() and (rb[4:7] == ob.scene_box[3:]).all()
    no_device_errors()


@pytest.mark.parametrize("bits", [1, 3, 7, 21])
@pytest.mark.parametrize("n", [2, 4097, 65543])
def test_build_parity_other_key_widths(cuda, n, bits):
    """Key widths either side of the common 10 and 20 bits per axis: 1 bit
    (eight distinct Morton keys, so most of the tree splits on the sorted
    positions), 3 and 7 bits (one and three sort passes) and 21 bits (63-bit
    keys, eight passes)."""
    vx, vy, vz = W.triangle_soup(n, seed=7 + n)
    _, _, ref = gpu_build(cuda, vx, vy, vz, None, n, bits)
    assert_build_equal(ref, oracle.lbvh_build(vx, vy, vz, None, n, bits), n)
    no_device_errors()


@pytest.mark.parametrize("n", [(2 << 20), (2 << 20) + 1])
def test_build_parity_either_side_of_the_climb_threshold(cuda, n):
    """Trees up to 2 Mi triangles finish their block-crossing climbs inside the
    tree pass, larger ones in k_build_tree_top: both exact."""
    vx, vy, vz = W.triangle_soup(n, seed=5 + n)
    _, _, ref = gpu_build(cuda, vx, vy, vz, None, n, 10)
    assert_build_equal(ref, oracle.lbvh_build(vx, vy, vz, None, n, 10), n)
    no_device_errors()


@pytest.mark.parametrize("n, bits", [(4097, 10), (300001, 10), (65537, 20)])
def test_tma_and_plain_record_gathers_agree(cuda, n, bits):
    """The tree pass gathers its leaves' staging records with TMA copies or,
    where the driver lacks the tensor-map encoder, with plain loads: the same
    tree, byte for byte, and the oracle's."""
    vx, vy, vz = W.triangle_soup(n, seed=77 + n)
    refs = []
    try:
        for tma in (1, 0):
            _lib.call("clr_debug_set_tma_gather", tma)
            _, _, ref = gpu_build(cuda, vx, vy, vz, None, n, bits)
            refs.append(ref)
    finally:
        _lib.call("clr_debug_set_tma_gather", 1)
    for k in refs[0]:
        assert np.array_equal(refs[0][k], refs[1][k]), k
    assert_build_equal(refs[0], oracle.lbvh_build(vx, vy, vz, None, n, bits), n)
    no_device_errors()


def test_build_parity_indexed_and_planar(cuda):
    # indexed input with shared vertices, duplicate centroids and a flat z axis
    rng = np.random.default_rng(5)
    nv, n = 3000, 8000
    vx = rng.random(nv).astype(np.float32)
    vy = rng.random(nv).astype(np.float32)
    vz = np.zeros(nv, dtype=np.float32)
    tri = rng.integers(0, nv, size=(n, 3)).astype(np.uint32)
    tri[:100] = tri[100:200]  # identical triangles -> equal keys
    _, _, ref = gpu_build(cuda, vx, vy, vz, tri, n, 10)
    ob = oracle.lbvh_build(vx, vy, vz, tri.reshape(-1), n, 10)
    assert_build_equal(ref, ob, n)
    no_device_errors()


def test_build_is_deterministic_and_reusable(cuda):
    n = 200000
    vx, vy, vz = W.triangle_soup(n, seed=77)
    b = lbvh.LBVHBuilder(1000, cuda)  # grows on demand
    v = tuple(torch.from_numpy(a).to(cuda) for a in (vx, vy, vz))
    bvh1 = b.perform(v, None, n, 10)
    nodes1, tris1 = bvh1.nodes.clone(), bvh1.tris.clone()
    bvh2 = b.perform(v, None, n, 10)
    torch.cuda.synchronize()
    assert torch.equal(nodes1, bvh2.nodes) and torch.equal(tris1, bvh2.tris)
    no_device_errors()


@pytest.mark.parametrize("case", ["soup_2", "soup_3", "soup_64", "soup_65", "soup_1000", "soup_4097",
                                  "soup_3000_b20", "soup_777_b4", "indexed_dups_600"])
def test_build_matches_reference_kernels(cuda, case):
    """The device build, exported to the reference's layouts, equals the
    reference's own construction kernels (lbvh_construction.cl run on the CPU,
    tests/golden/lbvh_build_ref.npz): sorted order, internal and leaf nodes
    and parents, byte for byte."""
    import os
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden_build as GB

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "lbvh_build_ref.npz"))
    kind, n, bits, seed = GB.CASES[case]
    vx, vy, vz, tri = GB.case_inputs(kind, n, seed)
    _, _, ref = gpu_build(cuda, vx, vy, vz, tri, n, bits)
    got = {"sorted_idx": ref["sorted_idx"].view(np.uint32), "inodes": ref["inodes"].view(np.uint8).reshape(-1),
           "lnodes": ref["lnodes"].view(np.uint8).reshape(-1), "parents": ref["parents"].view(np.uint32)}
    for k, a in got.items():
        assert GB.digest(k, a, n) == str(g[f"{case}/{k}_sha256"]), k
    no_device_errors()


@pytest.mark.parametrize("n", [1, 2, 7, 5000, 300001])
def test_trace_parity(cuda, n):
    vx, vy, vz = W.triangle_soup(n, seed=2000 + n)
    b, bvh, _ = gpu_build(cuda, vx, vy, vz, None, n, 10)
    ob = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    rays = W.closest_rays(20000, seed=n)
    rays[::7, 3] = 0.05  # some finite tmax
    oids, ots = oracle.trace_closest(vx, vy, vz, None, ob, rays)
    for ordered, sort in ((False, False), (True, False), (True, True)):
        ids, ts = lbvh.trace_closest(bvh, torch.from_numpy(rays).to(cuda), ordered=ordered, sort=sort)
        np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint32), oids)
        np.testing.assert_array_equal(ts.cpu().numpy(), ots)
    srays = W.shadow_rays(20000, seed=n + 1)
    oocc = oracle.trace_shadow(vx, vy, vz, None, ob, srays)
    for sort in (False, True):
        occ = lbvh.trace_shadow(bvh, torch.from_numpy(srays).to(cuda), sort=sort).cpu().numpy()
        np.testing.assert_array_equal(occ, oocc)
    no_device_errors()


def test_trace_sorted_order_edge_cases(cuda):
    """Searches in origin order: the same answers as the given order for ray
    counts around the sort's tile size, origins far outside the scene and
    non-finite ones, a scene whose box is flat on one axis, and no rays."""
    n = 5000
    vx, vy, vz = W.triangle_soup(n, seed=31)
    vy = np.full_like(vy, 0.5)  # flat: the root box has no extent in y
    b, bvh, _ = gpu_build(cuda, vx, vy, vz, None, n, 10)
    for m in (1, 4095, 4096, 4097, 70001):
        rays = W.closest_rays(m, seed=m)
        rays[: m // 3, :3] *= 1e6
        if m > 10:
            rays[5, 0] = np.nan
            rays[6, 1] = np.inf
        r = torch.from_numpy(rays).to(cuda)
        ids, ts = lbvh.trace_closest(bvh, r)
        ids_s, ts_s = lbvh.trace_closest(bvh, r, sort=True)
        assert torch.equal(ids, ids_s) and torch.equal(ts.view(torch.int32), ts_s.view(torch.int32)), m
        assert torch.equal(lbvh.trace_shadow(bvh, r), lbvh.trace_shadow(bvh, r, sort=True)), m
    lbvh.trace_closest(bvh, torch.empty((0, 8), device=cuda), sort=True)
    no_device_errors()


@pytest.mark.parametrize("n", [1, 2, 5000, 300001])
def test_trace_counted_matches_oracle_visits(cuda, n):
    """Per-ray visiting counts in the reference's order: internal boxes
    accepted and leaf boxes accepted (triangles tested) equal the oracle's,
    and the hit is the plain closest-hit query's."""
    vx, vy, vz = W.triangle_soup(n, seed=3000 + n)
    b, bvh, _ = gpu_build(cuda, vx, vy, vz, None, n, 10)
    ob = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    rays = W.closest_rays(20000, seed=n + 5)
    ids, counts = lbvh.trace_closest_counted(bvh, torch.from_numpy(rays).to(cuda))
    oids, _, st = oracle.trace_closest(vx, vy, vz, None, ob, rays, stats=True)
    np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint32), oids)
    c = counts.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(c[:, 0], st[:, 1])
    np.testing.assert_array_equal(c[:, 1], st[:, 3])
    assert (st[:, 1] <= st[:, 0]).all() and (st[:, 3] <= st[:, 2]).all()
    no_device_errors()


def _box_rays(vx, vy, vz, m, seed):
    """Rays from points uniform in the scene's box in directions uniform on
    the sphere (tmax = inf)."""
    r = np.random.default_rng(seed)
    lo = np.array([vx.min(), vy.min(), vz.min()])
    hi = np.array([vx.max(), vy.max(), vz.max()])
    d = r.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((m, 8), np.float32)
    rays[:, :3] = lo + (hi - lo) * r.random((m, 3))
    rays[:, 3] = np.inf
    rays[:, 4:7] = d
    return rays


def _fast_vs_oracle(cuda, vx, vy, vz, tri, n, rays):
    b, bvh, _ = gpu_build(cuda, vx, vy, vz, tri, n, 10)
    ob = oracle.lbvh_build(vx, vy, vz, tri, n, 10)
    lbvh.trace_replays(clear=True)
    ids, ts = lbvh.trace_closest(bvh, torch.from_numpy(rays).to(cuda), ordered=True)
    replays = lbvh.trace_replays(clear=True)
    oids, ots = oracle.trace_closest(vx, vy, vz, tri, ob, rays)
    np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint32), oids)
    np.testing.assert_array_equal(ts.cpu().numpy(), ots)
    no_device_errors()
    return replays


def test_trace_fast_equals_reference_order(cuda):
    """The nearer-first query with replay returns the reference's ids and
    distances bit for bit (no tolerance) on a random soup, where ties are
    rare and next to no ray is replayed."""
    n = 300001
    vx, vy, vz = W.triangle_soup(n, seed=99)
    rays = W.closest_rays(50000, seed=98)
    replays = _fast_vs_oracle(cuda, vx, vy, vz, None, n, rays)
    assert replays <= 50  # 0.1 %


def test_trace_fast_equals_reference_order_on_ties(cuda):
    """Scenes full of exact and near ties, where the reference's answer
    depends on its visiting order: every triangle of a mesh present twice
    (each hit an exact tie between two ids), and the Cornell box (shared
    edges, flat axis-aligned boxes) -- bit-exact, with the tied rays replayed."""
    from clear_gb300 import scenes

    sc = scenes.cornell_box(16, 16)
    vx, vy, vz, tri = sc.soa()
    tri = np.ascontiguousarray(tri.astype(np.uint32).reshape(-1))
    n = tri.size // 3
    rays = _box_rays(vx, vy, vz, 200000, 7)
    _fast_vs_oracle(cuda, vx, vy, vz, tri, n, rays)
    twice = np.concatenate([tri, tri])
    replays = _fast_vs_oracle(cuda, vx, vy, vz, twice, 2 * n, rays)
    assert replays > 100000  # nearly every hit is a tie


def test_trace_empty_scene_and_no_rays(cuda):
    b = lbvh.LBVHBuilder(1, cuda)
    e = torch.empty(0, dtype=torch.float32, device=cuda)
    bvh = b.perform((e, e, e), None, 0, 10)
    rays = torch.from_numpy(W.closest_rays(100, seed=1)).to(cuda)
    ids, ts = lbvh.trace_closest(bvh, rays)
    assert (ids.cpu().numpy().view(np.uint32) == MISS).all()
    assert lbvh.trace_shadow(bvh, rays).sum().item() == 0
    lbvh.trace_closest(bvh, rays[:0])
    no_device_errors()


def test_invalid_arguments_fail_loudly(cuda):
    b = lbvh.LBVHBuilder(10, cuda)
    vx, vy, vz = (torch.zeros(30, device=cuda) for _ in range(3))
    with pytest.raises(_lib.ClrError):
        b.perform((vx, vy, vz), None, 10, 0)
    with pytest.raises(_lib.ClrError):
        b.perform((vx, vy, vz), None, 10, 22)


def test_full_size_properties(cuda):
    """16 Mi triangles (the largest benchmark scene): properties that hold at
    any size, plus bit-exact hits on a ray sample against the oracle tree."""
    n = 1 << 24
    vx, vy, vz = W.triangle_soup(n, seed=24)
    b, bvh, ref = gpu_build(cuda, vx, vy, vz, None, n, 10)
    keys = ref["keys"].view(np.uint64)
    assert (keys[1:] >= keys[:-1]).all()
    sidx = ref["sorted_idx"].view(np.uint32)
    assert np.bincount(sidx, minlength=n).max() == 1
    inn = ref["inodes"].view(oracle.INODE_DTYPE)
    leaf_hits = np.bincount(inn["c"][inn["isChild"] == 1], minlength=n)
    inner_hits = np.bincount(inn["c"][inn["isChild"] == 0], minlength=n - 1)
    assert (leaf_hits == 1).all() and inner_hits[0] == 0 and (inner_hits[1:] == 1).all()
    ob = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    assert_build_equal(ref, ob, n)
    rays = W.closest_rays(50000, seed=3)
    oids, ots = oracle.trace_closest(vx, vy, vz, None, ob, rays)
    for ordered in (False, True):
        ids, ts = lbvh.trace_closest(bvh, torch.from_numpy(rays).to(cuda), ordered=ordered)
        np.testing.assert_array_equal(ids.cpu().numpy().view(np.uint32), oids)
        np.testing.assert_array_equal(ts.cpu().numpy(), ots)
    # the two device searches agree on a million more rays
    big = torch.from_numpy(W.closest_rays(1 << 20, seed=4)).to(cuda)
    a_id, a_t = lbvh.trace_closest(bvh, big, ordered=False)
    b_id, b_t = lbvh.trace_closest(bvh, big, ordered=True)
    assert torch.equal(a_id, b_id) and torch.equal(a_t, b_t)
    no_device_errors()

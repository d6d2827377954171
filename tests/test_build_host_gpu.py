"""Builds from host arrays (clr_lbvh_build_host): the upload-and-build entry a
reference host uses in place of creating its vertex and face buffers from
host memory and calling LBVHBuilder::perform.

Its trees must be bit-identical to clr_lbvh_build on the same data (itself
pinned to the oracle), including across a pipelined run where each call's
copy overlaps the previous call's build and the two device input buffers are
reused in turn.
"""
import numpy as np
import pytest
import torch

import oracle
from clear_gb300 import _lib, lbvh
from clear_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def device_build(cuda, vx, vy, vz, tri, n, bits):
    b = lbvh.LBVHBuilder(max(n, 1), cuda)
    v = tuple(torch.from_numpy(np.asarray(a)).to(cuda) for a in (vx, vy, vz))
    t = None if tri is None else torch.from_numpy(np.asarray(tri, dtype=np.int32)).to(cuda)
    bvh = b.perform(v, t, n, bits)
    torch.cuda.synchronize()
    return bvh


def pinned(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dtype).pin_memory()


def assert_same_tree(a: lbvh.BVH, b: lbvh.BVH):
    assert a.num_tris == b.num_tris
    n = a.num_tris
    assert torch.equal(a.tris.view(torch.int32), b.tris.view(torch.int32))
    assert torch.equal(a.root_box.view(torch.int32), b.root_box.view(torch.int32))
    if n > 1:
        assert torch.equal(a.nodes.view(torch.int32)[: (n - 1) * 16], b.nodes.view(torch.int32)[: (n - 1) * 16])


@pytest.mark.parametrize("n", [1, 2, 65, 4097, 300001])
def test_host_build_equals_device_build(cuda, n):
    vx, vy, vz = W.triangle_soup(n, seed=77 + n)
    ref = device_build(cuda, vx, vy, vz, None, n, 10)
    b = lbvh.LBVHBuilder(n, cuda)
    root = torch.zeros(8, dtype=torch.float32).pin_memory()
    got = b.perform_host(tuple(pinned(a) for a in (vx, vy, vz)), None, n, 10, root_host=root)
    torch.cuda.synchronize()
    assert_same_tree(got, ref)
    assert torch.equal(root.view(torch.int32), ref.root_box.cpu().view(torch.int32))
    assert _lib.device_status(clear=True) == 0


def test_host_build_indexed_matches_oracle(cuda):
    rng = np.random.default_rng(11)
    nv, n = 5000, 12000
    vx, vy, vz = (rng.random(nv).astype(np.float32) for _ in range(3))
    tri = rng.integers(0, nv, size=(n, 3)).astype(np.int32)
    ref = device_build(cuda, vx, vy, vz, tri, n, 10)
    b = lbvh.LBVHBuilder(n, cuda)
    got = b.perform_host(tuple(pinned(a) for a in (vx, vy, vz)), pinned(tri, torch.int32), n, 10)
    torch.cuda.synchronize()
    assert_same_tree(got, ref)
    ob = oracle.lbvh_build(vx, vy, vz, tri.astype(np.uint32).reshape(-1), n, 10)
    rb = got.root_box.cpu().numpy()
    assert (rb[:3] == ob.scene_box[:3]).all() and (rb[4:7] == ob.scene_box[3:]).all()


def test_pipelined_stream_of_builds(cuda):
    """Seven calls over three inputs of different sizes with no host
    synchronisation between them: every copy overlaps the previous build and
    each input buffer is refilled while the other is being read.  Every tree
    equals the device build of its own input."""
    inputs = []
    for k, n in enumerate([50000, 3001, 120000]):
        vx, vy, vz = W.triangle_soup(n, seed=500 + k)
        inputs.append((n, tuple(pinned(a) for a in (vx, vy, vz)), device_build(cuda, vx, vy, vz, None, n, 10)))
    b = lbvh.LBVHBuilder(1000, cuda)  # grows on demand
    order = [0, 1, 2, 0, 2, 1, 0]
    outs = [b.perform_host(inputs[i][1], None, inputs[i][0], 10) for i in order]
    torch.cuda.synchronize()
    for i, got in zip(order, outs):
        assert_same_tree(got, inputs[i][2])
    b.host_copy_wait()
    assert _lib.device_status(clear=True) == 0


def test_copy_after_orders_copies_behind_stream(cuda):
    n = 20000
    vx, vy, vz = W.triangle_soup(n, seed=9)
    ref = device_build(cuda, vx, vy, vz, None, n, 10)
    b = lbvh.LBVHBuilder(n, cuda)
    torch.cuda._sleep(10_000_000)  # queue work on the stream ahead of the copies
    b.host_copy_after_stream()
    got = b.perform_host(tuple(pinned(a) for a in (vx, vy, vz)), None, n, 10)
    torch.cuda.synchronize()
    assert_same_tree(got, ref)


def test_host_build_empty_and_invalid(cuda):
    b = lbvh.LBVHBuilder(16, cuda)
    e = torch.zeros(0, dtype=torch.float32)
    bvh = b.perform_host((e, e, e), None, 0, 10)
    assert bvh.num_tris == 0
    vx, vy, vz = (pinned(a) for a in W.triangle_soup(8, seed=3))
    with pytest.raises(_lib.ClrError):  # a soup of 8 triangles has 24 vertices, not 24 - 3
        b.perform_host((vx[:-3].contiguous(), vy[:-3].contiguous(), vz[:-3].contiguous()), None, 8, 10)
    with pytest.raises(_lib.ClrError):
        b.perform_host((vx, vy, vz), None, 8, 0)
    with pytest.raises(ValueError):
        b.perform_host((vx.to(cuda), vy, vz), None, 8, 10)

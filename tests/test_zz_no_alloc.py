"""The allocation-free build entry point, called through the C ABI.

clr_lbvh_build_noalloc is for callers that may not allocate device memory
(hosts that own a fixed device-memory budget, per-frame loops that cannot
afford cudaMalloc's synchronisation).  It must give exactly the output of
clr_lbvh_build -- the parity bar of every build test here is bit-exact --
and keep doing so on back-to-back calls that reuse its shared scratch array.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from clear_gb300 import _lib, lbvh
from clear_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc_build(dev, verts, n, bits):
    out = lbvh.BVH(n, dev)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ptr = [C.c_void_p(v.data_ptr()) for v in verts]
    _lib.call("clr_lbvh_build_noalloc", *ptr, None, C.c_uint32(n), C.c_uint32(bits), C.byref(out.c), stream)
    return out


def _same(a: lbvh.BVH, b: lbvh.BVH):
    torch.cuda.synchronize()
    n = a.num_tris
    assert torch.equal(a.tris[: 48 * n], b.tris[: 48 * n])
    if n > 1:
        assert torch.equal(a.nodes[: 64 * (n - 1)], b.nodes[: 64 * (n - 1)])
    assert torch.equal(a.root_box, b.root_box)


@pytest.mark.parametrize("bits", [10, 21])
def test_noalloc_matches_allocating_build_twice(cuda, bits):
    """32-bit keys (10 bits per axis) and 64-bit keys (21 bits per axis, eight
    sort passes, the most look-back words): first a large input, then a
    smaller one, so stale scratch from the first call would show up if
    anything were not cleared."""
    builder = lbvh.LBVHBuilder(1, cuda)
    for n, seed in ((200000, 31), (4097, 32)):
        vx, vy, vz = W.triangle_soup(n, seed=seed)
        verts = [torch.from_numpy(a).to(cuda) for a in (vx, vy, vz)]
        ref = builder.perform(verts, None, n, bits)
        got = _noalloc_build(cuda, verts, n, bits)
        _same(ref, got)
    assert _lib.device_status() == 0


@pytest.mark.parametrize("bits", [10, 21])
@pytest.mark.parametrize("n", [1, 2, 1 << 18])
def test_noalloc_edge_sizes(cuda, bits, n):
    """One triangle (no internal node), two (a single internal node) and the
    largest count the fixed array takes, each called twice in a row."""
    builder = lbvh.LBVHBuilder(1, cuda)
    vx, vy, vz = W.triangle_soup(n, seed=40 + n % 7)
    verts = [torch.from_numpy(a).to(cuda) for a in (vx, vy, vz)]
    ref = builder.perform(verts, None, n, bits)
    for _ in range(2):
        _same(ref, _noalloc_build(cuda, verts, n, bits))
    assert _lib.device_status() == 0


def test_noalloc_rejects_oversized_input(cuda):
    n = (1 << 18) + 1
    e = torch.zeros(3, dtype=torch.float32, device=cuda)
    out = lbvh.BVH(1, cuda)
    rc = _lib.lib().clr_lbvh_build_noalloc(C.c_void_p(e.data_ptr()), C.c_void_p(e.data_ptr()),
                                           C.c_void_p(e.data_ptr()), None, C.c_uint32(n), C.c_uint32(10),
                                           C.byref(out.c), None)
    assert rc == 6  # CLR_ECAPACITY
    assert b"262144" in _lib.lib().clr_last_error_string()

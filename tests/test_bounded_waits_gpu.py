"""Bounded waits that run out, on the GPU, without a fault or a hang.

Two places wait on work that another block or another iteration must
finish: the radix sort's decoupled look-back (a tile waits for its
predecessors' digit counts) and the batched renderer's frame loop (it runs
while paths remain).  Both waits are bounded; when a bound runs out the
kernel raises a device error bit and returns, and the context stays usable.
These tests make each bound run out on purpose -- a predecessor tile that
never publishes, an iteration bound of one -- read the error bit, and check
that the next normal call gives the right result.  (The reference has no
such bounds; its host only catches cl::Error, main.cpp:546-551.)
"""
import ctypes as C

import numpy as np
import pytest
import torch

from clear_gb300 import _lib, lbvh
from clear_gb300 import workloads as W
from clear_gb300.batch import BatchRenderer, PerSceneLoop, random_scene

import oracle

pytestmark = pytest.mark.gpu

TILE = 4096


def _limits(sort_spins: int, iterations: int) -> None:
    _lib.call("clr_debug_set_wait_limits", C.c_uint32(sort_spins), C.c_uint32(iterations))


def test_sort_lookback_runs_out_and_reports(cuda):
    _lib.device_status()  # start clean
    keys = torch.from_numpy(np.random.default_rng(3).integers(0, 1 << 30, 2 * TILE, dtype=np.uint32).view(np.int32))
    keys = keys.to(cuda)
    scratch = torch.zeros(4 * TILE + 769, dtype=torch.int32, device=cuda)
    _limits(1000, 0)
    try:
        _lib.call("clr_debug_lookback_stall", C.c_void_p(keys.data_ptr()), C.c_void_p(scratch.data_ptr()),
                  C.c_uint32(TILE), C.c_void_p(torch.cuda.current_stream(cuda).cuda_stream))
        torch.cuda.synchronize()  # the kernel returned
        bits = _lib.device_status()
    finally:
        _limits(0, 0)
    assert bits & _lib.DEVERR_SORT_TIMEOUT
    # the context is usable and a normal build is exact again
    n = 100_000
    vx, vy, vz = W.triangle_soup(n, seed=5)
    b = lbvh.LBVHBuilder(n, cuda)
    bvh = b.perform(tuple(torch.from_numpy(a).to(cuda) for a in (vx, vy, vz)), None, n, 10)
    ref = b.export_reference(bvh)
    torch.cuda.synchronize()
    ob = oracle.lbvh_build(vx, vy, vz, None, n, 10)
    assert (ref["sorted_idx"].cpu().numpy().view(np.uint32) == ob.sorted_idx).all()
    assert _lib.device_status() == 0


@pytest.mark.parametrize("graph", [False, True])
def test_batched_frame_loop_bound_runs_out_and_reports(cuda, graph):
    scenes = [random_scene(n, w, h, seed) for n, w, h, seed in ((300, 24, 24, 1), (900, 32, 32, 2))]
    loop = PerSceneLoop(scenes, cuda)
    rngs, pixs = loop.new_frame()
    loop.render(rngs, pixs, 2, 5)
    torch.cuda.synchronize()
    ref = torch.cat(pixs)
    _lib.device_status()
    br = BatchRenderer(scenes, cuda)
    _limits(0, 1)
    try:
        rng, pix = br.new_frame()
        br.render(rng, pix, 2, 5, graph=graph)
        torch.cuda.synchronize()
        bits = _lib.device_status()
    finally:
        _limits(0, 0)
    assert bits & _lib.DEVERR_QUEUE
    rng, pix = br.new_frame()
    br.render(rng, pix, 2, 5, graph=graph)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    assert torch.equal(pix, ref)
    br.close()

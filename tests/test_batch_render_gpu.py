"""Batched wavefront: every scene's image and final random states are
bit-identical to the per-scene wavefront render, with and without the CUDA
graph, with a slot pool smaller than the pixels (pixel succession) and with
different block sizes."""
import numpy as np
import pytest
import torch

from clear_gb300 import _lib
from clear_gb300.batch import BatchRenderer, PerSceneLoop, batch_workload, random_scene

SPP = 2
DEPTH = 5


def _scenes():
    wl = [(200, 32, 32, 1), (1500, 48, 48, 2), (3000, 64, 64, 3), (17, 16, 16, 4), (5000, 40, 40, 5),
          (800, 64, 64, 6), (2500, 24, 24, 7)]
    return [random_scene(n, w, h, seed) for n, w, h, seed in wl]


@pytest.fixture(scope="module")
def reference(cuda):
    scenes = _scenes()
    loop = PerSceneLoop(scenes, cuda)
    rngs, pixs = loop.new_frame()
    loop.render(rngs, pixs, SPP, DEPTH)
    torch.cuda.synchronize()
    return scenes, torch.cat(pixs), torch.cat(rngs)


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("config", [{}, {"pool_slots": 1000, "trace_block": 64, "shade_block": 64},
                                    {"pool_slots": 4099, "trace_block": 256}])
def test_batched_render_equals_per_scene(cuda, reference, graph, config):
    scenes, ref_pix, ref_rng = reference
    br = BatchRenderer(scenes, cuda, config=config)
    rng, pix = br.new_frame()
    br.render(rng, pix, SPP, DEPTH, graph=graph)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    assert torch.equal(pix, ref_pix)
    assert torch.equal(rng, ref_rng)
    if graph:  # the captured graph is reused for a second frame
        rng2, pix2 = br.new_frame()
        br.render(rng2, pix2, SPP, DEPTH, graph=True)
        torch.cuda.synchronize()
        assert torch.equal(pix2, ref_pix)
    br.close()


@pytest.mark.gpu
def test_batched_build_feeds_the_same_trees(cuda, reference):
    scenes, _, _ = reference
    br = BatchRenderer(scenes, cuda)
    loop = PerSceneLoop(scenes, cuda)
    torch.cuda.synchronize()
    for s, d in enumerate(loop.ds):
        b = br.bvh.scene(s)
        n = d.num_faces
        assert torch.equal(b.root_box, d.bvh.root_box)
        assert torch.equal(b.tris, d.bvh.tris[:n * _lib.TRI_BYTES])
        assert torch.equal(b.nodes[:(n - 1) * _lib.NODE_BYTES], d.bvh.nodes[:(n - 1) * _lib.NODE_BYTES])


def test_batch_workload_distribution():
    wl = batch_workload(512, seed=7)
    n = np.array([w[0] for w in wl])
    assert len(wl) == 512 and n.min() >= 1000 and n.max() <= 200_000
    assert {w[1] for w in wl} <= {128, 256, 384, 512} and all(w[1] == w[2] for w in wl)
    # log-uniform: the median is near the geometric mean of the bounds
    assert 8000 < np.median(n) < 20000
    assert wl == batch_workload(512, seed=7)


def test_random_scene_is_deterministic():
    a, b = random_scene(300, 16, 16, 9).blobs(), random_scene(300, 16, 16, 9).blobs()
    for k in ("vertices", "faces", "materials", "textures", "others"):
        assert np.array_equal(a[k], b[k])

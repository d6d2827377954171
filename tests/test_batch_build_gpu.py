"""Segmented (batched) LBVH build: every scene's tree, triangle records and
root box are bit-identical to a standalone build of that scene, for every
radix width, soups and indexed meshes, scenes of 1, 2, 3 ... triangles and
scene counts that are not powers of two."""
import numpy as np
import pytest
import torch

from clear_gb300 import _lib, lbvh
from clear_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _soups(sizes, seed0=10):
    parts = [W.triangle_soup(n, seed=seed0 + i) for i, n in enumerate(sizes)]
    # scenes in different places and scales: each is quantised in its own box
    out = []
    for i, (x, y, z) in enumerate(parts):
        s = 1.0 + 0.5 * i
        out.append((x * s + 3.0 * i, y * s - i, z * s))
    vx = np.concatenate([p[0] for p in out])
    vy = np.concatenate([p[1] for p in out])
    vz = np.concatenate([p[2] for p in out])
    return vx, vy, vz, out


def _compare(cuda, bb, scenes, faces_of, bits):
    for s, (x, y, z) in enumerate(scenes):
        n = bb.offsets[s + 1] - bb.offsets[s]
        b = lbvh.LBVHBuilder(n, cuda)
        ref = b.perform(tuple(torch.from_numpy(a).to(cuda) for a in (x, y, z)), faces_of(s), n, bits)
        got = bb.scene(s)
        torch.cuda.synchronize()
        assert torch.equal(got.root_box, ref.root_box), s
        assert torch.equal(got.tris, ref.tris), s
        if n > 1:
            assert torch.equal(got.nodes[:(n - 1) * _lib.NODE_BYTES], ref.nodes[:(n - 1) * _lib.NODE_BYTES]), s


@pytest.mark.parametrize("radix_bits", [8, 7, 6])
def test_batched_build_equals_standalone(cuda, radix_bits):
    sizes = [1, 2, 3, 5, 64, 1000, 4097, 3, 20000, 777, 1]
    vx, vy, vz, scenes = _soups(sizes)
    offs = np.concatenate([[0], np.cumsum(sizes)]).tolist()
    b = lbvh.LBVHBuilder(sum(sizes), cuda)
    bb = b.perform_batched(tuple(torch.from_numpy(a).to(cuda) for a in (vx, vy, vz)), None, offs, 10, radix_bits)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    _compare(cuda, bb, scenes, lambda s: None, 10)


def test_batched_build_indexed_meshes_and_many_scenes(cuda):
    rng = np.random.default_rng(5)
    sizes = rng.integers(1, 400, size=300).tolist()
    vx, vy, vz, scenes = _soups(sizes, seed0=100)
    # index the concatenated vertices through a permutation of each scene's own vertices
    faces, local, base = [], [], 0
    for n in sizes:
        perm = rng.permutation(3 * n).reshape(n, 3).astype(np.int64)
        local.append(perm)
        faces.append(perm + base)
        base += 3 * n
    faces = np.concatenate(faces)
    offs = np.concatenate([[0], np.cumsum(sizes)]).tolist()
    b = lbvh.LBVHBuilder(sum(sizes), cuda)
    bb = b.perform_batched(tuple(torch.from_numpy(a).to(cuda) for a in (vx, vy, vz)),
                           torch.from_numpy(faces).to(cuda), offs, 10, 8)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    _compare(cuda, bb, scenes, lambda s: torch.from_numpy(local[s]).to(cuda), 10)


def test_batched_build_rejects_bad_offsets(cuda):
    vx, vy, vz, _ = _soups([4, 4])
    b = lbvh.LBVHBuilder(8, cuda)
    v = tuple(torch.from_numpy(a).to(cuda) for a in (vx, vy, vz))
    with pytest.raises(_lib.ClrError):
        b.perform_batched(v, None, [0, 4, 4, 8], 10)  # empty scene
    with pytest.raises(_lib.ClrError):
        b.perform_batched(v, None, [1, 8], 10)
    with pytest.raises(_lib.ClrError):
        b.perform_batched(v, None, [0, 4, 8], 10, radix_bits=5)
